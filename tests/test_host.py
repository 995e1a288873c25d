"""Host-side logic of the product (no GPU): set-up numerics against the oracle,
and the C ABI library's exports."""
import ctypes
import os
import re

import numpy as np
import pytest

import sem_oracle as O
from semgb300 import _lib, host

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("n", range(2, 18))
def test_gll_and_derivmat_match_oracle(n):
    z, w = host.gausslobatto(n)
    zo, wo = O.gausslobatto(n)
    np.testing.assert_allclose(z, zo, rtol=0, atol=4e-16)
    np.testing.assert_allclose(w, wo, rtol=4e-16, atol=0)
    D, Do = host.derivMat(zo), O.derivMat(zo)
    np.testing.assert_allclose(D, Do, rtol=1e-13, atol=1e-13 * np.abs(Do).max())


def test_interp_semmesh_semq_bdf():
    xi, _ = O.gausslobatto(7)
    xo = np.linspace(-1, 1, 11)
    np.testing.assert_allclose(host.interpMat(xo, xi), O.interpMat(xo, xi), rtol=1e-13, atol=1e-14)
    for E, n in ((3, 4), (5, 9)):
        z, w = host.semmesh(E, n)
        zo, wo = O.semmesh(E, n)
        np.testing.assert_allclose(z, zo, rtol=0, atol=1e-15)
        np.testing.assert_allclose(w, wo, rtol=1e-15)
        for per in (False, True):
            g, ng = host.semq_index(E, n, per)
            go, ngo = O.semq_index(E, n, per)
            np.testing.assert_array_equal(g, go)
            assert ng == ngo
    for t, k in (([0.0] * 4, 3), ([0.1, 0.0], 1), ([0.3, 0.2, 0.1, 0.0], 3), ([0.2, 0.1, 0.0, 0.0], 3)):
        a, b = host.bdfExtK(t, k)
        ao, bo = O.bdfExtK(t, k)
        np.testing.assert_allclose(a, ao, rtol=1e-13)
        np.testing.assert_allclose(b, bo, rtol=1e-13)


def _header_functions():
    src = open(os.path.join(ROOT, "include", "sem_b200.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sem_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def built():
    _lib.build()
    return _lib.load()


def test_library_exports_every_declared_symbol(built):
    lib = built
    names = _header_functions()
    assert "sem_pcg" in names and "sem_lapl" in names
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)
    assert lib.sem_abi_version() == 1


def test_header_constants_match_binding():
    src = open(os.path.join(ROOT, "include", "sem_b200.h")).read()
    defines = dict(re.findall(r"#define\s+(SEM_[A-Z_]+)\s+(\d+)", src))
    assert int(defines["SEM_VARIANTS"]) == _lib.SEM_VARIANTS
    assert int(defines["SEM_BDF_MAX_ORDER"]) == _lib.SEM_BDF_MAX_ORDER
    assert int(defines["SEM_NOALLOC_MAX_LOCAL"]) > 0


def test_argument_validation_needs_no_gpu(built):
    lib = built
    h = ctypes.c_void_p()
    assert lib.sem_mesh_create(None, ctypes.byref(h)) == _lib.SEM_ERR_BAD_ARG
    assert b"NULL" in lib.sem_last_error()
    d = _lib.MeshDesc()
    d.nr, d.ns, d.Ex, d.Ey = 9, 7, 2, 2
    assert lib.sem_mesh_create(ctypes.byref(d), ctypes.byref(h)) == _lib.SEM_ERR_UNSUPPORTED
    d.nr, d.ns = 1, 1
    assert lib.sem_mesh_create(ctypes.byref(d), ctypes.byref(h)) == _lib.SEM_ERR_BAD_ARG
    assert lib.sem_mask(None, None, None, -1, None) == _lib.SEM_ERR_BAD_ARG
    a = np.zeros(4)
    assert lib.sem_abu(None, 0, 0, None, 0, 0, a.ctypes.data, 2, 2, a.ctypes.data, None) == _lib.SEM_ERR_BAD_ARG
    # ABu sizes are checked before any launch: empty factors, length(u) not a
    # multiple of size(Br,2), size(u,2) not a multiple of size(As,2); factors
    # of any size are otherwise accepted (no 32 x 32 limit)
    u, v = np.zeros(66 * 66), np.zeros(66 * 66)
    big = np.eye(40)
    assert lib.sem_abu(None, 0, 0, big.ctypes.data, 0, 40, u.ctypes.data, 66, 66, v.ctypes.data,
                       None) == _lib.SEM_ERR_BAD_ARG
    assert lib.sem_abu(None, 0, 0, big.ctypes.data, 40, 40, u.ctypes.data, 66, 66, v.ctypes.data,
                       None) == _lib.SEM_ERR_BAD_ARG
    assert b"multiple" in lib.sem_last_error()
    assert lib.sem_abu(big.ctypes.data, 40, 40, None, 0, 0, u.ctypes.data, 66, 66, v.ctypes.data,
                       None) == _lib.SEM_ERR_BAD_ARG


def test_bdf_coeffs_in_library_match_oracle(built):
    """sem_bdf_coeffs (host code of the library) against the oracle's
    bdfExtK (src/time.jl:31-53), including the steady branch and the
    zero-padded first steps of BDF3."""
    lib = built
    dt = 1e-3
    cases = [([0.0] * 4, 3), ([dt, 0.0, 0.0, 0.0], 3), ([2 * dt, dt, 0.0, 0.0], 3),
             ([3 * dt, 2 * dt, dt, 0.0], 3), ([0.1, 0.0], 1), ([0.5, 0.4, 0.25], 2),
             ([0.7, 0.6, 0.45, 0.3, 0.2, 0.1, 0.0], 6)]
    t = 0.0
    hist = [0.0] * 4
    for _ in range(5):  # the additions of TimeStepper.advance
        hist = [hist[0]] + hist[:-1]
        t += dt
        hist[0] = t
        cases.append((list(hist), 3))
    for tt, k in cases:
        a = (ctypes.c_double * k)()
        b = (ctypes.c_double * (k + 1))()
        assert lib.sem_bdf_coeffs(k, (ctypes.c_double * (k + 1))(*tt), a, b) == _lib.SEM_OK
        ao, bo = O.bdfExtK(tt, k)
        np.testing.assert_allclose(np.array(a[:]), ao, rtol=1e-15, atol=0)
        np.testing.assert_allclose(np.array(b[:]), bo, rtol=1e-15, atol=0)
    z = (ctypes.c_double * 8)()
    assert lib.sem_bdf_coeffs(0, z, z, z) == _lib.SEM_ERR_BAD_ARG
    assert lib.sem_bdf_coeffs(_lib.SEM_BDF_MAX_ORDER + 1, z, z, z) == _lib.SEM_ERR_BAD_ARG
    d = _lib.BdfDesc()
    assert lib.sem_bdf_run(None, ctypes.byref(d), z, None, None, None, None) == _lib.SEM_ERR_BAD_ARG


def test_product_has_no_oracle_imports():
    pkg = os.path.join(ROOT, "spectralelements.jl_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".jl")):
                txt = open(os.path.join(dirpath, f)).read()
                assert "sem_oracle" not in txt and "oracle/" not in txt, f


def test_simulate_step_count_follows_the_reference_loop():
    """Diffusion.simulate() without closures runs the number of steps the
    reference's while loop would (src/diffusion.jl:130-137), computed with the
    same additions as TimeStepper.advance."""
    from semgb300.solver import simulate_steps

    def loop(t0, dt, Tf):
        t, n = t0, 0
        while t <= Tf:
            t += dt
            n += 1
            if t < 1e-12:
                break
        return n
    for t0, dt, Tf in ((0.0, 1e-3, 0.2), (0.0, 2e-3, 2e-2), (0.0, 0.1, 0.3), (0.5, 0.25, 1.0), (0.0, 0.0, 0.0),
                       (0.0, 1e-3, 0.0), (1.0, 0.1, 0.5)):
        assert simulate_steps(t0, dt, Tf) == loop(t0, dt, Tf)
    assert simulate_steps(0.0, 0.0, 1.0) == 1  # steady: one step, then time < 1e-12 ends the loop
    with pytest.raises(ValueError):
        simulate_steps(0.5, 0.0, 1.0)  # the reference would never leave its loop


def test_julia_binding_matches_the_header():
    """SEMB200.jl (not executable here) against include/sem_b200.h: every
    ccall names a declared entry point, and the Julia and ctypes mirrors of
    the C structs have the C field names, in order."""
    jl = open(os.path.join(ROOT, "spectralelements.jl_gb300", "julia", "SEMB200.jl")).read()
    hdr = open(os.path.join(ROOT, "include", "sem_b200.h")).read()
    declared = set(_header_functions())
    called = set(re.findall(r"ccall\(\(:(sem_[a-z0-9_]+),", jl))
    assert called and called <= declared, called - declared
    hdr_nc = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)

    def c_fields(tag):
        end = re.search(r"\}\s*" + tag + r"\s*;", hdr_nc).start()
        start = hdr_nc.rfind("typedef struct {", 0, end) + len("typedef struct {")
        names = []
        for decl in hdr_nc[start:end].split(";"):
            decl = decl.strip()
            if not decl:
                continue
            # "const double* const* F" -> F; "int nr, ns, Ex, Ey" -> nr, ns, Ex, Ey
            head, _, rest = decl.partition(",")
            names.append(re.findall(r"\w+", head)[-1])
            names += [re.findall(r"\w+", n)[-1] for n in rest.split(",") if rest]
        return names

    def jl_fields(name):
        body = re.search(r"\nstruct " + name + r"\n(.*?)\nend", jl, flags=re.S).group(1)
        return re.findall(r"(\w+)::", body)
    for jl_name, c_name, py in (("PcgOpts", "sem_pcg_opts", _lib.PcgOpts),
                                ("SolveInfo", "sem_solve_info", _lib.SolveInfo),
                                ("BdfDesc", "sem_bdf_desc", _lib.BdfDesc),
                                ("MeshDesc", "sem_mesh_desc", _lib.MeshDesc)):
        assert jl_fields(jl_name) == c_fields(c_name), jl_name
        assert [f[0] for f in py._fields_] == c_fields(c_name), c_name  # the ctypes mirror too

    # every ccall passes as many argument types as the C declaration has parameters
    decl_arity = {}
    for name, params in re.findall(r"\b(sem_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", hdr_nc):
        params = params.strip()
        decl_arity[name] = 0 if params in ("", "void") else params.count(",") + 1

    def top_level_items(text):
        depth, items, cur = 0, 0, ""
        for ch in text:
            if ch in "({[":
                depth += 1
            elif ch in ")}]":
                depth -= 1
            if ch == "," and depth == 0:
                items += 1
                cur = ""
            else:
                cur += ch
        return items + (1 if cur.strip() else 0)

    for m in re.finditer(r"ccall\(\(:(sem_[a-z0-9_]+), libsem\),\s*\w+,\s*\(", jl):
        i, depth = m.end(), 1
        while depth:
            depth += {"(": 1, ")": -1}.get(jl[i], 0)
            i += 1
        types = jl[m.end():i - 1]
        assert top_level_items(types) == decl_arity[m.group(1)], (m.group(1), types)

    # the Julia methods the drop-in boundary names (functional forms, linsolve + rrule)
    for pattern in (r"function lapl\(u::CuArray\{Float64,2\}, M, Jr, Js, QQtx, QQty, Dr::AbstractMatrix, "
                    r"Ds::AbstractMatrix,\s*G11::CuArray\{Float64,2\}, G12::CuArray\{Float64,2\}, "
                    r"G22::CuArray\{Float64,2\}, mult",
                    r"function mass\(u::CuArray\{Float64,2\}, M, B, Jr, Js, QQtx, QQty, mult\)",
                    r"function gatherScatter\(u::CuArray\{Float64,2\}, QQtx::AbstractMatrix, QQty::AbstractMatrix\)",
                    r"function linsolve\(a::CuArray\{Float64,2\}, problem::VarCoefProblem, solver::PcgSolver\)",
                    r"ChainRulesCore\.rrule\(config::ChainRulesCore\.RuleConfig\{>:ChainRulesCore\.HasReverseMode\},"
                    r"\s*::typeof\(linsolve\)",
                    r"ChainRulesCore\.rrule\(::typeof\(lapl\)", r"ChainRulesCore\.rrule\(::typeof\(mass\)",
                    r"ChainRulesCore\.rrule\(::typeof\(varcoef_solve\)"):
        assert re.search(pattern, jl), pattern
