"""PCG on the device against the oracle's restatement of src/pcg.jl:16-60.

The reference loop is reproduced exactly (absolute Inf-norm tolerance,
zero initial guess, mult-weighted dots, maxiter = length(b)); iteration
counts agree to within 2 (summation order changes the last digits of the
dot products), solutions agree to the solver tolerance.
"""
import numpy as np
import pytest

import sem_oracle as O
from _helpers import host, meshes, rel_l2

pytestmark = pytest.mark.gpu


def _poisson_rhs(mo, M):
    ut = np.sin(np.pi * mo.x) * np.sin(np.pi * mo.y)
    f = 2 * np.pi ** 2 * ut
    return ut, O.gatherScatter(O.mask(O.mass(f, mo), M), mo)


@pytest.mark.parametrize("prec,variant", [("F64", 0), ("DF", 0), ("DF", 5)])
def test_poisson_cfg1_jacobi(gpu, prec, variant):
    import semgb300 as S
    mo, md = meshes(9, 8, 8, (False, False), "DDDD", 0.1,
                    precision=S.SEM_F64 if prec == "F64" else S.SEM_F64_DF)
    md.set_variant(variant)
    M = O.generateMask(["D"] * 4, mo)
    ut, b = _poisson_rhs(mo, M)
    tol = 1e-10 * np.abs(b).max()
    d = O.jacobi_diag(mo, 1.0, 0.0, M)
    info_o = {}
    x_o = O.pcg(b, lambda v: O.mask(O.gatherScatter(O.lapl(v, mo), mo), M), opM=lambda r: r / d,
                mult=mo.mult, tol=tol, info=info_o)
    op = S.HelmholtzOp(md, 1.0, 0.0)
    jac = S.Jacobi(op)
    np.testing.assert_allclose(host(jac.diag()), d, rtol=1e-13)
    info = {}
    x = host(S.pcg(S.as_local(b), op, opM=jac, mult=md.mult, tol=tol, info=info))
    assert info["converged"] and abs(info["iters"] - info_o["iters"]) <= 2, (info, info_o)
    assert np.abs(x - x_o).max() < 1e-10
    assert np.abs(x - ut).max() < 1e-8
    assert info["res_inf"] <= tol


def test_helmholtz_cfg2_shape_vs_c_oracle(gpu):
    """nu=1e-2, lambda=1 Helmholtz, Jacobi PCG to 1e-8 relative on 32x32, N=8."""
    import sem_oracle_c as C
    import semgb300 as S
    mo, md = meshes(9, 32, 32, (False, False), "DDDD", 0.05)
    M = O.generateMask(["D"] * 4, mo)
    rng = np.random.default_rng(2)
    f = np.zeros(mo.shape)
    for _ in range(16):
        kx, ky = rng.integers(1, 9, size=2)
        f += rng.standard_normal() / (kx ** 2 + ky ** 2) * np.sin(kx * np.pi * mo.x) * np.sin(ky * np.pi * mo.y)
    b = O.gatherScatter(O.mask(O.mass(f, mo), M), mo)
    tol = 1e-8 * np.abs(b).max()
    d = O.jacobi_diag(mo, 1e-2, 1.0, M)
    g = C.grid(9, 32, 32, (False, False), "DDDD")
    x_c, it_c, res_c = C.pcg(g, mo.Dr, mo.Ds, mo.G11, mo.G12, mo.G22, mo.B, b, nu=1e-2, k=1.0, d=d, tol=tol)
    op = S.HelmholtzOp(md, 1e-2, 1.0)
    info = {}
    x = host(S.pcg(S.as_local(b), op, opM=S.Jacobi(op), mult=md.mult, tol=tol, info=info))
    assert info["converged"] and abs(info["iters"] - it_c) <= 2, (info, it_c)
    assert rel_l2(x, x_c) < 1e-8
    # mixed precision reaches the same tolerance; error against the FP64 solution stated
    info_m = {}
    xm = host(S.pcg(S.as_local(b), op, opM=S.Jacobi(op), mult=md.mult, tol=tol, info=info_m,
                    precision=S.SEM_MIXED))
    assert info_m["converged"] and info_m["outer"] <= 6, info_m
    assert info_m["res_inf"] <= tol
    assert rel_l2(xm, x_c) < 1e-7
    # residual replacement: one FP32 CG, FP64 residual swapped in every time the
    # FP32 residual has fallen by 0.3; the iteration count stays near FP64 CG's
    info_r = {}
    xr = host(S.pcg(S.as_local(b), op, opM=S.Jacobi(op), mult=md.mult, tol=tol, info=info_r,
                    precision=S.SEM_MIXED_RR))
    assert info_r["converged"] and info_r["res_inf"] <= tol, info_r
    assert info_r["outer"] >= 2 and info_r["iters"] <= 1.5 * it_c, (info_r, it_c)
    assert rel_l2(xr, x_c) < 1e-7


@pytest.mark.parametrize("path,variant", [(0, 0), (1, 0), (1, 2), (1, 5), (2, 0)])
def test_unweighted_default_and_identity_precond(gpu, path, variant):
    """pcg's default mult = ones (unweighted dots) and opM = identity, on every
    solver path: the small-mesh launch, the chunked launches, and the chunked
    launches with the CG-fused kernel variants (which must not use their
    unassembled p.Ap for unweighted dots)."""
    import semgb300 as S
    mo, md = meshes(5, 4, 3, (False, False), "DDDD", 0.05)
    md.set_variant(variant)
    M = O.generateMask(["D"] * 4, mo)
    ut, b = _poisson_rhs(mo, M)
    info_o = {}
    x_o = O.pcg(b, lambda v: O.mask(O.gatherScatter(O.hlmz(v, 0.5, 2.0, mo), mo), M), tol=1e-9,
                info=info_o)
    op = S.HelmholtzOp(md, 0.5, 2.0)
    info = {}
    x = host(S.pcg(S.as_local(b), op, tol=1e-9, info=info, path=path))
    assert abs(info["iters"] - info_o["iters"]) <= 2
    assert np.abs(x - x_o).max() < 1e-8


def test_maxiter_warns_and_returns_x(gpu, capsys):
    import semgb300 as S
    mo, md = meshes(9, 8, 8, (False, False), "DDDD", 0.1)
    M = O.generateMask(["D"] * 4, mo)
    _, b = _poisson_rhs(mo, M)
    info_o = {}
    x_o = O.pcg(b, lambda v: O.mask(O.gatherScatter(O.lapl(v, mo), mo), M), mult=mo.mult,
                tol=1e-30, maxiter=7, info=info_o)
    op = S.HelmholtzOp(md, 1.0, 0.0)
    info = {}
    x = host(S.pcg(S.as_local(b), op, mult=md.mult, tol=1e-30, maxiter=7, info=info))
    assert "warning: res:" in capsys.readouterr().out
    assert info["iters"] == 7 and not info["converged"]
    assert rel_l2(x, x_o) < 1e-12
    # pcg! writes into x
    y = md.empty()
    S.pcg_(y, S.as_local(b), op, mult=md.mult, tol=1e-30, maxiter=7)
    assert rel_l2(host(y), x_o) < 1e-12


def test_nan_is_reported(gpu):
    import semgb300 as S
    mo, md = meshes(5, 3, 3)
    b = np.ones(mo.shape)
    b[4, 4] = np.nan
    op = S.HelmholtzOp(md, 1.0, 1.0)
    with pytest.raises(S.SemError) as e:
        S.pcg(S.as_local(b), op, mult=md.mult)
    assert e.value.status == 3


def test_zero_rhs_returns_zero(gpu):
    import semgb300 as S
    mo, md = meshes(5, 3, 3)
    op = S.HelmholtzOp(md, 1.0, 1.0)
    info = {}
    x = host(S.pcg(S.as_local(np.zeros(mo.shape)), op, mult=md.mult, info=info))
    assert info["iters"] == 0 and not x.any()


def test_rejects_host_closures(gpu):
    import semgb300 as S
    mo, md = meshes(5, 3, 3)
    with pytest.raises(TypeError):
        S.pcg(S.as_local(np.ones(mo.shape)), lambda v: v)


@pytest.mark.parametrize("precision", ["DF", "MIXED"])
def test_graph_replay_matches_direct_launches(gpu, precision):
    """The CG iteration chunks replay as CUDA graphs; with kernel timing on they
    are launched one by one.  Both give bit-identical solves, and a second
    solve into a different x buffer (re-captured graph) matches the first."""
    import semgb300 as S
    mo, md = meshes(9, 8, 8, (False, False), "DDDD", 0.1)
    M = O.generateMask(["D"] * 4, mo)
    _, b = _poisson_rhs(mo, M)
    bd = S.as_local(b)
    op = S.HelmholtzOp(md, 1.0, 0.0)
    prec = S.SEM_F64_DF if precision == "DF" else S.SEM_MIXED
    tol = 1e-10 * np.abs(b).max()
    runs = []
    lib = S.load()
    for timing in (0, 1, 0):
        lib.sem_timing_enable(timing)
        try:
            info = {}
            x = host(S.pcg(bd, op, opM=S.Jacobi(op), mult=md.mult, tol=tol, info=info, precision=prec,
                           path=S.SEM_PATH_CHUNKED))
        finally:
            lib.sem_timing_enable(0)
            lib.sem_timing_read(None, None)
        runs.append((x, info["iters"]))
    for x, it in runs[1:]:
        assert it == runs[0][1]
        np.testing.assert_array_equal(x, runs[0][0])
    # pcg! into a fixed buffer twice: same graph replayed
    y = md.empty()
    S.pcg_(y, bd, op, opM=S.Jacobi(op), mult=md.mult, tol=tol, precision=prec, path=S.SEM_PATH_CHUNKED)
    y1 = host(y).copy()
    y.zero_()
    S.pcg_(y, bd, op, opM=S.Jacobi(op), mult=md.mult, tol=tol, precision=prec, path=S.SEM_PATH_CHUNKED)
    np.testing.assert_array_equal(host(y), y1)
    np.testing.assert_array_equal(y1, runs[0][0])


@pytest.mark.parametrize("case", [
    (9, 8, 8, (False, False), "DDDD", 0.1, 1.0, 0.0),
    (5, 7, 3, (True, False), "NNDD", 0.05, 0.5, 2.0),
    (7, 3, 5, (False, True), "DDNN", 0.05, 1.0, 1.0),
    (4, 6, 6, (True, True), "NNNN", 0.0, 1.0, 3.0),
    (11, 4, 3, (False, False), "DNDN", 0.05, 0.2, 0.0),
    (2, 20, 9, (False, False), "DDDD", 0.05, 1.0, 0.5),
])
@pytest.mark.parametrize("precision", ["DF", "MIXED", "MIXED_RR"])
def test_small_path_matches_chunked_and_oracle(gpu, case, precision):
    """The single-launch small-mesh solver against the chunked graph path and
    the oracle: same iterations within 1 %, solutions to the tolerance."""
    import semgb300 as S
    n, Ex, Ey, per, bc, amp, nu, lam = case
    mo, md = meshes(n, Ex, Ey, per, bc, amp)
    M = O.generateMask(list(bc), mo)
    rng = np.random.default_rng(n + Ex)
    b = O.mask(O.gatherScatter(mo.B * rng.standard_normal(mo.shape), mo), M)
    tol = 1e-10 * np.abs(b).max()
    op = S.HelmholtzOp(md, nu, lam)
    prec = getattr(S, "SEM_" + ("F64_DF" if precision == "DF" else precision))
    res = {}
    for path in (S.SEM_PATH_SMALL, S.SEM_PATH_CHUNKED):
        info = {}
        x = host(S.pcg(S.as_local(b), op, opM=S.Jacobi(op), mult=md.mult, tol=tol, info=info,
                       precision=prec, path=path))
        assert info["converged"] and info["res_inf"] <= tol, (path, info)
        res[path] = (x, info)
    xs, i_s = res[S.SEM_PATH_SMALL]
    xc, i_c = res[S.SEM_PATH_CHUNKED]
    if precision == "DF":
        assert abs(i_s["iters"] - i_c["iters"]) <= max(2, i_c["iters"] // 100), (i_s, i_c)
    assert rel_l2(xs, xc) < 1e-7
    # the oracle's residual of the small path's solution
    r = b - O.mask(O.gatherScatter(O.hlmz(xs, nu, lam, mo), mo), M)
    assert np.abs(r).max() <= 2 * tol
    # repeated solves give identical results
    x2 = host(S.pcg(S.as_local(b), op, opM=S.Jacobi(op), mult=md.mult, tol=tol, precision=prec,
                    path=S.SEM_PATH_SMALL))
    np.testing.assert_array_equal(x2, xs)


def test_small_path_options_and_limits(gpu):
    import semgb300 as S
    mo, md = meshes(9, 8, 8, (False, False), "DDDD", 0.1)
    M = O.generateMask(["D"] * 4, mo)
    _, b = _poisson_rhs(mo, M)
    op = S.HelmholtzOp(md, 1.0, 0.0)
    # unweighted dots, no preconditioner, maxiter reached
    info_o = {}
    x_o = O.pcg(b, lambda v: O.mask(O.gatherScatter(O.lapl(v, mo), mo), M), tol=1e-30, maxiter=9,
                info=info_o)
    info = {}
    x = host(S.pcg(S.as_local(b), op, tol=1e-30, maxiter=9, info=info, path=S.SEM_PATH_SMALL))
    assert info["iters"] == 9 and not info["converged"]
    assert rel_l2(x, x_o) < 1e-12
    # a nu field is not served by the small path
    with pytest.raises(S.SemError):
        opn = S.HelmholtzOp(md, 1.0, 0.0, nu_field=S.as_local(np.ones(mo.shape)))
        S.pcg(S.as_local(b), opn, opM=S.Jacobi(opn), mult=md.mult, path=S.SEM_PATH_SMALL)
    # nor a mesh above the size limit
    _, big = meshes(9, 40, 40)
    with pytest.raises(S.SemError):
        opb = S.HelmholtzOp(big, 1.0, 0.0)
        S.pcg(S.as_local(np.zeros(big.shape)), opb, mult=big.mult, path=S.SEM_PATH_SMALL)


@pytest.mark.parametrize("path", [0, 1])
@pytest.mark.parametrize("prec_name", ["SEM_MIXED", "SEM_MIXED_RR"])
def test_mixed_budget_exhausted_finishes_in_fp64(gpu, path, prec_name):
    """With one sweep / one replacement allowed, the mixed solve cannot reach
    the tolerance in FP32; the FP64 CG finishes it from the current x, on the
    single-launch small-mesh path and on the chunked path alike."""
    import semgb300 as S
    mo, md = meshes(9, 8, 8, (False, False), "DDDD", 0.1)
    M = O.generateMask(["D"] * 4, mo)
    b = O.gatherScatter(O.mask(O.mass(2 * np.pi ** 2 * np.sin(np.pi * mo.x) * np.sin(np.pi * mo.y), mo), M), mo)
    tol = 1e-11 * np.abs(b).max()
    op = S.HelmholtzOp(md, 1.0, 0.0)
    info, info64 = {}, {}
    x = S.pcg(S.as_local(b), op, opM=S.Jacobi(op), mult=md.mult, tol=tol, precision=getattr(S, prec_name),
              max_outer=1, path=path, info=info)
    x64 = S.pcg(S.as_local(b), op, opM=S.Jacobi(op), mult=md.mult, tol=tol, path=path, info=info64)
    assert info["converged"] and info["res_inf"] <= tol, info
    assert info["outer"] >= 2, info  # the budgeted sweep/segment plus the FP64 finish
    assert rel_l2(host(x), host(x64)) < 1e-9


def test_tma_variant_in_captured_cg_chunks_fresh_process(gpu):
    """A mesh pinned to the TMA-fed operator (variant 6) before its first
    solve, in a process where no TMA launch has run yet: the CG chunks are
    captured into a CUDA graph around variant-6 operator launches, the solve
    converges in both FP64 arithmetics, none of the kernel's bounded waits
    gives up, and x equals the variant-2 solve to the solver tolerance."""
    import os
    import subprocess
    import sys
    import textwrap
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = textwrap.dedent("""
        import ctypes
        import numpy as np
        import torch
        import sem_oracle as O
        import semgb300 as S
        from _helpers import meshes, host, rel_l2
        lib = S.load()
        for prec in (S.SEM_F64, S.SEM_F64_DF):
            mo, md = meshes(9, 32, 24, (False, False), "DDDD", 0.05, precision=prec)
            M = O.generateMask(["D"] * 4, mo)
            rng = np.random.default_rng(4)
            b = S.as_local(O.gatherScatter(O.mask(O.mass(rng.standard_normal(mo.shape), mo), M), mo))
            tol = 1e-9 * float(b.abs().max())
            op = S.HelmholtzOp(md, 1e-2, 1.0)
            xs = {}
            for v in (6, 2):
                md.set_variant(v, prec)
                info = {}
                xs[v] = host(S.pcg(b, op, opM=S.Jacobi(op), mult=md.mult, tol=tol, info=info,
                                   precision=prec, path=S.SEM_PATH_CHUNKED))
                assert info["converged"] and info["res_inf"] <= tol, (v, info)
            assert rel_l2(xs[6], xs[2]) < 1e-7, rel_l2(xs[6], xs[2])
        cnt = ctypes.c_uint(0)
        S._lib.check(lib.sem_wait_timeouts(0, ctypes.byref(cnt)))
        assert cnt.value == 0
        print("ok")
    """)
    paths = [os.path.join(root, "spectralelements.jl_gb300"), os.path.join(root, "oracle"),
             os.path.join(root, "tests"), root]
    env = dict(os.environ)
    env["PYTHONPATH"] = os.pathsep.join(paths + [env.get("PYTHONPATH", "")])
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, env=env,
                       cwd=root)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout[-2000:] + r.stderr[-4000:]
