"""Range guard of the double-float arithmetic (SEM_F64_DF, the mixed
precisions' FP64 parts): values the pair format cannot carry (it holds about 47
significand bits in the FP32 exponent range) must never give a silently wrong
result.  An operator call whose input rows are all tiny (below 2^-60), or
whose inputs or intermediates overflow, is re-run in native FP64 by a gated
launch that follows it; scalar coefficients outside [2^-70, 2^90) send the
call to native FP64; and a solve that ends in NaN/Inf with a finite
right-hand side is solved again in native FP64.  Each case is checked against
native FP64 (SEM_F64) on the same inputs; fields are scaled by powers of two,
which native FP64 carries exactly.
"""
import numpy as np
import pytest

import sem_oracle as O
from _helpers import host, meshes, rel_l2

pytestmark = pytest.mark.gpu

SCALES = [2.0 ** -130, 2.0 ** 130, 2.0 ** -700, 2.0 ** 700, 2.0 ** -75, 1.0]


def _apply(S, md, prec, u, nu=1e-2, k=1.0, nu_field=None):
    md.set_precision(prec)
    op = S.HelmholtzOp(md, nu, k, nu_field=nu_field)
    return host(op(S.as_local(u)))


@pytest.mark.parametrize("scale", SCALES)
def test_apply_out_of_window_fields_match_fp64(gpu, scale):
    import semgb300 as S
    mo, md = meshes(9, 10, 7, (False, True), "DDNN", 0.05)
    u = np.random.default_rng(1).uniform(-1, 1, mo.shape) * scale
    ref = _apply(S, md, S.SEM_F64, u)
    assert np.isfinite(ref).all()
    for v in range(S._lib.SEM_VARIANTS):
        md.set_variant(v, S.SEM_F64_DF)
        got = _apply(S, md, S.SEM_F64_DF, u)
        assert np.isfinite(got).all(), (scale, v)
        assert rel_l2(got / scale, ref / scale) < 1e-12, (scale, v, rel_l2(got / scale, ref / scale))
    # and against the oracle on the unscaled field (power-of-two scaling is exact)
    M = O.generateMask(list("DDNN"), mo)
    ref_o = O.mask(O.gatherScatter(O.hlmz(u / scale, 1e-2, 1.0, mo), mo), M)
    assert rel_l2(ref / scale, ref_o) < 1e-12


def test_apply_field_with_tiny_and_huge_entries(gpu):
    """A field of order one holding a few entries far outside the window: only
    the element tiles that hold them run in FP64, and the result matches."""
    import semgb300 as S
    mo, md = meshes(9, 16, 12, (False, False), "DDDD", 0.05)
    u = np.random.default_rng(2).uniform(-1, 1, mo.shape)
    u[5, 7] = 1e-300
    u[40, 3] = -3e-45
    u[100, 90] = 1e60
    ref = _apply(S, md, S.SEM_F64, u)
    for v in range(S._lib.SEM_VARIANTS):
        md.set_variant(v, S.SEM_F64_DF)
        got = _apply(S, md, S.SEM_F64_DF, u)
        assert rel_l2(got, ref) < 1e-12, v


@pytest.mark.parametrize("nu,k", [(1e-30, 1.0), (1.0, 1e-50), (1e40, 1e40), (2.0 ** 95, 0.0)])
def test_apply_out_of_window_scalars(gpu, nu, k):
    import semgb300 as S
    mo, md = meshes(9, 6, 6, (False, False), "DDDD", 0.05)
    u = np.random.default_rng(3).uniform(-1, 1, mo.shape)
    ref = _apply(S, md, S.SEM_F64, u, nu, k)
    got = _apply(S, md, S.SEM_F64_DF, u, nu, k)
    assert np.isfinite(ref).all() and rel_l2(got, ref) < 1e-12


@pytest.mark.parametrize("gscale,bscale,nu,k", [(2.0 ** 120, 1.0, 1.0, 0.0), (2.0 ** -120, 1.0, 1.0, 0.0),
                                                (1.0, 2.0 ** -110, 0.0, 1.0), (1.0, 2.0 ** -60, 0.0, 2.0 ** -60)])
def test_apply_out_of_window_geometry(gpu, gscale, bscale, nu, k):
    """Metric terms or a mass term outside the pair format's accurate range (a
    mesh whose G or B was uploaded scaled): huge metric terms split into NaN
    pairs, metric terms below 2^-40 and k B products below 2^-100 flag the
    call, so every variant returns the native FP64 result.  The mass cases
    take nu = 0, so that the tiny term is the whole result."""
    import semgb300 as S
    mo = O.Mesh(9, 9, 5, 4, (False, False), O.sin_deform(0.05))
    arrays = {key: getattr(mo, key) for key in ("zr", "wr", "zs", "ws", "Dr", "Ds", "x", "y")}
    for key in ("G11", "G12", "G22"):
        arrays[key] = getattr(mo, key) * gscale
    arrays["B"] = mo.B * bscale
    md = S.Mesh.from_arrays(9, 5, 4, (False, False), arrays, bc="DDDD")
    u = np.random.default_rng(4).uniform(-1, 1, mo.shape)
    ref = _apply(S, md, S.SEM_F64, u, nu=nu, k=k)
    assert np.isfinite(ref).all() and np.abs(ref).max() > 0
    for v in range(S._lib.SEM_VARIANTS):
        md.set_variant(v, S.SEM_F64_DF)
        got = _apply(S, md, S.SEM_F64_DF, u, nu=nu, k=k)
        assert rel_l2(got, ref) < 1e-12, (v, rel_l2(got, ref))


def test_nan_input_stays_nan(gpu):
    import semgb300 as S
    mo, md = meshes(9, 5, 5, (False, False), "DDDD", 0.05)
    u = np.random.default_rng(5).uniform(-1, 1, mo.shape)
    u[12, 13] = np.nan
    ref = _apply(S, md, S.SEM_F64, u)
    got = _apply(S, md, S.SEM_F64_DF, u)
    np.testing.assert_array_equal(np.isnan(got), np.isnan(ref))


@pytest.mark.parametrize("E", [8, 40])  # 8: single-launch small-mesh paths; 40: chunked path
@pytest.mark.parametrize("prec_name", ["SEM_F64_DF", "SEM_MIXED", "SEM_MIXED_RR"])
@pytest.mark.parametrize("scale", [2.0 ** -140, 2.0 ** 140])
def test_solve_out_of_window_rhs(gpu, E, prec_name, scale):
    """pcg on b scaled outside the window equals the scaled native FP64 solve
    of the unscaled problem."""
    import semgb300 as S
    mo, md = meshes(9, E, E, (False, False), "DDDD", 0.1)
    M = O.generateMask(["D"] * 4, mo)
    f = 2 * np.pi ** 2 * np.sin(np.pi * mo.x) * np.sin(np.pi * mo.y)
    b = O.gatherScatter(O.mask(O.mass(f, mo), M), mo)
    tol = 1e-10 * np.abs(b).max()
    op = S.HelmholtzOp(md, 1.0, 0.5)
    x1 = host(S.pcg(S.as_local(b), op, opM=S.Jacobi(op), mult=md.mult, tol=tol, precision=S.SEM_F64))
    info = {}
    xs = host(S.pcg(S.as_local(b * scale), op, opM=S.Jacobi(op), mult=md.mult, tol=tol * scale,
                    precision=getattr(S, prec_name), info=info))
    assert info["converged"] and np.isfinite(xs).all(), info
    assert rel_l2(xs / scale, x1) < 1e-8, rel_l2(xs / scale, x1)


def test_solve_nan_rhs_reports_nan(gpu):
    import semgb300 as S
    mo, md = meshes(9, 8, 8, (False, False), "DDDD", 0.1)
    b = np.zeros(mo.shape)
    b[20, 20] = np.nan
    op = S.HelmholtzOp(md, 1.0, 0.0)
    with pytest.raises(S.SemError):
        S.pcg(S.as_local(b), op, opM=S.Jacobi(op), mult=md.mult, tol=1e-10, precision=S.SEM_F64_DF)


def test_batch_out_of_window(gpu):
    """Batched solves: a problem with a right-hand side outside the window and
    one with k outside it are solved again in native FP64 and match it."""
    import semgb300 as S
    ms, bs, tols, nus, ks = [], [], [], [], []
    for E, k, sc in [(6, 1.0, 1.0), (7, 1.0, 2.0 ** -140), (5, 1e-60, 1.0), (6, 2.0, 2.0 ** 140)]:
        mo, md = meshes(7, E, E + 1, (False, False), "DDDD", 0.05)
        M = O.generateMask(["D"] * 4, mo)
        b = O.gatherScatter(O.mask(O.mass(np.cos(3 * mo.x) + mo.y, mo), M), mo) * sc
        ms.append(md)
        bs.append(S.as_local(b))
        tols.append(1e-9 * np.abs(b).max())
        nus.append(0.5)
        ks.append(k)
    solver = S.BatchSolver(ms, nus, ks, jacobi=True)
    infos = []
    xs = solver.solve(bs, tols, precision=S.SEM_F64_DF, infos=infos)
    for md, b, t, nu, k, x, inf in zip(ms, bs, tols, nus, ks, xs, infos):
        assert inf["converged"], inf
        op = S.HelmholtzOp(md, nu, k)
        x64 = host(S.pcg(b, op, opM=S.Jacobi(op), mult=md.mult, tol=t, precision=S.SEM_F64))
        assert rel_l2(host(x), x64) < 1e-7


@pytest.mark.parametrize("slabs", [0, -1, 3])
def test_host_buffer_apply_out_of_window(gpu, slabs):
    import torch

    import semgb300 as S
    mo, md = meshes(9, 9, 11, (False, False), "DDDD", 0.05)
    u = np.random.default_rng(6).uniform(-1, 1, mo.shape) * 2.0 ** -150
    ref = _apply(S, md, S.SEM_F64, u)
    md.set_precision(S.SEM_F64_DF)
    nx, ny = mo.shape
    u_pin = torch.empty_strided((nx, ny), (1, nx), dtype=torch.float64, pin_memory=True)
    u_pin.copy_(torch.from_numpy(np.asfortranarray(u)))
    got = S.HelmholtzOp(md, 1e-2, 1.0).apply_host(u_pin, slabs=slabs)
    torch.cuda.synchronize()
    assert rel_l2(got.numpy(), ref) < 1e-12
