"""Parity of the device operators (through libsem_b200's C ABI) with the oracle.

Tolerances: relative L2 <= 1e-12 for FP64 operator applies (both the native
FP64 and the double-float arithmetic); bit-exact for masks, multiplicities
and gather-scatter of summed copies (the same summation order as the oracle).
"""
import numpy as np
import torch
import pytest

import sem_oracle as O
from _helpers import host, meshes, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-12

CASES = [
    # n, Ex, Ey, periodic, bc, deform amplitude
    (9, 8, 8, (False, False), "DDDD", 0.1),
    (9, 17, 13, (False, False), "DNDN", 0.05),
    (5, 3, 2, (True, False), "DDDD", 0.05),
    (4, 1, 1, (True, True), "NNNN", 0.0),
    (2, 9, 5, (False, True), "DDNN", 0.05),
    (3, 20, 11, (False, False), "NDDN", 0.05),
    (8, 10, 9, (True, True), "DDDD", 0.0),
    (12, 5, 7, (False, False), "DDDD", 0.05),
    (13, 3, 4, (True, False), "NNDD", 0.05),
    (16, 4, 3, (False, False), "DDDD", 0.05),
    (17, 3, 5, (False, True), "DDDD", 0.05),
    (6, 25, 1, (False, False), "DDDD", 0.05),
    (7, 1, 19, (False, False), "DDDD", 0.05),
]


def _ids(c):
    return f"n{c[0]}_{c[1]}x{c[2]}_p{int(c[3][0])}{int(c[3][1])}_{c[4]}"


@pytest.mark.parametrize("case", CASES, ids=_ids)
@pytest.mark.parametrize("prec", ["F64", "DF"])
@pytest.mark.parametrize("variant", [0, 2, 4, 5, 6])
def test_fused_operators(gpu, case, prec, variant):
    import semgb300 as S
    n, Ex, Ey, per, bc, amp = case
    mo, md = meshes(n, Ex, Ey, per, bc, amp, precision=getattr(S, "SEM_" + ("F64" if prec == "F64" else "F64_DF")))
    md.set_variant(variant)
    M = O.generateMask(list(bc), mo)
    rng = np.random.default_rng(3)
    u = rng.uniform(-1, 1, mo.shape)
    nu = rng.uniform(0.5, 2.0, mo.shape)
    ud = S.as_local(u)
    # lapl(u, msh)
    assert rel_l2(host(S.lapl(ud, md)), O.lapl(u, mo)) < TOL
    # lapl(u, nu, msh) = nu .* lapl
    assert rel_l2(host(S.lapl(ud, S.as_local(nu), md)), O.lapl(u, mo, nu)) < TOL
    # hlmz(u, nu, k, msh)
    assert rel_l2(host(S.hlmz(ud, 1e-2, 1.0, md)), O.hlmz(u, 1e-2, 1.0, mo)) < TOL
    # opLHS: mask(QQ'(hlmz)) fused
    ref = O.mask(O.gatherScatter(O.hlmz(u, 1e-2, 1.0, mo), mo), M)
    got = host(S.HelmholtzOp(md, 1e-2, 1.0)(ud))
    assert rel_l2(got, ref) < TOL
    # every copy of a global node carries the same value
    np.testing.assert_array_equal(got, O.gatherScatter(got, mo) * mo.mult)
    # variable coefficient folded into G: D'(nu G)D
    ref = O.mask(O.gatherScatter(O.laplace(u, mo.Dr, mo.Ds, nu * mo.G11, nu * mo.G12, nu * mo.G22), mo), M)
    got = host(S.HelmholtzOp(md, 1.0, 0.0, nu_field=S.as_local(nu))(ud))
    assert rel_l2(got, ref) < TOL
    # functional lapl(u, M, [], [], QQtx, QQty, Dr, Ds, G11, G12, G22, mult)
    Md = S.generateMask(list(bc), md)
    got = host(S.lapl(ud, Md, [], [], md.QQtx, md.QQty, md.Dr, md.Ds, S.as_local(mo.G11),
                      S.as_local(mo.G12), S.as_local(mo.G22), md.mult))
    ref = O.mask(O.gatherScatter(O.lapl(u, mo), mo), M)
    assert rel_l2(got, ref) < TOL
    # block-diagonal kron(I, Dr) accepted as in examples/p2d_explicit.jl:28; no QQ', no mask
    got = host(S.lapl(ud, [], [], [], [], [], np.kron(np.eye(Ex), mo.Dr), np.kron(np.eye(Ey), mo.Ds),
                      S.as_local(mo.G11), S.as_local(mo.G12), S.as_local(mo.G22), md.mult))
    assert rel_l2(got, O.lapl(u, mo)) < TOL


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_kernel_variants_bit_identical(gpu, case):
    """Every fused-kernel variant computes the same operations in the same
    order, so its output is bit-identical to variant 0 (FP64, double-float,
    and the FP32 operator through the mixed-precision solve)."""
    import semgb300 as S
    import torch
    n, Ex, Ey, per, bc, amp = case
    mo, md = meshes(n, Ex, Ey, per, bc, amp)
    rng = np.random.default_rng(5)
    ud = S.as_local(rng.uniform(-1, 1, mo.shape))
    nu = S.as_local(rng.uniform(0.5, 2.0, mo.shape))
    for prec in (S.SEM_F64, S.SEM_F64_DF):
        md.set_precision(prec)
        outs = []
        for v in range(S._lib.SEM_VARIANTS):
            md.set_variant(v)
            outs.append([host(S.lapl(ud, md)), host(S.lapl(ud, nu, md)), host(S.mass(ud, md)),
                         host(S.HelmholtzOp(md, 1e-2, 1.0)(ud)),
                         host(S.HelmholtzOp(md, 1.0, 0.5, nu_field=nu)(ud))])
        for v in range(1, len(outs)):
            for a, b in zip(outs[0], outs[v]):
                np.testing.assert_array_equal(a, b)
        # in-kernel completion (variant 5) over many launches: the arrival
        # counters stay consistent from launch to launch
        md.set_variant(5)
        op = S.HelmholtzOp(md, 1e-2, 1.0)
        for _ in range(25):
            np.testing.assert_array_equal(host(op(ud)), outs[0][3])
        # the fused QQ' and mask sum every node in the order of the standalone
        # gatherScatter: fused == mask(gatherScatter(hlmz(u)))
        Md = S.generateMask(list(bc), md)
        unfused = host(S.mask(S.gatherScatter(S.hlmz(ud, 1e-2, 1.0, md), md), Md))
        np.testing.assert_array_equal(outs[0][3], unfused)
    # FP32 inner operator: identical mixed-precision solves for every variant
    # of one CG form.  Variants 2 and 5 run the CG-fused operator launch and
    # variants 0 and 1 the operator launch with the p.Ap parts; both sum p.Ap
    # over the unassembled products.  Variants 3 and 4 take a separate dot
    # pass over the assembled A p, and so does variant 6 (the TMA-fed kernel).
    # Each form's solves agree bit for bit, and the forms agree to the
    # tolerance.
    md.set_precision(S.SEM_F64_DF)
    md.set_variant(0)
    M = O.generateMask(list(bc), mo)
    b = S.as_local(O.mask(O.gatherScatter(mo.B * rng.standard_normal(mo.shape), mo), M))
    op = S.HelmholtzOp(md, 0.5, 1.0)
    tol = 1e-10 * float(torch.max(torch.abs(b)))
    xs = []
    for v in range(S._lib.SEM_VARIANTS):
        md.set_variant(v, S.SEM_F32)
        info = {}
        xs.append((host(S.pcg(b, op, opM=S.Jacobi(op), mult=md.mult, tol=tol, info=info,
                              precision=S.SEM_MIXED)), info["iters"]))
    for form in ((0, 1), (2, 5), (3, 4, 6)):
        ref_x, ref_it = xs[form[0]]
        for v in form[1:]:
            x, it = xs[v]
            assert it == ref_it, (v, it, ref_it)
            np.testing.assert_array_equal(x, ref_x)
    # FP32 inner iterations react to the dot's summation order (13 % apart on a
    # periodic case); the solutions agree to the outer tolerance
    for v in (0, 2):
        assert abs(xs[v][1] - xs[3][1]) <= max(4, xs[3][1] // 4)
        assert rel_l2(xs[v][0], xs[3][0]) < 1e-6


def test_tma_kernel_waits_never_time_out(gpu):
    """Variant 6 moves its element tiles by TMA copies and bounds every
    mbarrier wait; on meshes whose rows suit tensor maps (n*Ex*8 bytes a
    multiple of 16, here also for FP32) none of its waits gives up, and its
    results equal variant 4's (which it replaces where TMA cannot serve)."""
    import ctypes
    import semgb300 as S
    lib = S._lib.load()
    cnt = ctypes.c_uint(0)
    S._lib.check(lib.sem_wait_timeouts(1, ctypes.byref(cnt)))
    for n, Ex, Ey in ((9, 40, 30), (5, 64, 9), (13, 12, 7), (17, 8, 5)):
        mo, md = meshes(n, Ex, Ey, (False, False), "DDDD", 0.05)
        ud = S.as_local(np.random.default_rng(n).uniform(-1, 1, mo.shape))
        for prec in (S.SEM_F64, S.SEM_F64_DF):
            md.set_precision(prec)
            outs = []
            for v in (4, 6):
                md.set_variant(v, prec)
                op = S.HelmholtzOp(md, 1e-2, 1.0)
                outs.append(host(op(ud)))
                for _ in range(3):
                    np.testing.assert_array_equal(host(op(ud)), outs[-1])
            np.testing.assert_array_equal(outs[0], outs[1])
    torch.cuda.synchronize()
    S._lib.check(lib.sem_wait_timeouts(1, ctypes.byref(cnt)))
    assert cnt.value == 0


def test_autotune_reports_every_variant(gpu):
    import semgb300 as S
    _, md = meshes(8, 40, 30, (False, False), "DDDD", 0.05)
    for prec in (S.SEM_F64, S.SEM_F64_DF, S.SEM_F32):
        t = md.autotune(prec)
        assert len(t["ms"]) == S._lib.SEM_VARIANTS and all(m > 0 for m in t["ms"]), t
        assert t["ms"][t["chosen"]] == min(t["ms"])


@pytest.mark.parametrize("case", CASES[:6], ids=_ids)
def test_structured_kernels_bit_exact(gpu, case):
    import semgb300 as S
    n, Ex, Ey, per, bc, amp = case
    mo, md = meshes(n, Ex, Ey, per, bc, amp)
    M = O.generateMask(list(bc), mo)
    rng = np.random.default_rng(4)
    u = rng.uniform(-1, 1, mo.shape)
    ud = S.as_local(u)
    np.testing.assert_array_equal(host(S.gatherScatter(ud, md)),
                                  O.gatherScatter_index(u, mo.l2gx, mo.nxg, mo.l2gy, mo.nyg))
    np.testing.assert_array_equal(host(S.gatherScatter(ud, md.QQtx, md.QQty)), O.gatherScatter(u, mo))
    # the functional form on the reference's dense QQtx/QQty (no handle)
    np.testing.assert_array_equal(host(S.gatherScatter(ud, mo.QQtx, mo.QQty)), host(S.gatherScatter(ud, md)))
    Md = S.generateMask(list(bc), md)
    np.testing.assert_array_equal(host(Md), M)
    np.testing.assert_array_equal(host(S.mask(ud, Md)), O.mask(u, M))
    np.testing.assert_array_equal(host(S.mask(ud, [])), u)
    np.testing.assert_array_equal(host(md.mult), mo.mult)
    np.testing.assert_array_equal(host(S.mass(ud, md)), O.mass(u, mo))
    mf = host(md.field("mask"))
    np.testing.assert_array_equal(mf, M.astype(float))
    # functional mass(u, M, B, [], [], QQtx, QQty, mult)
    got = host(S.mass(ud, Md, S.as_local(mo.B), [], [], md.QQtx, md.QQty, md.mult))
    ref = O.mask(O.gatherScatter(mo.B * u, mo), M)
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("nr,ns,Ex,Ey,per", [(4, 7, 5, 3, (True, False)), (9, 3, 2, 6, (False, True)),
                                              (2, 5, 1, 4, (True, True)), (6, 6, 1, 1, (False, False))])
def test_gather_scatter_grid_nr_ne_ns(gpu, nr, ns, Ex, Ey, per):
    """gatherScatter(u, QQtx, QQty) without a handle, nr != ns allowed: the
    reference's dense QQtx u QQty' (src/gatherScatter.jl:8-16), bit for bit."""
    import semgb300 as S
    Qx = O.semq(Ex, nr, per[0])
    Qy = O.semq(Ey, ns, per[1])
    QQx, QQy = Qx @ Qx.T, Qy @ Qy.T
    u = np.random.default_rng(9).uniform(-1, 1, (nr * Ex, ns * Ey))
    got = host(S.gatherScatter(S.as_local(u), QQx, QQy))
    np.testing.assert_array_equal(got, O.gatherScatter(u, QQx, QQy))


@pytest.mark.parametrize("n,Ex,Ey,per", [(9, 8, 8, (False, False)), (5, 7, 3, (True, False)),
                                         (17, 3, 2, (False, True))])
def test_device_geometry(gpu, n, Ex, Ey, per):
    import semgb300 as S
    mo = O.Mesh(n, n, Ex, Ey, per, O.sin_deform(0.1))
    md = S.Mesh(n, n, Ex, Ey, per, O.sin_deform(0.1))
    np.testing.assert_array_equal(host(md.x), mo.x)
    for k in ("Jac", "rx", "ry", "sx", "sy", "B", "G11", "G12", "G22", "Bi", "Jaci"):
        assert rel_l2(host(getattr(md, k)), getattr(mo, k)) < 1e-12, k


@pytest.mark.parametrize("shape_u,As,Br", [
    ((18, 27), (9, 9), (9, 9)),
    ((18, 27), None, (9, 9)),
    ((18, 27), (9, 9), None),
    ((12, 10), (3, 5), (7, 4)),
    ((8, 6), (4, 2), None),
    ((6, 4), None, (2, 4)),  # reshape(u, 4, :) spans columns
    ((64, 96), (32, 32), (32, 32)),
    # factors above 32 x 32 (strided GEMM path), rectangular ones included
    ((66, 40), None, (33, 33)),
    ((72, 90), (45, 45), None),
    ((100, 60), (20, 30), (130, 50)),
    ((6, 4), (3, 2), (2, 4)),  # both factors, rows not whole chunks of nb: reshape(u, 4, :) spans columns
])
def test_abu(gpu, shape_u, As, Br):
    import semgb300 as S
    rng = np.random.default_rng(7)
    u = rng.standard_normal(shape_u)
    A = None if As is None else rng.standard_normal(As)
    B = None if Br is None else rng.standard_normal(Br)
    got = host(S.ABu(A, B, S.as_local(u)))
    assert rel_l2(got, O.ABu(A, B, u)) < 1e-14


def test_abu_dense_gather_scatter_form(gpu):
    """The reference's gatherScatter is ABu(QQty, QQtx, u) with the dense
    global matrices of the mesh (src/gatherScatter.jl:8-16); the same call
    through sem_abu (factors of n*Ex x n*Ex, the GEMM path) equals the
    oracle's and the structured kernel's QQ'."""
    import semgb300 as S
    mo, md = meshes(5, 12, 9, (False, True), "DDDD", 0.05)
    Qx = O.semq(12, 5, False)
    Qy = O.semq(9, 5, True)
    QQtx, QQty = Qx @ Qx.T, Qy @ Qy.T
    u = np.random.default_rng(11).standard_normal(mo.shape)
    got = host(S.ABu(QQty, QQtx, S.as_local(u)))
    assert rel_l2(got, O.ABu(QQty, QQtx, u)) < 1e-14
    assert rel_l2(got, O.gatherScatter(u, mo)) < 1e-14
    assert rel_l2(got, host(S.gatherScatter(S.as_local(u), md))) < 1e-14


def test_abu_rejects_inconsistent_sizes(gpu):
    import semgb300 as S
    u = S.as_local(np.ones((66, 66)))
    with pytest.raises(S.SemError):
        S.ABu(None, np.eye(40), u)  # 66*66 is not a multiple of 40


def test_full_size_properties_cfg2(gpu):
    """256x256 elements, N=8: F64 vs double-float, C-oracle parity, symmetry,
    linearity (size-independent properties at the benchmark size)."""
    import sem_oracle_c as C
    import semgb300 as S
    import torch
    mo, md = meshes(9, 256, 256, (False, False), "DDDD", 0.05)
    rng = np.random.default_rng(3)
    u = rng.uniform(-1, 1, mo.shape)
    ud = S.as_local(u)
    op = S.HelmholtzOp(md, 1e-2, 1.0)
    md.set_precision(S.SEM_F64_DF)
    a_df = host(op(ud))
    md.set_precision(S.SEM_F64)
    a_64 = host(op(ud))
    assert rel_l2(a_df, a_64) < TOL
    ref = C.apply(C.grid(9, 256, 256, (False, False), "DDDD"), mo.Dr, mo.Ds, mo.G11, mo.G12,
                  mo.G22, mo.B, u, nu=1e-2, k=1.0)
    assert rel_l2(a_64, ref) < TOL
    assert rel_l2(a_df, ref) < TOL
    md.set_precision(S.SEM_F64_DF)
    # symmetry <v, A u>_mult == <u, A v>_mult on continuous masked fields
    Md = S.generateMask(["D"] * 4, md)
    cont = lambda w: S.mask(md.mult * S.gatherScatter(w, md), Md)  # noqa: E731
    uc = cont(ud)
    vc = cont(S.as_local(rng.uniform(-1, 1, mo.shape)))
    s1 = torch.sum(vc * op(uc) * md.mult).item()
    s2 = torch.sum(uc * op(vc) * md.mult).item()
    assert abs(s1 - s2) < 1e-11 * abs(s1)
    # linearity
    lhs = op(2.5 * uc - 0.75 * vc)
    rhs = 2.5 * op(uc) - 0.75 * op(vc)
    assert (torch.linalg.norm(lhs - rhs) / torch.linalg.norm(rhs)).item() < 1e-13


def test_errors(gpu):
    import semgb300 as S
    mo, md = meshes(5, 3, 3)
    u = S.as_local(np.ones(mo.shape))
    lib = S.load()
    st = lib.sem_lapl(md.handle, u.data_ptr(), u.data_ptr(), 0, None)
    assert st == 1 and b"alias" in lib.sem_last_error()
    md.set_bc(None)
    with pytest.raises(S.SemError):
        lib_st = lib.sem_mask_bc(md.handle, u.data_ptr(), S.local_empty(*mo.shape).data_ptr(), None)
        S._lib.check(lib_st)
    with pytest.raises(ValueError):
        S.lapl(S.as_local(np.ones((5, 5))), md)


@pytest.mark.parametrize("n,Ex,Ey,per,slabs", [(9, 10, 14, (False, False), 0), (9, 7, 9, (False, True), 3),
                                               (5, 6, 17, (True, True), 16), (12, 4, 7, (True, False), 2),
                                               (9, 3, 2, (False, False), 8), (9, 11, 6, (True, False), -1),
                                               (7, 5, 9, (False, True), -1)])
def test_host_buffer_apply_bit_identical(gpu, n, Ex, Ey, per, slabs):
    """sem_hlmz_host equals sem_hlmz on device buffers bit for bit, for every
    kernel variant and both FP64 arithmetics, from pinned and from pageable
    host memory: the field streamed in and out in slabs of tile rows (each
    slab's interfaces finished by its own fixup), or read and written in place
    by the kernels (slabs = -1)."""
    import semgb300 as S
    mo, md = meshes(n, Ex, Ey, per, "DDDD", 0.05)
    rng = np.random.default_rng(n * Ex + Ey)
    u = rng.uniform(-1, 1, mo.shape)
    u_dev = S.as_local(u)
    nx, ny = mo.shape
    u_pin = torch.empty_strided((nx, ny), (1, nx), dtype=torch.float64, pin_memory=True)
    u_pin.copy_(torch.from_numpy(np.asfortranarray(u)))
    u_page = torch.empty_strided((nx, ny), (1, nx), dtype=torch.float64)
    u_page.copy_(u_pin)
    for prec in (S.SEM_F64_DF, S.SEM_F64):
        md.set_precision(prec)
        op = S.HelmholtzOp(md, 0.7, 1.3)
        for v in range(S._lib.SEM_VARIANTS):
            md.set_variant(v, prec)
            ref = host(op(u_dev))
            got = op.apply_host(u_pin, slabs=slabs)
            torch.cuda.synchronize()
            assert np.array_equal(got.numpy(), ref), (prec, v)
            out_page = torch.empty_strided((nx, ny), (1, nx), dtype=torch.float64)
            try:
                op.apply_host(u_page, out=out_page, slabs=slabs)
            except S.SemError as e:  # direct access to pageable memory needs host page-table access
                assert slabs == S._lib.SEM_HOST_DIRECT and "cannot address" in str(e), e
                continue
            torch.cuda.synchronize()
            assert np.array_equal(out_page.numpy(), ref), (prec, v, "pageable")
    # the G-folded nu field (SEM_NU_IN_G) through the host-buffer call
    nu = S.as_local(np.exp(0.3 * np.sin(3 * mo.x) * np.cos(2 * mo.y)))
    opv = S.HelmholtzOp(md, 1.0, 0.4, nu_field=nu)
    ref = host(opv(u_dev))
    got = opv.apply_host(u_pin, slabs=slabs)
    torch.cuda.synchronize()
    assert np.array_equal(got.numpy(), ref)
