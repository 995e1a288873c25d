"""Operators beside the fused path, on the device against the oracle: the
dealiased (over-integrated) Laplacian and mass of the functional lapl/mass
(src/lapl.jl:54-68,83-103, src/mass.jl:32-50) with interpolation to a finer
GLL grid, grad / gradᵀ (src/grad.jl:16-63) and advect (src/advect.jl:27-78).
Tolerance: relative L2 1e-12
(the tensor-product sums run in another order than the oracle's BLAS)."""
import numpy as np
import pytest

import sem_oracle as O
from _helpers import host, meshes, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _fine(n, m, Ex, Ey, per, amp):
    """The coarse GLL mesh, its fine (m-point) twin with the same deformation,
    and the interpolation matrix coarse -> fine."""
    mo, md = meshes(n, Ex, Ey, per, "DDDD", amp)
    deform = O.sin_deform(amp) if amp else O.identity_deform
    mf = O.Mesh(m, m, Ex, Ey, per, deform)
    J = O.interpMat(mf.zr, mo.zr)
    return mo, md, mf, J


@pytest.mark.parametrize("n,m,Ex,Ey,per,blockdiag", [
    (5, 8, 3, 4, (False, False), False),
    (4, 7, 2, 3, (True, False), True),
    (7, 11, 2, 2, (False, True), False),
])
def test_dealiased_lapl_and_mass(gpu, n, m, Ex, Ey, per, blockdiag):
    import semgb300 as S
    mo, md, mf, J = _fine(n, m, Ex, Ey, per, 0.05)
    M = O.generateMask(["D"] * 4, mo)
    Md = S.generateMask("DDDD", md)
    rng = np.random.default_rng(n * m)
    u = rng.uniform(-1, 1, mo.shape)
    Jr = np.kron(np.eye(Ex), J) if blockdiag else J
    Js = np.kron(np.eye(Ey), J) if blockdiag else J
    Dr = np.kron(np.eye(Ex), mo.Dr) if blockdiag else mo.Dr
    Ds = np.kron(np.eye(Ey), mo.Ds) if blockdiag else mo.Ds
    # lapl(u, M, Jr, Js, QQtx, QQty, Dr, Ds, G11, G12, G22, mult) with fine-grid G
    ref = O.mask(O.gatherScatter(O.laplace_dealias(u, Jr, Js, Dr, Ds, mf.G11, mf.G12, mf.G22), mo), M)
    got = host(S.lapl(S.as_local(u), Md, Jr, Js, md.QQtx, md.QQty, Dr, Ds, S.as_local(mf.G11),
                      S.as_local(mf.G12), S.as_local(mf.G22), md.mult))
    assert rel_l2(got, ref) < TOL
    # mass(u, M, B, Jr, Js, QQtx, QQty, mult) with the fine-grid B, and B = []
    for B in (mf.B, None):
        ref = O.mask(O.gatherScatter(O.ABu(O._t(Js), O._t(Jr), (B if B is not None else 1.0) * O.ABu(Js, Jr, u)), mo), M)
        got = host(S.mass(S.as_local(u), Md, [] if B is None else S.as_local(B), Jr, Js, md.QQtx, md.QQty,
                          md.mult))
        assert rel_l2(got, ref) < TOL


def test_dealiased_mass_integrates_exactly(gpu):
    """With J to a finer GLL grid and the fine B, the sum of all local entries
    of J'(B J u) is the integral of u (J 1 = 1), exact for low degree."""
    import semgb300 as S
    mo, md, mf, J = _fine(5, 9, 2, 2, (False, False), 0.0)
    u = mo.x ** 2 + mo.y
    got = host(S.mass(S.as_local(u), [], S.as_local(mf.B), J, J, [], [], md.mult))
    exact = 4.0 / 3.0  # over the undeformed reference square [-1, 1]^2
    assert abs(np.sum(got) - exact) < 1e-13


@pytest.mark.parametrize("n,Ex,Ey,per,amp", [(9, 4, 3, (False, False), 0.1), (6, 5, 2, (True, False), 0.05),
                                             (4, 3, 6, (False, True), 0.0)])
def test_grad_and_grad_transpose(gpu, n, Ex, Ey, per, amp):
    import semgb300 as S
    mo, md = meshes(n, Ex, Ey, per, "DDDD", amp)
    rng = np.random.default_rng(n)
    u = rng.uniform(-1, 1, mo.shape)
    ur = O.ABu(None, mo.Dr, u)
    us = O.ABu(mo.Ds, None, u)
    ux, uy = (host(t) for t in S.grad(S.as_local(u), md))
    assert rel_l2(ux, mo.rx * ur + mo.sx * us) < TOL
    assert rel_l2(uy, mo.ry * ur + mo.sy * us) < TOL
    # exactness on the mesh coordinates: grad x = (1, 0), grad y = (0, 1)
    gx, gy = (host(t) for t in S.grad(S.as_local(mo.x), md))
    assert np.abs(gx - 1).max() < 1e-11 and np.abs(gy).max() < 1e-11
    # gradᵀ as src/grad.jl:55-61 writes it
    tx, ty = (host(t) for t in S.gradT(S.as_local(u), md))
    rx_ = O.ABu(mo.Dr.T, None, mo.rx * u) + O.ABu(None, mo.Ds.T, mo.sx * u)
    ry_ = O.ABu(mo.Dr.T, None, mo.ry * u) + O.ABu(None, mo.Ds.T, mo.sy * u)
    assert rel_l2(tx, rx_) < TOL
    assert rel_l2(ty, ry_) < TOL


@pytest.mark.parametrize("n,m,Ex,Ey,per,amp", [(6, 9, 3, 2, (False, False), 0.1), (5, 8, 2, 4, (True, True), 0.05)])
def test_advect_plain_and_dealiased(gpu, n, m, Ex, Ey, per, amp):
    """advect (src/advect.jl:27-78) against the oracle: plain B .* (u.grad T)
    and the dealiased form through a finer mesh of the same elements; the
    dealiased form integrates the advection of a polynomial exactly."""
    import semgb300 as S
    mo, md = meshes(n, Ex, Ey, per, "DDDD", amp)
    mfo, mfd = meshes(m, Ex, Ey, per, "DDDD", amp)
    rng = np.random.default_rng(n + m)
    T, ux, uy = (rng.uniform(-1, 1, mo.shape) for _ in range(3))
    got = host(S.advect(S.as_local(T), S.as_local(ux), S.as_local(uy), md))
    assert rel_l2(got, O.advect(T, ux, uy, mo)) < TOL
    J = O.interpMat(mfo.zr, mo.zr)
    got = host(S.advect(S.as_local(T), S.as_local(ux), S.as_local(uy), md, mfd))
    ref = O.advect_dealiased(T, ux, uy, mo, mfo.B, J, J)
    assert rel_l2(got, ref) < TOL
    # explicit Jr, Js (the oracle's interpMat, which may differ from the
    # package's in the last bit) give the same result
    got2 = host(S.advect(S.as_local(T), S.as_local(ux), S.as_local(uy), md, mfd, J, J))
    assert rel_l2(got2, got) < 1e-14


def test_advect_dealiased_integrates_exactly(gpu):
    """On the undeformed square [-1,1]^2 with T = x^2 and u = (x, 0):
    u.grad T = 2x^2, whose integral is 8/3; the sum of all local entries of
    the dealiased advection is that integral (J'1 sums the fine quadrature)."""
    import semgb300 as S
    mo, md = meshes(5, 2, 3, (False, False), "DDDD", 0.0)
    _, mfd = meshes(9, 2, 3, (False, False), "DDDD", 0.0)
    T, ux, uy = mo.x ** 2, mo.x, np.zeros(mo.shape)
    got = host(S.advect(S.as_local(T), S.as_local(ux), S.as_local(uy), md, mfd))
    assert abs(np.sum(got) - 8.0 / 3.0) < 1e-13
