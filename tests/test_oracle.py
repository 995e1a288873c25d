"""The CPU oracle pinned against known answers (no vectors produced by the
Julia reference exist: parity is unpinned at the GLL/BLAS/Zygote boundary)."""
import numpy as np
import pytest

import sem_oracle as O


@pytest.mark.parametrize("n,z,w", [
    (2, [-1, 1], [1, 1]),
    (3, [-1, 0, 1], [1 / 3, 4 / 3, 1 / 3]),
    (4, [-1, -np.sqrt(1 / 5), np.sqrt(1 / 5), 1], [1 / 6, 5 / 6, 5 / 6, 1 / 6]),
    (5, [-1, -np.sqrt(3 / 7), 0, np.sqrt(3 / 7), 1], [1 / 10, 49 / 90, 32 / 45, 49 / 90, 1 / 10]),
])
def test_gll_closed_form(n, z, w):
    zz, ww = O.gausslobatto(n)
    np.testing.assert_allclose(zz, z, rtol=0, atol=2e-16)
    np.testing.assert_allclose(ww, w, rtol=2e-16, atol=0)


def test_gll_high_precision():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 50
    for n in (6, 9, 13, 17):
        N = n - 1
        # interior nodes = roots of P'_N
        roots = sorted(mpmath.polyroots(mpmath.taylor(lambda t: mpmath.diff(lambda s: mpmath.legendre(N, s), t), 0, N - 1)[::-1], maxsteps=200, extraprec=200))
        zz, ww = O.gausslobatto(n)
        np.testing.assert_array_equal(zz[1:-1], [float(mpmath.re(r)) for r in roots])
        for i, x in enumerate(zz):
            ref = 2 / (N * n * mpmath.legendre(N, mpmath.mpf(x)) ** 2)
            assert abs(ww[i] - float(ref)) <= 2e-16 * abs(float(ref)) * 4


@pytest.mark.parametrize("n", [3, 5, 9, 12, 17])
def test_derivmat_exact_on_polynomials(n):
    z, _ = O.gausslobatto(n)
    D = O.derivMat(z)
    for p in range(n):
        err = np.abs(D @ z ** p - (p * z ** (p - 1) if p else 0 * z)).max()
        assert err < 1e-13 * max(1, p ** 2), (p, err)


def test_abu_is_kron():
    rng = np.random.default_rng(0)
    As, Br = rng.standard_normal((3, 4)), rng.standard_normal((5, 2))
    u = rng.standard_normal((6, 8))
    v = O.ABu(As, Br, u)
    # block form: v[blocks] = Br u_blk As'
    ref = np.zeros((15, 6))
    for bx in range(3):
        for by in range(2):
            ref[5 * bx:5 * bx + 5, 3 * by:3 * by + 3] = Br @ u[2 * bx:2 * bx + 2, 4 * by:4 * by + 4] @ As.T
    np.testing.assert_allclose(v, ref, rtol=1e-14, atol=1e-14)
    np.testing.assert_array_equal(O.ABu(None, None, u), u)


@pytest.mark.parametrize("shape_u,As,Br", [((6, 4), (3, 2), (2, 4)), ((40, 12), (2, 6), (33, 8)),
                                            ((66, 4), None, (33, 33)), ((8, 90), (45, 45), None)])
def test_abu_as_kronecker_operators(shape_u, As, Br):
    """src/ABu.jl:13-34 as linear algebra on vec(u) (column-major): the Br
    step is (I ⊗ Br) on consecutive chunks of nb entries, which span columns
    when nb does not divide size(u,1); the As step is (I ⊗ As ⊗ I_m') on the
    column blocks.  Covers the sizes the device's GEMM path serves."""
    rng = np.random.default_rng(1)
    u = rng.standard_normal(shape_u)
    A = None if As is None else rng.standard_normal(As)
    B = None if Br is None else rng.standard_normal(Br)
    m, n = shape_u
    x = u.flatten(order="F")
    if B is not None:
        x = np.kron(np.eye(m * n // B.shape[1]), B) @ x
        m = m * B.shape[0] // B.shape[1]
    if A is not None:
        x = np.kron(np.eye(n // A.shape[1]), np.kron(A, np.eye(m))) @ x
        n = n // A.shape[1] * A.shape[0]
    ref = x.reshape((m, n), order="F")
    np.testing.assert_allclose(O.ABu(A, B, u), ref, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("Ex,Ey,n,per", [(3, 2, 4, (False, False)), (2, 3, 5, (True, False)),
                                         (1, 2, 3, (True, True)), (4, 1, 2, (False, True))])
def test_gather_scatter_structured_equals_dense(Ex, Ey, n, per):
    msh = O.Mesh(n, n, Ex, Ey, per, dense_qq=True)
    rng = np.random.default_rng(1)
    u = rng.standard_normal(msh.shape)
    dense = O.gatherScatter(u, msh.QQtx, msh.QQty)
    idx = O.gatherScatter_index(u, msh.l2gx, msh.nxg, msh.l2gy, msh.nyg)
    np.testing.assert_allclose(idx, dense, rtol=1e-15, atol=1e-15)
    # multiplicities 1/2/4 and mult * (QQ' 1) = 1
    copies = O.gatherScatter(np.ones(msh.shape), msh)
    assert set(np.unique(copies)) <= {1.0, 2.0, 4.0}
    np.testing.assert_array_equal(msh.mult * copies, 1.0)


def test_mass_integrates_area_and_mask():
    msh = O.Mesh(9, 9, 8, 8, (False, False), O.sin_deform(0.1))
    assert abs(msh.B.sum() - 1.0) < 1e-13
    M = O.generateMask(["D", "N", "D", "D"], msh)
    assert M.dtype == bool
    assert not M[0, :].any() and M[-1, 1:-1].all() and not M[:, 0].any() and not M[:, -1].any()
    Mp = O.generateMask(["D"] * 4, O.Mesh(3, 3, 2, 2, (True, False)))
    assert Mp[0, 1:-1].all() and not Mp[:, 0].any()


def _poisson(E, n):
    msh = O.Mesh(n, n, E, E, (False, False), O.sin_deform(0.1))
    M = O.generateMask(["D"] * 4, msh)
    ut = np.sin(np.pi * msh.x) * np.sin(np.pi * msh.y)
    f = 2 * np.pi ** 2 * ut
    b = O.gatherScatter(O.mask(O.mass(f, msh), M), msh)
    d = O.jacobi_diag(msh, 1.0, 0.0, M)
    info = {}
    x = O.pcg(b, lambda v: O.mask(O.gatherScatter(O.lapl(v, msh), msh), M), opM=lambda r: r / d,
              mult=msh.mult, tol=1e-12 * np.abs(b).max(), info=info)
    return np.abs(x - ut).max(), info


def test_manufactured_poisson_spectral_convergence():
    errs = [_poisson(4, n)[0] for n in (4, 6, 8)]
    assert errs[0] > 10 * errs[1] > 100 * errs[2] / 10
    err, info = _poisson(8, 9)
    assert info["converged"] and err < 1e-9


def test_operator_symmetric_with_mult_inner_product():
    msh = O.Mesh(5, 5, 3, 3, (False, False), O.sin_deform(0.05))
    M = O.generateMask(["D"] * 4, msh)
    rng = np.random.default_rng(5)
    # continuous masked fields
    u = O.mask(msh.mult * O.gatherScatter(rng.standard_normal(msh.shape), msh), M)
    v = O.mask(msh.mult * O.gatherScatter(rng.standard_normal(msh.shape), msh), M)
    A = lambda w: O.mask(O.gatherScatter(O.hlmz(w, 0.3, 2.0, msh), msh), M)  # noqa: E731
    a, b = np.sum(v * A(u) * msh.mult), np.sum(u * A(v) * msh.mult)
    assert abs(a - b) < 1e-12 * abs(a)


def test_neumann_constant_null_space():
    msh = O.Mesh(6, 6, 3, 4, (False, False), O.sin_deform(0.05))
    Au = O.gatherScatter(O.lapl(np.ones(msh.shape), msh), msh)
    assert np.abs(Au).max() < 1e-11


def test_bdf_coefficients():
    a, b = O.bdfExtK([0.0, 0.0, 0.0, 0.0])
    np.testing.assert_array_equal(a, [1, 0, 0])
    np.testing.assert_array_equal(b, [0, 0, 0, 0])
    a, b = O.bdfExtK([0.1, 0.0], k=1)
    np.testing.assert_allclose(a, [1.0])
    np.testing.assert_allclose(b, [10.0, -10.0], rtol=1e-14)
    a, b = O.bdfExtK([0.3, 0.2, 0.1, 0.0], k=3)
    np.testing.assert_allclose(b, np.array([11 / 6, -3, 3 / 2, -1 / 3]) / 0.1, rtol=1e-12)
    np.testing.assert_allclose(a, [3, -3, 1], rtol=1e-12)


def test_c_oracle_matches_numpy():
    import sem_oracle_c as C
    for Ex, Ey, n, per, bc in [(3, 2, 5, (False, False), "DDDD"), (2, 3, 4, (True, False), "DNDD"),
                               (2, 2, 6, (True, True), "NNNN")]:
        msh = O.Mesh(n, n, Ex, Ey, per, O.sin_deform(0.05) if not any(per) else O.identity_deform)
        M = O.generateMask(list(bc), msh)
        rng = np.random.default_rng(2)
        u = rng.uniform(-1, 1, msh.shape)
        ref = O.mask(O.gatherScatter(O.hlmz(u, 0.7, 1.5, msh), msh), M)
        g = C.grid(n, Ex, Ey, per, bc)
        got = C.apply(g, msh.Dr, msh.Ds, msh.G11, msh.G12, msh.G22, msh.B, u, nu=0.7, k=1.5)
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-14
        np.testing.assert_allclose(C.gather_scatter(g, u), O.gatherScatter(u, msh), rtol=1e-15)


def test_grad_and_advect_known_answers():
    """grad (src/grad.jl:16-34) is exact on polynomials of the element order,
    and advect (src/advect.jl:27-64) integrates u.grad T over [-1, 1]^2, in
    the plain and the dealiased form (through a finer GLL grid)."""
    mo = O.Mesh(7, 7, 3, 2, (False, False), O.identity_deform)
    gx, gy = O.grad(mo.x ** 3 * mo.y, mo)
    np.testing.assert_allclose(gx, 3 * mo.x ** 2 * mo.y, atol=1e-11)
    np.testing.assert_allclose(gy, mo.x ** 3, atol=1e-11)
    # [-1, 1]^2: T = x^2 y, u = (1, x): integrand 2xy + x^3 is odd -> 0;
    # T = x^2, u = (x, 0): 2x^2 -> 8/3
    ones, zeros = np.ones(mo.shape), np.zeros(mo.shape)
    assert abs(np.sum(O.advect(mo.x ** 2 * mo.y, ones, mo.x, mo))) < 1e-13
    assert abs(np.sum(O.advect(mo.x ** 2, mo.x, zeros, mo)) - 8.0 / 3.0) < 1e-13
    mf = O.Mesh(11, 11, 3, 2, (False, False), O.identity_deform)
    J = O.interpMat(mf.zr, mo.zr)
    # T = x^4, u = (x^3, 0): 4 x^6 -> 2 * 4/7 * 2; on straight elements the
    # product of the interpolants stays within the 2n - 3 degrees GLL
    # integrates, so both forms are exact
    exact = 16.0 / 7.0
    dealiased = np.sum(O.advect_dealiased(mo.x ** 4, mo.x ** 3, zeros, mo, mf.B, J, J))
    plain = np.sum(O.advect(mo.x ** 4, mo.x ** 3, zeros, mo))
    assert abs(dealiased - exact) < 1e-12 and abs(plain - exact) < 1e-12
    # on the deformed map the Jacobian is not polynomial: the two forms differ
    md = O.Mesh(7, 7, 3, 2, (False, False), O.sin_deform(0.1))
    mdf = O.Mesh(11, 11, 3, 2, (False, False), O.sin_deform(0.1))
    a = np.sum(O.advect_dealiased(md.x ** 4, md.x ** 3, zeros, md, mdf.B, J, J))
    b = np.sum(O.advect(md.x ** 4, md.x ** 3, zeros, md))
    assert 1e-12 < abs(a - b) < 1e-3 * abs(a)


def _oracle_bdf_error(k, dt, T=0.4, n=8, E=3):
    """The oracle's Diffusion stepping (src/diffusion.jl:51-106 restated) on
    u = sin(pi x) sin(pi y) exp(-t) with its forcing; max error at T."""
    mo = O.Mesh(n, n, E, E, (False, False), O.identity_deform)
    M = O.generateMask(["D"] * 4, mo)
    nu = 0.5
    sp = np.sin(np.pi * mo.x) * np.sin(np.pi * mo.y)
    u = sp.copy()
    uh = [np.zeros(mo.shape) for _ in range(k)]
    t = [0.0] * (k + 1)
    for _ in range(int(round(T / dt))):
        uh = [u.copy()] + uh[:-1]
        t = [t[0]] + t[:-1]
        t[0] += dt
        _, bb = O.bdfExtK(t, k)
        f = (-1.0 + 2 * np.pi ** 2 * nu) * sp * np.exp(-t[0])
        rhs = O.diffusion_makeRHS(mo, nu, f, np.zeros(mo.shape), uh, bb, M)
        u = O.pcg(rhs, lambda v, bb=bb: O.diffusion_opLHS(v, mo, nu, bb[0], M), mult=mo.mult, tol=1e-13)
    return np.abs(u - sp * np.exp(-t[0])).max()


@pytest.mark.parametrize("k,order", [(1, 1.0), (2, 2.0), (3, 2.0)])
def test_oracle_bdf_time_order(k, order):
    """BDFk with the start of bdfExtK (src/time.jl:31-53: a BDF1 first step,
    then BDF2, ...) on a manufactured solution: order 1 for k = 1 and 2 for
    k = 2; for k = 3 the lower-order start steps keep the global order at 2."""
    e1 = _oracle_bdf_error(k, 0.02)
    e2 = _oracle_bdf_error(k, 0.01)
    rate = np.log2(e1 / e2)
    assert abs(rate - order) < 0.25, (e1, e2, rate)


def test_stiffness_integrals_plain_and_dealiased():
    """v' A u summed over local copies is the integral of grad v . grad u
    (src/lapl.jl:70-81, and the over-integrated form of :83-103 with the
    fine grid's metric): on [-1, 1]^2, u = v = x gives 4, u = v = x^2 gives
    16/3, and u = x^2, v = 1 gives 0 (the constant is in the kernel)."""
    mo = O.Mesh(6, 6, 3, 2, (False, False), O.identity_deform)
    mf = O.Mesh(10, 10, 3, 2, (False, False), O.identity_deform)
    J = O.interpMat(mf.zr, mo.zr)
    cases = ((mo.x, mo.x, 4.0), (mo.x ** 2, mo.x ** 2, 16.0 / 3.0), (mo.x ** 2, np.ones(mo.shape), 0.0))
    for u, v, exact in cases:
        plain = np.sum(v * O.laplace(u, mo.Dr, mo.Ds, mo.G11, mo.G12, mo.G22))
        deal = np.sum(v * O.laplace_dealias(u, J, J, mo.Dr, mo.Ds, mf.G11, mf.G12, mf.G22))
        assert abs(plain - exact) < 1e-12 and abs(deal - exact) < 1e-12, (plain, deal, exact)
