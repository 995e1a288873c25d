"""Adjoint gradients of J(nu) = 1/2 sum B (u - u_target)^2 with respect to a
nodal, G-folded diffusivity nu (the linsolve + @adjoint pattern of
src/adjoint.jl:5-24, examples/semPS.jl:157-192), checked against the oracle's
exact discrete adjoint and against central finite differences (h = 1e-6), for
the steady problem and for implicit-Euler time stepping with checkpoints.
"""
import numpy as np
import pytest

import sem_oracle as O
from _helpers import host, meshes, rel_l2

pytestmark = pytest.mark.gpu


def gaussian_field(mo, seed, sigma=0.5, nk=8):
    """Seeded random field sum_{kx,ky<=8} c k^-2 (cos|sin)(...), normalised to std sigma."""
    rng = np.random.default_rng(seed)
    g = np.zeros(mo.shape)
    for kx in range(1, nk + 1):
        for ky in range(1, nk + 1):
            a, b = rng.standard_normal(2) / (kx * kx + ky * ky)
            ph = rng.uniform(0, 2 * np.pi)
            g += a * np.cos(np.pi * (kx * mo.x + ky * mo.y) + ph) + b * np.sin(np.pi * (kx * mo.x - ky * mo.y))
    return sigma * (g - g.mean()) / g.std()


def oracle_varcoef_solve(mo, M, nu, rhs, k=0.0, tol=1e-13):
    G = (nu * mo.G11, nu * mo.G12, nu * mo.G22)
    A = lambda v: O.mask(O.gatherScatter(O.laplace(v, mo.Dr, mo.Ds, *G) + k * mo.B * v, mo), M)  # noqa: E731
    d = O.jacobi_diag(mo, 1.0, k, M, G=G)
    return O.pcg(rhs, A, opM=lambda r: r / d, mult=mo.mult, tol=tol)


def test_steady_adjoint_matches_oracle_and_fd(gpu):
    import torch

    import semgb300 as S
    mo, md = meshes(9, 10, 10, (False, False), "DDDD", 0.05)
    M = O.generateMask(["D"] * 4, mo)
    nu = np.exp(gaussian_field(mo, 5))
    ut = 0.05 * gaussian_field(mo, 6)
    b = O.gatherScatter(O.mask(O.mass(np.ones(mo.shape), mo), M), mo)
    tol = 1e-12 * np.abs(b).max()
    bd = S.as_local(b)
    Bd = md.B

    def J_dev(nu_np):
        u = S.linsolve_varcoef(S.as_local(nu_np), bd, md, tol=tol)
        return 0.5 * torch.sum(Bd * (u - S.as_local(ut)) ** 2).item()

    nu_t = S.as_local(nu).requires_grad_(True)
    u = S.linsolve_varcoef(nu_t, bd, md, tol=tol)
    J = 0.5 * torch.sum(Bd * (u - S.as_local(ut)) ** 2)
    J.backward()
    g = host(nu_t.grad)

    # oracle: exact discrete adjoint  A lam = mask(QQ'(B (u - ut))), g = -G:(grad lam)(grad u)
    u_o = oracle_varcoef_solve(mo, M, nu, b, tol=tol)
    assert rel_l2(host(u), u_o) < 1e-10
    rhs_adj = O.mask(O.gatherScatter(mo.B * (u_o - ut), mo), M)
    lam = oracle_varcoef_solve(mo, M, nu, rhs_adj, tol=1e-12 * np.abs(rhs_adj).max())
    g_o = O.grad_dot(lam, u_o, mo)
    assert rel_l2(g, g_o) < 1e-8

    # central finite differences along continuous directions; the J evaluations
    # run native FP64 operators, so that rounding (amplified by 1/h) stays well
    # below the 1e-5 tolerance
    md.set_precision(S.SEM_F64)
    rng = np.random.default_rng(7)
    for _ in range(4):
        delta = mo.mult * O.gatherScatter(rng.standard_normal(mo.shape), mo)
        h = 1e-6
        fd = (J_dev(nu + h * delta) - J_dev(nu - h * delta)) / (2 * h)
        ad = float(np.sum(g * delta))
        assert abs(fd - ad) <= 1e-5 * abs(ad) + 1e-14, (fd, ad)

    # the right-hand side examples/semPS.jl:184-186 uses for the adjoint solve,
    # mult .* QQ'(mask(u_bar)), averages the copies instead of summing them; its
    # gradient misses the finite differences where the exact one matches them
    rhs_ps = mo.mult * O.gatherScatter(O.mask(mo.B * (u_o - ut), M), mo)
    lam_ps = oracle_varcoef_solve(mo, M, nu, rhs_ps, tol=1e-12 * np.abs(rhs_ps).max())
    g_ps = O.grad_dot(lam_ps, u_o, mo)
    assert rel_l2(g_ps, g_o) > 1e-3


def test_rhs_cotangent_and_linsolve_match_fd(gpu):
    """The whole residual rhs(a) - lhs(a)(u) is pulled back (src/adjoint.jl:13-16):
    (1) the cotangent of b, mult .* lam, gives the gradient of J with respect
    to f for b = mask(QQ'(B f)) that central differences in f give; (2)
    linsolve(a, problem, solver) with a right-hand side that depends on a
    (built by differentiable torch operations, QQ' as the reference's dense
    QQtx/QQty) matches central differences in a."""
    import torch

    import semgb300 as S
    mo, md = meshes(7, 6, 5, (False, False), "DDDD", 0.05)
    M = O.generateMask(["D"] * 4, mo)
    nu = np.exp(gaussian_field(mo, 11))
    ut = 0.05 * gaussian_field(mo, 12)
    f0 = 1.0 + 0.3 * gaussian_field(mo, 13)
    Bd, utd = md.B, S.as_local(ut)
    md.set_precision(S.SEM_F64)

    def J_of_u(u):
        return 0.5 * torch.sum(Bd * (u - utd) ** 2)

    # (1) gradient in f through b
    def b_of(f):
        return O.gatherScatter(O.mask(mo.B * f, M), mo)

    tol = 1e-12 * np.abs(b_of(f0)).max()
    b_t = S.as_local(b_of(f0)).requires_grad_(True)
    u = S.linsolve_varcoef(S.as_local(nu), b_t, md, tol=tol)
    J_of_u(u).backward()
    bbar = host(b_t.grad)
    fbar = mo.B * O.mask(O.gatherScatter(bbar, mo), M)  # pullback of mask(QQ'(B f))
    rng = np.random.default_rng(21)
    for _ in range(3):
        df_ = rng.standard_normal(mo.shape)
        h = 1e-6
        Jp = J_of_u(S.linsolve_varcoef(S.as_local(nu), S.as_local(b_of(f0 + h * df_)), md, tol=tol)).item()
        Jm = J_of_u(S.linsolve_varcoef(S.as_local(nu), S.as_local(b_of(f0 - h * df_)), md, tol=tol)).item()
        fd = (Jp - Jm) / (2 * h)
        ad = float(np.sum(fbar * df_))
        assert abs(fd - ad) <= 1e-5 * abs(ad) + 1e-14, (fd, ad)

    # (2) linsolve with rhs(a) = mask(QQ'(B (1 + a/2))) as torch operations
    QX = torch.tensor(mo.QQtx, device="cuda")
    QY = torch.tensor(mo.QQty, device="cuda")
    Mt = S.as_local(M.astype(np.float64))

    def rhs_fn(a):
        return QX @ (Mt * Bd * (1.0 + 0.5 * a)) @ QY.T

    problem = S.VarCoefProblem(md, rhs_fn)
    solver = S.PcgSolver(tol=tol)
    a_t = S.as_local(nu).requires_grad_(True)
    J_of_u(S.linsolve(a_t, problem, solver)).backward()
    g = host(a_t.grad)
    for _ in range(3):
        delta = mo.mult * O.gatherScatter(rng.standard_normal(mo.shape), mo)
        h = 1e-6
        Jp = J_of_u(S.linsolve(S.as_local(nu + h * delta), problem, solver)).item()
        Jm = J_of_u(S.linsolve(S.as_local(nu - h * delta), problem, solver)).item()
        fd = (Jp - Jm) / (2 * h)
        ad = float(np.sum(g * delta))
        assert abs(fd - ad) <= 1e-5 * abs(ad) + 1e-14, (fd, ad)
    with pytest.raises(TypeError):
        S.linsolve(a_t, lambda a: None, solver)


@pytest.mark.parametrize("prec_name", ["SEM_MIXED_RR", "SEM_MIXED"])
@pytest.mark.parametrize("k", [0.0, 50.0])
def test_varcoef_mixed_precision_solves(gpu, prec_name, k):
    """The G-folded variable-coefficient solve in mixed precision: the FP32
    inner CG runs on nu .* G rounded to FP32, the FP64 residual on the
    double-float G-folded operator; both stop on the same FP64 tolerance as
    the FP64 solve, against the oracle."""
    import semgb300 as S
    mo, md = meshes(9, 12, 10, (False, False), "DDDD", 0.05)
    M = O.generateMask(["D"] * 4, mo)
    nu = np.exp(gaussian_field(mo, 7))
    b = O.gatherScatter(O.mask(O.mass(np.ones(mo.shape) + mo.x, mo), M), mo)
    tol = 1e-12 * np.abs(b).max()
    op = S.HelmholtzOp(md, 1.0, k, nu_field=S.as_local(nu))
    info, info64 = {}, {}
    x = S.pcg(S.as_local(b), op, opM=S.Jacobi(op), mult=md.mult, tol=tol,
              precision=getattr(S, prec_name), info=info)
    x64 = S.pcg(S.as_local(b), op, opM=S.Jacobi(op), mult=md.mult, tol=tol, precision=S.SEM_F64_DF,
                info=info64)
    assert info["converged"] and info["res_inf"] <= tol
    u_o = oracle_varcoef_solve(mo, M, nu, b, k=k, tol=tol)
    assert rel_l2(host(x), u_o) < 1e-9, rel_l2(host(x), u_o)
    assert rel_l2(host(x), host(x64)) < 1e-9
    # on this pure-diffusion problem the FP32 recurrences stall near 1e-10
    # relative to b; the FP64 CG finishes the solve (the iteration count then
    # exceeds the FP64 solve's, which is what a caller weighs against the
    # cheaper FP32 iterations)
    assert info["iters"] <= 5 * info64["iters"] + 100, (info, info64)


def test_transient_adjoint_with_checkpoints(gpu):
    import torch

    import semgb300 as S
    mo, md = meshes(7, 6, 6, (False, False), "DDDD", 0.05)
    M = O.generateMask(["D"] * 4, mo)
    nu = np.exp(gaussian_field(mo, 5))
    ut = 0.05 * gaussian_field(mo, 6)
    u0 = O.mask(np.sin(np.pi * mo.x) * np.sin(np.pi * mo.y), M)
    f = np.ones(mo.shape)
    dt, T, every = 1e-3, 12, 4
    tol = 1e-13

    # oracle time loop: (K + B/dt) u_n = B u_{n-1}/dt + B f, assembled
    bf = O.gatherScatter(O.mask(mo.B * f, M), mo)
    u_o = u0.copy()
    for _ in range(T):
        rhs = O.gatherScatter(O.mask(mo.B * u_o / dt, M), mo) + bf
        u_o = oracle_varcoef_solve(mo, M, nu, rhs, k=1.0 / dt, tol=tol)

    def J_dev(nu_np):
        u = S.transient_varcoef(S.as_local(nu_np), S.as_local(u0), S.as_local(f), md, dt, T, every, tol=tol)
        return 0.5 * torch.sum(md.B * (u - S.as_local(ut)) ** 2).item()

    nu_t = S.as_local(nu).requires_grad_(True)
    uT = S.transient_varcoef(nu_t, S.as_local(u0), S.as_local(f), md, dt, T, every, tol=tol)
    assert rel_l2(host(uT), u_o) < 1e-10
    J = 0.5 * torch.sum(md.B * (uT - S.as_local(ut)) ** 2)
    J.backward()
    g = host(nu_t.grad)
    assert np.isfinite(g).all() and np.abs(g).max() > 0
    md.set_precision(S.SEM_F64)  # FD evaluations in native FP64 (see the steady test)
    rng = np.random.default_rng(8)
    for _ in range(2):
        delta = mo.mult * O.gatherScatter(rng.standard_normal(mo.shape), mo)
        h = 1e-6
        fd = (J_dev(nu + h * delta) - J_dev(nu - h * delta)) / (2 * h)
        ad = float(np.sum(g * delta))
        assert abs(fd - ad) <= 1e-5 * abs(ad) + 1e-16, (fd, ad)

    # cotangents of the initial state and of the forcing
    u0_t = S.as_local(u0).requires_grad_(True)
    f_t = S.as_local(f).requires_grad_(True)
    uT = S.transient_varcoef(S.as_local(nu), u0_t, f_t, md, dt, T, every, tol=tol)
    (0.5 * torch.sum(md.B * (uT - S.as_local(ut)) ** 2)).backward()
    gu0, gf = host(u0_t.grad), host(f_t.grad)

    def J_uf(u0_np, f_np):
        u = S.transient_varcoef(S.as_local(nu), S.as_local(u0_np), S.as_local(f_np), md, dt, T, every, tol=tol)
        return 0.5 * torch.sum(md.B * (u - S.as_local(ut)) ** 2).item()

    h = 1e-6
    du = O.mask(mo.mult * O.gatherScatter(rng.standard_normal(mo.shape), mo), M)
    fd = (J_uf(u0 + h * du, f) - J_uf(u0 - h * du, f)) / (2 * h)
    ad = float(np.sum(gu0 * du))
    assert abs(fd - ad) <= 1e-5 * abs(ad) + 1e-16, (fd, ad)
    dfv = rng.standard_normal(mo.shape)
    fd = (J_uf(u0, f + h * dfv) - J_uf(u0, f - h * dfv)) / (2 * h)
    ad = float(np.sum(gf * dfv))
    assert abs(fd - ad) <= 1e-5 * abs(ad) + 1e-16, (fd, ad)


def test_diffusion_driver_matches_oracle(gpu):
    """Diffusion(bc, msh; Ti, Tf, dt, k) stepping (src/diffusion.jl:51-137) with
    the manufactured solution of examples/d2d.jl:13-33, against the oracle's
    restatement of opLHS/makeRHS and against the exact solution."""
    import semgb300 as S
    n, E = 9, 4
    mo, md = meshes(n, E, E, (False, False), "DDDD", 0.0)
    kx = ky = kt = 2.0
    nu = 1.0

    def ut(x, y, t):
        return np.sin(kx * np.pi * x) * np.sin(ky * np.pi * y) * np.cos(kt * np.pi * t)

    def forcing(x, y, t):
        return (ut(x, y, t) * ((kx ** 2 + ky ** 2) * np.pi ** 2 * nu)
                - np.sin(kx * np.pi * x) * np.sin(ky * np.pi * y) * np.sin(kt * np.pi * t) * (kt * np.pi))

    dt, steps, k = 1e-3, 10, 1
    dfn = S.Diffusion("DDDD", md, Ti=0.0, Tf=steps * dt, dt=dt, k=k, nu=nu, jacobi=True)
    x, y = host(md.x), host(md.y)
    dfn.u.copy_(S.as_local(ut(x, y, 0.0)))
    M = O.generateMask(["D"] * 4, mo)
    u_o = ut(mo.x, mo.y, 0.0)
    t = 0.0
    for _ in range(steps):
        dfn.evolve(setForcing=lambda fdev, xx, yy, tt: fdev.copy_(S.as_local(forcing(x, y, tt))), tol=1e-12)
        t += dt
        a, bb = O.bdfExtK([t, t - dt], k=1)
        rhs = O.diffusion_makeRHS(mo, nu, forcing(mo.x, mo.y, t), np.zeros(mo.shape), [u_o], bb, M)
        d = O.jacobi_diag(mo, nu, bb[0], M)
        u_o = O.pcg(rhs, lambda v: O.diffusion_opLHS(v, mo, nu, bb[0], M), opM=lambda r: r / d,
                    mult=mo.mult, tol=1e-12)
    assert rel_l2(host(dfn.u), u_o) < 1e-9
    assert np.abs(host(dfn.u) - ut(x, y, t)).max() < 5e-3  # implicit Euler, dt = 1e-3
