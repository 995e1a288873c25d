"""Device time stepping: makeRHS! (src/diffusion.jl:51-65) as sem_bdf_rhs and
whole runs of evolve! (src/diffusion.jl:81-137) as sem_bdf_run, against the
oracle's restatement of opLHS/makeRHS/pcg stepped on the CPU."""
import numpy as np
import pytest
import torch

import sem_oracle as O
from _helpers import host, meshes, rel_l2

pytestmark = pytest.mark.gpu

KX = KY = KT = 2.0
NU = 1.0


def _spatial(x, y):
    return np.sin(KX * np.pi * x) * np.sin(KY * np.pi * y)


def _exact(x, y, t):
    """examples/d2d.jl:13-33: sin(kx pi x) sin(ky pi y) cos(kt pi t)."""
    return _spatial(x, y) * np.cos(KT * np.pi * t)


def _forcing(x, y, t):
    return _spatial(x, y) * ((KX ** 2 + KY ** 2) * np.pi ** 2 * NU * np.cos(KT * np.pi * t)
                             - KT * np.pi * np.sin(KT * np.pi * t))


def _oracle_run(mo, M, u0, dt, steps, k, tol, f_of_t, ub_of_t=None, jacobi=False):
    """The reference's Diffusion stepping restated on the oracle: histories,
    time history, bdfExtK, makeRHS, pcg from zero with mult = msh.mult, u += ub."""
    uh = [np.zeros(mo.shape) for _ in range(k)]
    u = u0.copy()
    time = [0.0] * (k + 1)
    infos = []
    for _ in range(steps):
        uh = [u.copy()] + uh[:-1]
        time = [time[0]] + time[:-1]
        time[0] += dt
        t = time[0]
        _, bb = O.bdfExtK(time, k)
        ub = np.zeros(mo.shape) if ub_of_t is None else ub_of_t(t)
        rhs = O.diffusion_makeRHS(mo, NU, f_of_t(t), ub, uh, bb, M)
        if jacobi:
            d = O.jacobi_diag(mo, NU, bb[0], M)
            opM = lambda r, d=d: r / d  # noqa: E731
        else:
            opM = lambda r: r  # noqa: E731
        info = {}
        u = O.pcg(rhs, lambda v, bb=bb: O.diffusion_opLHS(v, mo, NU, bb[0], M), opM=opM,
                  mult=mo.mult, tol=tol, info=info) + ub
        infos.append(info)
    return u, time, infos


def test_bdf_rhs_matches_oracle(gpu):
    import semgb300 as S
    n, E = 9, 5
    mo, md = meshes(n, E, 4, (False, False), "DDDD", 0.05)
    rng = np.random.default_rng(11)
    M = O.generateMask(["D"] * 4, mo)
    k = 3
    dfn = S.Diffusion("DDDD", md, Ti=0.0, Tf=1.0, dt=1e-2, k=k, nu=NU)
    f = rng.standard_normal(mo.shape)
    ub = (1.0 - M) * rng.standard_normal(mo.shape)
    uh = [rng.standard_normal(mo.shape) for _ in range(k)]
    for hist in ([0.03, 0.02, 0.01, 0.0], [0.01, 0.0, 0.0, 0.0]):
        dfn.tstep.time = hist
        dfn.tstep.bdfA, dfn.tstep.bdfB = O.bdfExtK(hist, k)
        dfn.f = S.as_local(f)
        dfn.ub = S.as_local(ub)
        dfn.uh = [S.as_local(v) for v in uh]
        got = host(dfn.makeRHS())
        _, bb = O.bdfExtK(hist, k)
        ref = O.diffusion_makeRHS(mo, NU, f, ub, uh, bb, M)
        assert rel_l2(got, ref) < 1e-13, rel_l2(got, ref)
        # the copies of a global node agree to the bit (x-first gather order)
        for e in range(1, E):
            assert np.array_equal(got[e * n - 1, :], got[e * n, :])
        for e in range(1, 4):
            assert np.array_equal(got[:, e * n - 1], got[:, e * n])


@pytest.mark.parametrize("k,path,precision", [(1, 0, None), (3, 0, None), (3, 1, None),
                                              (2, 0, 3), (3, 1, 0)])
def test_bdf_run_matches_oracle_stepping(gpu, k, path, precision):
    """d2d.jl's manufactured solution; forcing as two separable modes;
    the whole run in one sem_bdf_run call (small-mesh path: no host wait per
    step; chunked path: one wait per CG chunk)."""
    import semgb300 as S
    n, E = 9, 4
    mo, md = meshes(n, E, E, (False, False), "DDDD", 0.0)
    kw = {} if precision is None else {"precision": precision}
    dt, steps, tol = 1e-3, 12, 1e-11
    dfn = S.Diffusion("DDDD", md, Ti=0.0, Tf=steps * dt, dt=dt, k=k, nu=NU, path=path, **kw)
    x, y = host(md.x), host(md.y)
    dfn.u.copy_(S.as_local(_exact(x, y, 0.0)))
    sp = _spatial(x, y)
    modes = [(S.as_local(sp * (KX ** 2 + KY ** 2) * np.pi ** 2 * NU), lambda t: np.cos(KT * np.pi * t)),
             (S.as_local(-sp * KT * np.pi), lambda t: np.sin(KT * np.pi * t))]
    infos = dfn.run(steps, forcing=modes, tol=tol)
    assert len(infos) == steps and all(i["converged"] for i in infos)
    u_o, time_o, infos_o = _oracle_run(mo, O.generateMask(["D"] * 4, mo), _exact(mo.x, mo.y, 0.0), dt,
                                       steps, k, tol, lambda t: _forcing(mo.x, mo.y, t))
    got = host(dfn.u)
    assert rel_l2(got, u_o) < 1e-9, rel_l2(got, u_o)
    assert dfn.tstep.time == time_o and dfn.tstep.istep == steps
    # iteration counts follow the oracle's CG (identity preconditioner, mult-weighted dots)
    for a, b in zip(infos, infos_o):
        if precision in (None, 0, 1):
            assert abs(a["iters"] - b["iters"]) <= max(2, b["iters"] // 20), (a, b)
    t = time_o[0]
    assert np.abs(got - _exact(x, y, t)).max() < 5e-3


def test_bdf_run_equals_evolve_loop_and_boundary_data(gpu):
    """One sem_bdf_run call against the per-step evolve() path, with
    non-homogeneous Dirichlet data ub (its lapl term and u += ub), and against
    the oracle with the same ub."""
    import semgb300 as S
    n, E = 8, 3
    mo, md = meshes(n, E, E + 1, (False, False), "DDDD", 0.05)
    M = O.generateMask(["D"] * 4, mo)
    rng = np.random.default_rng(5)
    g = (1.0 - M) * O.gatherScatter(rng.uniform(-1, 1, mo.shape), mo) * mo.mult
    F = mo.mult * O.gatherScatter(rng.uniform(-1, 1, mo.shape), mo)
    dt, steps, k, tol = 5e-3, 9, 3, 1e-12
    fc = lambda t: 1.0 + t  # noqa: E731
    bc = lambda t: np.cos(3.0 * t)  # noqa: E731
    a = S.Diffusion("DDDD", md, Ti=0.0, Tf=1.0, dt=dt, k=k, nu=NU)
    infos = a.run(steps, forcing=[(S.as_local(F), fc)], boundary=[(S.as_local(g), bc)], tol=tol)
    assert all(i["converged"] for i in infos)
    b = S.Diffusion("DDDD", md, Ti=0.0, Tf=1.0, dt=dt, k=k, nu=NU)
    Fd, gd = S.as_local(F), S.as_local(g)
    for _ in range(steps):
        b.evolve(setBC=lambda ub, xx, yy, t: ub.copy_(bc(t) * gd),
                 setForcing=lambda f, xx, yy, t: f.copy_(fc(t) * Fd), tol=tol)
    assert rel_l2(host(a.u), host(b.u)) < 1e-11
    for ua, ubb in zip(a.uh, b.uh):
        assert rel_l2(host(ua), host(ubb)) < 1e-11
    u_o, _, _ = _oracle_run(mo, M, np.zeros(mo.shape), dt, steps, k, tol, lambda t: fc(t) * F,
                            ub_of_t=lambda t: bc(t) * g)
    assert rel_l2(host(a.u), u_o) < 1e-9, rel_l2(host(a.u), u_o)
    assert rel_l2(host(a.ub), bc(a.tstep.time[0]) * g) < 1e-15


def test_simulate_runs_on_device_and_matches_loop(gpu):
    import semgb300 as S
    n, E = 9, 4
    _, md = meshes(n, E, E, (False, False), "DDDD", 0.0)
    x, y = host(md.x), host(md.y)
    dt, Tf = 2e-3, 2e-2
    a = S.Diffusion("DDDD", md, Ti=0.0, Tf=Tf, dt=dt, k=3, nu=NU)
    b = S.Diffusion("DDDD", md, Ti=0.0, Tf=Tf, dt=dt, k=3, nu=NU)
    for d in (a, b):
        d.f.copy_(S.as_local(_spatial(x, y)))
    a.simulate(setIC=lambda u, xx, yy, t: u.copy_(S.as_local(_exact(x, y, t))), tol=1e-12)
    seen = []
    b.simulate(callback=lambda d: seen.append(d.tstep.istep),
               setIC=lambda u, xx, yy, t: u.copy_(S.as_local(_exact(x, y, t))), tol=1e-12)
    assert a.tstep.istep == b.tstep.istep == seen[-1] and a.tstep.time == b.tstep.time
    assert rel_l2(host(a.u), host(b.u)) < 1e-11


def test_bdf_run_rejects_bad_arguments(gpu):
    import semgb300 as S
    from semgb300 import _lib
    _, md = meshes(5, 2, 2, (False, False), "DDDD", 0.0)
    with pytest.raises(ValueError):
        S.Diffusion("DDDD", md, dt=1e-3, k=S.SEM_BDF_MAX_ORDER + 1)
    d = S.Diffusion("DDDD", md, Ti=0.0, Tf=1.0, dt=1e-3, k=2)
    too_many = [(d.f, lambda t: 1.0)] * 9
    with pytest.raises(_lib.SemError):
        d.run(2, forcing=too_many)
    assert d.tstep.istep == 0
    assert torch.count_nonzero(d.u) == 0
