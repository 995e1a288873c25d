"""Batched solves (sem_batch_pcg): problems of different element counts, orders,
viscosities and mass coefficients in one persistent launch per order, each
checked against the single-problem solver sem_pcg and the oracle."""
import numpy as np
import pytest

import sem_oracle as O
from _helpers import host, meshes, rel_l2

pytestmark = pytest.mark.gpu


def _problems(seed, count):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        Ex, Ey = (int(v) for v in rng.integers(2, 13, size=2))
        n = int(rng.choice([3, 5, 7, 9, 11]))
        nu = float(10 ** rng.uniform(-3, 0))
        lam = float(rng.uniform(0, 10))
        out.append((n, Ex, Ey, nu, lam))
    return out


def _rhs(mo, M):
    f = 2 * np.pi ** 2 * np.sin(np.pi * mo.x) * np.sin(np.pi * mo.y)
    return O.gatherScatter(O.mask(O.mass(f, mo), M), mo)


@pytest.mark.parametrize("precision", ["DF", "MIXED", "MIXED_RR"])
def test_batch_matches_single_solves(gpu, precision):
    import semgb300 as S
    probs = _problems(11, 14)
    ms, bs, tols, refs = [], [], [], []
    for (n, Ex, Ey, nu, lam) in probs:
        mo, md = meshes(n, Ex, Ey, (False, False), "DDDD", 0.05)
        M = O.generateMask(["D"] * 4, mo)
        b = _rhs(mo, M)
        tol = 1e-10 * np.abs(b).max()
        op = S.HelmholtzOp(md, nu, lam)
        info = {}
        x_ref = host(S.pcg(S.as_local(b), op, opM=S.Jacobi(op), mult=md.mult, tol=tol, info=info))
        ms.append(md)
        bs.append(S.as_local(b))
        tols.append(tol)
        refs.append((x_ref, info["iters"], mo, M, b, nu, lam))
    solver = S.BatchSolver(ms, [p[3] for p in probs], [p[4] for p in probs], jacobi=True)
    infos = []
    prec = getattr(S, "SEM_" + ("F64_DF" if precision == "DF" else precision))
    xs = solver.solve(bs, tols, precision=prec, infos=infos)
    for (x, inf, (x_ref, it_ref, mo, M, b, nu, lam)) in zip(xs, infos, refs):
        assert inf["converged"] and inf["res_inf"] <= max(tols), inf
        if precision == "DF":
            # same iteration within 1 % (the dot products are summed in another order)
            assert abs(inf["iters"] - it_ref) <= max(2, it_ref // 100), (inf, it_ref)
        assert rel_l2(host(x), x_ref) < 1e-7, (inf, it_ref)
        # residual against the oracle's operator
        r = b - O.mask(O.gatherScatter(O.hlmz(host(x), nu, lam, mo), mo), M)
        assert np.abs(r).max() <= 2 * np.abs(b).max() * 1e-10 + 1e-300
    # a second solve on the same batch reuses its workspace
    xs2 = solver.solve(bs, tols, precision=prec)
    for x, x2 in zip(xs, xs2):
        np.testing.assert_array_equal(host(x), host(x2))


def test_batch_periodic_and_bc_variants(gpu):
    import semgb300 as S
    cases = [(5, 4, 3, (True, False), "NNDD", 0.5, 1.0), (7, 3, 5, (False, True), "DDNN", 1.0, 2.0),
             (4, 6, 2, (False, False), "DNDN", 0.1, 0.5), (9, 2, 2, (True, True), "NNNN", 1.0, 3.0)]
    ms, bs, tols, refs = [], [], [], []
    for (n, Ex, Ey, per, bc, nu, lam) in cases:
        mo, md = meshes(n, Ex, Ey, per, bc, 0.0 if any(per) else 0.05)
        M = O.generateMask(list(bc), mo)
        rng = np.random.default_rng(n)
        b = O.mask(O.gatherScatter(mo.B * rng.standard_normal(mo.shape), mo), M)
        tol = 1e-11 * np.abs(b).max()
        op = S.HelmholtzOp(md, nu, lam)
        x_ref = host(S.pcg(S.as_local(b), op, opM=S.Jacobi(op), mult=md.mult, tol=tol))
        ms.append(md)
        bs.append(S.as_local(b))
        tols.append(tol)
        refs.append(x_ref)
    solver = S.BatchSolver(ms, [c[5] for c in cases], [c[6] for c in cases])
    infos = []
    xs = solver.solve(bs, tols, infos=infos)
    for x, x_ref, inf in zip(xs, refs, infos):
        assert inf["converged"]
        assert rel_l2(host(x), x_ref) < 1e-8


def test_batch_rejects_large_orders(gpu):
    import semgb300 as S
    _, md = meshes(13, 2, 2)
    with pytest.raises(S.SemError):
        S.BatchSolver([md], [1.0], [1.0])
