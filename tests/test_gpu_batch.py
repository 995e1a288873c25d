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


@pytest.mark.parametrize("cluster_size,ctas_per_sm", [(2, 2), (4, 1), (16, 2), (16, 1)])
def test_batch_launch_shapes_give_the_same_solution(gpu, cluster_size, ctas_per_sm):
    """Every launch shape solves the batch: the cluster size changes which CTA
    owns a tile and so the grouping of the dot products' partial sums, so the
    solutions agree to the solve's accuracy, not bit for bit.  One cluster
    per group runs the group's problems one after another (the timeline)."""
    import semgb300 as S
    probs = _problems(12, 8)
    ms, bs, tols = [], [], []
    for (n, Ex, Ey, nu, lam) in probs:
        mo, md = meshes(n, Ex, Ey, (False, False), "DDDD", 0.05)
        b = _rhs(mo, O.generateMask(["D"] * 4, mo))
        ms.append(md)
        bs.append(S.as_local(b))
        tols.append(1e-10 * np.abs(b).max())
    solver = S.BatchSolver(ms, [p[3] for p in probs], [p[4] for p in probs], jacobi=True)
    ref_infos = []
    ref = [host(x) for x in solver.solve(bs, tols, precision=S.SEM_F64_DF, infos=ref_infos)]
    cfg = solver.config()
    assert [c["n"] for c in cfg] == sorted({p[0] for p in probs})
    assert all(c["cluster_size"] == 8 and c["ctas_per_sm"] == 2 and c["clusters"] == 0 for c in cfg)
    solver.set_config([dict(c, cluster_size=cluster_size, ctas_per_sm=ctas_per_sm, clusters=1) for c in cfg])
    infos = []
    xs = solver.solve(bs, tols, precision=S.SEM_F64_DF, infos=infos)
    for x, x0, inf, inf0 in zip(xs, ref, infos, ref_infos):
        assert inf["converged"]
        assert rel_l2(host(x), x0) < 1e-9, (inf, inf0)
    tl = solver.timeline()
    assert (tl["end_ns"] >= tl["start_ns"]).all() and (tl["start_ns"] >= 0).all()
    assert tl["total_ms"] > 0 and (tl["cluster"] >= 0).all()
    # one cluster per group: every group's problems carry one cluster id
    assert len(set(tl["cluster"].tolist())) == len(solver.config())
    # one cluster per group: a group's problems run one after another
    for c in solver.config():
        idx = [i for i, p in enumerate(probs) if p[0] == c["n"]]
        spans = sorted((tl["start_ns"][i], tl["end_ns"][i]) for i in idx)
        assert all(a[1] <= b[0] for a, b in zip(spans, spans[1:]))


def test_batch_set_config_rejects_bad_shapes(gpu):
    import semgb300 as S
    from semgb300._lib import SemError
    mo, md = meshes(5, 3, 3, (False, False), "DDDD", 0.05)
    solver = S.BatchSolver([md], [1.0], [1.0])
    cfg = solver.config()
    for bad in (dict(cluster_size=3), dict(ctas_per_sm=3), dict(clusters=-1), dict(n=7)):
        with pytest.raises(SemError):
            solver.set_config([dict(cfg[0], **bad)])
    assert solver.config() == cfg


def test_batch_autotune_chooses_persists_and_reloads(gpu, tmp_path):
    import semgb300 as S
    probs = _problems(13, 16)
    ms, bs, tols, refs = [], [], [], []
    for (n, Ex, Ey, nu, lam) in probs:
        mo, md = meshes(n, Ex, Ey, (False, False), "DDDD", 0.05)
        M = O.generateMask(["D"] * 4, mo)
        b = _rhs(mo, M)
        ms.append(md)
        bs.append(S.as_local(b))
        tols.append(1e-10 * np.abs(b).max())
        refs.append((mo, M, b, nu, lam))
    cache = tmp_path / "batch_tune.txt"
    solver = S.BatchSolver(ms, [p[3] for p in probs], [p[4] for p in probs], jacobi=True)
    r = solver.autotune(bs, tols, precision=S.SEM_MIXED, cache=cache)
    assert r["runs"] >= 3 and r["best_ms"] > 0
    chosen, order, wide = solver.config(), solver.order(), solver.wide()
    assert sorted(order) == list(range(len(probs)))
    assert len(wide) == len(probs) and set(wide) <= {0, 1} and r["wide"] == wide
    for c in chosen:
        assert c["cluster_size"] in (2, 4, 8, 16) and c["ctas_per_sm"] in (1, 2) and c["clusters"] >= 0
    # the tuned batch solves correctly
    infos = []
    xs = solver.solve(bs, tols, precision=S.SEM_MIXED, infos=infos)
    for x, inf, (mo, M, b, nu, lam) in zip(xs, infos, refs):
        assert inf["converged"]
        res = b - O.mask(O.gatherScatter(O.hlmz(host(x), nu, lam, mo), mo), M)
        assert np.abs(res).max() <= 2 * np.abs(b).max() * 1e-10 + 1e-300
    # a new batch of the same signature loads the choice without solving
    again = S.BatchSolver(ms, [p[3] for p in probs], [p[4] for p in probs], jacobi=True)
    r2 = again.autotune(bs, tols, precision=S.SEM_MIXED, cache=cache)
    assert r2["runs"] == 0
    assert again.config() == chosen and again.order() == order and again.wide() == wide
    # another tolerance is another signature
    other = S.BatchSolver(ms, [p[3] for p in probs], [p[4] for p in probs], jacobi=True)
    r3 = other.autotune(bs, [2 * t for t in tols], precision=S.SEM_MIXED, cache=cache)
    assert r3["runs"] >= 3


@pytest.mark.parametrize("precision", ["DF", "MIXED"])
def test_batch_wide_problems_solve_on_the_whole_gpu(gpu, precision):
    """Problems marked wide are solved alone on the whole GPU before the
    persistent launches; the batch's results stay converged and match the
    all-cluster solve to the tolerance, and the timeline puts them first."""
    import semgb300 as S
    probs = _problems(14, 10)
    ms, bs, tols, refs = [], [], [], []
    for (n, Ex, Ey, nu, lam) in probs:
        mo, md = meshes(n, Ex, Ey, (False, False), "DDDD", 0.05)
        M = O.generateMask(["D"] * 4, mo)
        b = _rhs(mo, M)
        ms.append(md)
        bs.append(S.as_local(b))
        tols.append(1e-10 * np.abs(b).max())
        refs.append((mo, M, b, nu, lam))
    prec = getattr(S, "SEM_" + ("F64_DF" if precision == "DF" else precision))
    solver = S.BatchSolver(ms, [p[3] for p in probs], [p[4] for p in probs], jacobi=True)
    x0 = [host(x) for x in solver.solve(bs, tols, precision=prec)]
    wide = [1 if i in (0, 3, 7) else 0 for i in range(len(probs))]
    solver.set_wide(wide)
    assert solver.wide() == wide
    infos = []
    xs = solver.solve(bs, tols, precision=prec, infos=infos)
    for x, xr, inf, (mo, M, b, nu, lam) in zip(xs, x0, infos, refs):
        assert inf["converged"], inf
        assert rel_l2(host(x), xr) < 1e-8
        res = b - O.mask(O.gatherScatter(O.hlmz(host(x), nu, lam, mo), mo), M)
        assert np.abs(res).max() <= 2 * np.abs(b).max() * 1e-10 + 1e-300
    tl = solver.timeline()
    widx = [i for i, w in enumerate(wide) if w]
    rest = [i for i, w in enumerate(wide) if not w]
    assert all(tl["cluster"][i] == -2 for i in widx)
    assert all(tl["cluster"][i] >= 0 for i in rest)
    assert max(tl["end_ns"][i] for i in widx) <= min(tl["start_ns"][i] for i in rest)
