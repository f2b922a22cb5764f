"""Batched uneven workload and serving loop on the GPU: every result must
equal the result of the same call made alone."""

import numpy as np
import pytest

from oracle import tb_oracle as O
from rustb_gb300 import batch, serve, workloads as W
from rustb_gb300.params import Parameters, Precision

pytestmark = pytest.mark.gpu


def test_batch_runner_matches_single_calls(tmp_path):
    specs = [(2, 4, False, (9, 9)), (3, 9, False, (4, 4, 3)), (2, 20, True, (6, 5)), (3, 40, False, (3, 3, 3)),
             (2, 64, True, (4, 4)), (2, 100, False, (3, 4))]
    jobs = []
    for i, (dim, norb, spin, mesh) in enumerate(specs):
        m = W.random_model(dim, norb, spin, 1, seed=300 + i)
        dirs = np.eye(dim)[:2]
        jobs.append(batch.Job(m, Parameters(kmesh=mesh, direction=dirs, mu=[-0.2, 0.0, 0.3])))
    lib = batch._lib.load()
    prev = lib.tbg_set_jacobi_max_n(8)
    for prec in (Precision.FP64, Precision.MIXED):
        runner = batch.BatchRunner(prec, autotune=True, cache_path=str(tmp_path / "tune.json"), max_workers=3)
        res = runner.hall_many(jobs)
        assert runner.stats["items"] >= len(jobs)
        if prec == Precision.FP64:  # the 9-band model puts the 16-band bucket up for the Jacobi crossover
            assert runner.stats["jacobi_crossover"] in (8, 16)
        for j, r in zip(jobs, res):
            single = j.model.hall_conductivity(j.params, prec).conductivity
            assert np.max(np.abs(r.conductivity - single)) <= 1e-12 * max(np.max(np.abs(single)), 1e-12)
    ref = O.hall_conductivity(jobs[0].model, (9, 9), np.eye(2), [-0.2, 0.0, 0.3])
    assert np.max(np.abs(res[0].conductivity - ref)) <= 1e-8 * np.max(np.abs(ref))
    lib.tbg_set_jacobi_max_n(prev)


def test_server_results_equal_alone_and_in_the_mix():
    models = {i: W.random_model(2 + (i % 2), n, i % 3 == 0, 1, seed=400 + i)
              for i, n in enumerate([4, 12, 30, 64, 7])}
    rng = np.random.default_rng(9)
    reqs = []
    for i in range(24):
        mid = int(rng.integers(0, len(models)))
        m = models[mid]
        nk = int(rng.integers(1, 200))
        obs = serve.OBSERVABLES[i % 3]
        reqs.append(serve.Request(mid, rng.uniform(0, 1, (nk, m.dim)), obs, precision=int(Precision.MIXED)))
    alone = [serve.execute(models[r.model_id], r) for r in reqs]
    srv = serve.Server(models, hbm_budget_bytes=2 << 30, max_inflight=3)
    futs = [srv.submit(r) for r in reqs]
    mixed = [f.result(timeout=300) for f in futs]
    srv.close()
    for a, b in zip(alone, mixed):
        if isinstance(a, tuple):
            assert all(np.array_equal(x, y) for x, y in zip(a, b))
        elif isinstance(a, np.ndarray):
            assert np.array_equal(a, b)
        else:
            assert a == b
    lat = srv.latencies()
    assert len(lat) == len(reqs) and np.all(lat > 0)


def test_concurrent_calls_on_different_band_counts():
    """Threads solving models of different sizes at once (each size launches
    the eigensolver with a different shared-memory footprint)."""
    import concurrent.futures as cf

    sizes = [(2, 40), (2, 100), (3, 64), (2, 200), (2, 256), (3, 24)]
    models = [W.random_model(dim, n, False, 1, seed=700 + i) for i, (dim, n) in enumerate(sizes)]
    rng = np.random.default_rng(11)
    ks = [rng.uniform(0, 1, (48, m.dim)) for m in models]
    params = [Parameters(kmesh=(1,) * m.dim, direction=np.eye(m.dim)[:2], mu=[0.0]) for m in models]
    alone = [m.berry_curvature_on(k, p, Precision.MIXED) for m, k, p in zip(models, ks, params)]

    def run(i):
        return [models[i].berry_curvature_on(ks[i], params[i], Precision.MIXED) for _ in range(3)]

    with cf.ThreadPoolExecutor(len(models)) as ex:
        out = list(ex.map(run, range(len(models))))
    for a, rs in zip(alone, out):
        for r in rs:
            assert all(np.array_equal(x, y) for x, y in zip(a, r))


def test_native_async_queue_matches_synchronous_calls():
    from rustb_gb300 import errors

    models = [W.random_model(2, 6, True, 1, seed=810), W.random_model(3, 40, False, 1, seed=811),
              W.random_model(2, 128, False, 1, seed=812)]
    rng = np.random.default_rng(5)
    jobs, expect = [], []
    for i, m in enumerate(models):
        dirs = np.eye(m.dim)[:2]
        ph = Parameters(kmesh=(4,) * m.dim, direction=dirs, mu=[-0.1, 0.0, 0.2])
        k = rng.uniform(0, 1, (37, m.dim))
        pb = Parameters(kmesh=(1,) * m.dim, direction=dirs, mu=[0.05])
        for prec in (Precision.FP64, Precision.MIXED):
            jobs.append(batch.submit_hall(m, ph, prec))
            expect.append(m.hall_conductivity(ph, prec).conductivity)
            jobs.append(batch.submit_berry(m, k, pb, prec))
            expect.append(m.berry_curvature_on(k, pb, prec))
            jobs.append(batch.submit_occupied(m, k, pb, prec))
            expect.append(m.occupied_berry_curvature_on(k, pb, prec))
        jobs.append(batch.submit_bands(m, k))
        expect.append(m.solve_band_all_parallel(k))
    # poll the first job until done, wait for the rest
    first = None
    while first is None:
        first = jobs[0].poll()
    got = [first] + [j.wait() for j in jobs[1:]]
    for g, e in zip(got, expect):
        if isinstance(e, tuple):
            assert all(np.array_equal(x, y) for x, y in zip(g, e))
        else:
            assert np.array_equal(g, e)
    # a job that fails reports its status and message through wait()
    bad = Parameters(kmesh=(4, 4), direction=np.eye(2), mu=[0.0])
    j = batch.submit_hall(models[0], bad, precision=7)
    with pytest.raises(errors.TbError):
        j.wait()
    lib = batch._lib.load()
    st = batch.ctypes.c_int(0)
    assert lib.tbg_batch_wait(123456789, batch.ctypes.byref(st)) == 9  # unknown ticket


@pytest.mark.parametrize("precision", [Precision.MIXED, Precision.FP64])
def test_berry_curvature_many_matches_per_model(precision, monkeypatch):
    """Models of one band count stacked into one pipeline
    (tbg_berry_curvature_multi) give each model's berry_curvature_on results:
    tables of different size, k-lists of different length (one empty), chunks
    that end inside a model's k-list (TBG_MAX_CHUNK), a model of another
    dimension (its own group) and a small model (the one-thread-per-k path,
    run alone).  One model is also checked against the oracle."""
    models = [W.random_model(3, 12, True, 1, seed=11), W.random_model(3, 12, True, 2, seed=12),
              W.random_model(2, 12, True, 1, seed=13), W.random_model(3, 3, False, 1, seed=14),
              W.random_model(3, 12, True, 1, seed=15), W.random_model(3, 12, True, 1, seed=16)]
    rng = np.random.default_rng(7)
    sizes = [37, 300, 50, 20, 0, 91]
    ks = [rng.uniform(0, 1, (n, m.dim)) for n, m in zip(sizes, models)]
    dirs3 = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])
    p3 = Parameters.rank2((1, 1, 1), dirs3[0], dirs3[1], [0.0])
    # the 2D model takes its own rank-2 directions: split by dimension
    monkeypatch.setenv("TBG_MAX_CHUNK", "100")
    idx3 = [0, 1, 3, 4, 5]
    res = batch.berry_curvature_many([models[i] for i in idx3], [ks[i] for i in idx3], p3, precision)
    for r, i in zip(res, idx3):
        Om, E = r
        Om1, E1 = models[i].berry_curvature_on(ks[i], p3, precision) if sizes[i] else (np.zeros((0, 1)),) * 2
        assert Om.shape[0] == sizes[i]
        if sizes[i] == 0:
            continue
        scale = max(np.abs(Om1).max(), 1e-300)
        assert np.max(np.abs(Om - Om1)) <= 1e-12 * scale, i
        assert np.max(np.abs(E - E1)) <= 1e-12 * max(np.abs(E1).max(), 1.0), i
    Om, E = res[1]
    Omr, Er = O.berry_on(models[1], ks[1][:4], dirs3)
    tol = 1e-6 if precision == Precision.MIXED else 1e-8
    assert np.max(np.abs(Om[:4] - Omr)) <= tol * np.abs(Omr).max()
    assert np.max(np.abs(E[:4] - Er)) <= 1e-9 * np.abs(Er).max()
    p2 = Parameters.rank2((1, 1), [1.0, 0.0], [0.0, 1.0], [0.0])
    (Om2, E2), = batch.berry_curvature_many([models[2]], [ks[2]], p2, precision)
    Om2r, E2r = models[2].berry_curvature_on(ks[2], p2, precision)
    assert np.max(np.abs(Om2 - Om2r)) <= 1e-12 * np.abs(Om2r).max()
