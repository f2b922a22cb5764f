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
    for prec in (Precision.FP64, Precision.MIXED):
        runner = batch.BatchRunner(prec, autotune=True, cache_path=str(tmp_path / "tune.json"), max_workers=3)
        res = runner.hall_many(jobs)
        assert runner.stats["items"] >= len(jobs)
        for j, r in zip(jobs, res):
            single = j.model.hall_conductivity(j.params, prec).conductivity
            assert np.max(np.abs(r.conductivity - single)) <= 1e-12 * max(np.max(np.abs(single)), 1e-12)
    ref = O.hall_conductivity(jobs[0].model, (9, 9), np.eye(2), [-0.2, 0.0, 0.3])
    assert np.max(np.abs(res[0].conductivity - ref)) <= 1e-8 * np.max(np.abs(ref))


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
