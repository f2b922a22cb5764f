"""Serving-loop admission logic on the CPU with a fake executor (no GPU):
the number of running requests and their footprint never exceed the limits,
requests are started in arrival order, and every request completes."""

import threading
import time

import numpy as np

from rustb_gb300 import batch, serve
from rustb_gb300.model import Model


class FakeModel(Model):
    def __init__(self, norb):
        super().__init__(np.eye(2), np.zeros((norb, 2)), False)

    def device_handle(self):
        return None


def test_admission_limits(monkeypatch):
    running = {"n": 0, "bytes": 0, "max_n": 0, "max_bytes": 0}
    lock = threading.Lock()
    order = []

    def fake_execute(m, req):
        need = serve.footprint_bytes(m, len(req.k), req.observable, req.precision)
        with lock:
            running["n"] += 1
            running["bytes"] += need
            running["max_n"] = max(running["max_n"], running["n"])
            running["max_bytes"] = max(running["max_bytes"], running["bytes"])
            order.append(req.model_id)
        time.sleep(0.02)
        with lock:
            running["n"] -= 1
            running["bytes"] -= need
        return req.model_id

    monkeypatch.setattr(serve, "execute", fake_execute)
    models = {i: FakeModel(n) for i, n in enumerate([4, 64, 128])}
    one = serve.footprint_bytes(models[2], 100, "berry", 1)
    srv = serve.Server(models, hbm_budget_bytes=int(2.5 * one), max_inflight=3)
    reqs = [serve.Request(i % 3, np.zeros((100, 2)), "berry") for i in range(12)]
    futs = [srv.submit(r) for r in reqs]
    assert [f.result(timeout=30) for f in futs] == [r.model_id for r in reqs]
    srv.close()
    assert running["max_n"] <= 3
    assert running["max_bytes"] <= int(2.5 * one) + serve.footprint_bytes(models[1], 100, "berry", 1)
    assert len(srv.latencies()) == 12


def test_bucket_of():
    assert [batch.bucket_of(n) for n in (1, 8, 9, 100, 128, 129, 256)] == [8, 8, 16, 128, 128, 256, 256]
