"""Serving-loop scheduling on the CPU with a fake per-call computation (no
GPU): admission limits (calls in flight, device footprint), cutting requests
into pieces and reassembling them in order, merging compatible pieces into
one call, round-robin service of active requests, and error propagation."""

import math
import threading
import time

import numpy as np
import pytest

from rustb_gb300 import batch, serve
from rustb_gb300.model import Model


class FakeModel(Model):
    def __init__(self, norb, nR=1):
        super().__init__(np.eye(2), np.zeros((norb, 2)), False)
        self.ham = np.zeros((nR, norb, norb), dtype=np.complex128)
        self.hamR = np.zeros((nR, 2), dtype=np.int64)

    def device_handle(self):
        return None


def per_k(k):
    """A per-k value that identifies the k-point (checks the reassembly order)."""
    return k[:, 0] * 1000.0 + k[:, 1]


class Recorder:
    def __init__(self, delay=0.01):
        self.lock = threading.Lock()
        self.n = self.bytes = self.max_n = self.max_bytes = 0
        self.calls = []
        self.delay = delay

    def compute(self, m, req, k):
        need = serve.footprint_bytes(m, len(k), req.observable, req.precision)
        with self.lock:
            self.n += 1
            self.bytes += need
            self.max_n = max(self.max_n, self.n)
            self.max_bytes = max(self.max_bytes, self.bytes)
            self.calls.append((req.model_id, len(k)))
        time.sleep(self.delay)
        with self.lock:
            self.n -= 1
            self.bytes -= need
        v = per_k(k)
        if req.observable == "berry":
            return np.repeat(v[:, None], m.nsta, 1), np.repeat(-v[:, None], m.nsta, 1)
        if req.observable == "bands":
            return np.repeat(v[:, None], m.nsta, 1)
        return v


def test_admission_limits_and_reassembly(monkeypatch):
    rec = Recorder()
    monkeypatch.setattr(serve, "_compute", rec.compute)
    models = {i: FakeModel(n) for i, n in enumerate([4, 64, 128])}
    one = serve.footprint_bytes(models[2], 100, "berry", 1)
    srv = serve.Server(models, hbm_budget_bytes=int(2.5 * one), max_inflight=3, chunk_flops=1.0, min_chunk_k=40,
                       merge=False)
    rng = np.random.default_rng(0)
    reqs = [serve.Request(i % 3, rng.uniform(0, 1, (100, 2)), serve.OBSERVABLES[i % 3]) for i in range(12)]
    futs = [srv.submit(r) for r in reqs]
    out = [f.result(timeout=30) for f in futs]
    srv.close()
    assert rec.max_n <= 3
    assert rec.max_bytes <= int(2.5 * one) + serve.footprint_bytes(models[2], 40, "berry", 1)
    assert srv.calls == 12 * 3  # 100 k-points in pieces of 40, 40, 20
    for r, o in zip(reqs, out):
        v = per_k(r.k)
        if r.observable == "berry":
            assert np.array_equal(o[0][:, 0], v) and np.array_equal(o[1][:, 0], -v)
        elif r.observable == "bands":
            assert np.array_equal(o[:, 0], v)
        else:
            assert o == math.fsum(v) / len(v) / 1.0
    assert len(srv.latencies()) == 12


def test_compatible_pieces_are_merged(monkeypatch):
    rec = Recorder(delay=0.05)
    monkeypatch.setattr(serve, "_compute", rec.compute)
    models = {0: FakeModel(16), 1: FakeModel(16)}
    srv = serve.Server(models, max_inflight=1, chunk_flops=1.0, min_chunk_k=64)
    rng = np.random.default_rng(1)
    blocker = serve.Request(1, rng.uniform(0, 1, (64, 2)), "bands")
    small = [serve.Request(0, rng.uniform(0, 1, (10, 2)), "sigma_xy") for _ in range(6)]
    futs = [srv.submit(blocker)] + [srv.submit(r) for r in small]
    res = [f.result(timeout=30) for f in futs]
    srv.close()
    # the six small sigma_xy requests on model 0 queue behind the blocker and run as one 60-point call
    assert (0, 60) in rec.calls and srv.merged_pieces >= 5
    for r, o in zip(small, res[1:]):
        assert o == math.fsum(per_k(r.k)) / 10


def test_round_robin_lets_small_requests_pass(monkeypatch):
    rec = Recorder(delay=0.02)
    monkeypatch.setattr(serve, "_compute", rec.compute)
    models = {0: FakeModel(8), 1: FakeModel(8)}
    srv = serve.Server(models, max_inflight=1, chunk_flops=1.0, min_chunk_k=10, merge=False)
    big = serve.Request(0, np.random.default_rng(2).uniform(0, 1, (200, 2)), "bands")  # 20 pieces
    fb = srv.submit(big)
    time.sleep(0.03)
    small = serve.Request(1, np.random.default_rng(3).uniform(0, 1, (5, 2)), "bands")
    fs = srv.submit(small)
    fs.result(timeout=30)
    assert not fb.done()  # the small request finished while the large one was still being served
    fb.result(timeout=30)
    srv.close()
    assert small.t_done < big.t_done


def test_errors_reach_every_request_of_the_call(monkeypatch):
    def boom(m, req, k):
        raise RuntimeError("device failure")

    monkeypatch.setattr(serve, "_compute", boom)
    srv = serve.Server({0: FakeModel(4)}, max_inflight=2)
    futs = [srv.submit(serve.Request(0, np.zeros((3, 2)), "bands")) for _ in range(3)]
    for f in futs:
        with pytest.raises(RuntimeError):
            f.result(timeout=30)
    srv.close()


def test_bucket_of():
    assert [batch.bucket_of(n) for n in (1, 8, 9, 100, 128, 129, 256)] == [8, 8, 16, 128, 128, 256, 256]


def test_requests_with_different_k_counts_merge(monkeypatch):
    """Merging removes requests from the middle of the queue: requests compare
    by identity, whatever their k-lists."""
    rec = Recorder(delay=0.03)
    monkeypatch.setattr(serve, "_compute", rec.compute)
    models = {0: FakeModel(16), 1: FakeModel(16)}
    srv = serve.Server(models, max_inflight=1, chunk_flops=1.0, min_chunk_k=200)
    rng = np.random.default_rng(4)
    blocker = serve.Request(1, rng.uniform(0, 1, (50, 2)), "bands")
    others = [serve.Request(i % 2, rng.uniform(0, 1, (7 + 13 * i, 2)), "berry") for i in range(8)]
    futs = [srv.submit(blocker)] + [srv.submit(r) for r in others]
    res = [f.result(timeout=30) for f in futs]
    srv.close()
    for r, o in zip(others, res[1:]):
        assert np.array_equal(o[0][:, 0], per_k(r.k))
