"""Request loop with continuous batching: resident models, requests cut into
k-chunks, chunks of the active requests served in turn, compatible chunks
merged into one library call, admission by device-memory footprint.

A request names a resident model, a k-list and an observable:

* ``bands``     -- band energies (``solve_band_all_parallel``, src/solve_ham.rs:94-107);
* ``berry``     -- band-resolved Berry curvature and energies
                   (``berry_curvature_at`` per k, src/response/traits.rs:60-78);
* ``sigma_xy``  -- the Direct Hall sum over the request's k-list,
                   sum_k sum_n Omega_n f(E_n, mu) / nk / det(lat)
                   (src/response/linear/mod.rs:204-223 on a k-list).

Scheduling.  On arrival a request's k-list is cut into pieces of at most
``chunk_k(model)`` points, sized so that one piece is about ``chunk_flops`` of
algorithmic work (F(N, nR) = 24 nR N^2 + 46 N^3 per k-point) but at least a
few waves of the per-matrix kernels.  Active requests are served round-robin,
one piece at a time, by a pool of ``max_inflight`` device workers (each call
runs on its own CUDA stream inside the thread-safe C-ABI, so the calls of
different workers overlap on the device): a request that arrives while large
ones run gets its first piece at the next free worker instead of waiting for
them to finish, and a request alone on the server gets every worker.  When a
worker takes a piece it also takes the next pieces of other active requests
with the same (model, observable, precision, mu, eta) while their k-points fit
one piece: many small requests on one model become one launch sequence.  A
call starts when its device footprint (buffers for its k-points plus the
model's tables) fits the budget next to the calls in flight, or when nothing
is in flight.

Results do not depend on what else runs or on how the k-list is cut: every
k-point's outputs are computed by per-matrix kernels from that k-point alone,
and sigma_xy is the exactly rounded sum (``math.fsum``) of the per-k values.
"""

from __future__ import annotations

import collections
import math
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np

from .model import Model
from .params import Parameters, Precision

OBSERVABLES = ("bands", "berry", "sigma_xy")


@dataclass(eq=False)  # requests are compared by identity (the scheduler removes them from its queue)
class Request:
    model_id: int
    k: np.ndarray
    observable: str
    mu: float = 0.0
    eta: float = 1e-3
    precision: int = int(Precision.MIXED)
    t_submit: float = 0.0
    t_start: float = 0.0
    t_done: float = 0.0
    future: Future = field(default_factory=Future)
    # scheduler state
    pieces: collections.deque = field(default_factory=collections.deque)  # (start, stop) k ranges
    parts: dict = field(default_factory=dict)  # start -> result of that range
    left: int = 0  # pieces not yet finished

    def key(self):
        return (self.model_id, self.observable, int(self.precision), float(self.mu), float(self.eta))


def work_per_k(model: Model) -> float:
    """Algorithmic flops per k-point, F(N, nR) = 24 nR N^2 + 46 N^3."""
    N = model.nsta
    return 24.0 * model.nR * N * N + 46.0 * N ** 3


def footprint_bytes(model: Model, nk: int, observable: str, precision: int) -> int:
    """Device bytes a call over nk k-points holds: the per-k buffers of the
    library's pipeline (it never takes more than nk k-points at a time) plus
    the model's paired hopping table."""
    N = model.nsta
    per_k = 16 * N * N * (2 if observable == "bands" else (15 if precision == int(Precision.MIXED) else 5))
    return int(nk) * per_k + 16 * model.nR * N * N


class Server:
    def __init__(self, models: dict, hbm_budget_bytes: int = 64 << 30, max_inflight: int = 8,
                 chunk_flops: float = 4e11, min_chunk_k: int = 456, merge: bool = True):
        self.models = models
        for m in models.values():
            m.device_handle()  # resident hopping tables
        self.budget = hbm_budget_bytes
        self.max_inflight = max_inflight
        self.chunk_flops = chunk_flops
        self.min_chunk_k = min_chunk_k
        self.merge = merge
        self.active = collections.deque()  # requests with pieces left to start, round-robin order
        self.lock = threading.Condition()
        self.inflight = 0
        self.inflight_bytes = 0
        self.closed = False
        self.done = []
        self.calls = 0
        self.merged_pieces = 0
        self.workers = [threading.Thread(target=self._worker, daemon=True) for _ in range(max_inflight)]
        for w in self.workers:
            w.start()

    # ------------------------------------------------------------------ API
    def chunk_k(self, model: Model) -> int:
        """k-points per piece for this model."""
        return int(max(self.min_chunk_k, min(65535, math.ceil(self.chunk_flops / work_per_k(model)))))

    def submit(self, req: Request) -> Future:
        if req.observable not in OBSERVABLES:
            raise ValueError(f"observable must be one of {OBSERVABLES}")
        if req.model_id not in self.models:
            raise KeyError(f"unknown model {req.model_id}")
        req.k = np.ascontiguousarray(req.k, dtype=np.float64)
        nk = len(req.k)
        c = self.chunk_k(self.models[req.model_id])
        req.pieces = collections.deque((a, min(nk, a + c)) for a in range(0, max(nk, 1), c))
        req.left = len(req.pieces)
        req.t_submit = time.perf_counter()
        with self.lock:
            if self.closed:
                raise RuntimeError("server is closed")
            self.active.append(req)
            self.lock.notify_all()
        return req.future

    def close(self):
        """Finish every submitted request, then stop the workers."""
        with self.lock:
            self.closed = True
            self.lock.notify_all()
        for w in self.workers:
            w.join()

    def latencies(self):
        return np.array([r.t_done - r.t_submit for r in self.done])

    # ------------------------------------------------------------ internals
    def _take(self):
        """Next call (under the lock): the first piece of the request at the
        head of the round-robin, merged with the next pieces of compatible
        requests while they fit one piece; None if nothing may start now."""
        if not self.active:
            return None
        head = self.active[0]
        m = self.models[head.model_id]
        cap = self.chunk_k(m)
        a, b = head.pieces[0]
        need = footprint_bytes(m, b - a, head.observable, head.precision)
        if self.inflight and self.inflight_bytes + need > self.budget:
            return None
        head.pieces.popleft()
        if head.t_start == 0.0:
            head.t_start = time.perf_counter()
        self.active.rotate(-1)  # the head goes to the back (round-robin)
        if not head.pieces:
            self.active.pop()
        taken = [(head, a, b)]
        total = b - a
        if self.merge:
            for r in list(self.active):
                if r is head or r.key() != head.key() or not r.pieces:
                    continue
                ra, rb = r.pieces[0]
                if total + (rb - ra) > cap:
                    continue
                r.pieces.popleft()
                if r.t_start == 0.0:
                    r.t_start = time.perf_counter()
                if not r.pieces:
                    self.active.remove(r)
                taken.append((r, ra, rb))
                total += rb - ra
            self.merged_pieces += len(taken) - 1
        need = footprint_bytes(m, total, head.observable, head.precision)
        self.inflight += 1
        self.inflight_bytes += need
        self.calls += 1
        return taken, need

    def _worker(self):
        while True:
            with self.lock:
                while True:
                    got = self._take()
                    if got is not None:
                        break
                    if self.closed and not self.active and self.inflight == 0:
                        self.lock.notify_all()
                        return
                    self.lock.wait(0.05)
            taken, need = got
            head = taken[0][0]
            m = self.models[head.model_id]
            err = None
            try:
                k = np.concatenate([r.k[a:b] for r, a, b in taken])
                out = _compute(m, head, k)
            except Exception as exc:  # surfaced through the futures of the requests in this call
                err = exc
            with self.lock:
                self.inflight -= 1
                self.inflight_bytes -= need
                off = 0
                for r, a, b in taken:
                    n = b - a
                    if err is None:
                        r.parts[a] = _slice(out, off, off + n)
                    elif not r.future.done():
                        r.future.set_exception(err)
                    off += n
                    r.left -= 1
                    if r.left == 0:
                        self._finish(r)
                self.lock.notify_all()

    def _finish(self, r: Request):
        if not r.future.done():
            try:
                parts = [r.parts[a] for a in sorted(r.parts)]
                r.future.set_result(_assemble(self.models[r.model_id], r, parts))
            except Exception as exc:
                r.future.set_exception(exc)
        r.t_done = time.perf_counter()
        self.done.append(r)


def _params(m: Model, req: Request) -> Parameters:
    dirs = np.eye(m.dim)[:2] if m.dim > 1 else np.array([[1.0], [1.0]])
    p = Parameters(kmesh=(1,) * m.dim, direction=dirs, mu=[req.mu])
    p.eta = req.eta
    return p


def _compute(m: Model, req: Request, k: np.ndarray):
    """Per-k outputs of one library call over the k-points k."""
    if len(k) == 0:
        if req.observable == "berry":
            return np.empty((0, m.nsta)), np.empty((0, m.nsta))
        return np.empty((0, m.nsta)) if req.observable == "bands" else np.empty(0)
    if req.observable == "bands":
        return m.solve_band_all_parallel(k, req.precision)
    p = _params(m, req)
    if req.observable == "berry":
        return m.berry_curvature_on(k, p, req.precision)
    return m.occupied_berry_curvature_on(k, p, req.precision)


def _slice(out, a: int, b: int):
    if isinstance(out, tuple):
        return tuple(x[a:b] for x in out)
    return out[a:b]


def _assemble(m: Model, req: Request, parts):
    if req.observable == "berry":
        return tuple(np.concatenate([p[i] for p in parts]) for i in range(2))
    cat = np.concatenate(parts)
    if req.observable == "bands":
        return cat
    return math.fsum(cat) / len(req.k) / float(np.linalg.det(m.lat))


def execute(m: Model, req: Request):
    """Run one request synchronously in a single call (the reference for the
    alone-vs-in-the-mix check)."""
    k = np.ascontiguousarray(req.k, dtype=np.float64)
    return _assemble(m, req, [_compute(m, req, k)])
