"""Request loop: resident models, admission by device-memory footprint,
continuous admission of new requests while others run.

A request names a resident model, a k-list and an observable:

* ``bands``     -- band energies (``solve_band_all_parallel``, src/solve_ham.rs:94-107);
* ``berry``     -- band-resolved Berry curvature and energies
                   (``berry_curvature_at`` per k, src/response/traits.rs:60-78);
* ``sigma_xy``  -- the Direct Hall sum over the request's k-list,
                   sum_k sum_n Omega_n f(E_n, mu) / nk / det(lat)
                   (src/response/linear/mod.rs:204-223 on a k-list).

Admission: a request is started when the estimated device footprint of the
running requests plus its own fits the budget and a slot is free; requests
that arrive while others are on the GPU wait in arrival order and are started
as soon as slots and memory free up.  Each running request is a thread that
calls the thread-safe C-ABI, which runs it on its own CUDA stream, so the work
of concurrent requests overlaps on the device.  Results do not depend on what
else runs: every call uses its own buffers and deterministic reductions.
"""

from __future__ import annotations

import collections
import math
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .model import Model
from .params import Parameters, Precision

OBSERVABLES = ("bands", "berry", "sigma_xy")


@dataclass
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


def footprint_bytes(model: Model, nk: int, observable: str, precision: int) -> int:
    """Device bytes a request holds while running (chunked as the library does)."""
    N = model.nsta
    per_k = 16 * N * N * (2 if observable == "bands" else (15 if precision == int(Precision.MIXED) else 5))
    chunk = max(1, min(nk, int(_lib.load().tbg_chunk_budget_bytes()) // max(per_k, 1), 65535))
    return chunk * per_k + 16 * model.nR * N * N


class Server:
    def __init__(self, models: dict, hbm_budget_bytes: int = 64 << 30, max_inflight: int = 8):
        self.models = models
        for m in models.values():
            m.device_handle()  # resident hopping tables
        self.budget = hbm_budget_bytes
        self.max_inflight = max_inflight
        self.queue = collections.deque()
        self.lock = threading.Condition()
        self.inflight = 0
        self.inflight_bytes = 0
        self.closed = False
        self.done = []
        self.dispatcher = threading.Thread(target=self._dispatch, daemon=True)
        self.dispatcher.start()

    # ------------------------------------------------------------------ API
    def submit(self, req: Request) -> Future:
        if req.observable not in OBSERVABLES:
            raise ValueError(f"observable must be one of {OBSERVABLES}")
        req.t_submit = time.perf_counter()
        with self.lock:
            self.queue.append(req)
            self.lock.notify_all()
        return req.future

    def close(self):
        with self.lock:
            self.closed = True
            self.lock.notify_all()
        self.dispatcher.join()
        with self.lock:
            while self.inflight:
                self.lock.wait(0.05)

    def latencies(self):
        return np.array([r.t_done - r.t_submit for r in self.done])

    # ------------------------------------------------------------ internals
    def _dispatch(self):
        while True:
            with self.lock:
                while True:
                    if self.queue:
                        req = self.queue[0]
                        m = self.models[req.model_id]
                        need = footprint_bytes(m, len(req.k), req.observable, req.precision)
                        fits = (self.inflight_bytes + need <= self.budget) or self.inflight == 0
                        if self.inflight < self.max_inflight and fits:
                            self.queue.popleft()
                            self.inflight += 1
                            self.inflight_bytes += need
                            break
                    elif self.closed:
                        return
                    self.lock.wait(0.01)
            threading.Thread(target=self._run, args=(req, need), daemon=True).start()

    def _run(self, req: Request, need: int):
        req.t_start = time.perf_counter()
        try:
            req.future.set_result(execute(self.models[req.model_id], req))
        except Exception as exc:  # surfaced through the future
            req.future.set_exception(exc)
        req.t_done = time.perf_counter()
        with self.lock:
            self.inflight -= 1
            self.inflight_bytes -= need
            self.done.append(req)
            self.lock.notify_all()


def execute(m: Model, req: Request):
    """Run one request synchronously (used by the server threads and for the
    alone-vs-in-the-mix check)."""
    k = np.ascontiguousarray(req.k, dtype=np.float64)
    if req.observable == "bands":
        return m.solve_band_all_parallel(k, req.precision)
    dirs = np.eye(m.dim)[:2] if m.dim > 1 else np.array([[1.0], [1.0]])
    p = Parameters(kmesh=(1,) * m.dim, direction=dirs, mu=[req.mu])
    p.eta = req.eta
    if req.observable == "berry":
        return m.berry_curvature_on(k, p, req.precision)
    occ = m.occupied_berry_curvature_on(k, p, req.precision)
    return math.fsum(occ) / len(k) / float(np.linalg.det(m.lat))
