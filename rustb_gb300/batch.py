"""Batched Hall conductivity over many models of uneven size.

Every model is uploaded once and stays resident.  The k-mesh of each model is
cut into work items (model, flat k-range); items are bucketed by band count
and run largest-first by a pool of host threads.  Each thread calls the
thread-safe C-ABI (``tbg_hall_sums_range``), which runs on its own CUDA stream,
so items of different models overlap on the device.  Partial sums of each
model are combined on the host with an exactly rounded sum (``math.fsum``) and
normalised as ``hall_conductivity`` does (src/response/linear/mod.rs:204-223).

The chunk size (k-points per item) and the number of concurrent items are
chosen per band-count bucket by :class:`Autotuner`, which times a few
candidates on the first models of a bucket and caches the winner in a JSON
file keyed by GPU name, bucket and precision.
"""

from __future__ import annotations

import concurrent.futures as cf
import ctypes
import json
import math
import os
import threading
import time
from dataclasses import dataclass

import numpy as np

from . import _lib
from .model import Model
from .params import HallConductivityResult, Parameters, Precision, spin_code

DEFAULT_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "autotune.json")


def bucket_of(nsta: int) -> int:
    """Band-count bucket: the next power of two (>= 8)."""
    b = 8
    while b < nsta:
        b *= 2
    return b


@dataclass
class Job:
    model: Model
    params: Parameters
    # only the first k_limit points of the mesh (flat gen_kmesh order): the
    # result is then that partial sum / (nk det), as tbg_hall_sums_range gives it
    k_limit: int | None = None

    def k_count(self) -> int:
        nk = int(np.prod(self.params.kmesh))
        return nk if self.k_limit is None else min(nk, int(self.k_limit))


class Autotuner:
    """Chooses (chunk k-points, concurrent items) per (bucket, precision), and
    for the FP64 path the band count up to which the warp-per-matrix Jacobi
    solver replaces the Householder one (timed on the 16- and 32-band buckets)."""

    CHUNKS = (256, 1024, 4096, 16384)
    WORKERS = (1, 2, 4)

    def __init__(self, path: str = DEFAULT_CACHE, gpu: str = "GPU"):
        self.path = path
        self.gpu = gpu
        self.lock = threading.Lock()
        self.table = {}
        if os.path.exists(path):
            try:
                self.table = json.load(open(path))
            except (OSError, ValueError):
                self.table = {}

    def key(self, bucket: int, precision: int) -> str:
        return f"{self.gpu}|{bucket}|{precision}"

    def get(self, bucket: int, precision: int):
        return self.table.get(self.key(bucket, precision))

    def crossover(self, jobs: list, buckets: dict, lib) -> int:
        """Jacobi/Householder crossover for the FP64 solver: for each of the
        16- and 32-band buckets present, time one job's first k-points with the
        Householder solver alone (crossover 8) and with Jacobi up to the bucket
        size; the crossover is the largest bucket where Jacobi was faster."""
        key = f"{self.gpu}|crossover"
        with self.lock:
            if key in self.table:
                return int(self.table[key])
        best = 8
        for b in (16, 32):
            if b not in buckets:
                continue
            j = jobs[max(buckets[b], key=lambda i: jobs[i].model.nsta)]
            nk = min(4096, int(np.prod(j.params.kmesh)))
            times = {}
            for cross in (8, b):
                lib.tbg_set_jacobi_max_n(cross)
                _run_range(lib, j.model, j.params, int(Precision.FP64), 0, min(nk, 64))
                t0 = time.perf_counter()
                _run_range(lib, j.model, j.params, int(Precision.FP64), 0, nk)
                times[cross] = time.perf_counter() - t0
            if times[b] < times[8]:
                best = b
        lib.tbg_set_jacobi_max_n(best)
        with self.lock:
            self.table[key] = best
            self._save()
        return best

    def _save(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            json.dump(self.table, open(self.path, "w"), indent=1)
        except OSError:
            pass

    def tune(self, bucket: int, precision: int, job: Job, lib) -> dict:
        """Time each candidate on a slice of this job's mesh."""
        m, p = job.model, job.params
        nk = job.k_count()
        best = None
        for chunk in self.CHUNKS:
            if chunk > max(256, nk):
                break
            for workers in self.WORKERS:
                n_items = max(1, min(workers * 2, nk // chunk))
                t0 = time.perf_counter()
                ranges = [(i * chunk % nk, min(chunk, nk - (i * chunk % nk))) for i in range(n_items)]
                with cf.ThreadPoolExecutor(workers) as ex:
                    list(ex.map(lambda r: _run_range(lib, m, p, precision, r[0], r[1]), ranges))
                dt = time.perf_counter() - t0
                rate = sum(r[1] for r in ranges) / dt
                if best is None or rate > best["rate"]:
                    best = {"chunk": chunk, "workers": workers, "rate": rate}
        with self.lock:
            self.table[self.key(bucket, precision)] = best
            self._save()
        return best


def _run_range(lib, model: Model, p: Parameters, precision: int, k0: int, cnt: int) -> np.ndarray:
    km = np.ascontiguousarray(p.kmesh, dtype=np.int64)
    d = _lib.as_f64(p.direction)
    mu = _lib.as_f64(p.mu)
    out = np.empty(len(mu))
    _lib.check(lib.tbg_hall_sums_range(model.device_handle(), _lib.iptr(km), int(k0), int(cnt), _lib.dptr(d),
                                       len(mu), _lib.dptr(mu), float(p.T[0]), float(p.eta), spin_code(p.spin),
                                       int(precision), _lib.dptr(out), None), lib)
    return out


class BatchRunner:
    def __init__(self, precision=Precision.MIXED, autotune: bool = True, cache_path: str = DEFAULT_CACHE,
                 max_workers: int = 4):
        self.lib = _lib.load()
        self.precision = int(precision)
        self.autotune = autotune
        self.tuner = Autotuner(cache_path, gpu=_gpu_name())
        self.max_workers = max_workers
        self.stats = {}

    def hall_many(self, jobs: list[Job]) -> list[HallConductivityResult]:
        for j in jobs:
            j.params.validate_rank2(j.model.dim)
            j.model.device_handle()  # upload once, resident
        buckets = {}
        for idx, j in enumerate(jobs):
            buckets.setdefault(bucket_of(j.model.nsta), []).append(idx)
        plan = {}
        if self.precision == int(Precision.FP64):
            # the crossover is process-wide; without tuning the library's setting stands
            self.crossover = self.tuner.crossover(jobs, buckets, self.lib) if self.autotune else None
        for b, idxs in buckets.items():
            cfg = self.tuner.get(b, self.precision)
            if cfg is None and self.autotune:
                probe = max(idxs, key=lambda i: jobs[i].k_count())
                cfg = self.tuner.tune(b, self.precision, jobs[probe], self.lib)
            plan[b] = cfg or {"chunk": 4096, "workers": 2}
        items = []
        for b, idxs in buckets.items():
            chunk = plan[b]["chunk"]
            for i in idxs:
                nk = jobs[i].k_count()
                for k0 in range(0, nk, chunk):
                    cost = min(chunk, nk - k0) * _work_per_k(jobs[i].model)
                    items.append((cost, i, k0, min(chunk, nk - k0)))
        items.sort(key=lambda it: -it[0])  # largest first
        partial = [[] for _ in jobs]
        lock = threading.Lock()
        workers = max(1, min(self.max_workers, max(p["workers"] for p in plan.values())))

        def run(it):
            _, i, k0, cnt = it
            s = _run_range(self.lib, jobs[i].model, jobs[i].params, self.precision, k0, cnt)
            with lock:
                partial[i].append(s)

        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(workers) as ex:
            list(ex.map(run, items))
        dt = time.perf_counter() - t0
        out = []
        for i, j in enumerate(jobs):
            arr = np.array(partial[i])
            nk = int(np.prod(j.params.kmesh))
            det = float(np.linalg.det(j.model.lat))
            sig = np.array([math.fsum(arr[:, c]) for c in range(arr.shape[1])]) / nk / det
            out.append(HallConductivityResult(chemical_potentials=j.params.mu.copy(), conductivity=sig))
        self.stats = {"seconds": dt, "items": len(items), "workers": workers, "plan": plan,
                      "jacobi_crossover": getattr(self, "crossover", None),
                      "k_points": sum(j.k_count() for j in jobs)}
        return out


def berry_curvature_many(models: list, k_lists: list, params: Parameters, precision=Precision.MIXED) -> list:
    """Band-resolved Berry curvature and energies of many models, each at its
    own k-points: ``berry_curvature_on`` per model, with the models of equal
    band count and dimension (a bucket) stacked into one pipeline
    (``tbg_berry_curvature_multi``): their H and velocities are formed from
    each model's table and the eigensolve, rotation and Omega run once over
    all of the bucket's k-points.  Returns [(Omega, E)] in input order."""
    if len(models) != len(k_lists):
        raise ValueError("one k-list per model")
    lib = _lib.load()
    out = [None] * len(models)
    groups = {}
    ks = []
    for i, (m, k) in enumerate(zip(models, k_lists)):
        kk = np.zeros((0, m.dim)) if np.size(k) == 0 else m._klist(k)
        m._check_berry_params(params)
        ks.append(kk)
        groups.setdefault((m.nsta, m.dim), []).append(i)
    d = _lib.as_f64(params.direction)
    for (nsta, _dim), idxs in sorted(groups.items()):
        handles = (ctypes.c_void_p * len(idxs))(*[models[i].device_handle() for i in idxs])
        nk = np.array([ks[i].shape[0] for i in idxs], dtype=np.int64)
        kcat = np.ascontiguousarray(np.concatenate([ks[i] for i in idxs], axis=0))
        Om = np.empty((int(nk.sum()), nsta))
        E = np.empty((int(nk.sum()), nsta))
        _lib.check(lib.tbg_berry_curvature_multi(len(idxs), handles, _lib.iptr(nk), _lib.dptr(kcat), _lib.dptr(d),
                                                 spin_code(params.spin), float(params.eta), int(precision),
                                                 _lib.dptr(Om), _lib.dptr(E)), lib)
        o = 0
        for i, n in zip(idxs, nk):
            out[i] = (Om[o:o + n], E[o:o + n])
            o += int(n)
    return out


def _work_per_k(m: Model) -> float:
    N = m.nsta
    return 24.0 * m.nR * N * N + 46.0 * N ** 3


def _gpu_name() -> str:
    try:
        import subprocess

        r = subprocess.run(["nvidia-smi", "--query-gpu=name", "--format=csv,noheader", "-i", "0"],
                           capture_output=True, text=True, timeout=10)
        return r.stdout.strip() or "GPU"
    except Exception:
        return "GPU"


# --------------------------------------------------- native asynchronous queue
class AsyncJob:
    """A job queued on the library's own worker threads (``tbg_batch_submit``).

    Holds the input and output arrays until the job is reported done."""

    def __init__(self, lib, ticket: int, keep: tuple, result):
        self._lib = lib
        self.ticket = ticket
        self._keep = keep
        self._result = result
        self._status = None

    def _finish(self, status: int):
        self._status = status
        _lib.check(status, self._lib)
        return self._result()

    def poll(self):
        """None while running, else the result (raises the job's error)."""
        if self._status is not None:
            return self._finish(self._status)
        done, st = ctypes.c_int(0), ctypes.c_int(0)
        _lib.check(self._lib.tbg_batch_poll(self.ticket, ctypes.byref(done), ctypes.byref(st)), self._lib)
        return self._finish(st.value) if done.value else None

    def wait(self):
        if self._status is not None:
            return self._finish(self._status)
        st = ctypes.c_int(0)
        _lib.check(self._lib.tbg_batch_wait(self.ticket, ctypes.byref(st)), self._lib)
        return self._finish(st.value)


def _submit(job, keep, result) -> AsyncJob:
    lib = _lib.load()
    t = ctypes.c_int64(0)
    _lib.check(lib.tbg_batch_submit(ctypes.byref(job), ctypes.byref(t)), lib)
    return AsyncJob(lib, t.value, keep + (job,), result)


def submit_hall(model: Model, p: Parameters, precision=Precision.FP64) -> AsyncJob:
    """Asynchronous ``hall_conductivity`` (Direct); wait() -> conductivity (nmu)."""
    p.validate_rank2(model.dim)
    km = np.ascontiguousarray(p.kmesh, dtype=np.int64)
    d = _lib.as_f64(p.direction)
    mu = _lib.as_f64(p.mu)
    out = np.empty(len(mu))
    job = _lib.TbgJob(kind=_lib.JOB_HALL, model=model.device_handle(), kmesh=_lib.iptr(km), dirs2=_lib.dptr(d),
                      nmu=len(mu), mu=_lib.dptr(mu), T=float(p.T[0]), eta=float(p.eta), spin=spin_code(p.spin),
                      precision=int(precision), out0=_lib.dptr(out))
    return _submit(job, (km, d, mu, out), lambda: out)


def submit_bands(model: Model, k) -> AsyncJob:
    """Asynchronous ``solve_band_all_parallel``; wait() -> E (nk, nsta)."""
    k = _lib.as_f64(np.atleast_2d(k))
    E = np.empty((k.shape[0], model.nsta))
    job = _lib.TbgJob(kind=_lib.JOB_BANDS, model=model.device_handle(), nk=k.shape[0], k=_lib.dptr(k),
                      out0=_lib.dptr(E))
    return _submit(job, (k, E), lambda: E)


def submit_berry(model: Model, k, p: Parameters, precision=Precision.FP64) -> AsyncJob:
    """Asynchronous band-resolved Berry curvature; wait() -> (Omega, E)."""
    k = _lib.as_f64(np.atleast_2d(k))
    d = _lib.as_f64(p.direction)
    Om = np.empty((k.shape[0], model.nsta))
    E = np.empty((k.shape[0], model.nsta))
    job = _lib.TbgJob(kind=_lib.JOB_BERRY, model=model.device_handle(), nk=k.shape[0], k=_lib.dptr(k),
                      dirs2=_lib.dptr(d), eta=float(p.eta), spin=spin_code(p.spin), precision=int(precision),
                      out0=_lib.dptr(Om), out1=_lib.dptr(E))
    return _submit(job, (k, d, Om, E), lambda: (Om, E))


def submit_occupied(model: Model, k, p: Parameters, precision=Precision.FP64) -> AsyncJob:
    """Asynchronous occupied Berry curvature at mu = p.mu[0]; wait() -> (nk,)."""
    k = _lib.as_f64(np.atleast_2d(k))
    d = _lib.as_f64(p.direction)
    mu = _lib.as_f64(p.mu)
    out = np.empty(k.shape[0])
    job = _lib.TbgJob(kind=_lib.JOB_OCCUPIED, model=model.device_handle(), nk=k.shape[0], k=_lib.dptr(k),
                      dirs2=_lib.dptr(d), nmu=len(mu), mu=_lib.dptr(mu), T=float(p.T[0]), eta=float(p.eta),
                      spin=spin_code(p.spin), precision=int(precision), out0=_lib.dptr(out))
    return _submit(job, (k, d, mu, out), lambda: out)
