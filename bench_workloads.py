"""Measurements of the other k-mesh workloads (used by ``bench.py --workload``).

* ``haldane``   -- Haldane model, 200 x 200 mesh, sigma_xy at mu = 0 (Chern
                   number checked); a step is the whole mesh.
* ``supercell`` -- 1024-orbital 2D supercell, 9 R vectors, 64 x 64 mesh; a step
                   is one batch of mesh points (FP64: models above 256 bands
                   run the plain path).
* ``batched``   -- the first ``--models`` of the 512 seeded uneven models
                   (norb log-uniform in [4, 256], half 2D / half 3D, their full
                   meshes); a step is the whole set through BatchRunner.
* ``serve``     -- resident models, Poisson arrivals of (model, k-list of
                   1-4096 points, observable) requests at 20-100 % of the
                   measured peak; p50 / p99 latency per load.
* ``dos``       -- Model::dos of the reference's benchmark model (two-band
                   honeycomb, -3..3 eV, 500 bins, sigma 1e-2) on a
                   1000 x 1000 mesh; a step is the whole mesh.
* ``wilson``    -- hybrid Wannier centres (Berry::wannier_centre) of a random
                   spinful 2D model with 64 bands, 32 occupied, 64 loops of
                   64 points; a step is the whole set of loops.
* ``ec``        -- Hall conductivity with Integration::EnergyCut on the
                   reference's own ec_vs_reference case (Haldane t2 = -0.3,
                   101 x 101 mesh, 201 chemical potentials, eta = 0.05); a step
                   is the whole mesh.
* ``eig-small`` -- the FP64 eigensolvers for 9-32 bands: the Householder
                   solver (one warp per matrix up to 16 bands) and the
                   warp-per-matrix cyclic Jacobi solver on 9728 random
                   Hermitian matrices per size; a step is one solve of the set.
* ``w90``       -- Wannier90 loading: a 64-orbital, 125-R seedname_hr.dat
                   (512 000 lines, Wannier90's 5I5,2F12.6 format) read into a
                   device-resident model; a step is one load.

Each prints one JSON line in the bench.py format.  The CPU baseline of each
(``--impl reference``) is the C port of the reference path on the host cores.
"""

from __future__ import annotations

import json
import math
import os
import time

import numpy as np

from rustb_gb300 import _lib, batch, serve, workloads as W
from rustb_gb300.params import Parameters, Precision

METRIC_K = "k-pts/s (H+eig+Berry, norb=128) mixed vs FP64 GPU @AHC err≤1e-6; serve p99"


def _line(args, world, metric, value, unit, ms_per_step, dtype, config, extra):
    out = {"metric": metric, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": unit != "ms",
           "scaling": "weak", "vs_baseline": None, "dtype": dtype,
           "data": "synthetic (seeded models, numpy default_rng)", "config": config}
    out.update(extra)
    print(json.dumps(out), flush=True)


def _cpu_port(model, dirs, mu, kmesh, k0, nk, threads=None):
    from oracle import build_port

    build_port.load()
    threads = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    build_port.hall_sums(model, dirs, mu, 0.0, 1e-3, -1, kmesh=kmesh, k0=k0, nk=nk, threads=threads)
    return nk / (time.perf_counter() - t0), threads


def run(args, rank, world, local):
    if rank != 0 and args.impl == "reference":
        return 0
    fn = {"haldane": haldane, "supercell": supercell, "batched": batched, "serve": serve_bench,
          "dos": dos_bench, "w90": w90_bench, "wilson": wilson_bench, "ec": ec_bench,
          "eig-small": eig_small_bench}[args.workload]
    return fn(args, rank, world, local)


# ----------------------------------------------------------------- haldane --
def haldane(args, rank, world, local):
    model = W.haldane_200()
    mesh = (200, 200)
    nk = 40000
    dirs = np.eye(2)
    cfg = {"workload": "Haldane model (lattice [sqrt3,-1],[sqrt3,1]; t1=-1, t2=0.15i, M=0.2), 200x200 mesh, "
                       "sigma_xy at mu=0, T=0, eta=1e-3", "k_mesh": list(mesh)}
    if args.impl == "reference":
        val, thr = _cpu_port(model, dirs, [0.0], mesh, 0, nk)
        _line(args, world, METRIC_K, val, "k-pts/s", nk / val * 1e3, "f64", cfg,
              {"impl": "reference", "cpu_baseline": {"value": val, "unit": "k-pts/s", "cores": thr, "kind": "port",
                                                     "sample": "the whole 200x200 mesh"},
               "e2e": {"value": val, "unit": "k-pts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
        return 0
    lib = _lib.load()
    lib.tbg_set_device(local)
    p = Parameters.rank2(mesh, [1.0, 0.0], [0.0, 1.0], [0.0])
    rep = {}
    for _ in range(args.warmup):
        model.hall_conductivity(p)
    t_dev = 0.0
    l0 = lib.tbg_kernel_launch_count(0)
    for _ in range(args.steps):
        s = model.hall_conductivity(p, report=rep).conductivity[0]
        t_dev += rep["device_ms"] / 1e3
    launches = lib.tbg_kernel_launch_count(0) - l0
    val = args.steps * nk * world / t_dev
    # e2e: model upload + the whole mesh + sigma readback per step
    t0 = time.perf_counter()
    for _ in range(args.steps):
        m2 = W.haldane_200()
        m2.hall_conductivity(p)
        m2._invalidate()
    e2e = args.steps * nk / (time.perf_counter() - t0)
    cpu, thr = _cpu_port(model, dirs, [0.0], mesh, 0, nk)
    _line(args, world, METRIC_K, val, "k-pts/s", t_dev / args.steps * 1e3, "f64", cfg,
          {"chern": 2 * math.pi * s, "gpu_launches": int(launches),
           "cpu_baseline": {"value": cpu, "unit": "k-pts/s", "cores": thr, "kind": "port",
                            "sample": "the whole 200x200 mesh"},
           "e2e": {"value": e2e, "unit": "k-pts/s", "h2d_bytes_per_step": int(model.ham.nbytes + model.hamR.nbytes),
                   "d2h_bytes_per_step": 8}})
    return 0


# --------------------------------------------------------------- supercell --
def supercell(args, rank, world, local):
    model = W.supercell_2d()
    mesh = (64, 64)
    B = args.batch if args.batch != 8192 else 152
    dirs = np.eye(2)
    cfg = {"workload": "2D supercell, 1024 orbitals, R in {-1,0,1}^2, t=exp(-d/0.8) N(0,1) complex, onsite "
                       "U(-0.5,0.5), 64x64 mesh, sigma_xy at mu=0", "k_mesh": list(mesh), "batch_kpts": B}
    if args.impl == "reference":
        n = max(1, (os.cpu_count() or 1))
        val, thr = _cpu_port(model, dirs, [0.0], mesh, 0, n)
        _line(args, world, METRIC_K, val, "k-pts/s", n / val * 1e3, "f64", cfg,
              {"impl": "reference", "cpu_baseline": {"value": val, "unit": "k-pts/s", "cores": thr, "kind": "port",
                                                     "sample": f"{n} k-points of the 64x64 mesh"},
               "e2e": {"value": val, "unit": "k-pts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
        return 0
    lib = _lib.load()
    lib.tbg_set_device(local)
    h = model.device_handle()
    import ctypes

    km = np.ascontiguousarray(mesh, dtype=np.int64)
    mu = np.array([0.0])
    out = np.zeros(1)
    rep = _lib.TbgReport()

    def step(s):
        k0 = (s * B) % 4096
        _lib.check(lib.tbg_hall_sums_range(h, _lib.iptr(km), k0, min(B, 4096 - k0), _lib.dptr(dirs), 1,
                                           _lib.dptr(mu), 0.0, 1e-3, -1, int(Precision.MIXED), _lib.dptr(out),
                                           ctypes.byref(rep)), lib)
        return rep.device_ms / 1e3

    for w in range(args.warmup):
        step(w)
    lib.tbg_kernel_timing_enable(1)
    _lib.kernel_timing(reset=True)
    t = sum(step(args.warmup + s) for s in range(args.steps))
    lib.tbg_kernel_timing_enable(0)
    timing = _lib.kernel_timing(reset=True)
    val = args.steps * B * world / t
    prec_ran = int(rep.precision)
    # mixed vs plain FP64 on the same 16 k-points (the FP64 solver takes about a second for them)
    acc = None
    if rank == 0 and prec_ran == int(Precision.MIXED):
        sums = {}
        for prec in (Precision.FP64, Precision.MIXED):
            _lib.check(lib.tbg_hall_sums_range(h, _lib.iptr(km), 0, 16, _lib.dptr(dirs), 1, _lib.dptr(mu), 0.0,
                                               1e-3, -1, int(prec), _lib.dptr(out), None), lib)
            sums[int(prec)] = float(out[0])
        p64 = sums[int(Precision.FP64)]
        acc = {"ahc_partial_rel_err_mixed_vs_fp64": abs(sums[int(Precision.MIXED)] - p64) / abs(p64),
               "sample": "flat k indices [0, 16) of the 64x64 mesh"}
        from oracle import build_port
        from oracle import tb_oracle as O

        port = float(np.sum(build_port.hall_sums(model, dirs, mu, 0.0, 1e-3, -1, kmesh=mesh, k0=0, nk=16)))
        acc["fp64_vs_port_rel"] = abs(p64 - port) / abs(port)
        acc["mixed_vs_port_rel"] = abs(sums[int(Precision.MIXED)] - port) / abs(port)
        # the configuration's stated output: Omega of the 20 bands nearest E = 0
        # (berry_curvature_at) at one mesh point, MIXED, against the numpy oracle
        kq = O.gen_kmesh(mesh)[1000:1001]
        pq = Parameters.rank2((1, 1), [1.0, 0.0], [0.0, 1.0], [0.0])
        Om, E = model.berry_curvature_on(kq, pq, Precision.MIXED)
        Omr, Er = O.berry_on(model, kq, dirs)
        sel = np.sort(np.argsort(np.abs(E[0]), kind="stable")[:20])
        acc["bands_near_zero"] = {
            "k": kq[0].tolist(), "bands": sel.tolist(), "E": E[0][sel].tolist(), "Omega": Om[0][sel].tolist(),
            "omega_rel_err_vs_oracle": float(np.max(np.abs(Om[0][sel] - Omr[0][sel])) / np.max(np.abs(Omr[0][sel]))),
            "E_err_over_normH": float(np.max(np.abs(E[0] - Er[0])) / np.linalg.norm(O.gen_ham(model, kq[0]), 2))}
    dtype = "f32 eigensolve + f64-class refinement (tcgen05, K in chunks of 256)" if prec_ran == int(Precision.MIXED) \
        else "f64"
    _line(args, world, METRIC_K, val, "k-pts/s", t / args.steps * 1e3, dtype, cfg,
          {"precision_ran": prec_ran, "accuracy": acc,
           "kernel_times_ms": {k: {"launches": v[0], "total_ms": v[1]} for k, v in timing.items()},
           "flops_per_k": 24.0 * model.nR * 1024 ** 2 + 46.0 * 1024 ** 3})
    return 0


# ----------------------------------------------------------------- batched --
def _batched_jobs(n_models):
    specs = W.batched_uneven_specs(512)[:n_models]
    jobs = []
    for dim, norb, mesh, seed in specs:
        m = W.random_model(dim, norb, False, 3, seed=seed)
        dirs = np.eye(dim)[:2]
        jobs.append(batch.Job(m, Parameters(kmesh=mesh, direction=dirs, mu=[0.0])))
    return jobs


def batched(args, rank, world, local):
    # 512 specs alternate 2D/3D by halves: take the subset from both halves
    n = args.models
    specs_all = W.batched_uneven_specs(512)
    idx = list(range(n // 2)) + list(range(256, 256 + n - n // 2))
    kcap = args.kcap if args.kcap > 0 else None
    jobs = []
    for i in idx:
        dim, norb, mesh, seed = specs_all[i]
        m = W.random_model(dim, norb, False, 3, seed=seed)
        jobs.append(batch.Job(m, Parameters(kmesh=mesh, direction=np.eye(dim)[:2], mu=[0.0]), k_limit=kcap))
    nk = sum(j.k_count() for j in jobs)
    flops = sum(j.k_count() * batch._work_per_k(j.model) for j in jobs)
    cfg = {"workload": f"batched uneven: {len(jobs)} of the 512 seeded models (norb log-uniform [4,256], half 2D "
                       "R|<=3 (49 R), half 3D (343 R), meshes 32^2-128^2 / 16^3-48^3), sigma_xy mu=0"
                       + (f", the first {kcap} points of each mesh" if kcap else ", whole meshes"),
           "models": len(jobs), "k_points": nk}
    if args.impl == "reference":
        j = max(jobs, key=lambda j: j.model.nsta)
        sample = 64
        val, thr = _cpu_port(j.model, j.params.direction, [0.0], j.params.kmesh, 0, sample)
        val_flops = val * batch._work_per_k(j.model)
        _line(args, world, "algorithmic GFLOP/s (batched uneven models)", val_flops / 1e9, "GFLOP/s", 0.0, "f64", cfg,
              {"impl": "reference", "cpu_baseline": {"value": val_flops / 1e9, "unit": "GFLOP/s", "cores": thr,
                                                     "kind": "port", "sample": f"{sample} k of the largest model"},
               "e2e": {"value": val_flops / 1e9, "unit": "GFLOP/s", "h2d_bytes_per_step": 0,
                       "d2h_bytes_per_step": 0}})
        return 0
    lib = _lib.load()
    lib.tbg_set_device(local)
    runner = batch.BatchRunner(Precision.MIXED, autotune=True)
    runner.hall_many(jobs)  # warm-up + autotune
    t0 = time.perf_counter()
    for _ in range(args.steps):
        runner.hall_many(jobs)
    dt = (time.perf_counter() - t0) / args.steps
    # per-bucket breakdown: the same jobs, one bucket at a time
    per_bucket = {}
    for b in sorted({batch.bucket_of(j.model.nsta) for j in jobs}):
        sub = [j for j in jobs if batch.bucket_of(j.model.nsta) == b]
        t1 = time.perf_counter()
        runner.hall_many(sub)
        tb = time.perf_counter() - t1
        fb = sum(j.k_count() * batch._work_per_k(j.model) for j in sub)
        per_bucket[str(b)] = {"models": len(sub), "seconds": tb, "tflops": fb / tb / 1e12}
    # the per-k outputs of the batched workload (eigenvalues and Berry curvature at every k): models of
    # equal band count stacked into one pipeline each (tbg_berry_curvature_multi)
    def mesh_head(mesh, n):
        idx = np.arange(min(n, int(np.prod(mesh))))
        cols, rest = [], idx
        for d in reversed(range(len(mesh))):  # gen_kmesh order: first dimension outermost
            cols.append((rest % mesh[d]) / mesh[d])
            rest = rest // mesh[d]
        return np.ascontiguousarray(np.stack(cols[::-1], axis=1))
    kper = [mesh_head(j.params.kmesh, j.k_count()) for j in jobs]
    pb = {2: Parameters(kmesh=(1, 1), direction=np.eye(2), mu=[0.0]),
          3: Parameters(kmesh=(1, 1, 1), direction=np.eye(3)[:2], mu=[0.0])}

    def berry_all():
        for dim in (2, 3):
            sel = [i for i, j in enumerate(jobs) if j.model.dim == dim]
            batch.berry_curvature_many([jobs[i].model for i in sel], [kper[i] for i in sel], pb[dim], Precision.MIXED)
    berry_all()  # warm-up
    t0 = time.perf_counter()
    berry_all()
    dtb = time.perf_counter() - t0
    groups = len({(j.model.nsta, j.model.dim) for j in jobs})
    _line(args, world, "algorithmic GFLOP/s (batched uneven models)", flops / dt / 1e9, "GFLOP/s", dt * 1e3,
          "f32 eigensolve + exact-slice tensor products", cfg,
          {"k_pts_per_s": nk / dt, "plan": runner.stats["plan"], "items": runner.stats["items"],
           "workers": runner.stats["workers"], "per_bucket": per_bucket,
           "per_k_outputs": {"what": "eigenvalues and Berry curvature at every k-point (berry_curvature_many: "
                                     "models of equal band count and dimension stacked into one pipeline)",
                             "seconds": dtb, "gflops": flops / dtb / 1e9, "k_pts_per_s": nk / dtb,
                             "stacked_groups": groups}})
    return 0


# ------------------------------------------------------------------- serve --
def serve_bench(args, rank, world, local):
    rng = np.random.default_rng(20260105)
    models = {}
    for i in range(16):
        dim = 2 if i % 2 == 0 else 3
        norb = int(round(math.exp(rng.uniform(math.log(4), math.log(256)))))
        models[i] = W.random_model(dim, norb, False, 3, seed=500 + i)
    cfg = {"workload": "serving: 16 resident seeded models (norb log-uniform [4,256]), requests of 1-4096 random "
                       "k-points, observable uniform in {bands, berry, sigma_xy}, Poisson arrivals",
           "models": len(models)}
    if args.impl == "reference":
        _line(args, world, "p99 latency (serving, 80% load)", None, "ms", 0.0, "f64", cfg,
              {"impl": "reference", "unavailable": "the reference has no serving loop; see the k-pts/s arms"})
        return 0
    lib = _lib.load()
    lib.tbg_set_device(local)

    def make_req():
        mid = int(rng.integers(0, len(models)))
        nk = int(rng.integers(1, 4097))
        obs = serve.OBSERVABLES[int(rng.integers(0, 3))]
        return serve.Request(mid, rng.uniform(0, 1, (nk, models[mid].dim)), obs)

    for _ in range(6):  # warm-up of every code path
        r = make_req()
        serve.execute(models[r.model_id], r)
    # peak: a saturating burst
    srv = serve.Server(models, hbm_budget_bytes=96 << 30, max_inflight=8)
    burst = [make_req() for _ in range(64)]
    t0 = time.perf_counter()
    futs = [srv.submit(r) for r in burst]
    for f in futs:
        f.result()
    t_burst = time.perf_counter() - t0
    srv.close()
    peak_req = len(burst) / t_burst
    peak_k = sum(len(r.k) for r in burst) / t_burst
    loads = {}
    for frac in (0.2, 0.4, 0.6, 0.8, 1.0):
        srv = serve.Server(models, hbm_budget_bytes=96 << 30, max_inflight=8)
        rate = frac * peak_req
        t_end = time.perf_counter() + args.serve_seconds
        futs = []
        kpts = 0
        t_start = time.perf_counter()
        while time.perf_counter() < t_end:
            r = make_req()
            kpts += len(r.k)
            futs.append(srv.submit(r))
            time.sleep(rng.exponential(1.0 / rate))
        for f in futs:
            f.result()
        wall = time.perf_counter() - t_start
        srv.close()
        lat = srv.latencies() * 1e3
        loads[f"{int(frac * 100)}%"] = {"requests": len(futs), "p50_ms": float(np.percentile(lat, 50)),
                                        "p99_ms": float(np.percentile(lat, 99)), "k_pts_per_s": kpts / wall}
    p99_80 = loads["80%"]["p99_ms"]
    _line(args, world, "p99 latency (serving, 80% load)", p99_80, "ms", p99_80, "f32 eigensolve + exact-slice tensor products",
          cfg, {"loads": loads, "peak_requests_per_s": peak_req, "peak_k_pts_per_s": peak_k})
    return 0


# --------------------------------------------------------------------- dos --
DOS_METRIC = "k-pts/s (Model::dos: band energies + Gaussian sum)"


def _cpu_dos(model, mesh, E_min, E_max, E_n, sigma, nk, threads=None):
    from oracle import build_port

    build_port.load()
    threads = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    build_port.dos_sums(model, mesh, E_min, E_max, E_n, sigma, 0, nk, threads=threads)
    return nk / (time.perf_counter() - t0), threads


# ncu: DRAM bytes (read + write) of one dos_kernel launch over the whole
# 1000 x 1000 mesh (one chunk)
DOS_KERNEL_DRAM_BYTES = 16.02e6


def _dos_roofline(lib, model, mesh, E_min, E_max, E_n, sigma, timing):
    """dos_kernel against the FP64 pipe.  Work unit: one in-window Gaussian term
    (|E_i - x| <= 38.6 sigma, the terms that are non-zero in FP64); the table
    method needs at least 3 FP64 operations per term (two recurrence multiplies,
    one add into the bin), so the peak is the measured FP64 FMA issue rate / 3."""
    import ctypes

    if "dos_kernel" not in timing:
        return None
    launches, ms, _ = timing["dos_kernel"]
    ev = model.solve_band_mesh(mesh).reshape(-1)
    step = (E_max - E_min) / (E_n - 1)
    w = 38.6 * sigma
    lo = np.clip(np.ceil((ev - w - E_min) / step), 0, E_n - 1)
    hi = np.clip(np.floor((ev + w - E_min) / step), 0, E_n - 1)
    inside = (ev + w >= E_min) & (ev - w <= E_min + step * (E_n - 1))
    terms = float(np.sum(np.where(inside, hi - lo + 1, 0)))
    p64 = ctypes.c_double(0.0)
    p32 = ctypes.c_double(0.0)
    lib.tbg_measure_fma_peaks(ctypes.byref(p64), ctypes.byref(p32))
    avg_s = ms / 1e3 / max(launches, 1)
    achieved = terms / avg_s / 1e9
    peak = p64.value * 1e12 / 2.0 / 3.0 / 1e9
    return {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "Gterms/s",
            "frac": achieved / peak if peak > 0 else None, "traffic": DOS_KERNEL_DRAM_BYTES,
            "traffic_unit": "bytes per launch (ncu dram read + write)", "kernel": "dos_kernel",
            "terms_per_launch": terms, "avg_launch_ms": avg_s * 1e3,
            "peak_source": "FP64 FMA loop on this GPU (tbg_measure_fma_peaks) / 2 flops / 3 ops per term"}


def dos_bench(args, rank, world, local):
    model = W.honeycomb_small()
    mesh = (1000, 1000)
    nk = mesh[0] * mesh[1]
    E_min, E_max, E_n, sigma = -3.0, 3.0, 500, 1e-2
    cfg = {"workload": "Model::dos, two-band honeycomb (onsite -0.7/+0.7, t=-1), 1000x1000 mesh, "
                       "E in [-3, 3] with 500 points, sigma = 1e-2", "k_mesh": list(mesh), "E_n": E_n,
           "sigma": sigma}
    sample = 40000
    if args.impl == "reference":
        val, thr = _cpu_dos(model, mesh, E_min, E_max, E_n, sigma, sample)
        _line(args, world, DOS_METRIC, val, "k-pts/s", nk / val * 1e3, "f64", cfg,
              {"impl": "reference", "cpu_baseline": {"value": val, "unit": "k-pts/s", "cores": thr, "kind": "port",
                                                     "sample": f"the first {sample} k-points of the mesh"},
               "e2e": {"value": val, "unit": "k-pts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
        return 0
    lib = _lib.load()
    lib.tbg_set_device(local)
    for _ in range(args.warmup):
        model.dos(mesh, E_min, E_max, E_n, sigma)
    lib.tbg_kernel_timing_enable(1)
    _lib.kernel_timing(reset=True)
    l0 = lib.tbg_kernel_launch_count(0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        E, d = model.dos(mesh, E_min, E_max, E_n, sigma)
    wall = time.perf_counter() - t0
    launches = lib.tbg_kernel_launch_count(0) - l0
    lib.tbg_kernel_timing_enable(0)
    timing = _lib.kernel_timing(reset=True)
    t_dev = sum(v[1] for v in timing.values()) / 1e3
    # whole call with the model resident: launches, the device work and the read-back
    val = args.steps * nk * world / wall
    # e2e: model upload, the whole mesh and the DOS read-back per step
    t0 = time.perf_counter()
    for _ in range(args.steps):
        m2 = W.honeycomb_small()
        m2.dos(mesh, E_min, E_max, E_n, sigma)
        m2._invalidate()
    e2e = args.steps * nk / (time.perf_counter() - t0)
    cpu, thr = _cpu_dos(model, mesh, E_min, E_max, E_n, sigma, sample)
    _line(args, world, DOS_METRIC, val, "k-pts/s", wall / args.steps * 1e3, "f64", cfg,
          {"roofline": _dos_roofline(lib, model, mesh, E_min, E_max, E_n, sigma, timing),
           "gpu_launches": int(launches), "states_integral": float(d.sum() * (E[1] - E[0])),
           "kernel_ms_per_step": t_dev / args.steps * 1e3,
           "kernel_times_ms": {k: {"launches": v[0], "total_ms": v[1]} for k, v in timing.items()},
           "cpu_baseline": {"value": cpu, "unit": "k-pts/s", "cores": thr, "kind": "port",
                            "sample": f"the first {sample} k-points of the mesh"},
           "e2e": {"value": e2e, "unit": "k-pts/s", "h2d_bytes_per_step": int(model.ham.nbytes + model.hamR.nbytes),
                   "d2h_bytes_per_step": 8 * E_n}})
    return 0


# --------------------------------------------------------------------- w90 --
W90_METRIC = "MB/s (Wannier90 _hr.dat -> device-resident model)"


def write_w90_dataset(d: str, seed_name: str, model) -> int:
    """Write ``model``'s tables as seedname_hr.dat (unit weights, Wannier90's
    5I5,2F12.6 lines, column-major blocks) plus a minimal .win; returns the
    _hr.dat size in bytes."""
    os.makedirs(d, exist_ok=True)
    n, nR = model.nsta, model.nR
    head = f"written for the w90 workload\n{n:12d}\n{nR:12d}\n"
    w = ["".join(f"{1:5d}" for _ in range(min(15, nR - i))) for i in range(0, nR, 15)]
    jj, ii = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")  # j outer, i inner
    rows = []
    for r in range(nR):
        R = model.hamR[r]
        h = model.ham[r][ii.reshape(-1), jj.reshape(-1)]
        block = np.empty((n * n, 7))
        block[:, 0:3] = R
        block[:, 3] = ii.reshape(-1) + 1
        block[:, 4] = jj.reshape(-1) + 1
        block[:, 5] = h.real
        block[:, 6] = h.imag
        rows.append(block)
    path = os.path.join(d, seed_name + "_hr.dat")
    with open(path, "w") as f:
        f.write(head + "\n".join(w) + "\n")
        np.savetxt(f, np.concatenate(rows), fmt="%5d%5d%5d%5d%5d%12.6f%12.6f")
    lat = model.lat
    win = ["begin unit_cell_cart", "Ang"] + [" ".join(f"{x:.10f}" for x in lat[i]) for i in range(3)]
    win += ["end unit_cell_cart", "", "begin projections", "Fe:" + ",".join(["s"] * n), "end projections", "",
            "begin atoms_frac", "Fe 0.0 0.0 0.0", "end atoms_frac"]
    with open(os.path.join(d, seed_name + ".win"), "w") as f:
        f.write("\n".join(win) + "\n")
    return os.path.getsize(path)


def w90_bench(args, rank, world, local):
    import ctypes
    import shutil
    import tempfile

    from rustb_gb300.model import Model

    src = W.random_model(3, 64, False, 2, seed=20260107)
    cfg = {"workload": "Wannier90 seedname_hr.dat of a random 64-orbital model, R in {-2..2}^3 (125 R, "
                       "512 000 lines, 5I5,2F12.6) + .win, loaded to a device-resident model",
           "nsta": src.nsta, "n_R": src.nR}
    tmp = tempfile.mkdtemp(prefix="w90_")
    try:
        size = write_w90_dataset(tmp, "bench", src)
        mb = size / 1e6
        hr = os.path.join(tmp, "bench_hr.dat")

        def port_once():
            from oracle import build_port

            build_port.load()
            t0 = time.perf_counter()
            build_port.read_hr(hr, src.nR * src.nsta ** 2)
            return mb / (time.perf_counter() - t0)

        if args.impl == "reference":
            vals = [port_once() for _ in range(max(1, args.steps))]
            val = float(np.median(vals))
            _line(args, world, W90_METRIC, val, "MB/s", mb / val * 1e3, "f64", cfg,
                  {"impl": "reference", "cpu_baseline": {"value": val, "unit": "MB/s", "cores": 1, "kind": "port",
                                                         "sample": f"the whole {mb:.1f} MB _hr.dat"},
                   "e2e": {"value": val, "unit": "MB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
            return 0
        lib = _lib.load()
        lib.tbg_set_device(local)

        def tables_once():
            # native table reader + upload of the tables (the device-resident part)
            h = ctypes.c_void_p()
            t0 = time.perf_counter()
            _lib.check(lib.tbg_w90_read_hr(hr.encode(), 0.0, ctypes.byref(h)), lib)
            nsta, nR = ctypes.c_int64(), ctypes.c_int64()
            lib.tbg_w90_info(h, ctypes.byref(nsta), ctypes.byref(nR), None)
            ham = np.empty((nR.value, nsta.value, nsta.value), dtype=np.complex128)
            hamR = np.empty((nR.value, 3), dtype=np.int64)
            lib.tbg_w90_copy(h, _lib.dptr(ham.view(np.float64)), _lib.iptr(hamR), None)
            lib.tbg_w90_free(h)
            m = Model(src.lat, np.zeros((nsta.value, 3)), False, ham=ham, hamR=hamR)
            m.device_handle()
            lib.tbg_set_device(local)
            dt = time.perf_counter() - t0
            m._invalidate()
            return dt

        for _ in range(args.warmup):
            tables_once()
        t = [tables_once() for _ in range(args.steps)]
        val = args.steps * mb * world / sum(t)
        # e2e: Model.from_hr (hr + win), then the upload, per step
        t0 = time.perf_counter()
        for _ in range(args.steps):
            m = Model.from_hr(tmp + "/", "bench", 0.0)
            m.device_handle()
            m._invalidate()
        e2e = args.steps * mb / (time.perf_counter() - t0)
        cpu = port_once()
        _line(args, world, W90_METRIC, val, "MB/s", sum(t) / args.steps * 1e3, "f64", cfg,
              {"roofline": None, "bound": "host parse (all host threads) + one H2D copy of the tables",
               "gpu_launches": 0, "threads": os.cpu_count(),
               "cpu_baseline": {"value": cpu, "unit": "MB/s", "cores": 1, "kind": "port",
                                "sample": f"the whole {mb:.1f} MB _hr.dat, line by line on one thread"},
               "e2e": {"value": e2e, "unit": "MB/s", "h2d_bytes_per_step": int(src.ham.nbytes + src.hamR.nbytes),
                       "d2h_bytes_per_step": 0}})
        return 0
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


# ------------------------------------------------------------------ wilson --
WILSON_METRIC = "Wilson loops/s (wannier_centre: eigenvectors, overlaps, unitary factors, eigenphases)"


def wilson_bench(args, rank, world, local):
    from oracle import tb_oracle as O

    model = W.random_model(2, 32, True, 1, seed=20260108)
    occ = list(range(32))
    nk1 = nk2 = 64
    cfg = {"workload": "Berry::wannier_centre of a random spinful 2D model (32 orbitals, 64 bands, R in "
                       "{-1,0,1}^2), occupied bands 0..31, 64 loops along k2 of 64 points; mixed eigenpairs",
           "nsta": model.nsta,
           "n_occ": len(occ), "loops": nk1, "points_per_loop": nk2}
    sample = 2

    def cpu_once():
        t0 = time.perf_counter()
        for i in range(sample):
            loop = np.array([[i / (nk1 - 1), j / (nk2 - 1)] for j in range(nk2)])
            O.wilson_loop(model, loop, occ)
        return sample / (time.perf_counter() - t0)

    if args.impl == "reference":
        val = cpu_once()
        _line(args, world, WILSON_METRIC, val, "loops/s", 1e3 / val, "f64", cfg,
              {"impl": "reference", "cpu_baseline": {"value": val, "unit": "loops/s", "cores": 1, "kind": "port",
                                                     "sample": f"{sample} of the loops (numpy + LAPACK per loop)"},
               "e2e": {"value": val, "unit": "loops/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
        return 0
    lib = _lib.load()
    lib.tbg_set_device(local)
    # FP64 eigenpairs (the drop-in) once for the accuracy and speed comparison
    args64 = (occ, [0.0, 0.0], [1.0, 0.0], [0.0, 1.0], nk1, nk2, Precision.FP64)
    model.wannier_centre(*args64)
    t0 = time.perf_counter()
    w64 = model.wannier_centre(*args64)
    fp64_val = nk1 / (time.perf_counter() - t0)
    args0 = (occ, [0.0, 0.0], [1.0, 0.0], [0.0, 1.0], nk1, nk2, Precision.MIXED)
    for _ in range(args.warmup):
        model.wannier_centre(*args0)
    lib.tbg_kernel_timing_enable(1)
    _lib.kernel_timing(reset=True)
    l0 = lib.tbg_kernel_launch_count(0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        wcc = model.wannier_centre(*args0)
    wall = time.perf_counter() - t0
    launches = lib.tbg_kernel_launch_count(0) - l0
    lib.tbg_kernel_timing_enable(0)
    timing = _lib.kernel_timing(reset=True)
    val = args.steps * nk1 * world / wall
    # e2e: model upload + the loops + the centres read back, per step
    t0 = time.perf_counter()
    for _ in range(args.steps):
        m2 = W.random_model(2, 32, True, 1, seed=20260108)
        m2.wannier_centre(*args0)
        m2._invalidate()
    e2e = args.steps * nk1 / (time.perf_counter() - t0)
    # roofline: the kernel family with the largest device time, against the FP64 pipe
    name, (ln, ms, work) = max(timing.items(), key=lambda kv: kv[1][1])
    import ctypes

    p64 = ctypes.c_double(0.0)
    p32 = ctypes.c_double(0.0)
    lib.tbg_measure_fma_peaks(ctypes.byref(p64), ctypes.byref(p32))
    ach = work / (ms / 1e3) / 1e12 if work > 0 and ms > 0 else None
    if name.startswith(("heev_kernel<float", "hetrd_tc", "bt_tc")):
        bound, peak, src = "fp32", p32.value, "FP32 FMA loop on this GPU (tbg_measure_fma_peaks); 14 N^3 per eigensolve"
    elif name.startswith("ozaki"):
        mp = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "MEASURED_PEAKS.json")
        bf16 = json.load(open(mp)).get("bf16_tflops", 1900.0) if os.path.exists(mp) else 1900.0
        pairs = 6 if "low" in name else (15 if "mid" in name else 21)
        bound, peak, src = "tensor", bf16 / pairs, f"MEASURED_PEAKS.json bf16_tflops / {pairs} slice products"
    else:
        bound, peak, src = "fp64", p64.value, "FP64 FMA loop on this GPU (tbg_measure_fma_peaks)"
    roof = {"bound": bound, "achieved": ach, "peak": peak, "unit": "TFLOP/s",
            "frac": ach / peak if ach and peak else None, "traffic": None, "kernel": name,
            "launches": ln, "avg_launch_ms": ms / max(ln, 1), "peak_source": src}
    cpu = cpu_once()
    dphi = np.abs(np.exp(1j * np.sort(wcc, axis=0)) - np.exp(1j * np.sort(w64, axis=0)))
    _line(args, world, WILSON_METRIC, val, "loops/s", wall / args.steps * 1e3,
          "f32 eigensolve + f64-class refinement; f64 overlaps and phases", cfg,
          {"roofline": roof, "gpu_launches": int(launches), "wcc_shape": list(wcc.shape),
           "fp64": {"value": fp64_val, "unit": "loops/s"},
           "accuracy": {"max_phase_diff_mixed_vs_fp64": float(dphi.max())},
           "kernel_times_ms": {k: {"launches": v[0], "total_ms": v[1]} for k, v in timing.items()},
           "cpu_baseline": {"value": cpu, "unit": "loops/s", "cores": 1, "kind": "port",
                            "sample": f"{sample} of the loops (numpy + LAPACK per loop, one thread)"},
           "e2e": {"value": e2e, "unit": "loops/s", "h2d_bytes_per_step": int(model.ham.nbytes + model.hamR.nbytes),
                   "d2h_bytes_per_step": int(wcc.nbytes)}})
    return 0


# ---------------------------------------------------------------------- ec --
EC_METRIC = "k-pts/s (hall_conductivity, Integration::EnergyCut)"


def _haldane_2d(t2_imag: float):
    from rustb_gb300.model import Model

    s3 = math.sqrt(3.0)
    m = Model.tb_model([[1.0, 0.0], [0.5, s3 / 2.0]], [[1.0 / 3.0, 1.0 / 3.0], [2.0 / 3.0, 2.0 / 3.0]])
    m.set_onsite([-0.7, 0.7])
    for R in [(0, 0), (-1, 0), (0, -1)]:
        m.add_hop(-1.0, 0, 1, R)
    for R in [(1, 0), (-1, 1), (0, -1)]:
        m.add_hop(t2_imag * 1j, 0, 0, R)
    for R in [(-1, 0), (1, -1), (0, 1)]:
        m.add_hop(t2_imag * 1j, 1, 1, R)
    return m


def ec_bench(args, rank, world, local):
    from rustb_gb300.params import Integration

    model = _haldane_2d(-0.3)
    mesh = (101, 101)
    nk = mesh[0] * mesh[1]
    mu = np.linspace(-3.0, 3.0, 201)
    p = Parameters.rank2(mesh, [1.0, 0.0], [0.0, 1.0], list(mu))
    p.eta = 0.05
    p.integration = Integration.EnergyCut
    cfg = {"workload": "Haldane (t2 = -0.3 i, onsite -/+0.7), 101x101 mesh, 201 mu in [-3, 3], eta = 0.05, T = 0, "
                       "Integration::EnergyCut", "k_mesh": list(mesh), "n_mu": len(mu)}
    sample = (21, 21)

    def cpu_once():
        from oracle import tb_oracle as O

        t0 = time.perf_counter()
        O.hall_energy_cut(model, list(sample), np.eye(2), mu, 0.0, 0.05)
        return sample[0] * sample[1] / (time.perf_counter() - t0)

    if args.impl == "reference":
        val = cpu_once()
        _line(args, world, EC_METRIC, val, "k-pts/s", nk / val * 1e3, "f64", cfg,
              {"impl": "reference", "cpu_baseline": {"value": val, "unit": "k-pts/s", "cores": 1, "kind": "port",
                                                     "sample": "the same model on a 21x21 mesh (numpy restatement)"},
               "e2e": {"value": val, "unit": "k-pts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
        return 0
    lib = _lib.load()
    lib.tbg_set_device(local)
    for _ in range(args.warmup):
        model.hall_conductivity(p)
    lib.tbg_kernel_timing_enable(1)
    _lib.kernel_timing(reset=True)
    l0 = lib.tbg_kernel_launch_count(0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sig = model.hall_conductivity(p).conductivity
    wall = time.perf_counter() - t0
    launches = lib.tbg_kernel_launch_count(0) - l0
    lib.tbg_kernel_timing_enable(0)
    timing = _lib.kernel_timing(reset=True)
    val = args.steps * nk * world / wall
    t0 = time.perf_counter()
    for _ in range(args.steps):
        m2 = _haldane_2d(-0.3)
        m2.hall_conductivity(p)
        m2._invalidate()
    e2e = args.steps * nk / (time.perf_counter() - t0)
    dev_ms = sum(v[1] for v in timing.values()) / args.steps
    name, (ln, ms, work) = max(timing.items(), key=lambda kv: kv[1][1])
    cpu = cpu_once()
    _line(args, world, EC_METRIC, val, "k-pts/s", wall / args.steps * 1e3, "f64", cfg,
          {"roofline": {"bound": "fp64 / latency", "achieved": None, "peak": None, "unit": None, "frac": None,
                        "traffic": None, "kernel": name, "share_of_device_time": ms / args.steps / max(dev_ms, 1e-9),
                        "note": "host band tracking and launch latency dominate at this size; per-kernel times "
                                "in kernel_times_ms"},
           "gpu_launches": int(launches), "device_ms_per_step": dev_ms,
           "chern_mu0": float(sig[100] * 2 * math.pi),
           "kernel_times_ms": {k: {"launches": v[0], "total_ms": v[1]} for k, v in timing.items()},
           "cpu_baseline": {"value": cpu, "unit": "k-pts/s", "cores": 1, "kind": "port",
                            "sample": "the same model on a 21x21 mesh (numpy restatement, one thread)"},
           "e2e": {"value": e2e, "unit": "k-pts/s", "h2d_bytes_per_step": int(model.ham.nbytes + model.hamR.nbytes),
                   "d2h_bytes_per_step": int(sig.nbytes)}})
    return 0


# --------------------------------------------------------------- eig-small --
def eig_small_bench(args, rank, world, local):
    """Matrices/s of the two FP64 solvers for 9-32 bands (CUDA events around
    the solver launch on a device copy; the headline is 32 bands through the
    solver the driver picks).  The reference arm times numpy's LAPACK eigh."""
    import ctypes

    sizes = [9, 12, 16, 20, 24, 32]
    nk = 152 * 64
    cfg = {"workload": f"random Hermitian complex matrices, {nk} per size, 9-32 bands", "sizes": sizes,
           "l2": "inputs copied to a fresh device buffer before each timed solve"}
    if args.impl == "reference":
        rng = np.random.default_rng(32)
        X = rng.standard_normal((512, 32, 32)) + 1j * rng.standard_normal((512, 32, 32))
        H = 0.5 * (X + np.conj(np.transpose(X, (0, 2, 1))))
        np.linalg.eigh(H[:8])
        t0 = time.perf_counter()
        for _ in range(args.steps):
            np.linalg.eigh(H)
        val = 512 * args.steps / (time.perf_counter() - t0)
        thr = os.cpu_count() or 1
        _line(args, world, "matrices/s (FP64 eigenpairs, 32 bands)", val, "matrices/s", 512 / val * 1e3, "f64", cfg,
              {"impl": "reference", "cpu_baseline": {"value": val, "unit": "matrices/s", "cores": thr, "kind": "port",
                                                      "sample": "512 random 32-band matrices, numpy LAPACK eigh"},
               "e2e": {"value": val, "unit": "matrices/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
        return 0
    lib = _lib.load()
    dp = ctypes.POINTER(ctypes.c_double)
    fn = lib.tbg_internal_eig_f64
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.c_int64, dp, dp, dp, ctypes.c_int, ctypes.c_int,
                   ctypes.POINTER(ctypes.c_float)]
    by_n = {}
    for n in sizes:
        rng = np.random.default_rng(n)
        X = rng.standard_normal((nk, n, n)) + 1j * rng.standard_normal((nk, n, n))
        H = np.ascontiguousarray(0.5 * (X + np.conj(np.transpose(X, (0, 2, 1)))))
        E = np.zeros((nk, n))
        U = np.zeros((nk, n, n), dtype=np.complex128)
        row = {}
        for method, name in ((0, "householder"), (1, "jacobi")):
            ms = ctypes.c_float(0.0)
            for reps in (max(args.warmup, 1), max(args.steps, 1)):
                _lib.check(fn(n, nk, H.view(np.float64).ctypes.data_as(dp), E.ctypes.data_as(dp),
                              U.view(np.float64).ctypes.data_as(dp), method, reps, ctypes.byref(ms)), lib)
            row[name] = {"ms": ms.value, "matrices_per_s": nk / ms.value * 1e3}
        by_n[str(n)] = row
    top = by_n[str(sizes[-1])]
    ms = top["householder"]["ms"] if lib_jacobi_max_n() < sizes[-1] else top["jacobi"]["ms"]
    _line(args, world, "matrices/s (FP64 eigenpairs, 32 bands)", nk / ms * 1e3, "matrices/s", ms, "f64", cfg,
          {"by_n": by_n, "jacobi_max_n": lib_jacobi_max_n(), "gpu_launches": 2 * len(sizes) * max(args.steps, 1)})
    return 0


def lib_jacobi_max_n() -> int:
    """The largest band count the FP64 driver gives to the Jacobi solver."""
    v = os.environ.get("TBG_JACOBI_MAX_N")
    return max(0, min(int(v), 32)) if v else 8
