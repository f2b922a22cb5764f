"""Benchmark of the k-mesh Hall path on the random spinful 3D workload.

Workload: Model<true,3>, 64 orbitals (128 bands), 343 R vectors (|R_i| <= 3),
cfg2 hopping statistics (numpy default_rng(20260101)), 64^3 k-mesh, sigma_xy
at mu = 0, T = 0, eta = 1e-3.  A step is one pass of the Hall path over one
batch of the mesh (a contiguous range of flat k indices): Fourier sum,
eigensolve, velocity rotation, Berry curvature and the occupation k-sum.
Ranks take disjoint ranges (weak scaling); the only exchange would be a sum of
n_mu doubles, done on the host.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--precision mixed|fp64] [--batch B]

Prints one JSON line (rank 0).
"""

from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "k-pts/s (H+eig+Berry, norb=128) mixed vs FP64 GPU @AHC err≤1e-6; serve p99"
KMESH = (64, 64, 64)
NK = 64 ** 3
MU = np.array([0.0])
DIRS = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])
ETA = 1e-3
WORKLOAD = ("random spinful 3D Model<true,3>: 64 orbitals (128 bands), 343 R (|R_i|<=3), "
            "64^3 k-mesh, sigma_xy at mu=0, T=0, eta=1e-3")


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Barrier and max-reduce across ranks (torch.distributed when world > 1)."""

    def __init__(self, world: int, backend: str):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as tdist

            tdist.init_process_group(backend=backend)
            self.tdist = tdist

    def barrier(self):
        if self.world > 1:
            self.tdist.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        if self.tdist.get_backend() == "nccl":
            t = t.cuda()
        self.tdist.all_reduce(t, op=self.tdist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, arr: np.ndarray) -> np.ndarray:
        if self.world == 1:
            return arr
        import torch

        t = torch.tensor(arr, dtype=torch.float64)
        if self.tdist.get_backend() == "nccl":
            t = t.cuda()
        self.tdist.all_reduce(t)
        return t.cpu().numpy()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def flush_l2(buf):
    """Overwrite a 256 MB device buffer (> the 129 MB L2) between steps."""
    buf.zero_()


def algorithmic_flops_per_k(N: int, nR: int) -> float:
    """F(N, nR) = 24 nR N^2 + 46 N^3 real flops per k-point (Fourier sum for H,
    Vx, Vy; nominal eigensolve 14 N^3; rotation 32 N^3)."""
    return 24.0 * nR * N * N + 46.0 * N ** 3


# DRAM bytes (read + write) per k-point of each kernel family, from ncu captures over 512 k-points
# of this workload: the FP32 solver's passes (TMEM-resident reduction, back-transformation), the
# three HIGH products of the refinement and the four MID products of the rotation of one k-point.
DRAM_BYTES_PER_MATRIX = {"hetrd_tc_kernel": 141.3e6 / 512, "bt_tc_kernel": 109.3e6 / 512,
                         "heev_kernel<float,smem>": 112.5e6 / 512, "heev_bt_kernel": 112.5e6 / 512,
                         "ozaki_tc_kernel<high>": 730.9e6 / 512, "ozaki_tc_kernel<mid>": 1466.6e6 / 512}


def slice_products(name: str) -> int:
    """BF16 digit products per FP64-class product of an exact-slice kernel
    family: 21 (HIGH, six digits), 15 (MID, five), 6 (LOW, three)."""
    return 6 if "low" in name else (15 if "mid" in name else 21)


def kernel_roofline(timing: dict, peaks: dict, units: int = 0) -> dict | None:
    """Roofline entry for the kernel family with the largest device time:
    achieved = its algorithmic flops / its device time (CUDA events around
    every launch, on the launching stream).  units = matrices (k-points) the
    timed launches of the family processed, for the per-launch traffic."""
    if not timing:
        return None
    name, (launches, ms, work) = max(timing.items(), key=lambda kv: kv[1][1])
    traffic = None
    if name in DRAM_BYTES_PER_MATRIX and units and launches:
        traffic = DRAM_BYTES_PER_MATRIX[name] * units / launches
    if name.startswith(("heev_kernel<float", "hetrd_tc", "bt_tc", "fp32")):
        bound, peak, src = "fp32", peaks["fp32_tflops"], "FP32 FMA loop on this GPU (tbg_measure_fma_peaks)"
    elif name.startswith("ozaki"):
        # FP64-class products from BF16 digit products: the attainable algorithmic
        # rate is the BF16 peak divided by the digit products per product
        pairs = slice_products(name)
        bound, peak = "tensor", (peaks.get("bf16_tflops") or 0.0) / pairs
        src = f"MEASURED_PEAKS.json bf16_tflops (burst) / {pairs} slice products"
    else:
        bound, peak, src = "fp64", peaks["fp64_tflops"], "FP64 FMA loop on this GPU (tbg_measure_fma_peaks)"
    achieved = work / (ms / 1e3) / 1e12 if ms > 0 and work > 0 else None
    return {"bound": bound, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": (achieved / peak) if (achieved and peak) else None, "traffic": traffic,
            "traffic_unit": "bytes per launch (DRAM read + write, ncu per-matrix figure x matrices per launch)",
            "kernel": name, "launches": launches, "avg_launch_ms": ms / max(launches, 1),
            "peak_source": src}


def measured_peaks(lib) -> dict:
    p64 = ctypes.c_double(0.0)
    p32 = ctypes.c_double(0.0)
    lib.tbg_measure_fma_peaks(ctypes.byref(p64), ctypes.byref(p32))
    out = {"fp64_tflops": p64.value, "fp32_tflops": p32.value}
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        mp = json.load(open(path))
        out["bf16_tflops"] = mp.get("bf16_tflops")
        out["hbm_gbs"] = mp.get("hbm_gbs")
    else:
        out["bf16_tflops"] = 1900.0
        out["hbm_gbs"] = 6800.0
    return out


def run_reference(args, rank, world):
    """CPU baseline on the host cores: the C port of Rustb's path (OpenBLAS
    zaxpy/zheev/zgemm, OpenMP over k)."""
    if rank != 0:
        return 0
    from oracle import build_port
    from rustb_gb300 import workloads as W

    model = W.random_spinful_3d()
    threads = os.cpu_count() or 1
    sample = args.ref_sample or threads * 64
    build_port.load()
    for w in range(args.warmup):
        build_port.hall_sums(model, DIRS, MU, 0.0, ETA, -1, kmesh=KMESH, k0=(w * sample) % NK, nk=min(sample, 16),
                             threads=threads)
    t0 = time.perf_counter()
    for s in range(args.steps):
        build_port.hall_sums(model, DIRS, MU, 0.0, ETA, -1, kmesh=KMESH, k0=(s * sample) % NK, nk=sample,
                             threads=threads)
    dt = time.perf_counter() - t0
    val = args.steps * sample / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "k-pts/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded random spinful 3D model, numpy default_rng(20260101))",
        "config": {"workload": WORKLOAD, "batch_kpts": sample, "k_mesh": list(KMESH), "precision": "fp64"},
        "cpu_baseline": {"value": val, "unit": "k-pts/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} k-points of the 64^3 mesh per step (flat index ranges)"},
        "e2e": {"value": val, "unit": "k-pts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "Rustb is Rust and cannot be built here; the C port restates its path over scipy's OpenBLAS",
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--batch", type=int, default=8192, help="k-points per rank per step")
    ap.add_argument("--fp64-sample", type=int, default=0, help="k-points of the plain FP64 run (0 = --batch)")
    ap.add_argument("--cpu-sample", type=int, default=0, help="k-points for the CPU baseline (0 = auto)")
    ap.add_argument("--ref-sample", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", choices=["random3d", "haldane", "batched", "supercell", "serve", "dos", "w90", "wilson", "ec", "eig-small"],
                    default="random3d")
    ap.add_argument("--models", type=int, default=64, help="batched: models taken from the 512-model set")
    ap.add_argument("--kcap", type=int, default=0, help="batched: first k-points of each mesh (0 = whole meshes)")
    ap.add_argument("--serve-seconds", type=float, default=8.0)
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.workload != "random3d":
        import bench_workloads

        return bench_workloads.run(args, rank, world, local)
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch

    from rustb_gb300 import _lib, workloads as W
    from rustb_gb300.params import Precision

    torch.cuda.set_device(local)
    dist = Dist(world, "nccl" if torch.cuda.is_available() else "gloo")
    lib = _lib.load()
    _lib.check(lib.tbg_set_device(local), lib)
    model = W.random_spinful_3d()
    N, nR = model.nsta, model.nR
    prec = Precision.MIXED if args.precision == "mixed" else Precision.FP64
    handle = model.device_handle()
    km = np.ascontiguousarray(KMESH, dtype=np.int64)
    B = args.batch
    sums = np.zeros(1)
    rep = _lib.TbgReport()

    from rustb_gb300 import shard

    def step(s, precision=prec, batch=B):
        k0, cnt = shard.step_range(NK, batch, world, rank, s)
        _lib.check(lib.tbg_hall_sums_range(handle, _lib.iptr(km), k0, cnt, _lib.dptr(DIRS), 1, _lib.dptr(MU), 0.0,
                                           ETA, -1, int(precision), _lib.dptr(sums), ctypes.byref(rep)), lib)
        return cnt

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    peaks = measured_peaks(lib)
    for w in range(args.warmup):
        step(w)
    # ------------------------------------------------------------- timed --
    lib.tbg_kernel_timing_enable(1)
    _lib.kernel_timing(reset=True)
    launches0 = lib.tbg_kernel_launch_count(0)
    clocks = ClockSampler(local)
    clocks.start()
    dev_ms = 0.0
    done = 0
    dist.barrier()
    torch.cuda.synchronize()
    for s in range(args.steps):
        flush_l2(flush)
        torch.cuda.synchronize()
        done += step(args.warmup + s)
        dev_ms += rep.device_ms
    torch.cuda.synchronize()
    dist.barrier()
    clk = clocks.stop()
    launches = lib.tbg_kernel_launch_count(0) - launches0
    lib.tbg_kernel_timing_enable(0)
    timing = _lib.kernel_timing(reset=True)
    t_max = dist.max(dev_ms / 1e3)
    value = done * world / t_max
    # ------------------------------------------------------------- e2e --
    # public API with host buffers: upload the model from pinned host memory,
    # run one batch, read the sums back; all inside the timed region
    ham_pin = torch.from_numpy(model.ham.view(np.float64)).pin_memory()
    hamR = np.ascontiguousarray(model.hamR, dtype=np.int64)
    orb = np.ascontiguousarray(model.orb)
    lat = np.ascontiguousarray(model.lat)
    h2d = ham_pin.numel() * 8 + hamR.nbytes + orb.nbytes + lat.nbytes + DIRS.nbytes + MU.nbytes + km.nbytes
    e2e_steps = args.steps
    dist.barrier()
    t0 = time.perf_counter()
    for s in range(e2e_steps):
        h = ctypes.c_void_p()
        _lib.check(lib.tbg_model_create(3, 1, model.norb, model.nR, _lib.iptr(hamR),
                                        ctypes.cast(ham_pin.data_ptr(), ctypes.POINTER(ctypes.c_double)),
                                        _lib.dptr(orb), _lib.dptr(lat), ctypes.byref(h)), lib)
        k0 = ((s * world + rank) * B) % NK
        _lib.check(lib.tbg_hall_sums_range(h, _lib.iptr(km), k0, min(B, NK - k0), _lib.dptr(DIRS), 1,
                                           _lib.dptr(MU), 0.0, ETA, -1, int(prec), _lib.dptr(sums), None), lib)
        lib.tbg_model_destroy(h)
    e2e_t = dist.max(time.perf_counter() - t0)
    e2e_val = e2e_steps * B * world / e2e_t
    out = None
    if rank == 0:
        # ---------------------------------------------- plain FP64 beside it --
        # plain FP64 path on a batch of the same size (flat indices [0, fs))
        fs = args.fp64_sample or B
        step(0, Precision.FP64, fs)
        fp64_val = fs / (rep.device_ms / 1e3)
        plain_sum = sums.copy()
        step(0, Precision.MIXED, fs)
        mixed_sum = sums.copy()
        acc = {"ahc_partial_rel_err_mixed_vs_fp64": float(abs(mixed_sum[0] - plain_sum[0]) / abs(plain_sum[0])),
               "sample": f"flat k indices [0, {fs}) of the 64^3 mesh"}
        roof_line = kernel_roofline(timing, peaks, units=done)
        cpu = None
        if not args.no_cpu_baseline:
            from oracle import build_port

            threads = os.cpu_count() or 1
            cs = args.cpu_sample or threads * 32
            build_port.load()
            build_port.hall_sums(model, DIRS, MU, 0.0, ETA, -1, kmesh=KMESH, k0=0, nk=threads, threads=threads)
            t0 = time.perf_counter()
            port_S = build_port.hall_sums(model, DIRS, MU, 0.0, ETA, -1, kmesh=KMESH, k0=0, nk=cs, threads=threads)
            cdt = time.perf_counter() - t0
            cpu = {"value": cs / cdt, "unit": "k-pts/s", "cores": threads, "kind": "port",
                   "sample": f"{cs} k-points of the 64^3 mesh (flat indices [0, {cs}))"}
            # the GPU's FP64 and MIXED sums over the port's k-points, against the port
            port_sum = float(math.fsum(port_S[:, 0]))
            step(0, Precision.FP64, cs)
            acc["fp64_vs_port_rel"] = float(abs(sums[0] - port_sum) / abs(port_sum))
            step(0, Precision.MIXED, cs)
            acc["mixed_vs_port_rel"] = float(abs(sums[0] - port_sum) / abs(port_sum))
            acc["port_sample"] = f"flat k indices [0, {cs}) of the 64^3 mesh (C port, OpenBLAS zheev)"
        flops_k = algorithmic_flops_per_k(N, nR)
        out = {
            "metric": METRIC, "value": value, "unit": "k-pts/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 eigensolve + f64 refinement/rotation" if prec == Precision.MIXED else "f64",
            "data": "synthetic (seeded random spinful 3D model, numpy default_rng(20260101))",
            "config": {"workload": WORKLOAD, "batch_kpts": B, "k_mesh": list(KMESH),
                       "precision": args.precision, "parallelism": f"k-range shards x{world}",
                       "l2": "working set per step >> L2 and a 256 MB buffer is overwritten before every step"},
            "algorithmic_tflops": value * flops_k / 1e12,
            "fp64_plain": {"value": fp64_val, "unit": "k-pts/s", "sample_kpts": fs,
                           "mixed_speedup": value / fp64_val},
            "accuracy": acc,
            "roofline": roof_line,
            "kernel_times_ms": {k: {"launches": v[0], "total_ms": v[1], "tflops": (v[2] / v[1] / 1e9 if v[1] else None)}
                                for k, v in sorted(timing.items(), key=lambda kv: -kv[1][1])},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_val, "unit": "k-pts/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(sums.nbytes), "steps": e2e_steps,
                    "note": "model upload from pinned host memory + one batch + sums readback per step"},
            "gpu_launches": int(launches),
            "clocks": clk,
            "measured_peaks": peaks,
        }
        print(json.dumps(out), flush=True)
    dist.barrier()
    return 0


if __name__ == "__main__":
    sys.exit(main())
