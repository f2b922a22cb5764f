"""The configuration models against the oracle, not against the library's own
FP64 path.

Rustb's k-mesh results on the benchmark models (the random spinful 3D model
of 128 bands and 343 R, the Haldane model on its 200 x 200 mesh, the
1024-orbital supercell, models of the batched uneven set, and the three
serving observables) are compared with the CPU restatements of the reference
path: the C port (OpenBLAS zheev, OpenMP over k; ``oracle/cpu_port.c``) for
k-sums over mesh ranges, the numpy oracle (LAPACK zheev) for band-resolved
quantities.  Tolerances (written in each test): eigenvalues <= 1e-10 ||H||
(FP64) / 1e-9 ||H|| (mixed); Omega and sigma <= 1e-8 relative (FP64); AHC
<= 1e-6 relative (mixed).  The reference path is src/response/traits.rs:160-200
(per-k Omega_n), src/response/linear/mod.rs:193-225 (the Direct k-sum).
"""

import math
import os

import numpy as np
import pytest

from oracle import build_port
from oracle import tb_oracle as O
from rustb_gb300 import _lib, batch, serve, workloads as W
from rustb_gb300.params import Parameters, Precision

pytestmark = pytest.mark.gpu

XY3 = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])
XY2 = np.array([[1.0, 0.0], [0.0, 1.0]])
THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def spinful3d():
    return W.random_spinful_3d()


def gpu_sums_range(model, kmesh, k0, cnt, dirs, mu, precision):
    """sum over flat mesh indices [k0, k0 + cnt) of sum_n Omega_n f(E_n, mu_j)
    through tbg_hall_sums_range (no 1/(nk det) normalisation)."""
    lib = _lib.load()
    km = np.ascontiguousarray(kmesh, dtype=np.int64)
    mu = _lib.as_f64(np.atleast_1d(mu))
    out = np.empty(len(mu))
    _lib.check(lib.tbg_hall_sums_range(model.device_handle(), _lib.iptr(km), int(k0), int(cnt),
                                       _lib.dptr(_lib.as_f64(dirs)), len(mu), _lib.dptr(mu), 0.0, 1e-3, -1,
                                       int(precision), _lib.dptr(out), None), lib)
    return out


def port_sums_range(model, kmesh, k0, cnt, dirs, mu):
    S = build_port.hall_sums(model, dirs, np.atleast_1d(mu), 0.0, 1e-3, -1, kmesh=kmesh, k0=k0, nk=cnt,
                             threads=THREADS)
    return S.sum(axis=0)


# ------------------------------------------------ random spinful 3D (128) --
@pytest.mark.parametrize("k0", [0, 131072 + 4096 + 37])
def test_spinful3d_sigma_sums_vs_port(spinful3d, k0):
    """Partial Direct sums over 256 consecutive flat indices of the 64^3 mesh:
    FP64 within 1e-8 and MIXED within 1e-6 of the C port."""
    km = (64, 64, 64)
    mus = np.array([-0.5, 0.0, 0.3])
    ref = port_sums_range(spinful3d, km, k0, 256, XY3, mus)
    plain = gpu_sums_range(spinful3d, km, k0, 256, XY3, mus, Precision.FP64)
    mixed = gpu_sums_range(spinful3d, km, k0, 256, XY3, mus, Precision.MIXED)
    for j in range(len(mus)):
        assert abs(plain[j] - ref[j]) <= 1e-8 * abs(ref[j]), (j, plain[j], ref[j])
        assert abs(mixed[j] - ref[j]) <= 1e-6 * abs(ref[j]), (j, mixed[j], ref[j])


def test_spinful3d_band_resolved_omega_vs_oracle(spinful3d):
    """Omega_n and E_n of every band at 4 mesh points: FP64 within 1e-8 of the
    largest |Omega_n| (eigenvalues 1e-10 ||H||), MIXED within 1e-6 (1e-9 ||H||)."""
    k = O.gen_kmesh((64, 64, 64))[[0, 1234, 99999, 262143]]
    p = Parameters.rank2((1, 1, 1), XY3[0], XY3[1], [0.0])
    Omr, Er = O.berry_on(spinful3d, k, XY3)
    nrm = max(np.linalg.norm(h, 2) for h in O.gen_ham_batch(spinful3d, k, 1))
    for prec, tol_om, tol_e in ((Precision.FP64, 1e-8, 1e-10), (Precision.MIXED, 1e-6, 1e-9)):
        Om, E = spinful3d.berry_curvature_on(k, p, prec)
        assert np.max(np.abs(E - Er)) <= tol_e * nrm
        for i in range(len(k)):
            assert np.max(np.abs(Om[i] - Omr[i])) <= tol_om * np.max(np.abs(Omr[i])), (prec, i)


# --------------------------------------------------------- Haldane 200^2 --
def test_haldane_200_sigma_vs_port():
    """The Haldane configuration on its full 200 x 200 mesh: sigma_xy at
    mu = 0 within 1e-8 of the C port, and C = round(2 pi sigma) = +-1."""
    h = W.haldane_200()
    km = (200, 200)
    p = Parameters.rank2(km, [1.0, 0.0], [0.0, 1.0], [0.0])
    s = h.hall_conductivity(p).conductivity[0]
    ref = port_sums_range(h, km, 0, 40000, XY2, [0.0])[0] / 40000 / float(np.linalg.det(h.lat))
    assert abs(s - ref) <= 1e-8 * abs(ref)
    assert abs(round(2 * math.pi * s)) == 1 and round(2 * math.pi * s) == round(2 * math.pi * ref)
    # per-k curvature on a sample of the mesh against the numpy oracle
    k = O.gen_kmesh(km)[::997]
    Om, E = h.berry_curvature_on(k, p)
    Omr, Er = O.berry_on(h, k, XY2)
    assert np.max(np.abs(E - Er)) <= 1e-12 * np.max(np.abs(Er))
    assert np.max(np.abs(Om - Omr)) <= 1e-8 * np.max(np.abs(Omr))


# ------------------------------------------------ 1024-orbital supercell --
def nearest_bands(E, n=20, energy=0.0):
    """Indices (ascending) of the n bands whose energies lie nearest `energy`."""
    return np.sort(np.argsort(np.abs(E - energy), kind="stable")[:n])


def test_supercell_1024_spectrum_and_omega_near_zero():
    """The supercell configuration (1024 bands, R in {-1,0,1}^2) at 2 k-points:
    the MIXED full spectrum within 1e-9 ||H|| of zheev, and Omega of the 20
    bands nearest E = 0 (berry_curvature_at, src/response/traits.rs:60-78)
    within 1e-8 (FP64) / 1e-6 (MIXED) of the oracle's largest value there."""
    m = W.supercell_2d()
    k = np.array([[0.125, 0.375], [0.5, 0.0625]])
    p = Parameters.rank2((1, 1), [1.0, 0.0], [0.0, 1.0], [0.0])
    Omr, Er = O.berry_on(m, k, XY2)
    Hs = O.gen_ham_batch(m, k, 1)
    for prec, tol_om, tol_e in ((Precision.FP64, 1e-8, 1e-10), (Precision.MIXED, 1e-6, 1e-9)):
        Om, E = m.berry_curvature_on(k, p, prec)
        for i in range(len(k)):
            assert np.max(np.abs(E[i] - Er[i])) <= tol_e * np.linalg.norm(Hs[i], 2), (prec, i)
            sel = nearest_bands(Er[i])
            assert np.array_equal(sel, nearest_bands(E[i]))
            scale = np.max(np.abs(Omr[i][sel]))
            assert np.max(np.abs(Om[i][sel] - Omr[i][sel])) <= tol_om * scale, (prec, i)


# ------------------------------------------------------ batched uneven set --
def test_batched_models_vs_port(tmp_path):
    """Three models drawn from the batched uneven set (shrunk meshes): the
    batch runner's sigma within 1e-8 (FP64) / 1e-6 (MIXED) of the C port."""
    specs = W.batched_uneven_specs(512)
    picks = [specs[i] for i in (3, 300, 17)]
    jobs, refs = [], []
    for dim, norb, mesh, seed in picks:
        m = W.random_model(dim, norb, False, 3, seed=seed)
        km = (6, 5) if dim == 2 else (3, 3, 2)
        dirs = np.eye(dim)[:2]
        mus = np.array([-0.2, 0.0, 0.3])
        jobs.append(batch.Job(m, Parameters(kmesh=km, direction=dirs, mu=mus)))
        nk = int(np.prod(km))
        refs.append(port_sums_range(m, km, 0, nk, dirs, mus) / nk / float(np.linalg.det(m.lat)))
    for prec, tol in ((Precision.FP64, 1e-8), (Precision.MIXED, 1e-6)):
        runner = batch.BatchRunner(prec, autotune=False, cache_path=str(tmp_path / "t.json"), max_workers=3)
        res = runner.hall_many(jobs)
        for r, ref in zip(res, refs):
            assert np.max(np.abs(r.conductivity - ref)) <= tol * np.max(np.abs(ref)), prec


# -------------------------------------------------------------- serving --
def test_serving_observables_vs_oracle():
    """One request of each observable kind through the serving loop, against
    the numpy oracle: bands (1e-9 ||H||), band-resolved Berry curvature
    (1e-6 of the largest |Omega_n|) and sigma_xy on the k-list (1e-6)."""
    models = {0: W.random_model(3, 40, True, 3, seed=4001), 1: W.random_model(2, 150, False, 3, seed=4002)}
    rng = np.random.default_rng(4)
    reqs = [serve.Request(0, rng.uniform(0, 1, (33, 3)), "bands"),
            serve.Request(1, rng.uniform(0, 1, (7, 2)), "berry"),
            serve.Request(0, rng.uniform(0, 1, (25, 3)), "sigma_xy"),
            serve.Request(1, rng.uniform(0, 1, (19, 2)), "sigma_xy", mu=0.1)]
    srv = serve.Server(models, hbm_budget_bytes=4 << 30, max_inflight=4)
    futs = [srv.submit(r) for r in reqs]
    out = [f.result(timeout=300) for f in futs]
    srv.close()
    for r, got in zip(reqs, out):
        m = models[r.model_id]
        dirs = np.eye(m.dim)[:2]
        if r.observable == "bands":
            Hs = O.gen_ham_batch(m, r.k, 1)
            nrm = max(np.linalg.norm(h, 2) for h in Hs)
            assert np.max(np.abs(got - np.array([O.eigvalsh(h) for h in Hs]))) <= 1e-9 * nrm
        elif r.observable == "berry":
            Om, E = got
            Omr, Er = O.berry_on(m, r.k, dirs)
            assert np.max(np.abs(Om - Omr)) <= 1e-6 * np.max(np.abs(Omr))
        else:
            occ = O.occupied_berry_curvature_on(m, r.k, dirs, r.mu)
            ref = math.fsum(occ) / len(r.k) / float(np.linalg.det(m.lat))
            assert abs(got - ref) <= 1e-6 * abs(ref)


# ------------------------------------------ fused Berry + occupation sums --
@pytest.mark.parametrize("T", [0.0, 300.0])
def test_mixed_hall_fused_sums_many_mu(T):
    """The mixed hall path sums Omega_n f(E_n, mu_j) in the fused kernel (upper
    triangles of the band-basis velocities, per-CTA compensated partials):
    against the oracle's Direct sums for 40 chemical potentials, T = 0 and
    300 K, within 1e-6 of the largest |sigma|."""
    m = W.random_model(3, 24, True, 1, seed=4100)  # 48 bands
    mus = np.linspace(-1.0, 1.0, 40)
    p = Parameters.rank2((3, 3, 2), XY3[0], XY3[1], mus).with_temperature(T)
    s = m.hall_conductivity(p, Precision.MIXED).conductivity
    ref = O.hall_conductivity(m, (3, 3, 2), XY3, mus, T)
    assert np.max(np.abs(s - ref)) <= 1e-6 * np.max(np.abs(ref))


@pytest.mark.parametrize("norb", [251, 300])
def test_large_model_band_resolved_omega_vs_oracle(norb):
    """Models beyond one CTA's shared memory (the FP32 solver's hybrid layout,
    the panel back-transformation, two row tiles of the exact-slice products
    and, at 300 bands, contractions longer than one exact chunk): band-resolved
    Omega and E of the mixed path at three k-points against the oracle."""
    m = W.random_model(3, norb, False, 1, seed=norb)
    k = np.random.default_rng(norb).uniform(0, 1, (3, 3))
    p = Parameters.rank2((1, 1, 1), XY3[0], XY3[1], [0.0])
    Om, E = m.berry_curvature_on(k, p, Precision.MIXED)
    Omr, Er = O.berry_on(m, k, XY3)
    nrm = np.abs(Er).max()
    assert np.max(np.abs(E - Er)) <= 1e-9 * nrm
    assert np.max(np.abs(Om - Omr)) <= 1e-6 * np.abs(Omr).max()
