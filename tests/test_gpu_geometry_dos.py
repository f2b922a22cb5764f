"""GPU parity for quantum geometry and the density of states: libtbgpu
(through the C-ABI) against the oracle on the same inputs.

Tolerances: FP64 metric and Berry curvature <= 1e-8 of their scale per band,
energies <= 1e-10 of ||H||; mixed path <= 1e-6 of the scale; DOS <= 1e-9 of
its maximum (the band energies enter through exp(-A^2/2) whose slope is
A / sigma, so eigenvalue rounding is amplified by at most 39 / sigma)."""

import ctypes
import math

import numpy as np
import pytest

import models as M
from oracle import tb_oracle as O
from rustb_gb300 import _lib, errors, workloads as W
from rustb_gb300.params import Integration, Parameters, Precision

pytestmark = pytest.mark.gpu

XY = np.array([[1.0, 0.0], [0.0, 1.0]])
XY3 = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


# Band-resolved values need non-degenerate bands: inside a degenerate pair the
# split between the two bands depends on the eigenbasis (the Kane-Mele bands
# are Kramers pairs), so spinful cases use generic random models here.
SKEW = np.array([[1.0, 0.0], [0.6, 0.8]])


def _models():
    return [
        ("haldane", M.haldane(), XY),                                   # nsta 2: fused small path
        ("random_2d_s3", W.random_model(2, 3, True, 1, seed=300), SKEW),  # nsta 6, spinful, fused
        ("random_2d_12", W.random_model(2, 12, False, 1, seed=301), XY),  # batched FP64 path
        ("random_3d_s10", W.random_model(3, 10, True, 1, seed=302), XY3),
    ]


@pytest.mark.parametrize("name,model,dirs", _models(), ids=[m[0] for m in _models()])
def test_quantum_geometry_on_matches_oracle(name, model, dirs):
    rng = np.random.default_rng(17)
    k = rng.random((37, model.dim))
    p = Parameters.rank2([1] * model.dim, dirs[0], dirs[1], [0.0])
    p.eta = 2e-3
    r = model.quantum_geometry_on(k, p)
    g, om, E = O.quantum_geometry_on(model, k, dirs, eta=2e-3)
    assert rel(r.energies, E) < 1e-10
    assert rel(r.metric, g) < 1e-8
    assert rel(r.berry_curvature, om) < 1e-8
    # the Berry component is the Kubo curvature of berry_curvature_on
    om2, _ = model.berry_curvature_on(k, p)
    assert rel(r.berry_curvature, om2) < 1e-10


def test_quantum_geometry_at_shapes_massive_dirac():
    """named_band_result_has_real_components (src/quantum_geometry.rs:318-328)."""
    m = M.massive_dirac()
    p = Parameters.rank2([1, 1], [1.0, 0.0], [0.0, 1.0], [0.0])
    r = m.quantum_geometry_at([0.0, 0.0], p)
    assert r.metric.shape == r.berry_curvature.shape == r.energies.shape == (m.nsta,)
    assert np.array_equal(r.energies, np.array([-0.5, 0.5]))
    assert np.all(r.metric == 0.0) and np.all(r.berry_curvature == 0.0)


@pytest.mark.parametrize("norb,spin", [(24, False), (12, True)])
def test_quantum_geometry_mixed_matches_oracle(norb, spin):
    m = W.random_model(2, norb, spin, 1, seed=303 + norb)
    rng = np.random.default_rng(19)
    k = rng.random((64, 2))
    p = Parameters.rank2([1, 1], XY[0], XY[1], [0.0])
    p.eta = 5e-3
    r = m.quantum_geometry_on(k, p, Precision.MIXED)
    g, om, E = O.quantum_geometry_on(m, k, XY, eta=5e-3)
    assert rel(r.energies, E) < 1e-9
    assert rel(r.metric, g) < 1e-6
    assert rel(r.berry_curvature, om) < 1e-6


@pytest.mark.parametrize("precision", [Precision.FP64, Precision.MIXED])
def test_quantum_geometry_mesh_matches_oracle(precision):
    # skewed directions: the C3-symmetric Haldane model integrates g_xy to zero
    cases = [(M.haldane(), [12, 12], SKEW), (W.random_model(2, 16, False, 1, seed=304), [6, 5], SKEW),
             (M.kane_mele(rashba=0.05), [9, 9], SKEW)]
    mu = [-1.0, 0.0, 0.35]
    for model, kmesh, dirs in cases:
        for T in (0.0, 300.0):
            p = Parameters.rank2(kmesh, dirs[0], dirs[1], mu)
            p.T = np.array([T])
            p.eta = 1e-2
            r = model.quantum_geometry(p, precision)
            g, om = O.quantum_geometry(model, kmesh, dirs, mu, T=T, eta=1e-2)
            tol = 1e-9 if precision == Precision.FP64 else 1e-6
            # the time-reversal-symmetric Kane-Mele model integrates Omega to
            # zero: the scale has a floor of 1e-3 (metric values are O(0.1))
            assert np.max(np.abs(r.metric - g)) <= tol * max(np.max(np.abs(g)), 1e-3)
            assert np.max(np.abs(r.berry_curvature - om)) <= tol * max(np.max(np.abs(om)), 1e-3)
            assert np.array_equal(r.chemical_potentials, np.asarray(mu))


def test_quantum_geometry_mesh_berry_equals_hall_sum():
    model = W.random_model(2, 12, False, 1, seed=305)
    p = Parameters.rank2([7, 9], XY[0], XY[1], [-0.5, 0.25])
    p.eta = 3e-3
    qg = model.quantum_geometry(p)
    hall = model.hall_conductivity(p)
    assert rel(qg.berry_curvature, hall.conductivity) < 1e-12


def test_qwz_chern_over_two_pi():
    m = M.qwz_2d(-1.0)
    p = Parameters.rank2([31, 31], XY[0], XY[1], [0.0])
    p.eta = 1e-4
    r = m.quantum_geometry(p)
    assert abs(abs(2 * math.pi * r.berry_curvature[0]) - 1.0) < 2e-2


DOS_CASES = [
    # model, kmesh, E_min, E_max, E_n, sigma
    ("bench_small_31", M.bench_small, [31, 31], -3.0, 3.0, 500, 1e-2),   # benches/bench_main.rs:297-305
    ("haldane_ragged", M.haldane, [7, 5], -9.0, 9.0, 1000, 0.05),
    ("random12", lambda: W.random_model(2, 12, False, 1, seed=306), [8, 6], -4.0, 4.0, 777, 0.02),
    ("random3d_s6", lambda: W.random_model(3, 6, True, 1, seed=307), [3, 4, 2], -5.0, 5.0, 256, 0.1),
    ("single_bin", M.haldane, [4, 4], 0.3, 0.4, 1, 0.2),
    ("narrow_sigma", M.bench_small, [9, 9], -3.0, 3.0, 301, 1e-4),
    ("wide_sigma", M.bench_small, [9, 9], -3.0, 3.0, 301, 10.0),
    ("gap_window", M.bench_small, [9, 9], -0.5, 0.5, 129, 1e-2),
]


@pytest.mark.parametrize("case", DOS_CASES, ids=[c[0] for c in DOS_CASES])
def test_dos_matches_oracle(case):
    _, build, kmesh, E_min, E_max, E_n, sigma = case
    model = build()
    E, d = model.dos(kmesh, E_min, E_max, E_n, sigma)
    E_o, d_o = O.dos(model, kmesh, E_min, E_max, E_n, sigma)
    assert np.array_equal(E, E_o)
    scale = max(np.max(np.abs(d_o)), 1e-300)
    tol = 1e-9 if sigma >= 1e-2 else 1e-7
    assert np.max(np.abs(d - d_o)) <= tol * scale


def test_dos_flat_bands_closed_form():
    levels = [-1.25, 0.0, 0.4, 2.0]
    model = M.flat_bands(levels)
    E, d = model.dos([5, 3], -3.0, 3.0, 601, 0.05)
    expect = sum(np.exp(-((E - x) / 0.05) ** 2 / 2.0) / 0.05 / math.sqrt(2 * math.pi) for x in levels)
    assert np.allclose(d, expect, rtol=1e-12, atol=1e-300)


def test_dos_integrates_to_state_count_large_model():
    model = W.random_model(2, 40, False, 1, seed=308)
    E, d = model.dos([10, 10], -40.0, 40.0, 16001, 0.05)
    assert abs(d.sum() * (E[1] - E[0]) - model.nsta) < 1e-6


def _raw_dos(model, kmesh, E_min, E_max, E_n, sigma):
    lib = _lib.load()
    km = np.ascontiguousarray(np.asarray(kmesh, dtype=np.int64))
    out = np.empty(max(int(E_n), 1))
    return lib.tbg_dos(model.device_handle(), _lib.iptr(km), float(E_min), float(E_max), int(E_n), float(sigma),
                       None, _lib.dptr(out))


def test_dos_c_abi_errors():
    m = M.haldane()
    assert _raw_dos(m, [4, 4], 1.0, 1.0, 10, 0.1) == errors.TBG_E_INVALID_ENERGY_RANGE
    assert _raw_dos(m, [4, 4], 2.0, 1.0, 0, -1.0) == errors.TBG_E_INVALID_ENERGY_RANGE  # range checked first
    assert _raw_dos(m, [4, 4], 0.0, 1.0, 0, 0.1) == errors.TBG_E_INVALID_DOS_PARAMETER
    assert _raw_dos(m, [4, 4], 0.0, 1.0, 10, 0.0) == errors.TBG_E_INVALID_DOS_PARAMETER
    assert _raw_dos(m, [4, 4], 0.0, 1.0, 10, float("nan")) == errors.TBG_E_INVALID_DOS_PARAMETER
    assert _raw_dos(m, [4, 4], 0.0, 1.0, 10, float("inf")) == errors.TBG_E_INVALID_DOS_PARAMETER
    assert _raw_dos(m, [4, 0], 0.0, 1.0, 10, 0.1) == errors.TBG_E_INVALID_KMESH
    assert _raw_dos(m, [4, 4], 0.0, 1.0, 10, 0.1) == errors.TBG_OK


def test_quantum_geometry_c_abi_errors():
    m = M.haldane()
    lib = _lib.load()
    k = np.zeros((1, 2))
    out = np.empty((3, 2))
    d = _lib.as_f64(XY)
    h = m.device_handle()
    assert lib.tbg_quantum_geometry(h, 1, _lib.dptr(k), _lib.dptr(d), -1.0, 0, _lib.dptr(out[0]),
                                    _lib.dptr(out[1]), _lib.dptr(out[2])) == errors.TBG_E_INVALID_RESPONSE_PARAMETER
    km = np.array([0, 3], dtype=np.int64)
    mu = np.zeros(1)
    res = np.empty(2)
    assert lib.tbg_quantum_geometry_mesh(h, _lib.iptr(km), _lib.dptr(d), 1, _lib.dptr(mu), 0.0, 1e-3, 0,
                                         _lib.dptr(res[:1]), _lib.dptr(res[1:]), None) == errors.TBG_E_INVALID_KMESH


# ------------------------------------------------------------ band meshes --
@pytest.mark.parametrize("name,build,kmesh", [
    ("haldane", M.haldane, [9, 7]),
    ("kane_mele", lambda: M.kane_mele(rashba=0.05), [5, 6]),
    ("random12", lambda: W.random_model(2, 12, False, 1, seed=309), [6, 4]),
    ("qwz3d", M.qwz_stacked_3d, [4, 3, 5]),
    ("random3d_s9", lambda: W.random_model(3, 9, True, 1, seed=310), [3, 2, 4]),
])
def test_bands_mesh_matches_oracle(name, build, kmesh):
    model = build()
    E = model.solve_band_mesh(kmesh)
    ref = O.solve_band_all(model, O.gen_kmesh(kmesh))
    scale = max(np.max(np.abs(ref)), 1.0)
    assert E.shape == ref.shape
    assert np.max(np.abs(E - ref)) <= 1e-10 * scale
    # the k-list path gives the same energies
    E2 = model.solve_band_all_parallel(O.gen_kmesh(kmesh))
    assert np.max(np.abs(E - E2)) <= 1e-12 * scale


def _parse_bxsf(path):
    lines = open(path, encoding="utf-8").read().split("\n")
    i = lines.index("  BEGIN_BANDGRID_3D_band_energies")
    nb = int(lines[i + 1])
    dims = [int(v) for v in lines[i + 2].split()]
    vals = []
    for ln in lines[i + 7:]:
        if ln.startswith("    BAND:") or not ln.strip() or ln.strip().startswith("END"):
            continue
        vals += [float(v) for v in ln.split()]
    return nb, dims, np.array(vals).reshape(nb, -1).T


def test_write_bxsf_round_trip(tmp_path):
    model = W.random_model(3, 5, False, 1, seed=311)
    km = [3, 4, 12]
    path = model.write_bxsf(km, 0.25, str(tmp_path / "bands"))
    assert path.endswith(".bxsf")
    nb, dims, E = _parse_bxsf(path)
    assert nb == model.nsta and dims == km
    ref = O.solve_band_all(model, O.gen_kmesh(km))
    assert np.allclose(E, ref, rtol=2e-10, atol=1e-12)  # 10 decimals in the file
    text = open(path, encoding="utf-8").read()
    assert "  Fermi Energy: 0.250000000000\n" in text


def test_write_spin_frmsf(tmp_path):
    from rustb_gb300 import write_spin_frmsf

    up = W.random_model(3, 3, False, 1, seed=312)
    dn = W.random_model(3, 3, False, 1, seed=313)
    dn.lat = up.lat.copy()
    km = [2, 3, 4]
    path = write_spin_frmsf(up, dn, km, 0.1, str(tmp_path / "spin"))
    lines = open(path).read().split("\n")
    assert lines[0] == "2 3 4" and lines[1] == "1" and lines[2] == "6"
    vals = np.array([float(v) for ln in lines[6:] for v in ln.split()])
    nk = 24
    energies, colors = vals[:6 * nk], vals[6 * nk:]
    eu = O.solve_band_all(up, O.gen_kmesh(km)) - 0.1
    ed = O.solve_band_all(dn, O.gen_kmesh(km)) - 0.1
    ref = np.concatenate([eu, ed], axis=1).T.reshape(-1)
    assert np.allclose(energies, ref, rtol=2e-10, atol=1e-12)
    assert np.array_equal(colors, np.where(np.arange(6 * nk) // nk < 3, 1.0, -1.0))
    with pytest.raises(errors.TbPanic):
        write_spin_frmsf(up, W.random_model(3, 4, False, 1, seed=314), km, 0.0, str(tmp_path / "bad"))
