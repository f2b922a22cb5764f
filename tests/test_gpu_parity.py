"""GPU parity: libtbgpu (through the C-ABI) against the oracle on the same
seeded inputs.  Tolerances: eigenvalues <= 1e-10 ||H|| (FP64) / 1e-9 ||H||
(mixed); gauge-invariant quantities (projectors, Omega, sigma) <= 1e-8
relative (FP64) and AHC <= 1e-6 relative (mixed); H and V to 1e-12 of their
scale; Chern numbers exactly equal after rounding."""

import json
import math
import os

import numpy as np
import pytest

import models as M
from oracle import tb_oracle as O
from rustb_gb300 import errors, workloads as W
from rustb_gb300.model import Model
from rustb_gb300.params import Gauge, Parameters, Precision, SpinDirection

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
KNOWN = json.load(open(os.path.join(HERE, "golden", "reference_known_answers.json")))
CASES = np.load(os.path.join(HERE, "golden", "oracle_cases.npz"))
XY3 = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])


def fixture_model():
    return Model(CASES["rs_lat"], CASES["rs_orb"], True, ham=CASES["rs_ham"], hamR=CASES["rs_hamR"])


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


# ------------------------------------------------------------------ H and V --
@pytest.mark.parametrize("gauge", [Gauge.Atom, Gauge.Lattice])
def test_gen_ham_matches_fixture(gauge):
    m = fixture_model()
    H = m.gen_ham_batch(CASES["rs_k"], gauge)
    ref = CASES["rs_H"] if gauge == Gauge.Atom else CASES["rs_HL"]
    assert rel(H, ref) < 1e-12


@pytest.mark.parametrize("gauge", [Gauge.Atom, Gauge.Lattice])
def test_gen_v_projected_matches_fixture(gauge):
    m = fixture_model()
    V, H = m.gen_v_projected_batch(CASES["rs_k"], gauge, XY3)
    refV = CASES["rs_V"] if gauge == Gauge.Atom else CASES["rs_VL"]
    assert rel(V, refV) < 1e-12


def test_gen_v_graphene_golden_values():
    ka = KNOWN["test_gen_v"]
    g = M.graphene()
    V, _ = g.gen_v(ka["gen_v_k"], Gauge.Atom)
    assert abs(V[0, 0, 1] - complex(*ka["gen_v_atom_x_01"])) < ka["gen_v_tol"]
    assert abs(V[1, 1, 0] - complex(*ka["gen_v_atom_y_10"])) < ka["gen_v_tol"]
    VL, _ = g.gen_v(ka["gen_v_k"], Gauge.Lattice)
    assert abs(VL[0, 0, 1] - complex(*ka["gen_v_lattice_x_01"])) < ka["gen_v_tol"]
    E = g.solve_band_onek([0.0, 0.0])
    assert np.allclose(E, ka["gamma_bands"], atol=1e-14)
    assert np.all(np.abs(g.solve_band_onek(ka["k_bands_zero"])) < ka["k_bands_tol"])


def test_gen_v_cfg2_size_matches_oracle():
    m = W.random_spinful_3d()
    k = np.random.default_rng(5).uniform(0, 1, (3, 3))
    dirs = np.array([[1.0, 0.5, 0.0], [0.0, 1.0, -0.25]])
    V, H = m.gen_v_projected_batch(k, Gauge.Atom, dirs)
    Vr, Hr = O.gen_v_projected_batch(m, k, 1, dirs)
    assert rel(H, Hr) < 1e-12 and rel(V, Vr) < 1e-12


def test_fourier_sums_with_repeated_and_unpaired_R():
    """The +-R paired table: a repeated R = 0 block and a repeated R give the same
    sums as the oracle; an R whose -R is missing is refused when the model is
    uploaded, as the reference's hopping check refuses it."""
    m = W.random_model(2, 6, False, 1, seed=77)
    ham, hamR = m.ham.copy(), m.hamR.copy()
    i0 = int(np.flatnonzero(np.all(hamR == 0, axis=1))[0])
    i1 = int(np.flatnonzero(np.any(hamR != 0, axis=1))[0])
    ham2 = np.concatenate([ham, 0.5 * ham[[i0]], 0.25 * ham[[i1]]])
    ham2[i0] *= 0.5
    ham2[i1] *= 0.75
    hamR2 = np.concatenate([hamR, hamR[[i0]], hamR[[i1]]])
    same = Model(m.lat, m.orb, False, ham=ham2, hamR=hamR2)
    k = np.random.default_rng(3).uniform(0, 1, (9, 2))
    ref = O.gen_ham_batch(m, k, 1)
    assert rel(same.gen_ham_batch(k), ref) < 1e-12
    V, H = same.gen_v_projected_batch(k, Gauge.Atom, np.eye(2))
    Vr, Hr = O.gen_v_projected_batch(m, k, 1, np.eye(2))
    assert rel(V, Vr) < 1e-12
    E = same.solve_band_all_parallel(k, Precision.MIXED)
    assert np.max(np.abs(E - np.linalg.eigvalsh(ref))) <= 1e-9 * np.max(np.abs(np.linalg.eigvalsh(ref)))
    lone = Model(m.lat, m.orb, False, ham=np.concatenate([ham, ham[[i1]] * 0.3j]),
                 hamR=np.concatenate([hamR, hamR[[i1]] * 3]))
    with pytest.raises(errors.InvalidModel):
        lone.gen_ham_batch(k)
    # 40 bands: the same duplicates through the tensor-core Fourier table
    b = W.random_model(3, 40, False, 1, seed=78)
    j0 = int(np.flatnonzero(np.all(b.hamR == 0, axis=1))[0])
    j1 = int(np.flatnonzero(np.any(b.hamR != 0, axis=1))[0])
    hb = np.concatenate([b.ham, 0.5 * b.ham[[j0]], 0.25 * b.ham[[j1]]])
    hb[j0] *= 0.5
    hb[j1] *= 0.75
    big = Model(b.lat, b.orb, False, ham=hb, hamR=np.concatenate([b.hamR, b.hamR[[j0]], b.hamR[[j1]]]))
    kb = np.random.default_rng(4).uniform(0, 1, (24, 3))
    Eb = big.solve_band_all_parallel(kb, Precision.MIXED)
    Hb = O.gen_ham_batch(b, kb, 1)
    for i in range(24):
        assert np.max(np.abs(Eb[i] - O.eigvalsh(Hb[i]))) <= 1e-9 * np.linalg.norm(Hb[i], 2)


def test_rmatrix_commutator_term():
    m = W.random_model(2, 3, False, 1, seed=21)
    rng = np.random.default_rng(4)
    rm = (rng.standard_normal((3, 2, 3, 3)) + 1j * rng.standard_normal((3, 2, 3, 3))) * 0.1
    m.set_rmatrix(rm)
    k = rng.uniform(0, 1, (5, 2))
    for gauge in (Gauge.Atom, Gauge.Lattice):
        V, H = m.gen_v_projected_batch(k, gauge, np.eye(2))
        Vr, Hr = O.gen_v_projected_batch(m, k, int(gauge), np.eye(2))
        assert rel(V, Vr) < 1e-11


# -------------------------------------------------------------- eigensolver --
@pytest.mark.parametrize("norb,spin,dim", [(1, False, 2), (2, False, 2), (7, False, 3), (8, True, 2),
                                          (33, False, 2), (64, True, 3), (150, False, 2)])
def test_solve_band_matches_zheev(norb, spin, dim):
    m = W.random_model(dim, norb, spin, 1, seed=100 + norb)
    k = np.random.default_rng(norb).uniform(0, 1, (6, dim))
    E = m.solve_band_all_parallel(k)
    Eref = O.solve_band_all(m, k)
    Hs = O.gen_ham_batch(m, k, 1)
    for i in range(len(k)):
        nrm = np.linalg.norm(Hs[i], 2)
        assert np.max(np.abs(E[i] - Eref[i])) <= 1e-10 * nrm


@pytest.mark.parametrize("norb,spin", [(3, False), (16, True), (64, True)])
def test_solve_eigenvectors_rows(norb, spin):
    m = W.random_model(2, norb, spin, 1, seed=7 + norb)
    k = np.random.default_rng(1).uniform(0, 1, (4, 2))
    E, U = m.solve_all_parallel(k)
    Hs = O.gen_ham_batch(m, k, 1)
    Er, Ur = O.solve_all(m, k)
    for i in range(len(k)):
        nrm = np.linalg.norm(Hs[i], 2)
        rows = U[i]                                  # row n = eigenvector n
        assert np.max(np.abs(rows.conj() @ rows.T - np.eye(m.nsta))) < 1e-12
        resid = Hs[i] @ rows.T - rows.T * E[i][None, :]
        assert np.max(np.abs(resid)) < 1e-10 * nrm
        # band projectors P_n = u u^H agree with zheev's for well separated bands
        gaps = np.diff(Er[i])
        for n in range(m.nsta):
            g = min(gaps[n - 1] if n > 0 else np.inf, gaps[n] if n < m.nsta - 1 else np.inf)
            if g < 1e-6 * nrm:
                continue
            P = np.outer(rows[n], rows[n].conj())
            Pr = np.outer(Ur[i][n], Ur[i][n].conj())
            assert np.max(np.abs(P - Pr)) < 1e-8


def test_degenerate_kramers_pairs():
    """Kane-Mele keeps time reversal and inversion: every band is doubly
    degenerate; the degenerate subspace projector must still be exact."""
    km = M.kane_mele()
    k = np.array([[0.1, 0.2], [0.3, 0.4], [0.25, 0.6]])
    E, U = km.solve_all_parallel(k)
    Hs = O.gen_ham_batch(km, k, 1)
    for i in range(len(k)):
        assert np.allclose(E[i], O.eigvalsh(Hs[i]), atol=1e-12)
        rows = U[i]
        assert np.max(np.abs(rows.conj() @ rows.T - np.eye(4))) < 1e-12
        assert np.max(np.abs(Hs[i] @ rows.T - rows.T * E[i][None, :])) < 1e-12


# ---------------------------------------------------------- Berry and Hall --
def test_berry_curvature_matches_fixture():
    m = fixture_model()
    p = Parameters.rank2((1, 1, 1), XY3[0], XY3[1], [0.0])
    Om, E = m.berry_curvature_on(CASES["rs_k"], p)
    assert np.max(np.abs(E - CASES["rs_E"])) < 1e-12
    assert rel(Om, CASES["rs_Om"]) < 1e-8


def test_spin_berry_curvature_matches_fixture():
    m = fixture_model()
    p = Parameters.rank2((1, 1, 1), XY3[0], XY3[1], [0.0]).with_spin(SpinDirection.Z)
    Om, _ = m.berry_curvature_on(CASES["rs_k"], p)
    assert rel(Om, CASES["rs_OmSz"]) < 1e-8


@pytest.mark.parametrize("spin", [SpinDirection.X, SpinDirection.Y])
def test_spin_berry_curvature_xy(spin):
    km = M.kane_mele(rashba=0.05)
    k = np.random.default_rng(3).uniform(0, 1, (7, 2))
    p = Parameters.rank2((1, 1), [1.0, 0.0], [0.0, 1.0], [0.0]).with_spin(spin)
    occ = km.occupied_berry_curvature_on(k, p)
    ref = O.occupied_berry_curvature_on(km, k, np.eye(2), 0.0, 0.0, int(spin), 1e-3)
    assert np.max(np.abs(occ - ref)) <= 1e-8 * max(np.max(np.abs(ref)), 1.0)


def test_occupied_berry_curvature_haldane():
    h = M.haldane()
    k = O.gen_kmesh((9, 9))
    p = Parameters.rank2((1, 1), [1.0, 0.0], [0.0, 1.0], [0.0])
    got = h.occupied_berry_curvature_on(k, p)
    ref = O.occupied_berry_curvature_on(h, k, np.eye(2), 0.0)
    assert rel(got, ref) < 1e-8
    one = h.occupied_berry_curvature_at(k[3], p)
    assert abs(one - ref[3]) <= 1e-8 * max(abs(ref[3]), 1.0)


def test_hall_haldane_chern_and_oracle():
    ka = KNOWN["Haldan_model"]
    h = M.haldane()
    p = Parameters.rank2(tuple(ka["kmesh"]), [1.0, 0.0], [0.0, 1.0], [0.0])
    s = h.hall_conductivity(p).conductivity
    assert abs(s[0] * 2 * math.pi - ka["chern"]) < ka["chern_tol"]
    assert abs(s[0] - CASES["haldane_sigma_31"][0]) <= 1e-8 * abs(CASES["haldane_sigma_31"][0])


def test_hall_time_reversal_antisymmetry():
    ka = KNOWN["hall_conductivity_ec_tr"]
    lo, hi, n = ka["mu_grid"]
    mus = np.linspace(lo, hi, n)
    p = Parameters.rank2(tuple(ka["kmesh"]), [1.0, 0.0], [0.0, 1.0], mus)
    p.eta = ka["eta"]
    a = M.haldane(-0.3).hall_conductivity(p).conductivity
    b = M.haldane(0.3).hall_conductivity(p).conductivity
    assert np.max(np.abs(a + b)) < ka["tol"]


def test_hall_qwz_plateau():
    ka = KNOWN["hall_conductivity_ec_3d_qwz"]
    lo, hi, n = ka["mu_grid"]
    mus = np.linspace(lo, hi, n)
    q = M.qwz_stacked_3d(-1.0)
    for km in ka["kmesh"]:
        p = Parameters.rank2(tuple(km), [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], mus)
        p.eta = ka["eta"]
        s = q.hall_conductivity(p).conductivity
        ref = O.hall_conductivity(q, km, XY3, mus, 0.0, ka["eta"])
        assert np.max(np.abs(s - ref)) <= 1e-8 * np.max(np.abs(ref))
        assert abs(s[n // 2] - ka["plateau"]) < ka["direct_vs_energy_cut_tol"] + ka["plateau_tol_energy_cut"]


@pytest.mark.parametrize("T,key", [(0.0, "rs_sigma_444"), (300.0, "rs_sigma_444_T300")])
def test_hall_random_spinful_matches_fixture(T, key):
    m = fixture_model()
    p = Parameters.rank2((4, 4, 4), XY3[0], XY3[1], CASES["rs_mu"]).with_temperature(T)
    s = m.hall_conductivity(p).conductivity
    assert rel(s, CASES[key]) < 1e-8


def test_hall_chunking_is_invariant(monkeypatch):
    h = M.haldane()
    p = Parameters.rank2((13, 11), [1.0, 0.0], [0.0, 1.0], [-0.5, 0.0, 0.5])
    a = h.hall_conductivity(p).conductivity
    monkeypatch.setenv("TBG_MAX_CHUNK", "17")
    b = h.hall_conductivity(p).conductivity
    assert np.max(np.abs(a - b)) <= 1e-13 * np.max(np.abs(a))


def test_cfg1_haldane_200_chern():
    h = W.haldane_200()
    p = Parameters.rank2((200, 200), [1.0, 0.0], [0.0, 1.0], [0.0])
    s = h.hall_conductivity(p).conductivity
    assert round(abs(s[0] * 2 * math.pi)) == 1
    assert abs(abs(s[0] * 2 * math.pi) - 1.0) < 1e-3


# ------------------------------------------------------------ mixed path --
def test_mixed_matches_plain_cfg2_model():
    m = W.random_spinful_3d()
    p = Parameters.rank2((3, 3, 2), XY3[0], XY3[1], [0.0])
    plain = m.hall_conductivity(p, Precision.FP64).conductivity
    mixed = m.hall_conductivity(p, Precision.MIXED).conductivity
    assert abs(mixed[0] - plain[0]) <= 1e-6 * abs(plain[0])
    k = O.gen_kmesh((3, 3, 2))[:4]
    Om, E = m.berry_curvature_on(k, p, Precision.MIXED)
    Hs = O.gen_ham_batch(m, k, 1)
    for i in range(len(k)):
        Er = O.eigvalsh(Hs[i])
        assert np.max(np.abs(E[i] - Er)) <= 1e-9 * np.linalg.norm(Hs[i], 2)


# band counts that reach each layout of the FP32 solver inside the mixed
# chain: two matrices per SM with the tiled back-transformation (67; 134 with
# padding to a multiple of 4), one per SM with the panel back-transformation
# (150, 200)
@pytest.mark.parametrize("norb,spin", [(67, False), (134, False), (75, True), (100, True)])
def test_mixed_matches_plain_across_solver_layouts(norb, spin):
    m = W.random_model(2, norb, spin, 1, seed=900 + norb)
    p = Parameters.rank2((4, 4), [1.0, 0.0], [0.0, 1.0], [-0.1, 0.0, 0.2])
    plain = m.hall_conductivity(p, Precision.FP64).conductivity
    mixed = m.hall_conductivity(p, Precision.MIXED).conductivity
    assert np.max(np.abs(mixed - plain)) <= 1e-6 * np.max(np.abs(plain))
    k = O.gen_kmesh((4, 4))[:3]
    _, E = m.berry_curvature_on(k, p, Precision.MIXED)
    Hs = O.gen_ham_batch(m, k, 1)
    for i in range(len(k)):
        assert np.max(np.abs(E[i] - O.eigvalsh(Hs[i]))) <= 1e-9 * np.linalg.norm(Hs[i], 2)


# mixed-precision band energies (tbg_solve_band_prec): the tensor-core
# Fourier sum (nR <= 408) or the FP64 sum converted (3D, |R_i| <= 4: nR = 729),
# solver layouts from 24 to 251 bands
@pytest.mark.parametrize("dim,norb,spin,rmax", [(2, 24, False, 1), (3, 64, True, 1), (2, 134, False, 1),
                                                (2, 251, False, 1), (3, 20, False, 4)])
def test_mixed_band_energies(dim, norb, spin, rmax):
    m = W.random_model(dim, norb, spin, rmax, seed=700 + norb)
    k = np.random.default_rng(norb).uniform(0, 1, (40, dim))
    E = m.solve_band_all_parallel(k, Precision.MIXED)
    Hs = O.gen_ham_batch(m, k[:6], 1)
    for i in range(6):
        assert np.max(np.abs(E[i] - O.eigvalsh(Hs[i]))) <= 1e-9 * np.linalg.norm(Hs[i], 2)
    E64 = m.solve_band_all_parallel(k)
    assert np.max(np.abs(E - E64)) <= 1e-9 * np.max(np.abs(E64))
    assert np.all(np.diff(E, axis=1) >= 0)


def test_mixed_beyond_256_bands():
    """300 bands: the FP32 solver with the matrix in global memory and the
    tensor-core products in chunks of 256 along K."""
    m = W.random_model(2, 300, False, 1, seed=1300)
    p = Parameters.rank2((3, 3), [1.0, 0.0], [0.0, 1.0], [-0.1, 0.0, 0.2])
    plain = m.hall_conductivity(p, Precision.FP64).conductivity
    mixed = m.hall_conductivity(p, Precision.MIXED).conductivity
    assert np.max(np.abs(mixed - plain)) <= 1e-6 * np.max(np.abs(plain))
    k = O.gen_kmesh((3, 3))[:2]
    E = m.solve_band_all_parallel(k, Precision.MIXED)
    Hs = O.gen_ham_batch(m, k, 1)
    for i in range(len(k)):
        assert np.max(np.abs(E[i] - O.eigvalsh(Hs[i]))) <= 1e-9 * np.linalg.norm(Hs[i], 2)


def test_mixed_supercell_1024_bands():
    """The 1024-orbital supercell workload: dense spectrum, two refinement sweeps."""
    m = W.supercell_2d()
    p = Parameters.rank2((2, 2), [1.0, 0.0], [0.0, 1.0], [0.0])
    plain = m.hall_conductivity(p, Precision.FP64).conductivity
    mixed = m.hall_conductivity(p, Precision.MIXED).conductivity
    assert abs(mixed[0] - plain[0]) <= 1e-6 * abs(plain[0])


def test_mixed_handles_kramers_clusters():
    km = M.kane_mele()
    p = Parameters.rank2((12, 12), [1.0, 0.0], [0.0, 1.0], [-0.5, 0.0, 0.5]).with_spin(SpinDirection.Z)
    plain = km.hall_conductivity(p, Precision.FP64).conductivity
    mixed = km.hall_conductivity(p, Precision.MIXED).conductivity
    assert np.max(np.abs(mixed - plain)) <= 1e-6 * max(np.max(np.abs(plain)), 1e-3)


# ------------------------------------------------------------ error paths --
def test_error_paths():
    h = M.haldane()
    p = Parameters.rank2((4, 4), [1.0, 0.0], [0.0, 1.0], [0.0]).with_spin(SpinDirection.Z)
    with pytest.raises(errors.SpinNotAllowed):
        h.hall_conductivity(p)
    with pytest.raises(errors.InvalidResponseParameter):
        h.hall_conductivity(Parameters.rank2((4, 4), [0.0, 0.0], [0.0, 1.0], [0.0]))
    with pytest.raises(errors.InvalidKmeshDimensions):
        h.hall_conductivity(Parameters.rank2((0, 4), [1.0, 0.0], [0.0, 1.0], [0.0]))
    with pytest.raises(errors.KVectorLengthMismatch):
        h.berry_curvature_at([0.1, 0.2, 0.3], Parameters.rank2((1, 1), [1.0, 0.0], [0.0, 1.0], [0.0]))
    with pytest.raises(errors.TbPanic):
        h.gen_ham([0.1])
    # the C-ABI itself rejects a spin current on a spinless model
    import ctypes
    from rustb_gb300 import _lib
    lib = _lib.load()
    k = np.zeros((1, 2))
    d = np.eye(2)
    out = np.zeros(2)
    st = lib.tbg_berry_curvature(h.device_handle(), 1, _lib.dptr(k), _lib.dptr(d), 2, 1e-3, 0,
                                 _lib.dptr(out), _lib.dptr(out))
    assert st == errors.TBG_E_SPIN_NOT_ALLOWED
    assert "spin" in _lib.last_error().lower()
    st = lib.tbg_berry_curvature(h.device_handle(), 1, _lib.dptr(k), _lib.dptr(d), -1, float("nan"), 0,
                                 _lib.dptr(out), _lib.dptr(out))
    assert st == errors.TBG_E_INVALID_RESPONSE_PARAMETER


def test_empty_k_list_is_ok():
    h = M.haldane()
    E = h.solve_band_all_parallel(np.zeros((0, 2)))
    assert E.shape == (0, 2)


# ----------------------------------------------------- small-N fused path --
@pytest.mark.parametrize("norb,spin_model,dim,spin", [(3, False, 2, None), (5, False, 3, None),
                                                      (4, True, 2, SpinDirection.Z), (4, True, 3, SpinDirection.X),
                                                      (2, True, 2, SpinDirection.Y), (1, False, 1, None)])
def test_small_fused_path_matches_oracle(norb, spin_model, dim, spin):
    m = W.random_model(dim, norb, spin_model, 1, seed=50 + norb + dim)
    rng = np.random.default_rng(norb)
    k = rng.uniform(0, 1, (37, dim))
    dirs = np.eye(dim)[:2] if dim > 1 else np.array([[1.0], [1.0]])
    p = Parameters(kmesh=(1,) * dim, direction=dirs, mu=[0.0])
    if spin is not None:
        p = p.with_spin(spin)
    Om, E = m.berry_curvature_on(k, p)
    Omr, Er = O.berry_on(m, k, dirs, -1 if spin is None else int(spin))
    assert np.max(np.abs(E - Er)) <= 1e-12 * max(1.0, np.max(np.abs(Er)))
    assert rel(Om, Omr) < 1e-8
    if dim > 1:
        mus = np.array([-0.3, 0.0, 0.4])
        ph = Parameters(kmesh=(5,) * dim, direction=dirs, mu=mus)
        if spin is not None:
            ph = ph.with_spin(spin)
        s = m.hall_conductivity(ph).conductivity
        ref = O.hall_conductivity(m, (5,) * dim, dirs, mus, 0.0, 1e-3, -1 if spin is None else int(spin))
        assert np.max(np.abs(s - ref)) <= 1e-8 * max(np.max(np.abs(ref)), 1e-12)


# ------------------------------------------------------------ large models --
@pytest.mark.parametrize("norb,spin", [(256, False), (160, True), (512, False)])
def test_large_models_eigenvalues_and_berry(norb, spin):
    m = W.random_model(2, norb, spin, 1, seed=norb)
    k = np.random.default_rng(2).uniform(0, 1, (2, 2))
    E = m.solve_band_all_parallel(k)
    Hs = O.gen_ham_batch(m, k, 1)
    for i in range(len(k)):
        nrm = np.linalg.norm(Hs[i], 2)
        assert np.max(np.abs(E[i] - O.eigvalsh(Hs[i]))) <= 1e-10 * nrm
    if m.nsta <= 320:
        p = Parameters.rank2((1, 1), [1.0, 0.0], [0.0, 1.0], [0.0])
        Om, E2 = m.berry_curvature_on(k[:1], p)
        Omr, Er = O.berry_on(m, k[:1], np.eye(2))
        assert rel(Om, Omr) < 1e-8
        Omm, Em = m.berry_curvature_on(k[:1], p, Precision.MIXED)
        assert np.max(np.abs(Em - Er)) <= 1e-9 * np.linalg.norm(Hs[0], 2)
        occ = Er[0] < 0
        assert abs((Omm[0] * occ).sum() - (Omr[0] * occ).sum()) <= 1e-6 * np.abs(Omr[0]).sum()


@pytest.mark.parametrize("norb,spin", [(6, False), (4, True)])
def test_small_models_with_large_tables_take_the_batched_path(norb, spin):
    """Models of at most 8 states with more than 32 R vectors (3D, |R_i| <= 3:
    343 R) run the batched FP64 pipeline instead of the one-thread-per-k
    kernel; MIXED requests on them run FP64.  Against the oracle."""
    m = W.random_model(3, norb, spin, 3, seed=910 + norb)
    assert m.nR == 343
    k = np.random.default_rng(norb).uniform(0, 1, (23, 3))
    p = Parameters.rank2((1, 1, 1), XY3[0], XY3[1], [0.0])
    Omr, Er = O.berry_on(m, k, XY3)
    for prec in (Precision.FP64, Precision.MIXED):
        Om, E = m.berry_curvature_on(k, p, prec)
        assert np.max(np.abs(E - Er)) <= 1e-10 * np.max(np.abs(Er))
        assert rel(Om, Omr) < 1e-8
        assert np.max(np.abs(m.solve_band_all_parallel(k, prec) - Er)) <= 1e-10 * np.max(np.abs(Er))
    mus = np.array([-0.3, 0.0, 0.4])
    ph = Parameters.rank2((3, 3, 2), XY3[0], XY3[1], mus)
    ref = O.hall_conductivity(m, (3, 3, 2), XY3, mus)
    for prec in (Precision.FP64, Precision.MIXED):
        s = m.hall_conductivity(ph, prec).conductivity
        assert np.max(np.abs(s - ref)) <= 1e-8 * np.max(np.abs(ref))
