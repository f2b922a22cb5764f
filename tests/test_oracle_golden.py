"""The oracle against the known answers held by Rustb's own tests (CPU).

Each test restates one assertion of src/lib.rs on the oracle; the values and
tolerances come from tests/golden/reference_known_answers.json.
"""

import json
import math
import os

import numpy as np
import pytest

import models as M
from oracle import tb_oracle as O
from rustb_gb300 import workloads as W

HERE = os.path.dirname(os.path.abspath(__file__))
KNOWN = json.load(open(os.path.join(HERE, "golden", "reference_known_answers.json")))
CASES = np.load(os.path.join(HERE, "golden", "oracle_cases.npz"))


def test_gen_v_golden_matrices():
    ka = KNOWN["test_gen_v"]
    g = M.graphene()
    assert np.array_equal(O.eigvalsh(O.gen_ham(g, [0.0, 0.0])), np.array(ka["gamma_bands"]))
    assert np.all(np.abs(O.eigvalsh(O.gen_ham(g, ka["k_bands_zero"]))) < ka["k_bands_tol"])
    V, _ = O.gen_v(g, ka["gen_v_k"], 1)
    tol = ka["gen_v_tol"]
    for key, (p, i, j) in {"gen_v_atom_x_01": (0, 0, 1), "gen_v_atom_x_10": (0, 1, 0),
                           "gen_v_atom_y_01": (1, 0, 1), "gen_v_atom_y_10": (1, 1, 0)}.items():
        assert abs(V[p, i, j] - complex(*ka[key])) < tol, key
    assert abs(V[0, 0, 0]) < tol and abs(V[1, 1, 1]) < tol
    VL, _ = O.gen_v(g, ka["gen_v_k"], 0)
    assert abs(VL[0, 0, 1] - complex(*ka["gen_v_lattice_x_01"])) < tol
    assert abs(VL[0, 1, 0] - complex(*ka["gen_v_lattice_x_10"])) < tol
    # solve_onek rows diagonalise gen_ham (lib.rs:742-754)
    E, U = O.solve_all(g, np.array([ka["gen_v_k"]]))
    H = O.gen_ham(g, ka["gen_v_k"], 1)
    D = U[0].conj() @ H @ U[0].T
    assert np.allclose(np.real(np.diag(D)), E[0], atol=ka["solve_onek_tol"])


def test_evec_transform_sanity():
    ka = KNOWN["evec_transform_sanity"]
    h = M.haldane()
    H = O.gen_ham(h, ka["k"], 1)
    E, W_ = O.eigh(H)
    D = W_.conj().T @ H @ W_
    assert np.max(np.abs(D - np.diag(E))) < ka["tol"]


def test_haldane_chern_number():
    ka = KNOWN["Haldan_model"]
    h = M.haldane()
    sigma = O.hall_conductivity(h, ka["kmesh"], np.eye(2), np.array([0.0]), 0.0, ka["eta"])
    assert abs(sigma[0] * 2 * math.pi - ka["chern"]) < ka["chern_tol"]
    lo, hi, n = ka["mu_grid"]
    mus = np.linspace(lo, hi, n)
    grid = O.hall_conductivity(h, ka["kmesh"], np.eye(2), mus, 0.0, ka["eta"])
    assert abs(grid[50] - sigma[0]) < ka["mu_grid_tol"]
    for idx, mu in [(0, -2.0), (100, 2.0)]:
        single = O.hall_conductivity(h, ka["kmesh"], np.eye(2), np.array([mu]), 0.0, ka["eta"])
        assert abs(grid[idx] - single[0]) < ka["mu_grid_tol"]


def test_kubo_matches_wilson_loop():
    ka = KNOWN["conductivity_test"]
    h = M.haldane()
    k = np.array(ka["k"])
    d1, d2 = np.array([1.0, 0.0]), np.array([0.0, 1.0])
    Om, E = O.berry_curvature_at(h, k, np.array([d1, d2]), -1, ka["eta"])
    result1 = Om[E <= 0.0].sum() * 2 * math.pi
    dk = ka["dk"]
    loop = [k + dk * d1, k + dk * d1 + dk * d2, k + dk * d2, k - dk * d1 + dk * d2, k - dk * d1,
            k - dk * d1 - dk * d2, k - dk * d2, k + dk * d1 - dk * d2, k + dk * d1]
    phase = O.berry_loop(h, np.array(loop), [0])
    result2 = phase / dk ** 2 / 4.0 / (2 * math.pi) * math.sqrt(3.0) / 2.0
    assert abs(result2 - result1) < ka["wilson_tol"]


def test_single_vs_multi_mu():
    ka = KNOWN["conductivity_test"]
    h = M.haldane()
    kmesh = (20, 20)  # the reference uses 100x100; the identity holds at any mesh
    a1 = O.hall_conductivity(h, kmesh, np.array([[0.0, 1.0], [1.0, 0.0]]), np.array([ka["mu"]]), 0.0, ka["eta"])
    a2 = O.hall_conductivity(h, kmesh, np.array([[0.0, 1.0], [1.0, 0.0]]), np.array([ka["mu"], 0.0]), 0.0,
                             ka["eta"])
    assert abs(a1[0] - a2[0]) < ka["single_vs_multi_tol"]


def test_time_reversal_antisymmetry():
    ka = KNOWN["hall_conductivity_ec_tr"]
    lo, hi, n = ka["mu_grid"]
    mus = np.linspace(lo, hi, n)
    kmesh = (25, 25)  # reference: 51x51; the antisymmetry is exact at any mesh
    a = O.hall_conductivity(M.haldane(-0.3), kmesh, np.eye(2), mus, 0.0, ka["eta"])
    b = O.hall_conductivity(M.haldane(0.3), kmesh, np.eye(2), mus, 0.0, ka["eta"])
    assert np.max(np.abs(a + b)) < ka["tol"]


def test_qwz_3d_plateau_direct():
    ka = KNOWN["hall_conductivity_ec_3d_qwz"]
    q = M.qwz_stacked_3d(-1.0)
    lo, hi, n = ka["mu_grid"]
    mus = np.linspace(lo, hi, n)
    for km in ka["kmesh"]:
        s = O.hall_conductivity(q, km, np.array([[1.0, 0, 0], [0, 1.0, 0]]), mus, 0.0, ka["eta"])
        # Direct integration agrees with the energy-cut plateau within the reference's tolerance
        assert abs(s[n // 2] - ka["plateau"]) < ka["direct_vs_energy_cut_tol"] + ka["plateau_tol_energy_cut"]


def test_berry_kernel_consistency():
    """Omega_n from the band-basis K_nm equals the direct sum (lib.rs:2519-2559)."""
    ka = KNOWN["berry_curvature_kernel_consistency"]
    h = M.haldane(-0.3)
    ks = O.gen_kmesh((7, 7))
    for k in ks:
        Om, E = O.berry_curvature_at(h, k, np.eye(2), -1, ka["eta"])
        V, H = O.gen_v_projected(h, k, 1, np.eye(2))
        E2, W_ = O.eigh(H)
        Ka = (W_.conj().T @ V[0] @ W_) * (W_.conj().T @ V[1] @ W_).T
        dE = E2[:, None] - E2[None, :]
        t = Ka / (dE * dE + ka["eta"] ** 2)
        np.fill_diagonal(t, 0)
        assert np.max(np.abs(-2.0 * t.sum(1).imag - Om)) < ka["tol"]


def test_fermi_function_rules():
    ka = KNOWN["thermodynamics"]
    assert O.fermi(np.array([0.0]), 0.0, 0.0)[0] == ka["step_at_mu"]
    assert O.fermi(np.array([-1.0, 1.0]), 0.0, 0.0).tolist() == [1.0, 0.0]
    w = 0.01
    assert O.fermi(np.array([0.6]), 0.0, w)[0] == 0.0       # x = 60 > 50
    assert O.fermi(np.array([-0.6]), 0.0, w)[0] == 1.0
    assert abs(O.fermi(np.array([0.1]), 0.0, w)[0] - 1.0 / (1.0 + math.exp(10.0))) < 1e-15


def test_gen_kmesh_order():
    k = O.gen_kmesh((2, 3))
    assert k.shape == (6, 2)
    assert k[:3, 0].tolist() == [0.0, 0.0, 0.0] and k[3:, 0].tolist() == [0.5, 0.5, 0.5]
    assert np.allclose(k[:3, 1], [0, 1 / 3, 2 / 3])


def test_oracle_reproduces_fixtures():
    """The oracle still produces the committed fixture values (no drift)."""
    m = W.Model(CASES["rs_lat"], CASES["rs_orb"], True, ham=CASES["rs_ham"], hamR=CASES["rs_hamR"])
    dirs = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])
    V, H = O.gen_v_projected_batch(m, CASES["rs_k"], 1, dirs)
    assert np.allclose(H, CASES["rs_H"], atol=1e-13) and np.allclose(V, CASES["rs_V"], atol=1e-13)
    Om, E = O.berry_on(m, CASES["rs_k"], dirs, -1, 1e-3)
    assert np.allclose(E, CASES["rs_E"], atol=1e-12)
    assert np.allclose(Om, CASES["rs_Om"], rtol=1e-8, atol=1e-8 * np.abs(CASES["rs_Om"]).max())


def test_cfg1_haldane_workload_is_topological():
    h = W.haldane_200()
    s = O.hall_conductivity(h, (40, 40), np.eye(2), np.array([0.0]), 0.0, 1e-3)
    assert round(abs(s[0] * 2 * math.pi)) == 1


@pytest.mark.parametrize("spin", [-1, 0, 1, 2])
def test_spin_matrix_is_sigma_over_two(spin):
    S = O.spin_matrix(2, spin)
    if spin < 0:
        assert np.array_equal(S, np.eye(4))
    else:
        assert np.allclose(S, S.conj().T)
        assert np.allclose(S @ S, 0.25 * np.eye(4))
