"""The quantum-geometry and DOS restatements of the oracle against analytic
known answers (CPU).

Rustb's own tests for these paths assert shapes only
(src/quantum_geometry.rs:318-328) and a Direct/Simplex agreement whose values
are not recorded (:330-342); the DOS is plotted, not asserted
(src/lib.rs:1352-1365).  The restatements are therefore pinned here by
closed forms:
- the Berry component of the geometric tensor equals the Kubo Berry curvature
  already pinned against the reference's known answers;
- for a two-band model H = d(k).sigma the metric of either band is
  g_ab = 1/4 d_a(d^) . d_b(d^) (d^ = d/|d|, derivatives along Cartesian k),
  and tr g >= |Omega| pointwise;
- the mesh-integrated Berry curvature of the QWZ model is C / (2 pi), C = +-1;
- flat bands give a mesh-independent DOS equal to the bare Gaussians, and the
  DOS integrates to the number of states.
"""

import math

import numpy as np
import pytest

import models as M
from oracle import tb_oracle as O

XY = np.array([[1.0, 0.0], [0.0, 1.0]])
XX = np.array([[1.0, 0.0], [1.0, 0.0]])
YY = np.array([[0.0, 1.0], [0.0, 1.0]])


def test_geometry_berry_component_equals_kubo_curvature():
    rng = np.random.default_rng(5)
    for model in (M.haldane(), M.kane_mele(rashba=0.05), M.qwz_2d(-1.0)):
        for k in rng.random((4, 2)):
            g, om, E = O.quantum_geometry_at(model, k, XY, eta=1e-3)
            om2, E2 = O.berry_curvature_at(model, k, XY, -1, 1e-3)
            assert np.array_equal(E, E2)
            assert np.allclose(om, om2, rtol=1e-12, atol=1e-12 * np.max(np.abs(om2)))
            assert g.shape == om.shape == (model.nsta,)


def _d_vector(model, kc):
    """d(k) of a two-band H = d0 + d.sigma at Cartesian k (lattice = identity, orbitals at 0)."""
    H = O.gen_ham(model, np.asarray(kc) / (2.0 * math.pi), 1)
    return np.array([H[0, 1].real, -H[0, 1].imag, 0.5 * (H[0, 0] - H[1, 1]).real])


@pytest.mark.parametrize("mass", [-1.0, 1.5, -2.5])
def test_two_band_metric_closed_form(mass):
    model = M.qwz_2d(mass)
    rng = np.random.default_rng(11)
    h = 1e-5
    for kf in rng.random((5, 2)):
        kc = 2.0 * math.pi * kf
        dh = []
        for a in range(2):
            e = np.zeros(2)
            e[a] = h
            dp = _d_vector(model, kc + e)
            dm = _d_vector(model, kc - e)
            dh.append((dp / np.linalg.norm(dp) - dm / np.linalg.norm(dm)) / (2 * h))
        g_exact = np.array([[0.25 * dh[a] @ dh[b] for b in range(2)] for a in range(2)])
        for dirs, (a, b) in ((XX, (0, 0)), (YY, (1, 1)), (XY, (0, 1))):
            g, om, _ = O.quantum_geometry_at(model, kf, dirs, eta=1e-9)
            assert np.allclose(g, g_exact[a, b], rtol=1e-6, atol=1e-8), (dirs, g, g_exact[a, b])
        gxx = O.quantum_geometry_at(model, kf, XX, eta=1e-9)[0]
        gyy = O.quantum_geometry_at(model, kf, YY, eta=1e-9)[0]
        om = O.quantum_geometry_at(model, kf, XY, eta=1e-9)[1]
        assert np.all(gxx + gyy >= np.abs(om) * (1 - 1e-9))


def test_metric_diagonal_is_non_negative():
    rng = np.random.default_rng(3)
    for model in (M.haldane(), M.kane_mele(rashba=0.1)):
        for k in rng.random((3, 2)):
            for dirs in (XX, YY):
                g, _, _ = O.quantum_geometry_at(model, k, dirs, eta=1e-3)
                assert np.all(g >= 0.0)


def test_qwz_mesh_berry_is_chern_over_two_pi():
    model = M.qwz_2d(-1.0)
    metric, berry = O.quantum_geometry(model, [31, 31], XY, [0.0], T=0.0, eta=1e-4)
    assert abs(abs(2.0 * math.pi * berry[0]) - 1.0) < 2e-2
    # the occupied band's metric integrates to a positive number (QWZ, m = -1)
    assert metric[0] > 0.0


def test_dos_flat_bands_closed_form():
    levels = [-1.25, 0.0, 0.4, 2.0]
    model = M.flat_bands(levels)
    E_min, E_max, E_n, sigma = -3.0, 3.0, 601, 0.05
    E, d = O.dos(model, [3, 4], E_min, E_max, E_n, sigma)
    expect = sum(np.exp(-((E - x) / sigma) ** 2 / 2.0) / sigma / math.sqrt(2 * math.pi) for x in levels)
    assert np.allclose(d, expect, rtol=1e-12, atol=1e-15)


def test_dos_integrates_to_state_count():
    model = M.haldane()
    E, d = O.dos(model, [24, 24], -12.0, 12.0, 4801, 0.05)  # bands within |E| < 9
    step = E[1] - E[0]
    assert abs(d.sum() * step - model.nsta) < 1e-6


def test_dos_energy_grid_is_ndarray_linspace():
    E = O.dos_energies(-3.0, 3.0, 500)
    step = 6.0 / 499.0
    assert E[0] == -3.0 and E[1] == -3.0 + step and E[-1] == -3.0 + step * 499.0
    assert np.array_equal(O.dos_energies(0.5, 1.0, 1), np.array([0.5]))
