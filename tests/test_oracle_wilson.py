"""The oracle's Wilson-loop restatement pinned by closed forms and the
reference's known answers (CPU).

- Flat bands with orbitals at tau: each eigenvector is k-independent, so the
  only non-trivial overlap is the loop's gauge phase: the Berry phase of band n
  along G is 2 pi G . tau_n (mod 2 pi).
- The det form is the sum of the unitary-product phases (mod 2 pi): the SVD
  only removes the positive singular values.
- berry_flux summed over the BZ / 2 pi is the Chern number (Haldane: |C| = 1,
  the value src/lib.rs's Haldan_model test prints), and a small plaquette's
  flux is Omega times its area (conductivity_test, src/lib.rs:757-830).
- Kramers pairs: on the time-reversal-invariant lines of the Kane-Mele model
  the two Wannier centres coincide (mod 2 pi).
"""

import math

import numpy as np

import models as M
from oracle import tb_oracle as O


def _wrap(x):
    return (x + math.pi) % (2 * math.pi) - math.pi


def test_flat_band_berry_phase_is_two_pi_g_tau():
    taus = [[0.1, 0.3], [1.0 / 3.0, 1.0 / 3.0], [0.75, 0.2]]
    m = M.Model.tb_model(np.eye(2), taus)
    m.set_onsite([-1.0, 0.5, 2.0])
    for G in ([0, 1], [1, 0], [1, 1], [2, -1]):
        loop = np.array([[0.2 + G[0] * t, 0.1 + G[1] * t] for t in np.linspace(0.0, 1.0, 9)])
        for n in range(3):
            ph = O.wilson_loop(m, loop, [n])[0]
            expect = 2 * math.pi * float(np.dot(G, taus[n]))
            assert abs(_wrap(ph - expect)) < 1e-12


def test_det_form_is_the_sum_of_the_unitary_phases():
    rng = np.random.default_rng(2)
    for model, occ in ((M.haldane(), [0]), (M.kane_mele(rashba=0.1), [0, 1]), (M.qwz_stacked_3d(), [0])):
        for _ in range(3):
            k0 = rng.random(model.dim)
            G = np.zeros(model.dim)
            G[rng.integers(model.dim)] = 1.0
            loop = np.array([k0 + G * t for t in np.linspace(0.0, 1.0, 31)])
            s = float(np.sum(O.wilson_loop(model, loop, occ)))
            d = O.wilson_loop_det(model, loop, occ)
            assert abs(_wrap(s - d)) < 1e-9


def test_haldane_chern_from_plaquette_fluxes():
    flux = O.berry_flux(M.haldane(), [0], [0.0, 0.0], [1.0, 0.0], [0.0, 1.0], 31, 31)
    C = flux.sum() / (2 * math.pi)
    assert abs(abs(C) - 1.0) < 1e-9


def test_small_plaquette_flux_is_curvature_times_area():
    m = M.haldane()
    k = np.array([0.21, 0.37])
    h = 1e-3
    flux = O.berry_flux(m, [0], k, [h, 0.0], [0.0, h], 1, 1)[0, 0, 0]
    om, _ = O.berry_curvature_at(m, k + h / 2, np.eye(2), -1, 1e-12)
    # reciprocal-lattice area of the plaquette: h^2 |det B|, B = 2 pi lat^-T
    area = h * h * abs(np.linalg.det(2 * math.pi * np.linalg.inv(m.lat).T))
    # counter-clockwise plaquette: flux = +Omega x area (the relation conductivity_test asserts)
    assert abs(flux - om[0] * area) < 1e-4 * abs(om[0] * area)


def test_kramers_pairs_on_time_reversal_lines():
    m = M.kane_mele(rashba=0.0)
    wcc = O.wannier_centre(m, [0, 1], [0.0, 0.0], [1.0, 0.0], [0.0, 1.0], 3, 41)  # k1 = 0, 0.5, 1
    for col in (0, 1, 2):
        a, b = wcc[:, col]
        assert abs(_wrap(a - b)) < 1e-8


def test_plaquette_det_matches_the_kubo_pin_restatement():
    # the Kubo-formula pin (conductivity_test) uses berry_loop on closed
    # plaquettes, where the gauge phase is 1: both forms agree there
    m = M.haldane()
    loop = np.array([[0.1, 0.1], [0.12, 0.1], [0.12, 0.12], [0.1, 0.12], [0.1, 0.1]])
    assert abs(_wrap(O.berry_loop(m, loop, [0]) - O.wilson_loop_det(m, loop, [0]))) < 1e-12
