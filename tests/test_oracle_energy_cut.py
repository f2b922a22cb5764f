"""The oracle's energy-cut Hall restatement against the known answers of
Rustb's own energy-cut tests (CPU):
- hall_conductivity_ec_vs_reference (src/lib.rs:2621-2661): Haldane t2 = -0.3,
  eta = 0.05, mu in [-3, 3]: |sigma_EC - sigma_Direct| < 3e-2;
- hall_conductivity_ec_tr (src/lib.rs:2663-2729): sigma_EC(t2) + sigma_EC(-t2)
  = 0 to 1e-10 on the 51 x 51 mesh;
- hall_conductivity_ec_3d_qwz (src/lib.rs:3222-3262): stacked QWZ m = -1,
  eta = 0.1: |EC - Direct| < 5e-2 and the mu = 0 plateau within 0.003 of 1/(2 pi)
  (the 10 x 10 x 4 mesh of the reference's pair);
and, for T > 0, the thermal convolution against the Direct sum."""

import math

import numpy as np

import models as M
from oracle import tb_oracle as O


def test_ec_vs_direct_haldane():
    m = M.haldane_2d(-0.3)
    mu = np.linspace(-3.0, 3.0, 201)
    ec = O.hall_energy_cut(m, [31, 31], np.eye(2), mu, 0.0, 0.05)
    d = O.hall_conductivity(m, [31, 31], np.eye(2), mu, 0.0, 0.05)
    assert np.max(np.abs(ec - d)) < 3e-2


def test_ec_time_reversal():
    mu = np.linspace(-3.0, 3.0, 101)
    a = O.hall_energy_cut(M.haldane_2d(-0.3), [51, 51], np.eye(2), mu, 0.0, 0.05)
    b = O.hall_energy_cut(M.haldane_2d(0.3), [51, 51], np.eye(2), mu, 0.0, 0.05)
    assert np.max(np.abs(a + b)) < 1e-10


def test_ec_3d_qwz_plateau():
    m = M.qwz_stacked_3d(-1.0)
    mu = np.linspace(-3.0, 3.0, 61)
    dirs = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])
    ec = O.hall_energy_cut(m, [10, 10, 4], dirs, mu, 0.0, 0.1)
    d = O.hall_conductivity(m, [10, 10, 4], dirs, mu, 0.0, 0.1)
    assert np.max(np.abs(ec - d)) < 5e-2
    assert abs(ec[30] - 1.0 / (2.0 * math.pi)) < 0.003


def test_ec_finite_temperature_matches_direct():
    m = M.haldane()
    mu = np.linspace(-1.0, 1.0, 11)
    ec = O.hall_energy_cut(m, [12, 12], np.eye(2), mu, 300.0, 0.05)
    d = O.hall_conductivity(m, [12, 12], np.eye(2), mu, 300.0, 0.05)
    assert np.max(np.abs(ec - d)) < 1e-4


def test_greedy_assignment_and_tracking_order():
    ov = np.array([[0.1, 0.9, 0.0], [0.8, 0.15, 0.05], [0.1, 0.1, 0.8]])
    assert O.greedy_assign(ov) == [1, 0, 2]
    # equal best values: rows keep their order (stable sort), columns the first maximum
    assert O.greedy_assign(np.array([[0.5, 0.5], [0.5, 0.5]])) == [0, 1]
    assert O.neighbour_indices(0, [3, 4]) == [4, 1]
    assert O.neighbour_indices(5, [3, 4]) == [9, 1, 6, 4]
