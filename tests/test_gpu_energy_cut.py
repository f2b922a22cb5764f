"""GPU parity for Integration::EnergyCut of hall_conductivity: the device
path (vertex data, edge overlaps, host tracking, simplex occupancy cut)
against the oracle's restatement on the same inputs (1e-9 of the scale for
gapped / generic models), and the known answers of Rustb's own energy-cut
tests at their full mesh sizes."""

import math

import numpy as np
import pytest

import models as M
from oracle import tb_oracle as O
from rustb_gb300 import errors, workloads as W
from rustb_gb300.params import Integration, Parameters, SpinDirection

pytestmark = pytest.mark.gpu

XY3 = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])


def ec(model, kmesh, dirs, mu, T=0.0, eta=0.05, spin=None):
    p = Parameters.rank2(kmesh, dirs[0], dirs[1], list(mu))
    p.T = np.array([T])
    p.eta = eta
    p.integration = Integration.EnergyCut
    if spin is not None:
        p.spin = spin
    return model.hall_conductivity(p).conductivity


def direct(model, kmesh, dirs, mu, eta):
    p = Parameters.rank2(kmesh, dirs[0], dirs[1], list(mu))
    p.eta = eta
    return model.hall_conductivity(p).conductivity


def close(a, b, tol):
    return np.max(np.abs(a - b)) <= tol * max(np.max(np.abs(b)), 1e-3)


@pytest.mark.parametrize("name,build,kmesh,dirs,eta", [
    ("haldane", lambda: M.haldane_2d(-0.3), [21, 21], np.eye(2), 0.05),
    ("haldane_ragged", M.haldane, [7, 11], np.eye(2), 0.02),
    ("random2d_n6", lambda: W.random_model(2, 6, False, 1, seed=501), [9, 8], np.eye(2), 0.05),
    ("qwz3d", lambda: M.qwz_stacked_3d(-1.0), [6, 6, 3], XY3, 0.1),
    ("random3d_n4", lambda: W.random_model(3, 4, False, 1, seed=502), [4, 5, 3], XY3, 0.05),
])
def test_energy_cut_matches_oracle(name, build, kmesh, dirs, eta):
    m = build()
    mu = np.linspace(-3.0, 3.0, 41)
    got = ec(m, kmesh, dirs, mu, eta=eta)
    ref = O.hall_energy_cut(m, kmesh, dirs, mu, 0.0, eta)
    assert close(got, ref, 1e-9)


def test_energy_cut_spin_current_matches_oracle():
    m = M.kane_mele(rashba=0.05)
    mu = np.linspace(-2.0, 2.0, 21)
    got = ec(m, [9, 9], np.eye(2), mu, eta=0.05, spin=SpinDirection.Z)
    ref = O.hall_energy_cut(m, [9, 9], np.eye(2), mu, 0.0, 0.05, spin=int(SpinDirection.Z))
    assert close(got, ref, 1e-8)


def test_energy_cut_finite_temperature_matches_oracle():
    m = M.haldane()
    mu = np.linspace(-1.0, 1.0, 11)
    got = ec(m, [12, 12], np.eye(2), mu, T=300.0, eta=0.05)
    ref = O.hall_energy_cut(m, [12, 12], np.eye(2), mu, 300.0, 0.05)
    assert close(got, ref, 1e-9)


@pytest.mark.parametrize("nk", [31, 51, 71, 101])
def test_ec_vs_direct_reference_bound(nk):
    """hall_conductivity_ec_vs_reference (src/lib.rs:2621-2661)."""
    m = M.haldane_2d(-0.3)
    mu = np.linspace(-3.0, 3.0, 201)
    assert np.max(np.abs(ec(m, [nk, nk], np.eye(2), mu) - direct(m, [nk, nk], np.eye(2), mu, 0.05))) < 3e-2


def test_ec_time_reversal_51():
    """hall_conductivity_ec_tr (src/lib.rs:2663-2729)."""
    mu = np.linspace(-3.0, 3.0, 101)
    a = ec(M.haldane_2d(-0.3), [51, 51], np.eye(2), mu)
    b = ec(M.haldane_2d(0.3), [51, 51], np.eye(2), mu)
    assert np.max(np.abs(a + b)) < 1e-10


@pytest.mark.parametrize("nk", [10, 14])
def test_ec_3d_qwz_plateau(nk):
    """hall_conductivity_ec_3d_qwz (src/lib.rs:3222-3262)."""
    m = M.qwz_stacked_3d(-1.0)
    mu = np.linspace(-3.0, 3.0, 61)
    e = ec(m, [nk, nk, 4], XY3, mu, eta=0.1)
    d = direct(m, [nk, nk, 4], XY3, mu, 0.1)
    assert np.max(np.abs(e - d)) < 5e-2
    assert abs(e[30] - 1.0 / (2.0 * math.pi)) < 0.003


def test_energy_cut_errors():
    m = M.haldane()
    with pytest.raises(errors.InvalidResponseParameter):
        ec(m, [4, 4], np.eye(2), [0.5, 0.0])
    m1 = M.Model.tb_model([[1.0]], [[0.0]])
    m1.set_onsite([0.0])
    p = Parameters.rank2([4], [1.0], [1.0], [0.0]).with_integration(Integration.EnergyCut)
    with pytest.raises(errors.InvalidDimension):
        m1.hall_conductivity(p)
