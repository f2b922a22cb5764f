"""A Wannier90-loaded model through the device path: band energies, the
velocity with the position-matrix commutator (HasRMatrix) and the Berry
curvature against the oracle on the same loaded tables."""

import numpy as np
import pytest

import w90_data as D
from oracle import tb_oracle as O
from rustb_gb300.model import Model
from rustb_gb300.params import Gauge, Parameters, Precision

pytestmark = pytest.mark.gpu

XY3 = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("spin,with_r,wsvec", [(False, False, True), (False, True, False), (True, True, True)])
def test_w90_model_on_the_device(tmp_path, spin, with_r, wsvec):
    nsta = 8 if spin else 10
    D.write_dataset(str(tmp_path), "wan", nsta, 1, seed=51, spin=spin, exact=True, with_r=with_r, wsvec=wsvec)
    m = Model.from_hr(str(tmp_path) + "/", "wan", 0.2, with_rmatrix=with_r)
    rng = np.random.default_rng(3)
    k = rng.random((24, 3))
    E = m.solve_band_all_parallel(k)
    assert rel(E, O.solve_band_all(m, k)) < 1e-10
    V, H = m.gen_v_projected_batch(k, Gauge.Atom, XY3)
    Vo = np.stack([O.gen_v_projected(m, kk, 1, XY3)[0] for kk in k])
    assert rel(V, Vo) < 1e-11
    p = Parameters.rank2([1, 1, 1], XY3[0], XY3[1], [0.0])
    om, _ = m.berry_curvature_on(k, p)
    om_o, _ = O.berry_on(m, k, XY3, -1, 1e-3)
    assert rel(om, om_o) < 1e-8


def test_w90_model_hall_mixed_matches_fp64(tmp_path):
    D.write_dataset(str(tmp_path), "hall", 16, 1, seed=52, exact=True, wsvec=True)
    m = Model.from_hr(str(tmp_path) + "/", "hall", 0.0)
    p = Parameters.rank2([6, 6, 4], XY3[0], XY3[1], [-0.5, 0.0, 0.5])
    s64 = m.hall_conductivity(p, Precision.FP64).conductivity
    smx = m.hall_conductivity(p, Precision.MIXED).conductivity
    assert np.max(np.abs(smx - s64)) <= 1e-6 * np.max(np.abs(s64))
    so = O.hall_conductivity(m, [6, 6, 4], XY3, [-0.5, 0.0, 0.5])
    assert rel(s64, so) < 1e-8
