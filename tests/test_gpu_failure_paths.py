"""Failure paths of the device code, driven without a GPU fault.

* Non-finite input.  The reference panics when LAPACK reports info != 0
  (src/ndarray_lapack.rs:446) and stops at ``todo!()`` when ``eigh`` fails
  (src/solve_ham.rs:125).  Here a NaN in the hopping table is found by the
  eigensolver while it bounds the spectrum; the call returns TBG_E_NOCONV
  (raised as DeviceError) on the FP64 and the mixed path, for eigenvalue-only
  and eigenpair calls, and the library stays usable.
* Bounded waits.  The tensor-core products' stage hand-off waits are given a
  limit of a few polls through an internal hook, so they run out: each CTA
  flags an abort, drains its own bulk copies and committed MMAs (those waits
  keep their full bound), frees its tensor memory, and the call returns
  TBG_E_TIMEOUT.  The next call with the normal limit matches the oracle.
"""

import numpy as np
import pytest

from oracle import tb_oracle as O
from rustb_gb300 import _lib, errors, workloads as W
from rustb_gb300.model import Model
from rustb_gb300.params import Parameters, Precision

pytestmark = pytest.mark.gpu


def _nan_model(norb=20, spin=False):
    m = W.random_model(2, norb, spin, 1, seed=2024)
    ham = m.ham.copy()
    ham[1, 3, 4] = np.nan  # one element of a hopping block; its -R partner stays finite
    return Model(m.lat, m.orb, spin, ham=ham, hamR=m.hamR.copy()), m


@pytest.mark.parametrize("precision", [Precision.FP64, Precision.MIXED])
def test_nan_hopping_reports_no_convergence(precision):
    bad, good = _nan_model()
    k = np.random.default_rng(3).uniform(0, 1, (9, 2))
    p = Parameters.rank2((4, 4), [1.0, 0.0], [0.0, 1.0], [0.0])
    calls = [lambda: bad.solve_band_all_parallel(k, precision),
             lambda: bad.berry_curvature_on(k, p, precision),
             lambda: bad.hall_conductivity(p, precision)]
    for call in calls:
        with pytest.raises(errors.DeviceError) as ei:
            call()
        assert ei.value.code == errors.TBG_E_NOCONV
        assert "NaN" in str(ei.value)
    # the library and the device stay usable
    E = good.solve_band_all_parallel(k, precision)
    Hs = O.gen_ham_batch(good, k, 1)
    tol = 1e-10 if precision == Precision.FP64 else 1e-9
    for i in range(len(k)):
        assert np.max(np.abs(E[i] - O.eigvalsh(Hs[i]))) <= tol * np.linalg.norm(Hs[i], 2)


def test_tensor_core_wait_timeout_is_reported_and_recovers():
    lib = _lib.load()
    m = W.random_model(2, 40, True, 1, seed=2025)  # 80 bands: every product on tcgen05
    p = Parameters.rank2((3, 3), [1.0, 0.0], [0.0, 1.0], [-0.1, 0.0, 0.2])
    prev = lib.tbg_internal_tc_wait_limit(2)
    try:
        with pytest.raises(errors.DeviceError) as ei:
            m.hall_conductivity(p, Precision.MIXED)
        assert ei.value.code == errors.TBG_E_TIMEOUT
    finally:
        lib.tbg_internal_tc_wait_limit(prev)
    assert lib.tbg_internal_tc_wait_limit(0) == prev  # the default was back in place
    s = m.hall_conductivity(p, Precision.MIXED).conductivity
    ref = O.hall_conductivity(m, (3, 3), np.eye(2), [-0.1, 0.0, 0.2])
    assert np.max(np.abs(s - ref)) <= 1e-6 * np.max(np.abs(ref))
