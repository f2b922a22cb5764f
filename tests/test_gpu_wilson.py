"""GPU parity for the Wilson loops (berry_loop, berry_loop_det, berry_flux,
berry_phase, wannier_centre) against the oracle restatement on the same loops.
Phases are compared on the unit circle (|e^{i a} - e^{i b}| <= 1e-9 after
matching each GPU phase to its nearest oracle phase); the reference's own
order of the phases within a loop is LAPACK zgeev's, so both sides are
compared as sets."""

import math

import numpy as np
import pytest

import models as M
from oracle import tb_oracle as O
from rustb_gb300 import errors, workloads as W

pytestmark = pytest.mark.gpu


def same_phases(a, b, tol=1e-9):
    a = np.atleast_1d(a)
    b = list(np.atleast_1d(b))
    for x in a:
        d = [abs(np.exp(1j * x) - np.exp(1j * y)) for y in b]
        j = int(np.argmin(d))
        if d[j] > tol:
            return False
        b.pop(j)
    return True


def _loops(model, n, n_k, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        k0 = rng.random(model.dim)
        G = np.zeros(model.dim)
        G[i % model.dim] = 1.0
        if i % 3 == 2:
            G[(i + 1) % model.dim] = -1.0
        out.append(np.array([k0 + G * t for t in np.linspace(0.0, 1.0, n_k)]))
    return out


CASES = [
    ("haldane", M.haldane, [0]),
    ("kane_mele", lambda: M.kane_mele(rashba=0.1), [0, 1]),
    ("random12", lambda: W.random_model(2, 12, False, 1, seed=401), [0, 1, 2, 3, 4]),
    ("random3d_s8", lambda: W.random_model(3, 8, True, 1, seed=402), list(range(7))),
    ("random2d_s32_occ60", lambda: W.random_model(2, 32, True, 1, seed=405), list(range(60))),
    ("qwz3d", M.qwz_stacked_3d, [0]),
]


@pytest.mark.parametrize("name,build,occ", CASES, ids=[c[0] for c in CASES])
def test_berry_loop_matches_oracle(name, build, occ):
    m = build()
    for loop in _loops(m, 4, 41, seed=7):
        ph = m.berry_loop(loop, occ)
        assert np.all(np.diff(ph) >= 0)
        assert same_phases(ph, O.wilson_loop(m, loop, occ))
        d = m.berry_loop_det(loop, occ)
        assert same_phases(d, O.wilson_loop_det(m, loop, occ))
        # the det form is the sum of the unitary phases (mod 2 pi)
        assert same_phases(d, float(np.sum(ph)), tol=1e-8)


def test_flat_band_berry_phase_closed_form():
    taus = [[0.1, 0.3], [1.0 / 3.0, 1.0 / 3.0], [0.75, 0.2]]
    m = M.Model.tb_model(np.eye(2), taus)
    m.set_onsite([-1.0, 0.5, 2.0])
    loop = np.array([[0.2, 0.1 + t] for t in np.linspace(0.0, 1.0, 9)])
    ph = m.berry_loop(loop, [0, 1, 2])
    assert same_phases(ph, [2 * math.pi * t[1] for t in taus], tol=1e-12)


def test_berry_flux_chern_haldane():
    m = M.haldane()
    flux = m.berry_flux([0], [0.0, 0.0], [1.0, 0.0], [0.0, 1.0], 31, 31)
    ref = O.berry_flux(m, [0], [0.0, 0.0], [1.0, 0.0], [0.0, 1.0], 31, 31)
    assert np.max(np.abs(flux - ref)) < 1e-9
    assert abs(abs(flux.sum() / (2 * math.pi)) - 1.0) < 1e-9


def test_berry_flux_multiband_plaquettes():
    m = W.random_model(2, 6, False, 1, seed=403)
    flux = m.berry_flux([0, 1, 2], [0.1, 0.2], [1.0, 0.0], [0.0, 1.0], 7, 5)
    ref = O.berry_flux(m, [0, 1, 2], [0.1, 0.2], [1.0, 0.0], [0.0, 1.0], 7, 5)
    for i in range(7):
        for j in range(5):
            assert same_phases(flux[i, j], ref[i, j])


def test_wannier_centre_and_berry_phase():
    m = M.kane_mele(rashba=0.05)
    wcc = m.wannier_centre([0, 1], [0.0, 0.0], [1.0, 0.0], [0.0, 1.0], 11, 31)
    ref = O.wannier_centre(m, [0, 1], [0.0, 0.0], [1.0, 0.0], [0.0, 1.0], 11, 31)
    assert wcc.shape == ref.shape == (2, 11)
    for i in range(11):
        assert same_phases(wcc[:, i], ref[:, i])
    kv = np.array([[[i / 10.0, j / 30.0] for j in range(31)] for i in range(11)])
    bp = m.berry_phase([0, 1], kv)
    assert bp.shape == (2, 11)
    for i in range(11):
        assert same_phases(bp[:, i], ref[:, i])


def test_wilson_errors():
    m = M.haldane()
    with pytest.raises(errors.TbPanic):  # not closed modulo a lattice vector
        m.berry_loop(np.array([[0.0, 0.0], [0.5, 0.0], [0.7, 0.1]]), [0])
    with pytest.raises(errors.TbPanic):  # band index out of range
        m.berry_loop(np.array([[0.0, 0.0], [0.5, 0.0], [1.0, 0.0]]), [2])
    with pytest.raises(errors.TbPanic):
        m.wannier_centre([0], [0.0, 0.0], [1.0, 0.0], [0.0, 1.0], 1, 5)
    big = W.random_model(2, 70, False, 1, seed=404)
    with pytest.raises(errors.TbPanic):  # more than 64 occupied bands
        big.berry_loop(np.array([[0.0, 0.0], [0.5, 0.0], [1.0, 0.0]]), list(range(66)))


@pytest.mark.parametrize("norb,spin,occ", [(24, False, list(range(10))), (16, True, list(range(16)))])
def test_berry_loop_mixed_precision(norb, spin, occ):
    """Mixed eigenpairs (FP32 + tensor-core refinement) against the oracle, 1e-6 on the circle."""
    from rustb_gb300.params import Precision

    m = W.random_model(2, norb, spin, 1, seed=406 + norb)
    for loop in _loops(m, 3, 33, seed=9):
        ph = m.berry_loop(loop, occ, Precision.MIXED)
        assert same_phases(ph, O.wilson_loop(m, loop, occ), tol=1e-6)
        d = m.berry_loop_det(loop, occ, Precision.MIXED)
        assert same_phases(d, O.wilson_loop_det(m, loop, occ), tol=1e-6)
    wcc = m.wannier_centre(occ, [0.0, 0.0], [1.0, 0.0], [0.0, 1.0], 5, 21, Precision.MIXED)
    ref = O.wannier_centre(m, occ, [0.0, 0.0], [1.0, 0.0], [0.0, 1.0], 5, 21)
    for i in range(5):
        assert same_phases(wcc[:, i], ref[:, i], tol=1e-6)
