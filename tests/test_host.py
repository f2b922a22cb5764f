"""Host-side logic (CPU): the Model builder mirrors src/model_build.rs, the
Parameters validators mirror src/response/config.rs, status codes map to the
TbError classes, and libtbgpu.so exports every symbol include/tbgpu.h declares."""

import ctypes
import os
import re

import numpy as np
import pytest

import models as M
from rustb_gb300 import _lib, errors, workloads as W
from rustb_gb300.model import Model
from rustb_gb300.params import Parameters, SpinDirection

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_add_hop_stores_hermitian_partner():
    m = Model.tb_model([[1.0, 0.0], [0.0, 1.0]], [[0.0, 0.0], [0.5, 0.0]])
    m.add_hop(1.0 + 0.5j, 0, 1, (1, 0))
    ip = m._find_R((1, 0))
    im = m._find_R((-1, 0))
    assert m.hamR[0].tolist() == [0, 0]
    assert m.ham[ip, 0, 1] == 1.0 + 0.5j and m.ham[im, 1, 0] == 1.0 - 0.5j
    m.add_hop(2.0, 0, 1, (1, 0))
    assert m.ham[ip, 0, 1] == 3.0 + 0.5j and m.ham[im, 1, 0] == 3.0 - 0.5j


def test_add_element_existing_r_updates_both_sides():
    """add_element_updates_existing_hopping_hermitically (src/lib.rs:611-650)."""
    m = Model.tb_model([[1.0, 0.0], [0.0, 1.0]], [[0.0, 0.0], [0.5, 0.0]])
    m.set_hop(1.0, 0, 0, (1, 0))
    m.set_hop(2.0, 0, 0, (1, 0))
    assert m.ham[m._find_R((1, 0)), 0, 0] == 2.0
    assert m.ham[m._find_R((-1, 0)), 0, 0] == 2.0
    m.set_hop(0.4 + 0.2j, 0, 1, (0, 0))
    assert m.ham[0, 0, 1] == 0.4 + 0.2j and m.ham[0, 1, 0] == 0.4 - 0.2j


def test_complex_onsite_rejected_before_writing():
    m = Model.tb_model([[1.0, 0.0], [0.0, 1.0]], [[0.0, 0.0]])
    before = m.ham.copy()
    with pytest.raises(errors.TbPanic):
        m.add_hop(1.0 + 2.0j, 0, 0, (0, 0))
    assert np.array_equal(m.ham, before)


@pytest.mark.parametrize("pauli", [None, SpinDirection.X, SpinDirection.Y, SpinDirection.Z])
def test_spin_decoration_is_hermitian(pauli):
    m = Model.tb_model([[1.0, 0.0], [0.0, 1.0]], [[0.0, 0.0], [0.5, 0.5]], spin=True)
    m.add_hop(0.3 + 0.1j, 0, 1, (1, 0), pauli)
    ip, im = m._find_R((1, 0)), m._find_R((-1, 0))
    assert np.allclose(m.ham[im], m.ham[ip].conj().T)
    n = m.norb
    if pauli == SpinDirection.Y:  # model_build.rs:57-60
        assert m.ham[ip, 0 + n, 1] == (0.3 + 0.1j) * 1j
        assert m.ham[ip, 0, 1 + n] == -(0.3 + 0.1j) * 1j
    if pauli == SpinDirection.Z:
        assert m.ham[ip, 0, 1] == 0.3 + 0.1j and m.ham[ip, n, 1 + n] == -(0.3 + 0.1j)


def test_random_model_is_hermitian_closed():
    m = W.random_model(3, 4, True, 1, seed=3)
    H0 = m.ham[0]
    assert np.allclose(H0, H0.conj().T)
    for r in range(1, m.nR, 2):
        assert np.array_equal(m.hamR[r + 1], -m.hamR[r])
        assert np.allclose(m.ham[r + 1], m.ham[r].conj().T)


def test_cfg2_shapes():
    m = W.random_spinful_3d()
    assert m.nsta == 128 and m.nR == 343 and m.dim == 3


def test_parameters_validation_errors():
    p = Parameters.rank2((4, 4), [1.0, 0.0], [0.0, 1.0], np.array([0.0]))
    p.validate_rank2(2)
    with pytest.raises(errors.InvalidKmeshDimensions):
        Parameters.rank2((0, 4), [1.0, 0.0], [0.0, 1.0], [0.0]).validate_rank2(2)
    with pytest.raises(errors.InvalidResponseParameter):
        Parameters.rank2((4, 4), [0.0, 0.0], [0.0, 1.0], [0.0]).validate_rank2(2)
    with pytest.raises(errors.DimensionMismatch):
        Parameters(kmesh=(4, 4), direction=np.eye(2)[:1], mu=[0.0]).validate_rank2(2)
    with pytest.raises(errors.InvalidResponseParameter):
        Parameters.rank2((4, 4), [1.0, 0.0], [0.0, 1.0], []).validate_rank2(2)
    p = Parameters.rank2((4, 4), [1.0, 0.0], [0.0, 1.0], [0.0])
    p.eta = -1.0
    with pytest.raises(errors.InvalidResponseParameter):
        p.validate_rank2(2)
    p = Parameters.rank2((4, 4), [1.0, 0.0], [0.0, 1.0], [0.0]).with_temperature(-5.0)
    with pytest.raises(errors.InvalidResponseParameter):
        p.validate_rank2(2)


def test_status_codes_map_to_error_classes():
    assert isinstance(errors.error_for(errors.TBG_E_SPIN_NOT_ALLOWED, "x"), errors.SpinNotAllowed)
    assert isinstance(errors.error_for(errors.TBG_E_KVECTOR_LENGTH, "x"), errors.KVectorLengthMismatch)
    assert isinstance(errors.error_for(errors.TBG_E_OOM, "x"), errors.DeviceError)
    errors.raise_for_status(0, "")


def _header_symbols():
    text = open(os.path.join(ROOT, "include", "tbgpu.h")).read()
    return sorted(set(re.findall(r"\b(tbg_[a-z0-9_]+)\s*\(", text)))


def test_header_and_binding_agree():
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert set(_header_symbols()) == bound


def test_library_exports_every_declared_symbol():
    lib_path = _lib.LIB_PATH
    if not os.path.exists(lib_path):
        from rustb_gb300 import build
        build.build_library()
    lib = ctypes.CDLL(lib_path)
    for name in _header_symbols():
        assert hasattr(lib, name), name
    lib.tbg_version.restype = ctypes.c_char_p
    assert lib.tbg_version().startswith(b"tbgpu")
