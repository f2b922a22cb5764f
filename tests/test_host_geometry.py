"""Host-side validation of the quantum-geometry and DOS entry points (CPU):
every error the reference raises before touching the k-mesh is raised here
before any device call, with the reference's error class."""

import numpy as np
import pytest

import models as M
from rustb_gb300 import errors
from rustb_gb300.params import Integration, Parameters

XY = np.array([[1.0, 0.0], [0.0, 1.0]])


def test_dos_parameter_errors_in_reference_order():
    m = M.haldane()
    with pytest.raises(errors.InvalidEnergyRange):
        m.dos([4, 4], 1.0, 1.0, 10, 0.1)
    with pytest.raises(errors.InvalidEnergyRange):  # range is checked before E_n and sigma
        m.dos([4, 4], 2.0, 1.0, 0, -1.0)
    with pytest.raises(errors.InvalidDosParameter):
        m.dos([4, 4], 0.0, 1.0, 0, 0.1)
    for sigma in (0.0, -1.0, float("nan"), float("inf")):
        with pytest.raises(errors.InvalidDosParameter):
            m.dos([4, 4], 0.0, 1.0, 10, sigma)
    for km in ([], [4, 0]):
        with pytest.raises(errors.InvalidKmeshDimensions):
            m.dos(km, 0.0, 1.0, 10, 0.1)
    with pytest.raises(errors.TbPanic):
        m.dos([4, 4, 4], 0.0, 1.0, 10, 0.1)


def test_quantum_geometry_parameter_errors():
    m = M.haldane()
    p = Parameters.rank2([4, 4], XY[0], XY[1], [0.0])
    p.integration = Integration.EnergyCut
    with pytest.raises(errors.InvalidResponseParameter):
        m.quantum_geometry(p)
    p.integration = Integration.Simplex
    with pytest.raises(errors.TbPanic):
        m.quantum_geometry(p)
    m1 = M.Model.tb_model([[1.0]], [[0.0]])
    m1.set_onsite([0.0])
    p1 = Parameters.rank2([4], [1.0], [1.0], [0.0]).with_integration(Integration.Simplex)
    with pytest.raises(errors.InvalidDimension):
        m1.quantum_geometry(p1)
    bad = Parameters.rank2([4, 4], XY[0], XY[1], [0.0])
    bad.eta = -1.0
    with pytest.raises(errors.InvalidResponseParameter):
        m.quantum_geometry(bad)
    with pytest.raises(errors.InvalidResponseParameter):
        m.quantum_geometry_on(np.zeros((2, 2)), bad)
    ok = Parameters.rank2([4, 4], XY[0], XY[1], [0.0])
    with pytest.raises(errors.DimensionMismatch):
        m.quantum_geometry_on(np.zeros((2, 3)), ok)
    with pytest.raises(errors.KVectorLengthMismatch):
        m.quantum_geometry_at([0.0, 0.0, 0.0], ok)


def test_dos_status_codes_map_to_error_classes():
    assert isinstance(errors.error_for(errors.TBG_E_INVALID_ENERGY_RANGE, "x"), errors.InvalidEnergyRange)
    assert isinstance(errors.error_for(errors.TBG_E_INVALID_DOS_PARAMETER, "x"), errors.InvalidDosParameter)
