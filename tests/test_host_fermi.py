"""BXSF / FRMSF text layout of the mesh exports (CPU): the documents are
rebuilt from given energies and compared with the layout the reference writes
(src/fermi_surface.rs:476-543, 571-585, 680-705)."""

import math

import numpy as np
import pytest

from rustb_gb300 import errors
from rustb_gb300.fermi import bxsf_text, frmsf_block, frmsf_text, rec_lat, rust_exp, rust_fixed


def test_rust_float_formatting():
    assert rust_exp(0.0) == "0.0000000000E0"
    assert rust_exp(1.25e-3) == "1.2500000000E-3"
    assert rust_exp(-1234.5) == "-1.2345000000E3"
    assert rust_exp(float("nan")) == "NaN"
    assert rust_fixed(2.0 * math.pi, 10) == "6.2831853072"
    assert rust_fixed(0.25, 12) == "0.250000000000"


def test_rec_lat_is_two_pi_inverse_transpose():
    lat = np.array([[1.0, 0.0, 0.0], [0.5, math.sqrt(3) / 2, 0.0], [0.0, 0.0, 2.0]])
    b = rec_lat(lat)
    assert np.allclose(lat @ b.T, 2 * math.pi * np.eye(3), atol=1e-14)
    with pytest.raises(errors.Linalg):
        rec_lat(np.zeros((3, 3)))


def test_bxsf_layout_breaks_lines_every_ten_z_points():
    b = 2 * math.pi * np.eye(3)
    km = (1, 2, 12)
    E = np.arange(24 * 2, dtype=np.float64).reshape(24, 2) * 0.5 - 3.0
    text = bxsf_text(b, km, 0.125, E)
    lines = text.split("\n")
    assert lines[:7] == ["BEGIN_INFO", "  # BXSF exported by Rustb", "  # Number of k-points: 1×2×12 = 24",
                         "  # Number of bands: 2", "  Fermi Energy: 0.125000000000", "END_INFO", ""]
    assert lines[7:13] == ["BEGIN_BLOCK_BANDGRID_3D", "  band_energies", "  BEGIN_BANDGRID_3D_band_energies",
                           "    2", "    1 2 12", "    0.0 0.0 0.0"]
    assert lines[13] == "    6.2831853072 0.0000000000 0.0000000000"
    assert lines[16] == "    BAND: 1"
    # one (ix, iy) row of 12 z-points: a break after the 10th value
    first = " ".join(rust_exp(v) for v in E[0:10, 0])
    assert lines[17] == " " + first
    assert lines[18] == " " + rust_exp(E[10, 0]) + " " + rust_exp(E[11, 0])
    assert lines[-3:] == ["  END_BANDGRID_3D", "END_BLOCK_BANDGRID_3D", ""]
    assert text.count("BAND:") == 2


def test_frmsf_layout():
    b = np.eye(3)
    up = np.array([[0.1, 0.2], [0.3, 0.4], [0.5, 0.6]])  # (nk = 3, nsta = 2)
    dn = -up
    text = frmsf_text(b, (1, 1, 3), up, dn)
    lines = text.split("\n")
    assert lines[:6] == ["1 1 3", "1", "4", "1.0000000000 0.0000000000 0.0000000000",
                         "0.0000000000 1.0000000000 0.0000000000", "0.0000000000 0.0000000000 1.0000000000"]
    # energies band-major: 12 values -> 10 + 2 per line
    vals = [0.1, 0.3, 0.5, 0.2, 0.4, 0.6, -0.1, -0.3, -0.5, -0.2, -0.4, -0.6]
    assert lines[6] == "".join(" " + rust_exp(v) for v in vals[:10])
    assert lines[7] == "".join(" " + rust_exp(v) for v in vals[10:])
    colors = [1.0] * 6 + [-1.0] * 6
    assert lines[8] == "".join(" " + rust_exp(v) for v in colors[:10])
    assert frmsf_block([1.0] * 10) == " 1.0000000000E0" * 10 + "\n"
