"""Wannier90 loading (CPU): the native table reader against the oracle's
line-by-line restatement (bit for bit), and the reference's own reader tests
(src/wannier90.rs:1221-1518) restated on the host mirror."""

import math
import os

import numpy as np
import pytest

import w90_data as D
from oracle import tb_oracle as O
from rustb_gb300 import errors
from rustb_gb300.model import Model
from rustb_gb300.wannier90 import BOHR_TO_ANGSTROM, win_data_line


@pytest.fixture(scope="module", autouse=True)
def _library():
    from rustb_gb300 import _lib, build

    if not os.path.exists(_lib.LIB_PATH):
        build.build_library()


def _w(d, name, text):
    with open(os.path.join(d, name), "w") as f:
        f.write(text)


CUBIC = "begin unit_cell_cart\n1.0 0.0 0.0\n0.0 1.0 0.0\n0.0 0.0 1.0\nend unit_cell_cart\n\n"
HR1 = "generated\n1\n1\n1\n0 0 0 1 1 0.0 0.0\n"


def _load(d):
    return Model.from_hr(str(d) + "/", "seedname", 0.0, spin=False)


# --------------------------------------------------- the reference's tests --
def test_from_hr_loads_minimal_dataset(tmp_path):
    _w(tmp_path, "seedname.win", CUBIC + "begin projections\nC:s\nend projections\n")
    _w(tmp_path, "seedname_hr.dat", HR1)
    _w(tmp_path, "seedname_centres.xyz", "2\nWannier centres\nC 0.0 0.0 0.0\nC 0.0 0.0 0.0\n")
    m = _load(tmp_path)
    assert m.norb == 1 and m.natom() == 1


def test_from_hr_drops_xyz_atom_without_orbitals(tmp_path):
    _w(tmp_path, "seedname.win", CUBIC + "begin projections\nC:s\nend projections\n")
    _w(tmp_path, "seedname_hr.dat", HR1)
    _w(tmp_path, "seedname_centres.xyz", "3\nWannier centres\nX 0.0 0.0 0.0\nC 0.1 0.0 0.0\nCs 0.2 0.0 0.0\n")
    m = _load(tmp_path)
    assert m.norb == 1 and m.natom() == 1


def test_from_hr_drops_multiple_atoms_of_same_unprojected_species(tmp_path):
    _w(tmp_path, "seedname.win", CUBIC + "begin projections\nC:s\nend projections\n")
    _w(tmp_path, "seedname_hr.dat", HR1)
    _w(tmp_path, "seedname_centres.xyz",
       "4\nWannier centres\nX 0.0 0.0 0.0\nC 0.1 0.0 0.0\nCs 0.2 0.0 0.0\nCs 0.3 0.0 0.0\n")
    m = _load(tmp_path)
    assert m.norb == 1 and m.natom() == 1


def test_from_hr_without_xyz_drops_atom_without_orbitals(tmp_path):
    _w(tmp_path, "seedname.win", CUBIC + "begin atoms_cart\nC 0.0 0.0 0.0\nCs 0.1 0.0 0.0\nend atoms_cart\n\n"
       "begin projections\nC:s\nend projections\n")
    _w(tmp_path, "seedname_hr.dat", HR1)
    m = _load(tmp_path)
    assert m.norb == 1 and m.natom() == 1


def test_from_hr_rejects_projection_species_missing_from_xyz(tmp_path):
    _w(tmp_path, "seedname.win", CUBIC + "begin projections\nC:s\nend projections\n")
    _w(tmp_path, "seedname_hr.dat", HR1)
    _w(tmp_path, "seedname_centres.xyz", "2\nWannier centres\nC 0.0 0.0 0.0\nFe 0.0 0.0 0.0\n")
    with pytest.raises(errors.FileParse, match="species mismatch"):
        _load(tmp_path)


def test_from_hr_rejects_unknown_projection_species(tmp_path):
    _w(tmp_path, "seedname.win", CUBIC + "begin projections\nXx:s\nend projections\n")
    _w(tmp_path, "seedname_hr.dat", HR1)
    _w(tmp_path, "seedname_centres.xyz", "1\nWannier centres\nC 0.0 0.0 0.0\n")
    with pytest.raises(errors.FileParse, match="Unknown atomic species 'Xx' in begin projections"):
        _load(tmp_path)


def test_win_data_line_strips_hash_and_bang_comments():
    assert win_data_line("spinors = .true.") == "spinors = .true."
    assert win_data_line("# spinors = .true.") == ""
    assert win_data_line("#spinors=true") == ""
    assert win_data_line("spinors = .true. ! enable spin") == "spinors = .true."
    assert win_data_line("Fe 1.0 0.0 0.0 # position") == "Fe 1.0 0.0 0.0"
    assert win_data_line("  \t") == ""


def test_from_hr_without_centres_xyz_uses_atoms_cart_fallback(tmp_path):
    _w(tmp_path, "seedname.win", CUBIC + "begin atoms_cart\nFe 0.0 0.0 0.0\nend atoms_cart\n\n"
       "begin projections\nFe:s\nend projections\n")
    _w(tmp_path, "seedname_hr.dat", HR1)
    m = _load(tmp_path)
    assert m.norb == 1 and m.natom() == 1


def test_from_hr_without_xyz_loads_multiple_atoms_of_same_species(tmp_path):
    _w(tmp_path, "seedname.win", CUBIC + "begin atoms_cart\nFe 0.0 0.0 0.0\nFe 1.0 0.0 0.0\nend atoms_cart\n\n"
       "begin projections\nFe:s\nFe:p\nend projections\n")
    hr = "generated\n8\n1\n1\n0 0 0 1 1 0.0 0.0\n"
    for i in range(1, 9):
        for j in range(1, 9):
            if i != 1 or j != 1:
                hr += f"0 0 0 {i} {j} 0.0 0.0\n"
    _w(tmp_path, "seedname_hr.dat", hr)
    m = _load(tmp_path)
    assert m.norb == 8 and m.natom() == 2
    assert m.atoms[0].norb() == 4 and m.atoms[1].norb() == 4


@pytest.mark.parametrize("unit,block,expected", [
    ("BoHr", "ATOMS_CART\nBOHR\nFe 1.0 0.0 0.0 ! inline comment\nEND ATOMS_CART", 2.0 * BOHR_TO_ANGSTROM),
    ("AnG", "atoms_cart\nAngstrom\nFe 1.0 0.0 0.0\nend atoms_cart", 2.0),
    ("Ang", "atoms_frac\nFe 0.5 0.0 0.0\nend atoms_frac", 2.0),
])
def test_from_hr_handles_coordinate_blocks_and_units_consistently(tmp_path, unit, block, expected):
    _w(tmp_path, "seedname.win", f"BEGIN UNIT_CELL_CART\n{unit}\n2.0 0.0 0.0\n0.0 2.0 0.0\n0.0 0.0 2.0\n"
       f"END UNIT_CELL_CART\n\nBEGIN {block}\n\nbegin projections\nFe:s\nend projections\n")
    _w(tmp_path, "seedname_hr.dat", HR1)
    m = _load(tmp_path)
    assert m.norb == 1 and m.natom() == 1
    assert abs(m.lat[0, 0] - expected) < 1e-12
    assert abs(m.atoms[0].position[0] - 0.5) < 1e-12
    assert abs(m.orb[0, 0] - 0.5) < 1e-12


def test_from_hr_rejects_malformed_atom_rows_without_panicking(tmp_path):
    _w(tmp_path, "seedname.win", "begin unit_cell_cart\n1 0 0\n0 1 0\n0 0 1\nend unit_cell_cart\n\n"
       "begin atoms_cart\nFe 0.0 0.0\nend atoms_cart\n\nbegin projections\nFe:s\nend projections\n")
    _w(tmp_path, "seedname_hr.dat", HR1)
    with pytest.raises(errors.FileParse):
        _load(tmp_path)


def test_from_hr_rejects_truncated_centres_xyz_without_panicking(tmp_path):
    _w(tmp_path, "seedname.win", "begin unit_cell_cart\n1 0 0\n0 1 0\n0 0 1\nend unit_cell_cart\n\n"
       "begin projections\nFe:s,p\nend projections\n")
    hr = "generated\n4\n1\n1\n" + "".join(f"0 0 0 {i} {j} 0.0 0.0\n" for i in range(1, 5) for j in range(1, 5))
    _w(tmp_path, "seedname_hr.dat", hr)
    _w(tmp_path, "seedname_centres.xyz", "5\nWannier centres\nX 0.0 0.0 0.0\nFe 0.0 0.0 0.0\n")
    with pytest.raises(errors.FileParse, match="Truncated"):
        _load(tmp_path)


def test_from_hr_merges_multi_line_projections_into_one_atom(tmp_path):
    _w(tmp_path, "seedname.win", CUBIC + "begin atoms_cart\nFe 0.0 0.0 0.0\nend atoms_cart\n\n"
       "begin projections\nFe:s\nFe:p\nend projections\n")
    hr = "generated\n4\n1\n1\n" + "".join(f"0 0 0 {i} {j} 0.0 0.0\n" for i in range(1, 5) for j in range(1, 5))
    _w(tmp_path, "seedname_hr.dat", hr)
    m = _load(tmp_path)
    assert m.norb == 4 and m.natom() == 1 and m.atoms[0].norb() == 4


# ------------------------------------------------- native tables vs oracle --
@pytest.mark.parametrize("exact,spin,with_r,wsvec", [
    (True, False, False, False), (False, False, True, False), (True, True, True, True), (False, False, False, True),
])
def test_native_tables_equal_the_line_by_line_restatement(tmp_path, exact, spin, with_r, wsvec):
    nsta = 6 if spin else 5
    D.write_dataset(str(tmp_path), "mat", nsta, 1, seed=41, spin=spin, exact=exact, with_r=with_r, wsvec=wsvec)
    zero = 0.375
    m = Model.from_hr(str(tmp_path) + "/", "mat", zero, with_rmatrix=with_r)
    ham, hamR, weights = O.w90_read_hr(str(tmp_path / "mat_hr.dat"), zero)
    rm = O.w90_read_r(str(tmp_path / "mat_r.dat"), hamR, weights, nsta) if with_r else None
    if wsvec:
        ham, hamR, rm = O.w90_apply_wsvec(str(tmp_path / "mat_wsvec.dat"), ham, hamR, rm)
    if with_r:
        rm = O.w90_hermitize_rmatrix(rm, hamR)
    assert np.array_equal(m.hamR, hamR)
    assert np.array_equal(m.ham, ham)
    if with_r:
        assert np.array_equal(m.rmatrix, rm)
    else:
        assert m.rmatrix is None
    assert m.spin == spin and m.nsta == nsta


def test_native_tables_match_the_generated_model(tmp_path):
    Rs, H, w, rm = D.write_dataset(str(tmp_path), "g", 4, 1, seed=42, exact=True)
    m = Model.from_hr(str(tmp_path) + "/", "g", 0.0)
    for r, R in enumerate(m.hamR):
        assert np.allclose(m.ham[r], H[tuple(R)], rtol=0, atol=1e-15)
    assert tuple(m.hamR[0]) == (0, 0, 0)
    lat = np.array([[3.1, 0.0, 0.0], [0.2, 2.9, 0.0], [0.0, 0.3, 4.2]])
    assert np.array_equal(m.lat, lat)


def test_reader_errors(tmp_path):
    with pytest.raises(errors.FileCreation):
        Model.from_hr(str(tmp_path) + "/", "missing", 0.0)
    _w(tmp_path, "bad_hr.dat", "x\nnot-a-number\n1\n1\n0 0 0 1 1 0.0 0.0\n")
    with pytest.raises(errors.FileParse, match="nsta"):
        Model.from_hr(str(tmp_path) + "/", "bad", 0.0)
    _w(tmp_path, "tr_hr.dat", "x\n2\n1\n1\n0 0 0 1 1 0.0 0.0\n0 0 0 2 1 0.0 0.0\n")
    with pytest.raises(errors.TbPanic):  # the reference indexes past the end: a panic
        Model.from_hr(str(tmp_path) + "/", "tr", 0.0)
    _w(tmp_path, "im_hr.dat", "x\n1\n1\n1\n0 0 0 1 1 0.0\n")
    with pytest.raises(errors.FileParse, match="Missing Hamiltonian imaginary part"):
        Model.from_hr(str(tmp_path) + "/", "im", 0.0)
    D.write_dataset(str(tmp_path), "nor", 3, 1, seed=43)
    with pytest.raises(errors.FileCreation, match="_r.dat"):
        Model.from_hr_with_rmatrix(str(tmp_path) + "/", "nor", 0.0)
    with pytest.raises(errors.Other, match="Spin mismatch"):
        Model.from_hr(str(tmp_path) + "/", "nor", 0.0, spin=True)
    _w(tmp_path, "pj_hr.dat", HR1)
    _w(tmp_path, "pj.win", CUBIC + "begin projections\nC:q\nend projections\n")
    with pytest.raises(errors.InvalidOrbitalProjection):
        Model.from_hr(str(tmp_path) + "/", "pj", 0.0)
