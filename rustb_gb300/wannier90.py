"""Wannier90 model loading -- host mirror of ``Wannier90::from_hr`` and
``Model::from_hr_with_rmatrix`` (src/wannier90.rs:42-1219).

The tight-binding tables (``seedname_hr.dat``, ``_r.dat``, ``_wsvec.dat``) are
read by the native reader of ``libtbgpu.so`` (``tbg_w90_*``, all host threads);
the small text files (``seedname.win``: lattice, spinors, projections, atoms;
``seedname_centres.xyz``: Wannier centres and atoms) are parsed here.  Files
are read in the reference's order, so the first error raised is the one the
reference raises, with the same ``TbError`` class.
"""

from __future__ import annotations

import ctypes
import os
import sys
from dataclasses import dataclass, field

import numpy as np

from . import _lib, errors

BOHR_TO_ANGSTROM = 0.52917721067  # src/wannier90.rs:9

# Chemical symbols H .. Ra, the species AtomType accepts (src/atom_struct.rs:485-580).
ELEMENTS = (
    "H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br Kr "
    "Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb "
    "Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn Fr Ra").split()

# Projection name -> orbitals (src/wannier90.rs:356-433).
PROJECTIONS = {
    "s": ["s"], "p": ["pz", "px", "py"], "d": ["dz2", "dxz", "dyz", "dx2y2", "dxy"],
    "f": ["fz3", "fxz2", "fyz2", "fzx2y2", "fxyz", "fxx23y2", "fy3x2y2"],
    "sp3": ["sp3_1", "sp3_2", "sp3_3", "sp3_4"], "sp2": ["sp2_1", "sp2_2", "sp2_3"], "sp": ["sp_1", "sp_2"],
    "sp3d": ["sp3d_1", "sp3d_2", "sp3d_3", "sp3d_4", "sp3d_5"],
    "sp3d2": ["sp3d2_1", "sp3d2_2", "sp3d2_3", "sp3d2_4", "sp3d2_5", "sp3d2_6"],
    "px": ["px"], "py": ["py"], "pz": ["pz"], "dxy": ["dxy"], "dxz": ["dxz"], "dyz": ["dyz"], "dz2": ["dz2"],
    "dx2-y2": ["dx2y2"],
}


@dataclass
class Atom:
    """An atom of the loaded model: fractional position, species, orbital indices."""

    position: np.ndarray
    species: str
    orbitals: list = field(default_factory=list)

    def norb(self) -> int:
        return len(self.orbitals)


def win_data_line(line: str) -> str:
    """``win_data_line`` (wannier90.rs:11-17): text before the first ``!`` or ``#``, trimmed."""
    return line.split("!", 1)[0].split("#", 1)[0].strip()


def length_unit_scale(token: str):
    """``length_unit_scale`` (wannier90.rs:19-25)."""
    t = token.lower()
    if t in ("ang", "angstrom", "angstroms"):
        return 1.0
    if t == "bohr":
        return BOHR_TO_ANGSTROM
    return None


def _parse_f64(token: str, file: str, context: str) -> float:
    try:
        t = token.strip()
        if not t or t.lower().startswith(("0x", "-0x", "+0x")) or "_" in t:
            raise ValueError("invalid float literal")
        return float(t)
    except ValueError:
        raise errors.FileParse(f"Failed to parse data from file '{file}': Failed to parse {context}: "
                               f"invalid float literal") from None


def _species(name: str, file: str, message: str) -> str:
    if name not in ELEMENTS:
        raise errors.FileParse(f"Failed to parse data from file '{file}': {message}")
    return name


class _Lines:
    def __init__(self, lines, file):
        self.lines = lines
        self.i = 0
        self.file = file

    def next(self):
        if self.i >= len(self.lines):
            return None
        s = self.lines[self.i]
        self.i += 1
        return s

    def need(self, message="Unexpected end of file"):
        s = self.next()
        if s is None:
            raise errors.FileParse(f"Failed to parse data from file '{self.file}': {message}")
        return s


def _read_lines(path: str, what: str):
    try:
        with open(path, "rb") as f:
            data = f.read()
    except OSError as e:
        raise errors.FileCreation(f"Failed to create file '{path}': Unable to open {what} file: {e}") from None
    text = data.decode("utf-8")
    lines = text.split("\n")
    if lines and lines[-1] == "":
        lines.pop()
    return [ln[:-1] if ln.endswith("\r") else ln for ln in lines]


@dataclass
class _Win:
    lat: np.ndarray
    spin: bool
    proj_name: list
    proj_list: list
    atom_proj: list
    atom_name: list
    atom_pos: np.ndarray


def parse_win(win_path: str) -> _Win:
    """The seedname.win keyword loop (wannier90.rs:246-537)."""
    it = _Lines(_read_lines(win_path, "win"), win_path)
    bad = lambda m: errors.FileParse(f"Failed to parse data from file '{win_path}': {m}")  # noqa: E731
    lat = np.zeros((3, 3))
    spin = False
    proj_name, proj_list, atom_proj, atom_name, atom_pos = [], [], [], [], []
    while True:
        a = it.next()
        if a is None:
            break
        keyword = win_data_line(a).lower()
        if "begin unit_cell_cart" in keyword:
            unit = 1.0
            rows = []
            while len(rows) < 3:
                line = win_data_line(it.need("Missing lattice vector line"))
                if not line:
                    continue
                tokens = line.split()
                if not rows and len(tokens) == 1:
                    unit = length_unit_scale(tokens[0])
                    if unit is None:
                        raise bad(f"Unknown unit_cell_cart unit '{tokens[0]}'")
                    continue
                if len(tokens) != 3:
                    raise bad(f"A unit_cell_cart row must contain 3 numbers, found {len(tokens)} in '{line}'")
                rows.append([_parse_f64(t, win_path, "lattice vector") * unit for t in tokens])
            lat = np.array(rows, dtype=np.float64)
        elif "spinors" in keyword and ("t" in keyword or "true" in keyword):
            spin = True
        elif "begin projections" in keyword:
            while True:
                string = win_data_line(it.need())
                if not string:
                    continue
                if "end projections" in string.lower():
                    break
                prj = [x.strip() for x in string.replace(";", ",").replace(":", ",").split(",")]
                if len(prj) < 2 or not prj[0]:
                    raise bad(f"Malformed projection line '{string}': expected species:orbital")
                n_orb = 0
                orbs = []
                for item in prj[1:]:
                    item = item.strip()
                    if item not in PROJECTIONS:
                        raise errors.InvalidOrbitalProjection(
                            f"Invalid orbital projection string: 'Unrecognized projection '{item}' in seedname.win'")
                    n_orb += len(PROJECTIONS[item])
                    orbs += PROJECTIONS[item]
                proj_list.append(n_orb)
                atom_proj.append(orbs)
                proj_name.append(_species(prj[0], win_path,
                                          f"Unknown atomic species '{prj[0]}' in begin projections"))
        elif "begin atoms_cart" in keyword:
            unit = 1.0
            first = True
            while True:
                string = win_data_line(it.need())
                if not string:
                    continue
                if "end atoms_cart" in string.lower():
                    break
                fields = string.split()
                if first and len(fields) == 1:
                    unit = length_unit_scale(fields[0])
                    if unit is None:
                        raise bad(f"Unknown atoms_cart unit '{fields[0]}'")
                    first = False
                    continue
                first = False
                if len(fields) != 4:
                    raise bad(f"An atoms_cart row must contain a species and 3 coordinates, found {len(fields)} "
                              f"fields in '{string}'")
                atom_name.append(fields[0])
                atom_pos.append([_parse_f64(t, win_path, "Cartesian atom position") * unit for t in fields[1:]])
        elif "begin atoms_frac" in keyword:
            while True:
                string = win_data_line(it.need())
                if not string:
                    continue
                if "end atoms_frac" in string.lower():
                    break
                fields = string.split()
                if len(fields) != 4:
                    raise bad(f"An atoms_frac row must contain a species and 3 coordinates, found {len(fields)} "
                              f"fields in '{string}'")
                atom_name.append(fields[0])
                frac = np.array([_parse_f64(t, win_path, "fractional atom position") for t in fields[1:]])
                atom_pos.append(list(frac @ lat))
    return _Win(lat, spin, proj_name, proj_list, atom_proj, atom_name,
                np.array(atom_pos, dtype=np.float64).reshape(-1, 3))


def _inv(lat):
    try:
        return np.linalg.inv(lat)
    except np.linalg.LinAlgError as e:
        raise errors.Linalg(f"Linear algebra operation failed: {e}") from None


def _assign_orbitals(win: _Win, name: str, orb_proj: list):
    """Orbitals of every projection line of one species, merged into one atom."""
    orbitals = []
    for j, jn in enumerate(win.proj_name):
        if jn == name:
            first = len(orb_proj)
            orbitals += list(range(first, first + win.proj_list[j]))
            orb_proj += win.atom_proj[j]
    return orbitals


def _orbitals_and_atoms(win: _Win, xyz_path: str, nsta: int):
    """Orbital positions, atoms and projections (wannier90.rs:546-769)."""
    spin = win.spin
    orb_proj: list = []
    atoms: list = []
    dropped: list = []
    if os.path.exists(xyz_path):
        lines = _read_lines(xyz_path, "xyz")
        bad = lambda m: errors.FileParse(f"Failed to parse data from file '{xyz_path}': {m}")  # noqa: E731
        if len(lines) < 2:
            raise bad("_centres.xyz must contain a count and comment line")
        try:
            declared = int(lines[0].strip())
            if declared < 0:
                raise ValueError
        except ValueError:
            raise bad("Invalid _centres.xyz entry count: invalid digit found in string") from None
        available = len(lines) - 2
        if declared < nsta or available < declared:
            raise bad(f"Truncated _centres.xyz: header declares {declared} entries, HR requires {nsta} "
                      f"Wannier-centre entries, but only {available} data lines are present")
        norb = nsta // 2 if spin else nsta
        orb = np.zeros((norb, 3))
        for i in range(norb):
            fields = lines[i + 2].split()
            if len(fields) < 4:
                raise bad(f"Malformed Wannier-centre row {i + 1}: expected a label and 3 coordinates")
            for axis in range(3):
                orb[i, axis] = _parse_f64(fields[axis + 1], xyz_path, "Wannier-centre position")
        inv = _inv(win.lat)
        orb = orb @ inv
        n_atom = declared - nsta
        pos = np.zeros((n_atom, 3))
        names = []
        for i in range(n_atom):
            fields = lines[i + 2 + nsta].split()
            if len(fields) < 4:
                raise bad(f"Malformed atom row {i + 1} in _centres.xyz: expected a species and 3 coordinates")
            for axis in range(3):
                pos[i, axis] = _parse_f64(fields[axis + 1], xyz_path, "atom position")
            names.append(_species(fields[0], xyz_path,
                                  f"Unknown atomic species '{fields[0]}' in _centres.xyz; species must be listed "
                                  f"in the win file's begin projections block"))
        for i, name in enumerate(names):
            orbitals = _assign_orbitals(win, name, orb_proj)
            if not orbitals:
                if name not in dropped:
                    print(f"warning: dropping '{name}' atoms from _centres.xyz (no orbitals in the projections "
                          f"block)", file=sys.stderr)
                    dropped.append(name)
                continue
            atoms.append(Atom(pos[i] @ inv, name, orbitals))
        if len(orb_proj) != norb:
            detail = (f"{norb} orbitals declared in the projections block, but only {len(orb_proj)} could be "
                      f"assigned to atoms" if len(orb_proj) < norb else
                      f"{norb} orbitals declared in the projections block, but {len(orb_proj)} were assigned to atoms")
            raise bad(f"species mismatch between _centres.xyz and the win projections block: {detail}. "
                      f"_centres.xyz species: {names}; projection species: {win.proj_name}")
        return orb, atoms, orb_proj
    # no _centres.xyz: orbitals sit on the atoms of the win file
    inv = _inv(win.lat)
    atom_pos = win.atom_pos @ inv
    orb_rows = []
    for i, raw in enumerate(win.atom_name):
        name = _species(raw, xyz_path.replace("_centres.xyz", ".win"),
                        f"Unknown atomic species '{raw}' in begin atoms_frac block")
        orbitals = []
        for j, jn in enumerate(win.proj_name):
            if jn == name:
                first = len(orb_proj)
                orbitals += list(range(first, first + win.proj_list[j]))
                orb_proj += win.atom_proj[j]
                orb_rows += [atom_pos[i]] * win.proj_list[j]
        if not orbitals:
            if name not in dropped:
                print(f"warning: dropping '{name}' atoms from begin atoms_frac/atoms_cart (no orbitals in the "
                      f"projections block)", file=sys.stderr)
                dropped.append(name)
            continue
        atoms.append(Atom(atom_pos[i].copy(), name, orbitals))
    expected = nsta // 2 if spin else nsta
    if len(orb_proj) != expected:
        win_path = xyz_path[: -len("_centres.xyz")] + ".win"
        detail = (f"{expected} orbitals declared in the HR file, but only {len(orb_proj)} could be assigned to atoms"
                  if len(orb_proj) < expected else
                  f"{expected} orbitals declared in the HR file, but {len(orb_proj)} were assigned to atoms")
        raise errors.FileParse(f"Failed to parse data from file '{win_path}': species mismatch between begin "
                               f"atoms_frac and the projections block: {detail}. atom species: {win.atom_name}; "
                               f"projection species: {win.proj_name}")
    orb = np.array(orb_rows, dtype=np.float64).reshape(-1, 3)
    return orb, atoms, orb_proj


class _Tables:
    """Owner of a native ``tbg_w90`` handle."""

    def __init__(self, hr_path: str, zero_energy: float):
        self.lib = _lib.load()
        self.h = ctypes.c_void_p()
        _lib.check(self.lib.tbg_w90_read_hr(hr_path.encode(), float(zero_energy), ctypes.byref(self.h)), self.lib)

    def read_r(self, path: str):
        _lib.check(self.lib.tbg_w90_read_r(self.h, path.encode()), self.lib)

    def wsvec(self, path: str) -> bool:
        applied = ctypes.c_int(0)
        _lib.check(self.lib.tbg_w90_apply_wsvec(self.h, path.encode(), ctypes.byref(applied)), self.lib)
        return bool(applied.value)

    def hermitize(self):
        _lib.check(self.lib.tbg_w90_hermitize_rmatrix(self.h), self.lib)

    def arrays(self):
        nsta, nR, has_r = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int()
        _lib.check(self.lib.tbg_w90_info(self.h, ctypes.byref(nsta), ctypes.byref(nR), ctypes.byref(has_r)), self.lib)
        n, r = nsta.value, nR.value
        ham = np.empty((r, n, n), dtype=np.complex128)
        hamR = np.empty((r, 3), dtype=np.int64)
        rm = np.empty((r, 3, n, n), dtype=np.complex128) if has_r.value else None
        _lib.check(self.lib.tbg_w90_copy(self.h, _lib.dptr(ham.view(np.float64)), _lib.iptr(hamR),
                                         _lib.dptr(rm.view(np.float64)) if rm is not None else None), self.lib)
        return ham, hamR, rm

    def nsta(self) -> int:
        nsta = ctypes.c_int64()
        _lib.check(self.lib.tbg_w90_info(self.h, ctypes.byref(nsta), None, None), self.lib)
        return nsta.value

    def close(self):
        if self.h:
            self.lib.tbg_w90_free(self.h)
            self.h = ctypes.c_void_p()


def from_hr(path: str, file_name: str, zero_energy: float = 0.0, spin: bool | None = None,
            with_rmatrix: bool = False):
    """``Wannier90::from_hr`` (src/wannier90.rs:49-1203): reads
    ``path + file_name`` + ``_hr.dat``, ``.win``, ``_centres.xyz`` (optional),
    ``_r.dat`` (when ``with_rmatrix``), ``_wsvec.dat`` (optional).  ``spin``
    plays the part of the model's SPIN parameter: ``None`` takes the .win
    file's ``spinors`` setting, a value that disagrees with it is an error."""
    from .model import Model

    prefix = f"{path}{file_name}"
    tables = _Tables(prefix + "_hr.dat", zero_energy)
    try:
        nsta = tables.nsta()
        win = parse_win(prefix + ".win")
        if spin is not None and bool(spin) != win.spin:
            raise errors.Other(f"Spin mismatch: Wannier90 .win file has spin={str(win.spin).lower()} but Model "
                               f"was constructed with SPIN={str(bool(spin)).lower()}")
        orb, atoms, orb_proj = _orbitals_and_atoms(win, prefix + "_centres.xyz", nsta)
        if with_rmatrix:
            tables.read_r(prefix + "_r.dat")
        tables.wsvec(prefix + "_wsvec.dat")
        tables.hermitize()
        ham, hamR, rm = tables.arrays()
    finally:
        tables.close()
    if orb.shape[0] == 0:
        raise errors.InvalidModel("model has no orbitals")
    if not (np.all(np.isfinite(win.lat)) and np.all(np.isfinite(orb))):
        raise errors.InvalidModel("finite_geometry: lattice and orbital positions must be finite")
    model = Model(win.lat, orb, win.spin, ham=ham, hamR=hamR)
    if rm is not None:
        model.set_rmatrix(rm)
    model.atoms = atoms
    model.orb_projection = orb_proj
    return model


def from_hr_with_rmatrix(path: str, file_name: str, zero_energy: float = 0.0, spin: bool | None = None):
    """``Model::from_hr_with_rmatrix`` (src/wannier90.rs:1208-1219): the _r.dat file is required."""
    return from_hr(path, file_name, zero_energy, spin, with_rmatrix=True)
