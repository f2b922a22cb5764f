"""Band-energy mesh exports consumed by Fermi-surface tools.

``write_bxsf`` mirrors ``BxsfExport::write_bxsf`` (src/fermi_surface.rs:441-546,
XCrySDen BXSF) and ``write_spin_frmsf`` mirrors ``write_spin_frmsf``
(fermi_surface.rs:637-706, FermiSurfer FRMSF).  The band energies come from
``tbg_bands_mesh`` (the device path of ``solve_band_all_parallel`` on
``gen_kmesh``); the text follows the reference byte for byte, including Rust's
float formatting (``{:.10}`` fixed, ``{:.10E}`` scientific with a bare exponent:
``1.2500000000E-3``, ``0.0000000000E0``).  Rendering of the contours
(``show_fermi_surface``) is plotting and is not provided.
"""

from __future__ import annotations

import math

import numpy as np

from . import _lib, errors


def rust_fixed(v: float, prec: int) -> str:
    """Rust ``format!("{:.prec}", v)`` for an f64."""
    v = float(v)
    if math.isnan(v):
        return "NaN"
    if math.isinf(v):
        return "inf" if v > 0 else "-inf"
    return f"{v:.{prec}f}"


def rust_exp(v: float, prec: int = 10) -> str:
    """Rust ``format!("{:.prec$E}", v)``: mantissa with ``prec`` decimals, then
    ``E`` and the decimal exponent without sign padding or leading zeros."""
    v = float(v)
    if math.isnan(v):
        return "NaN"
    if math.isinf(v):
        return "inf" if v > 0 else "-inf"
    mant, exp = f"{v:.{prec}E}".split("E")
    return f"{mant}E{int(exp)}"


def rec_lat(lat) -> np.ndarray:
    """``Model::rec_lat`` (src/model.rs:679-687): 2 pi (lat^T)^-1."""
    lat = np.asarray(lat, dtype=np.float64)
    try:
        inv_t = np.linalg.inv(lat.T)
    except np.linalg.LinAlgError as e:
        raise errors.Linalg(f"Failed to invert lattice: {e}") from None
    return 2.0 * math.pi * inv_t


def bands_mesh(model, k_mesh) -> np.ndarray:
    """Band energies (nk, nsta) on the uniform mesh, gen_kmesh order."""
    km = np.ascontiguousarray(np.asarray(k_mesh, dtype=np.int64).reshape(-1))
    if km.size == 0 or np.any(km <= 0):
        raise errors.InvalidKmeshDimensions(f"Invalid k-point mesh dimensions: {km.tolist()}")
    if km.size != model.dim:
        raise errors.TbPanic(f"k-mesh has {km.size} entries, the model has dimension {model.dim}")
    E = np.empty((int(np.prod(km)), model.nsta))
    lib = _lib.load()
    _lib.check(lib.tbg_bands_mesh(model.device_handle(), _lib.iptr(km), _lib.dptr(E)), lib)
    return E


def _require_3d(model):
    if model.dim != 3:
        raise errors.InvalidDimension(f"dimension {model.dim} is not supported; supported: [3]")


def bxsf_text(b, k_mesh, e_fermi: float, eval_) -> str:
    """The BXSF document of write_bxsf (fermi_surface.rs:476-543)."""
    nx, ny, nz = (int(v) for v in k_mesh)
    nk = nx * ny * nz
    nsta = eval_.shape[1]
    out = ["BEGIN_INFO\n", "  # BXSF exported by Rustb\n",
           f"  # Number of k-points: {nx}×{ny}×{nz} = {nk}\n", f"  # Number of bands: {nsta}\n",
           f"  Fermi Energy: {rust_fixed(e_fermi, 12)}\n", "END_INFO\n", "\n",
           "BEGIN_BLOCK_BANDGRID_3D\n", "  band_energies\n", "  BEGIN_BANDGRID_3D_band_energies\n",
           f"    {nsta}\n", f"    {nx} {ny} {nz}\n", "    0.0 0.0 0.0\n"]
    for r in range(3):
        out.append("    " + " ".join(rust_fixed(b[r, c], 10) for c in range(3)) + "\n")
    for ib in range(nsta):
        out.append(f"    BAND: {ib + 1}\n")
        col = eval_[:, ib]
        row = 0
        for _ in range(nx):
            for _ in range(ny):
                for iz in range(nz):
                    if iz % 10 == 0 and iz > 0:
                        out.append("\n")
                    out.append(" " + rust_exp(col[row]))
                    row += 1
                out.append("\n")
        out.append("\n")
    out.append("  END_BANDGRID_3D\n")
    out.append("END_BLOCK_BANDGRID_3D\n")
    return "".join(out)


def write_bxsf(model, k_mesh, e_fermi: float, filename: str) -> str:
    """``BxsfExport::write_bxsf`` (fermi_surface.rs:454-546); returns the path."""
    _require_3d(model)
    b = rec_lat(model.lat)
    E = bands_mesh(model, k_mesh)
    path = filename if filename.endswith(".bxsf") else f"{filename}.bxsf"
    with open(path, "wb") as f:
        f.write(bxsf_text(b, k_mesh, e_fermi, E).encode("utf-8"))
    return path


def frmsf_block(values) -> str:
    """format_frmsf_block (fermi_surface.rs:571-585): 10 values per line."""
    parts = []
    n = len(values)
    for i, v in enumerate(values):
        parts.append(" " + rust_exp(v))
        if (i + 1) % 10 == 0:
            parts.append("\n")
    if n % 10 != 0:
        parts.append("\n")
    return "".join(parts)


def frmsf_text(b, k_mesh, eval_up, eval_dn) -> str:
    """The FRMSF document of write_spin_frmsf (fermi_surface.rs:680-705);
    eval_up / eval_dn already shifted by -e_fermi."""
    nx, ny, nz = (int(v) for v in k_mesh)
    nsta = eval_up.shape[1]
    merged = np.concatenate([eval_up, eval_dn], axis=1)
    head = [f"{nx} {ny} {nz}\n", "1\n", f"{2 * nsta}\n"]
    for r in range(3):
        head.append(" ".join(rust_fixed(b[r, c], 10) for c in range(3)) + "\n")
    energy = merged.T.reshape(-1)  # band outermost, k in gen_kmesh order
    nk = merged.shape[0]
    color = np.where(np.arange(energy.size) // nk < nsta, 1.0, -1.0)
    return "".join(head) + frmsf_block(energy) + frmsf_block(color)


def write_spin_frmsf(up_model, dn_model, k_mesh, e_fermi: float, filename: str) -> str:
    """``write_spin_frmsf`` (fermi_surface.rs:637-706); returns the path."""
    _require_3d(up_model)
    _require_3d(dn_model)
    nsta = up_model.nsta
    if dn_model.nsta != nsta:
        raise errors.TbPanic(f"Spin models must have same band count: up={nsta}, dn={dn_model.nsta}")
    lat_diff = float(np.abs(np.asarray(up_model.lat) - np.asarray(dn_model.lat)).sum())
    if lat_diff > 1e-10:
        raise errors.TbPanic(f"up_model and dn_model must have the same lattice, diff = {lat_diff}")
    b = rec_lat(up_model.lat)
    eu = bands_mesh(up_model, k_mesh) - e_fermi
    ed = bands_mesh(dn_model, k_mesh) - e_fermi
    path = filename if filename.endswith(".frmsf") else f"{filename}.frmsf"
    with open(path, "wb") as f:
        f.write(frmsf_text(b, k_mesh, eu, ed).encode("utf-8"))
    return path
