"""Generate the golden fixtures under tests/golden/.

1. ``reference_known_answers.json`` -- the known answers that Rustb's own
   tests assert on the k-mesh path, transcribed from src/lib.rs (file:line in
   each entry).  Rustb cannot be compiled here (no Rust toolchain), so these
   values are the parity anchor for the oracle.
2. ``oracle_cases.npz`` -- oracle outputs (H, V, E, Omega, sigma) for small
   seeded models, used to pin the oracle against drift (CPU tests) and as the
   reference the GPU parity tests compare with.

Run from the repository root:  python tests/golden/make_golden.py
"""

import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import tb_oracle as O  # noqa: E402
from rustb_gb300 import workloads as W  # noqa: E402
import models as M  # noqa: E402

S3 = math.sqrt(3.0)

KNOWN = {
    "test_gen_v": {
        "source": "src/lib.rs:671-755",
        "model": "graphene t=1 delta=0, lat [[1,0],[0.5,sqrt3/2]], orb (1/3,1/3),(2/3,2/3)",
        "gamma_bands": [-3.0, 3.0],
        "gamma_tol": 0.0,
        "k_bands_zero": [1.0 / 3.0, 2.0 / 3.0],
        "k_bands_tol": 1e-5,
        "gen_v_k": [1.0 / 3.0, 1.0 / 3.0],
        "gen_v_atom_x_01": [-0.8137976813493737, -0.2961981327260237],
        "gen_v_atom_x_10": [-0.8137976813493737, 0.2961981327260237],
        "gen_v_atom_y_01": [-0.4698463103929542, -0.17101007166283436],
        "gen_v_atom_y_10": [-0.4698463103929542, 0.17101007166283436],
        "gen_v_lattice_x_01": [-3.0 * S3 / 4.0, 3.0 / 4.0],
        "gen_v_lattice_x_10": [-3.0 * S3 / 4.0, -3.0 / 4.0],
        "gen_v_tol": 1e-8,
        "solve_onek_tol": 1e-5,
    },
    "evec_transform_sanity": {
        "source": "src/lib.rs:1231-1277",
        "model": "haldane t=-1 t2=-1 delta=0.7",
        "k": [0.3, 0.4],
        "tol": 1e-10,
    },
    "Haldan_model": {
        "source": "src/lib.rs:902-1164 (asserts 955, 978-998)",
        "model": "haldane t=-1 t2=-1 delta=0.7",
        "kmesh": [31, 31],
        "eta": 1e-3,
        "chern": 1.0,
        "chern_tol": 1e-3,
        "mu_grid": [-2.0, 2.0, 101],
        "mu_grid_tol": 1e-3,
    },
    "conductivity_test": {
        "source": "src/lib.rs:757-846",
        "model": "haldane t=-1 t2=-1 delta=0.7",
        "k": [1.0 / 3.0, 2.0 / 3.0],
        "dk": 1e-4,
        "eta": 1e-3,
        "wilson_tol": 1e-4,
        "kmesh": [100, 100],
        "mu": -1.0,
        "single_vs_multi_tol": 1e-5,
    },
    "berry_curvature_kernel_consistency": {
        "source": "src/lib.rs:2519-2559",
        "model": "build_haldane_2d(-0.3)",
        "kmesh": [21, 21],
        "eta": 0.05,
        "tol": 1e-12,
    },
    "hall_conductivity_ec_tr": {
        "source": "src/lib.rs:2665-2739",
        "models": "build_haldane_2d(-0.3) vs build_haldane_2d(0.3)",
        "kmesh": [51, 51],
        "eta": 0.05,
        "mu_grid": [-3.0, 3.0, 101],
        "tol": 1e-10,
    },
    "hall_conductivity_ec_3d_qwz": {
        "source": "src/lib.rs:3222-3268",
        "model": "build_qwz_stacked_3d(-1.0)",
        "kmesh": [[10, 10, 4], [14, 14, 4]],
        "eta": 0.1,
        "mu_grid": [-3.0, 3.0, 61],
        "plateau": 1.0 / (2.0 * math.pi),
        "plateau_tol_energy_cut": 0.003,
        "direct_vs_energy_cut_tol": 5e-2,
    },
    "thermodynamics": {
        "source": "src/thermodynamics.rs:100-118, 152-181",
        "step_at_mu": 0.5,
        "clamp": 50.0,
    },
}


def oracle_cases():
    out = {}
    # random spinful 3D model (cfg2 statistics, small)
    m = W.random_model(3, 6, True, 1, seed=7)
    rng = np.random.default_rng(11)
    k = rng.uniform(0, 1, (12, 3))
    dirs = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])
    V, H = O.gen_v_projected_batch(m, k, 1, dirs)
    VL, HL = O.gen_v_projected_batch(m, k, 0, dirs)
    Om, E = O.berry_on(m, k, dirs, -1, 1e-3)
    OmS, _ = O.berry_on(m, k, dirs, 2, 1e-3)
    out.update(rs_ham=m.ham, rs_hamR=m.hamR, rs_orb=m.orb, rs_lat=m.lat, rs_k=k, rs_H=H, rs_V=V, rs_HL=HL,
               rs_VL=VL, rs_E=E, rs_Om=Om, rs_OmSz=OmS)
    mu = np.array([-0.5, 0.0, 0.5])
    out["rs_sigma_444"] = O.hall_conductivity(m, (4, 4, 4), dirs, mu, 0.0, 1e-3)
    out["rs_sigma_444_T300"] = O.hall_conductivity(m, (4, 4, 4), dirs, mu, 300.0, 1e-3)
    out["rs_mu"] = mu
    # Haldane (Rustb's test model)
    h = M.haldane()
    out["haldane_sigma_31"] = O.hall_conductivity(h, (31, 31), np.eye(2), np.array([0.0]), 0.0, 1e-3)
    return out


def main():
    with open(os.path.join(HERE, "reference_known_answers.json"), "w") as f:
        json.dump(KNOWN, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "oracle_cases.npz"), **oracle_cases())
    print("wrote", HERE)


if __name__ == "__main__":
    main()
