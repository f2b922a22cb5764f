"""Synthetic Wannier90 datasets for the reader tests: a seeded random
Hermitian-closed model written in the file formats Wannier90 emits
(_hr.dat 5I5,2F12.6 lines with 15 weights per line; _r.dat 5I5,6F12.6;
_wsvec.dat entry/weight/shift lines), or at full precision."""

import itertools
import os

import numpy as np


def random_tables(nsta, rmax, seed):
    rng = np.random.default_rng(seed)
    Rs = [R for R in itertools.product(range(-rmax, rmax + 1), repeat=3)]
    half = {}
    for R in Rs:
        mR = tuple(-x for x in R)
        if mR in half:
            continue
        m = (rng.normal(size=(nsta, nsta)) + 1j * rng.normal(size=(nsta, nsta))) * 0.3
        if R == (0, 0, 0):
            m = 0.5 * (m + m.conj().T)
        half[R] = m
    H = {}
    for R, m in half.items():
        H[R] = m
        H[tuple(-x for x in R)] = m.conj().T
    weights = {R: int(rng.integers(1, 4)) for R in Rs}
    for R in Rs:
        weights[tuple(-x for x in R)] = weights[R]
    rmat = {}
    for R in Rs:
        if R in rmat:
            continue
        a = (rng.normal(size=(3, nsta, nsta)) + 1j * rng.normal(size=(3, nsta, nsta))) * 0.1
        rmat[R] = a
        rmat[tuple(-x for x in R)] = np.conj(np.transpose(a, (0, 2, 1))) + 1e-3 * rng.normal(size=(3, nsta, nsta))
    return Rs, H, weights, rmat


def write_dataset(d, seed_name, nsta, rmax, seed, spin=False, exact=False, with_r=False, wsvec=False,
                  xyz=True, zero_shift=None):
    os.makedirs(d, exist_ok=True)
    Rs, H, w, rm = random_tables(nsta, rmax, seed)
    fmt = (lambda x: f"{x:25.17e}") if exact else (lambda x: f"{x:12.6f}")
    lines = ["written by a test generator", f"{nsta:12d}", f"{len(Rs):12d}"]
    ws = [w[R] for R in Rs]
    for i in range(0, len(ws), 15):
        lines.append("".join(f"{x:5d}" for x in ws[i:i + 15]))
    for R in Rs:
        for j in range(nsta):
            for i in range(nsta):
                v = H[R][i, j] * w[R]
                lines.append(f"{R[0]:5d}{R[1]:5d}{R[2]:5d}{i + 1:5d}{j + 1:5d}{fmt(v.real)}{fmt(v.imag)}")
    open(os.path.join(d, seed_name + "_hr.dat"), "w").write("\n".join(lines) + "\n")
    if with_r:
        rl = ["written by a test generator", f"{nsta:12d}", f"{len(Rs):12d}"]
        for R in Rs:
            for j in range(nsta):
                for i in range(nsta):
                    vals = "".join(fmt(c) for r in range(3) for c in ((rm[R][r, i, j] * w[R]).real,
                                                                      (rm[R][r, i, j] * w[R]).imag))
                    rl.append(f"{R[0]:5d}{R[1]:5d}{R[2]:5d}{i + 1:5d}{j + 1:5d}{vals}")
        open(os.path.join(d, seed_name + "_r.dat"), "w").write("\n".join(rl) + "\n")
    if wsvec:
        # (R, i, j) with shifts T pairs with (-R, j, i) with shifts -T, so the
        # refolded R set stays closed under R -> -R as Wannier90's is
        rng = np.random.default_rng(seed + 1)
        shifts = {}
        for R in Rs:
            for i in range(nsta):
                for j in range(nsta):
                    key = (R, i, j)
                    if key in shifts:
                        continue
                    self_partner = R == (0, 0, 0) and i == j  # on-site: distance 0, one image
                    T = ([(0, 0, 0)] if self_partner or rng.random() < 0.7 else
                         [(0, 0, 0), tuple(int(x) for x in rng.integers(-1, 2, 3))])
                    shifts[key] = T
                    shifts[(tuple(-x for x in R), j, i)] = [tuple(-x for x in t) for t in T]
        wl = ["## written by Wannier90 use_ws_distance=T"]
        for R in Rs:
            for i in range(nsta):
                for j in range(nsta):
                    T = shifts[(R, i, j)]
                    wl.append(f"{R[0]:5d}{R[1]:5d}{R[2]:5d}{i + 1:5d}{j + 1:5d}")
                    wl.append(f"{len(T):5d}")
                    for t in T:
                        wl.append(f"{t[0]:5d}{t[1]:5d}{t[2]:5d}")
        open(os.path.join(d, seed_name + "_wsvec.dat"), "w").write("\n".join(wl) + "\n")
    norb = nsta // 2 if spin else nsta
    win = ["begin unit_cell_cart", "  Ang", "  3.1 0.0 0.0", "  0.2 2.9 0.0", "  0.0 0.3 4.2", "end unit_cell_cart",
           ""]
    if spin:
        win.append("spinors = .true.   ! spinor Wannier functions")
    win += ["begin projections", f"Fe:{','.join(['s'] * norb)}", "end projections", "",
            "begin atoms_frac", "Fe 0.25 0.5 0.125", "end atoms_frac"]
    open(os.path.join(d, seed_name + ".win"), "w").write("\n".join(win) + "\n")
    if xyz:
        rng = np.random.default_rng(seed + 2)
        xl = [f"{nsta + 1:6d}", " Wannier centres, written by a test generator"]
        for i in range(nsta):
            c = rng.uniform(0, 3, 3)
            xl.append(f"X {c[0]:16.8f}{c[1]:16.8f}{c[2]:16.8f}")
        xl.append(f"Fe {1.0:16.8f}{1.5:16.8f}{0.5:16.8f}")
        open(os.path.join(d, seed_name + "_centres.xyz"), "w").write("\n".join(xl) + "\n")
    return Rs, H, w, rm
