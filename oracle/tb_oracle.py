"""CPU oracle for the Rustb k-mesh hot path -- TEST INFRASTRUCTURE ONLY.

This module restates, in numpy, the algorithm of Rustb's k-mesh path so that
the GPU library can be checked against it.  It is imported only by the tests,
by ``__graft_entry__.smoke()`` and by ``bench.py``'s CPU-baseline leg, always
as the checker; the product (``rustb_gb300``) never calls it.

Parity anchor.  Rustb is Rust and cannot be built here (no cargo/rustc), so
the oracle is pinned against the known answers held by Rustb's own tests
(``src/lib.rs``: ``test_gen_v`` golden velocity matrices and Gamma/K
eigenvalues, ``evec_transform_sanity``, ``Haldan_model`` C = 1,
``conductivity_test`` Kubo vs Wilson loop, ``hall_conductivity_ec_tr``
antisymmetry, ``hall_conductivity_ec_3d_qwz`` plateau); see
``tests/test_oracle_golden.py``.  The eigensolver is LAPACK ``zheev`` (scipy's
bundled OpenBLAS), the routine Rustb's openblas backend reaches through
ndarray-linalg ``Eigh`` (``src/response/traits.rs:168``).

Functions cite the reference file:line they follow.
"""

from __future__ import annotations

import numpy as np
from scipy.linalg import lapack

TWO_PI = 2.0 * np.pi
BOLTZMANN_CONSTANT_EV_PER_K = 8.617333262145e-5  # src/thermodynamics.rs:10


# --------------------------------------------------------------------------
# k-mesh and phases
# --------------------------------------------------------------------------

def gen_kmesh(kmesh) -> np.ndarray:
    """``gen_kmesh`` (src/kpoints.rs:49-87): k = (i/N1, j/N2, l/N3) with the
    first dimension outermost; row index = i*N2*N3 + j*N3 + l."""
    kmesh = [int(n) for n in kmesh]
    axes = [np.arange(n, dtype=np.float64) / float(n) for n in kmesh]
    grids = np.meshgrid(*axes, indexing="ij")
    return np.stack([g.reshape(-1) for g in grids], axis=1)


def phases(k: np.ndarray, hamR: np.ndarray) -> np.ndarray:
    """exp(i 2 pi k.R) for every R (src/model_physics.rs:58-90)."""
    kr = np.atleast_2d(k) @ hamR.T.astype(np.float64)
    return np.exp(1j * TWO_PI * kr)


def orb_phase(k: np.ndarray, orb_sta: np.ndarray) -> np.ndarray:
    """exp(i 2 pi k.tau) per state (src/model_physics.rs:103-128)."""
    return np.exp(1j * TWO_PI * (np.atleast_2d(k) @ orb_sta.T))


def orb_states(model) -> np.ndarray:
    """Orbital positions per state; spinful duplicates tau
    (src/model_physics.rs:131-137, src/velocity.rs:546-550)."""
    return np.concatenate([model.orb, model.orb], axis=0) if model.spin else model.orb


# --------------------------------------------------------------------------
# H(k) and velocity
# --------------------------------------------------------------------------

def gen_ham(model, k, gauge: int = 1) -> np.ndarray:
    """``gen_ham`` (src/model_physics.rs:43-148) for one k-point.
    gauge: 0 = Lattice, 1 = Atom."""
    return gen_ham_batch(model, np.atleast_2d(k), gauge)[0]


def gen_ham_batch(model, k: np.ndarray, gauge: int = 1) -> np.ndarray:
    """Batched ``gen_ham``: H_lat(k) = sum_R ham[R] e^{2 pi i k.R}
    (zaxpy loop, model_physics.rs:92-96), then for the Atom gauge
    H[m,n] *= conj(phi_m) phi_n (model_physics.rs:138-146)."""
    nsta = model.nsta
    u = phases(k, model.hamR)                                   # (nk, nR)
    H = (u @ model.ham.reshape(model.nR, nsta * nsta)).reshape(-1, nsta, nsta)
    if gauge == 1:
        phi = orb_phase(k, orb_states(model))                   # (nk, nsta)
        H = H * np.conj(phi)[:, :, None] * phi[:, None, :]
    return H


def gen_v_projected(model, k, gauge: int, directions) -> tuple[np.ndarray, np.ndarray]:
    """``gen_v_projected`` (src/velocity.rs:470-731) for one k-point.

    v_p = sum_R i (w_p . R_cart) ham[R] e^{2 pi i k.R}             (587-599)
    Atom gauge: v_p[m,n] = (v_p[m,n] + i (w_p.tau_n - w_p.tau_m) H_lat[m,n])
                           * conj(phi_m) phi_n                       (602-610)
    and H -> conj(phi_m) H phi_n                                    (616-622).
    Returns (v_proj (n_proj, nsta, nsta), H).
    """
    V, H = gen_v_projected_batch(model, np.atleast_2d(k), gauge, directions)
    return V[0], H[0]


def gen_v_projected_batch(model, k: np.ndarray, gauge: int, directions):
    directions = np.atleast_2d(np.asarray(directions, dtype=np.float64))
    nsta = model.nsta
    nk = k.shape[0]
    u = phases(k, model.hamR)                                   # (nk, nR)
    hop = model.ham.reshape(model.nR, nsta * nsta)
    R_cart = model.hamR.astype(np.float64) @ model.lat          # velocity.rs:530-531
    H = (u @ hop).reshape(nk, nsta, nsta)
    V = np.empty((nk, directions.shape[0], nsta, nsta), dtype=np.complex128)
    for p, w in enumerate(directions):
        coef = 1j * (R_cart @ w)                                # i (w . R_cart)
        V[:, p] = ((u * coef[None, :]) @ hop).reshape(nk, nsta, nsta)
    if gauge == 1:
        orb_sta = orb_states(model)
        phi = orb_phase(k, orb_sta)                             # (nk, nsta)
        tau_proj = directions @ (orb_sta @ model.lat).T         # (n_proj, nsta)
        g = np.conj(phi)[:, :, None] * phi[:, None, :]          # (nk, m, n)
        for p in range(directions.shape[0]):
            diff = tau_proj[p][None, :] - tau_proj[p][:, None]  # [m,n] = tau_n - tau_m
            V[:, p] = (V[:, p] + 1j * diff[None] * H) * g
        H = H * g
    if getattr(model, "rmatrix", None) is not None:
        V = V + _rmatrix_term(model, k, gauge, directions, H, u)
    return V, H


def _rmatrix_term(model, k, gauge, directions, Hk, u):
    """i [H, A_w] position-matrix term (src/velocity.rs:627-668): A_w is the
    direction-weighted Fourier sum of rmatrix over its first n_rmat R rows; in
    the Atom gauge it is gauge-transformed and its diagonal zeroed."""
    rm = model.rmatrix                                          # (n_rmat, dim, nsta, nsta)
    n_rmat = rm.shape[0]
    nsta = model.nsta
    nk = k.shape[0]
    out = np.zeros((nk, directions.shape[0], nsta, nsta), dtype=np.complex128)
    rk = np.einsum("kr,rdij->kdij", u[:, :n_rmat], rm)          # (nk, dim, nsta, nsta)
    if gauge == 1:
        phi = orb_phase(k, orb_states(model))
        g = np.conj(phi)[:, :, None] * phi[:, None, :]
    for p, w in enumerate(directions):
        a = np.einsum("d,kdij->kij", w, rk)
        if gauge == 1:
            a = a * g
            idx = np.arange(nsta)
            a[:, idx, idx] = 0.0
        out[:, p] = 1j * (Hk @ a - a @ Hk)
    return out


def gen_v(model, k, gauge: int = 1):
    """``gen_v`` (src/velocity.rs:236-441): the projected velocity with the
    Cartesian unit vectors as directions."""
    return gen_v_projected(model, k, gauge, np.eye(model.dim))


# --------------------------------------------------------------------------
# eigensolver
# --------------------------------------------------------------------------

def eigh(H: np.ndarray):
    """LAPACK zheev with JOBZ='V' (src/response/traits.rs:168 via ndarray-linalg,
    src/ndarray_lapack.rs:412-448).  Returns ascending E and eigenvectors in the
    COLUMNS of W with H W = W diag(E)."""
    w, v, info = lapack.zheev(np.asarray(H, dtype=np.complex128), compute_v=1, lower=1)
    if info != 0:
        raise RuntimeError(f"zheev info={info}")  # ndarray_lapack.rs:446 panics
    return w, v


def eigvalsh(H: np.ndarray) -> np.ndarray:
    w, _, info = lapack.zheev(np.asarray(H, dtype=np.complex128), compute_v=0, lower=0)
    if info != 0:
        raise RuntimeError(f"zheev info={info}")
    return w


def solve_band_all(model, k: np.ndarray) -> np.ndarray:
    """``solve_band_all_parallel`` (src/solve_ham.rs:94-107)."""
    Hs = gen_ham_batch(model, np.atleast_2d(k), 1)
    return np.stack([eigvalsh(H) for H in Hs])


def solve_all(model, k: np.ndarray):
    """``solve_all_parallel`` (src/solve_ham.rs:168-184); eigenvectors as ROWS
    (solve_onek conj-transposes, solve_ham.rs:122-128)."""
    Hs = gen_ham_batch(model, np.atleast_2d(k), 1)
    E, U = [], []
    for H in Hs:
        w, v = eigh(H)
        E.append(w)
        U.append(v.T)  # row n = eigenvector n
    return np.stack(E), np.stack(U)


# --------------------------------------------------------------------------
# Berry curvature and Hall conductivity
# --------------------------------------------------------------------------

def spin_matrix(norb: int, spin: int) -> np.ndarray:
    """``build_spin_matrix`` (src/response/helpers.rs:11-40): sigma (x) I / 2."""
    nsta = 2 * norb
    m = np.zeros((nsta, nsta), dtype=np.complex128)
    i = np.arange(norb)
    if spin == 0:
        m[i, i + norb] = 0.5
        m[i + norb, i] = 0.5
    elif spin == 1:
        m[i, i + norb] = -0.5j
        m[i + norb, i] = 0.5j
    elif spin == 2:
        m[i, i] = 0.5
        m[i + norb, i + norb] = -0.5
    else:
        m = np.eye(nsta, dtype=np.complex128)
    return m


def berry_curvature_at(model, k, directions, spin: int = -1, eta: float = 1e-3):
    """``berry_curvature_at_impl`` (src/response/traits.rs:160-200).

    (V, H) = gen_v_projected(k, Atom, direction)                      :166
    (E, U) = eigh(H)                                                  :168
    J = 1/2 {S, V_0} if spin else V_0                                 :170-175
    Jb = U^T J U*, Vb = U^T V_1 U* (eigenvectors of H in columns of U*) :177-180
    K = Jb o Vb^T;  Omega_n = sum_{m != n} -2 Im K_nm / ((E_n-E_m)^2 + eta^2)  :181-195
    Returns (Omega, E).
    """
    V, H = gen_v_projected(model, np.asarray(k, dtype=np.float64), 1, directions)
    E, W = eigh(H)
    J = V[0]
    if model.spin and spin is not None and spin >= 0:
        S = spin_matrix(model.norb, spin)
        J = 0.5 * (S @ J + J @ S)                                # math.rs anti_comm
    Jb = W.conj().T @ J @ W
    Vb = W.conj().T @ V[1] @ W
    K = Jb * Vb.T
    dE = E[:, None] - E[None, :]
    den = dE * dE + eta * eta
    term = -2.0 * K.imag / den
    np.fill_diagonal(term, 0.0)
    return term.sum(axis=1), E


def fermi(energy, mu: float, width: float):
    """``fermi_from_width`` (src/thermodynamics.rs:100-118): step with 1/2 at
    E == mu when width == 0; else 1/(1+e^x) clamped at |x| > 50."""
    energy = np.asarray(energy, dtype=np.float64)
    if width == 0.0:
        return np.where(energy < mu, 1.0, np.where(energy > mu, 0.0, 0.5))
    x = (energy - mu) / width
    with np.errstate(over="ignore"):
        f = 1.0 / (1.0 + np.exp(np.clip(x, -50.0, 50.0)))
    f = np.where(x > 50.0, 0.0, np.where(x < -50.0, 1.0, f))
    return f


def occupation_width(T: float) -> float:
    """``parameters_occupation`` (src/response/config.rs:173-181)."""
    return 0.0 if T <= 0.0 else T * BOLTZMANN_CONSTANT_EV_PER_K


def berry_on(model, k_list, directions, spin=-1, eta=1e-3):
    """Band-resolved Omega and E on a k-list (berry_curvature_at per k)."""
    k_list = np.atleast_2d(np.asarray(k_list, dtype=np.float64))
    Om = np.empty((k_list.shape[0], model.nsta))
    E = np.empty_like(Om)
    for i, k in enumerate(k_list):
        Om[i], E[i] = berry_curvature_at(model, k, directions, spin, eta)
    return Om, E


def occupied_berry_curvature_on(model, k_list, directions, mu: float, T=0.0, spin=-1, eta=1e-3):
    """``occupied_berry_curvature_on`` (src/response/traits.rs:104-150)."""
    Om, E = berry_on(model, k_list, directions, spin, eta)
    return (Om * fermi(E, mu, occupation_width(T))).sum(axis=1)


def hall_from_bands(Om, E, mu_list, T, nk, det):
    """Direct-integration reduction (src/response/linear/mod.rs:204-223):
    sigma(mu) = sum_k sum_n Omega_n f(E_n, mu) / nk / det(lat)."""
    width = occupation_width(T)
    out = np.empty(len(mu_list))
    for j, mu in enumerate(mu_list):
        per_k = (Om * fermi(E, float(mu), width)).sum(axis=1)
        out[j] = per_k.sum() / nk / det
    return out


def hall_conductivity(model, kmesh, directions, mu_list, T=0.0, eta=1e-3, spin=-1):
    """``hall_conductivity`` with Integration::Direct
    (src/response/linear/mod.rs:160-225); det is the signed lattice
    determinant (:188)."""
    k = gen_kmesh(kmesh)
    Om, E = berry_on(model, k, directions, spin, eta)
    det = float(np.linalg.det(model.lat))
    return hall_from_bands(Om, E, np.atleast_1d(mu_list), T, k.shape[0], det)


# --------------------------------------------------------------------------
# Quantum geometry (src/quantum_geometry.rs) and density of states
# (src/model_physics.rs)
# --------------------------------------------------------------------------

def quantum_geometry_at(model, k, directions, eta: float = 1e-3):
    """``quantum_geometry_at_impl`` (src/quantum_geometry.rs:149-193).

    (V, H) = gen_v_projected(k, Atom, direction)                      :154-155
    (E, U) = eigh(H)                                                  :156
    Ab = U^T V_0 U*, Bb = U^T V_1 U*                                  :157-163
    K = Ab o Bb^T; G_n = sum_{m != n} K_nm / ((E_n - E_m)^2 + eta^2)  :164-184
    metric_n = Re G_n, Omega_n = -2 Im G_n                            :185-186
    Charge current only: the spin field of the parameters is ignored.
    Returns (metric, Omega, E).
    """
    V, H = gen_v_projected(model, np.asarray(k, dtype=np.float64), 1, directions)
    E, W = eigh(H)
    Ab = W.conj().T @ V[0] @ W
    Bb = W.conj().T @ V[1] @ W
    K = Ab * Bb.T
    dE = E[:, None] - E[None, :]
    T = K / (dE * dE + eta * eta)
    np.fill_diagonal(T, 0.0)
    G = T.sum(axis=1)
    return G.real.copy(), -2.0 * G.imag, E


def quantum_geometry_on(model, k_list, directions, eta: float = 1e-3):
    """``quantum_geometry_on`` (src/quantum_geometry.rs:104-138): per k-point,
    returns (metric, Omega, E), each (nk, nsta)."""
    k_list = np.atleast_2d(np.asarray(k_list, dtype=np.float64))
    g = np.empty((k_list.shape[0], model.nsta))
    om = np.empty_like(g)
    E = np.empty_like(g)
    for i, k in enumerate(k_list):
        g[i], om[i], E[i] = quantum_geometry_at(model, k, directions, eta)
    return g, om, E


def quantum_geometry(model, kmesh, directions, mu_list, T=0.0, eta=1e-3):
    """``Model::quantum_geometry`` with Integration::Direct
    (src/quantum_geometry.rs:196-240): per mu,
    sum_k sum_n value_n f(E_n, mu) / nk / det(lat) for the metric and Omega."""
    k = gen_kmesh(kmesh)
    g, om, E = quantum_geometry_on(model, k, directions, eta)
    det = float(np.linalg.det(model.lat))
    mu_list = np.atleast_1d(np.asarray(mu_list, dtype=np.float64))
    return (hall_from_bands(g, E, mu_list, T, k.shape[0], det),
            hall_from_bands(om, E, mu_list, T, k.shape[0], det))


def dos_energies(E_min: float, E_max: float, E_n: int) -> np.ndarray:
    """``Array1::linspace(E_min, E_max, E_n)`` as ndarray 0.17 yields it
    (src/model_physics.rs:210): start + i * step, step = (end - start) / (n - 1)
    (0 for n == 1) -- the last point is not forced to E_max."""
    step = (E_max - E_min) / float(E_n - 1) if E_n > 1 else 0.0
    return E_min + step * np.arange(E_n, dtype=np.float64)


def dos_from_bands(eigs, E_min: float, E_max: float, E_n: int, sigma: float, nk: int, chunk: int = 4096):
    """The Gaussian sum of ``Model::dos`` (src/model_physics.rs:206-227):
    A = (E - x) / sigma, f = exp(-A^2 / 2) / sigma / sqrt(2 pi), summed over
    every band energy x, divided by nk."""
    E = dos_energies(E_min, E_max, E_n)
    sigma0 = 1.0 / sigma
    pi0 = 1.0 / np.sqrt(2.0 * np.pi)
    x = np.asarray(eigs, dtype=np.float64).reshape(-1)
    acc = np.zeros(E_n)
    for c0 in range(0, x.size, chunk):
        A = (E[None, :] - x[c0:c0 + chunk, None]) * sigma0
        acc += (np.exp(-A * A / 2.0) * sigma0 * pi0).sum(axis=0)
    return E, acc / float(nk)


def dos(model, kmesh, E_min: float, E_max: float, E_n: int, sigma: float):
    """``Model::dos`` (src/model_physics.rs:179-230): band energies on the
    uniform mesh (gen_kmesh order), then the Gaussian sum."""
    k = gen_kmesh(kmesh)
    eigs = solve_band_all(model, k)
    return dos_from_bands(eigs, E_min, E_max, E_n, sigma, k.shape[0])


# --------------------------------------------------------------------------
# Wilson loop (used only to pin the Kubo formula, src/geometry.rs:156-215)
# --------------------------------------------------------------------------

def berry_loop(model, k_loop, occ):
    """Berry phase of the occupied bands ``occ`` around a closed k-loop
    (``berry_loop``, src/geometry.rs:156-215): -Im log det prod of overlap
    matrices in the Atom gauge, with the loop's last point identified with its
    first."""
    k_loop = np.atleast_2d(np.asarray(k_loop, dtype=np.float64))
    vecs = []
    for k in k_loop[:-1]:
        _, W = eigh(gen_ham(model, k, 1))
        vecs.append(W[:, occ])
    vecs.append(vecs[0])
    prod = np.eye(len(occ), dtype=np.complex128)
    for a, b in zip(vecs[:-1], vecs[1:]):
        prod = prod @ (a.conj().T @ b)
    return -np.angle(np.linalg.det(prod))


# --------------------------------------------------------------------------
# Wannier90 tight-binding tables (src/wannier90.rs), line by line
# --------------------------------------------------------------------------

def _w90_lines(path):
    with open(path, "rb") as f:
        text = f.read().decode("utf-8")
    lines = text.split("\n")
    if lines and lines[-1] == "":
        lines.pop()
    return [ln[:-1] if ln.endswith("\r") else ln for ln in lines]


def w90_read_hr(path, zero_energy=0.0):
    """_hr.dat as ``from_hr`` reads it (src/wannier90.rs:85-245): returns
    (ham (nR, nsta, nsta) c128 with R = 0 first, hamR (nR, 3), weights)."""
    reads = _w90_lines(path)
    nsta = int(reads[1].strip())
    n_R = int(reads[2].strip())
    weights = []
    n_line = 0
    for i in range(3, len(reads)):
        if "." in reads[i]:
            n_line = i
            break
        weights += [int(x) for x in reads[i].split()]
    ham = [np.zeros((nsta, nsta), dtype=np.complex128)]
    hamR = [(0, 0, 0)]
    for i in range(n_R):
        first = reads[i * nsta * nsta + n_line].split()
        R = (int(first[0]), int(first[1]), int(first[2]))
        m = np.zeros((nsta, nsta), dtype=np.complex128)
        for ind_i in range(nsta):
            for ind_j in range(nsta):
                tok = reads[i * nsta * nsta + ind_i * nsta + ind_j + n_line].split()
                m[ind_j, ind_i] = complex(float(tok[5]), float(tok[6])) / float(weights[i])
        if R == (0, 0, 0):
            ham[0] = m
        else:
            ham.append(m)
            hamR.append(R)
    ham = np.array(ham)
    for i in range(nsta):
        ham[0, i, i] -= zero_energy
    return ham, np.array(hamR, dtype=np.int64), weights


def _find_R(hamR, R):
    for r in range(len(hamR)):
        if tuple(hamR[r]) == tuple(R):
            return r
    return None


def w90_read_r(path, hamR, weights, nsta):
    """_r.dat (src/wannier90.rs:771-880): rmatrix (nR, 3, nsta, nsta) aligned with hamR."""
    reads = _w90_lines(path)
    n_R = int(reads[2].strip())
    rm = np.zeros((len(hamR), 3, nsta, nsta), dtype=np.complex128)
    for i in range(n_R):
        first = reads[i * nsta * nsta + 3].split()
        index = _find_R(hamR, (int(first[0]), int(first[1]), int(first[2])))
        if index is None:
            raise KeyError("R vector not found in Hamiltonian")
        for ind_i in range(nsta):
            for ind_j in range(nsta):
                tok = reads[i * nsta * nsta + ind_i * nsta + ind_j + 3].split()
                for r in range(3):
                    rm[index, r, ind_j, ind_i] = complex(float(tok[5 + 2 * r]), float(tok[6 + 2 * r])) / float(weights[i])
    return rm


def w90_apply_wsvec(path, ham, hamR, rm=None):
    """_wsvec.dat refolding (src/wannier90.rs:882-1142)."""
    reads = _w90_lines(path)
    nsta = ham.shape[1]
    new_R = [(0, 0, 0)]
    new_ham = [np.zeros((nsta, nsta), dtype=np.complex128)]
    new_rm = [np.zeros((3, nsta, nsta), dtype=np.complex128)] if rm is not None else None
    i = 0
    while i < len(reads) - 1:
        i += 1
        tok = reads[i].split()
        R = (int(tok[0]), int(tok[1]), int(tok[2]))
        ii, jj = int(tok[3]) - 1, int(tok[4]) - 1
        i += 1
        weight = int(reads[i].split()[0])
        index = _find_R(hamR, R)
        if index is None:
            raise KeyError("R vector not found in Hamiltonian")
        hop = ham[index, ii, jj] / float(weight)
        hx = rm[index, :, ii, jj] / float(weight) if rm is not None else None
        for _ in range(weight):
            i += 1
            t = reads[i].split()
            nR = (R[0] + int(t[0]), R[1] + int(t[1]), R[2] + int(t[2]))
            j = _find_R(new_R, nR)
            if j is None:
                new_R.append(nR)
                new_ham.append(np.zeros((nsta, nsta), dtype=np.complex128))
                if rm is not None:
                    new_rm.append(np.zeros((3, nsta, nsta), dtype=np.complex128))
                j = len(new_R) - 1
            new_ham[j][ii, jj] += hop
            if rm is not None:
                new_rm[j][:, ii, jj] += hx
    return (np.array(new_ham), np.array(new_R, dtype=np.int64),
            np.array(new_rm) if rm is not None else None)


def w90_hermitize_rmatrix(rm, hamR):
    """(src/wannier90.rs:1146-1167): every R row but the last, in place."""
    nsta = rm.shape[2]
    for r in range(len(hamR) - 1):
        q = _find_R(hamR, tuple(-x for x in hamR[r]))
        if q is None:
            raise KeyError("Missing Hermitian conjugate")
        for i in range(nsta):
            for j in range(nsta):
                for c in range(3):
                    rm[r, c, i, j] = (rm[r, c, i, j] + np.conj(rm[q, c, j, i])) / 2.0
                    rm[q, c, j, i] = np.conj(rm[r, c, i, j])
    return rm


# --------------------------------------------------------------------------
# Wilson loops (src/geometry.rs:156-420), with the loop's periodic gauge
# --------------------------------------------------------------------------

def _loop_overlaps(model, k_loop, occ):
    """Overlap matrices <u_i(k_t)|u_j(k_t+1)> along the loop; the last point's
    eigenvectors are the first point's times exp(-2 pi i G . tau)
    (geometry.rs:160-196)."""
    k_loop = np.atleast_2d(np.asarray(k_loop, dtype=np.float64))
    n_k = k_loop.shape[0]
    diff = k_loop[-1] - k_loop[0]
    if np.any(np.abs(diff - np.round(diff)) > 1e-9):
        raise ValueError("the end of this loop must differ from the beginning by an integer grid vector")
    tau = orb_states(model)
    _, U = solve_all(model, k_loop)                       # rows = eigenvectors
    U = U.copy()
    U[n_k - 1] = U[0] * np.exp(-2j * np.pi * (tau @ diff))[None, :]
    ev = U[:, occ, :]                                     # (n_k, n_occ, nsta)
    return [ev[t].conj() @ ev[t + 1].T for t in range(n_k - 1)]


def wilson_loop(model, k_loop, occ):
    """``berry_loop`` (geometry.rs:156-215): product of the unitary parts U V^H
    of the overlaps, -arg of its eigenvalues; sorted ascending here."""
    prod = np.eye(len(occ), dtype=np.complex128)
    for O in _loop_overlaps(model, k_loop, occ):
        u, _, vh = np.linalg.svd(O)
        prod = prod @ (u @ vh)
    return np.sort(-np.angle(np.linalg.eigvals(prod)))


def wilson_loop_det(model, k_loop, occ):
    """``berry_loop_det`` (geometry.rs:217-270): -arg det of the raw product."""
    prod = np.eye(len(occ), dtype=np.complex128)
    for O in _loop_overlaps(model, k_loop, occ):
        prod = prod @ O
    return float(-np.angle(np.linalg.det(prod)))


def berry_flux(model, occ, k_start, dir_1, dir_2, nk1, nk2):
    """``berry_flux`` (geometry.rs:272-339): plaquette Wilson loops, (nk1, nk2, n_occ)."""
    ks, d1, d2 = (np.asarray(v, dtype=np.float64) for v in (k_start, dir_1, dir_2))
    out = np.empty((nk1, nk2, len(occ)))
    dx, dy = 1.0 / nk1, 1.0 / nk2
    for i in range(nk1):
        for j in range(nk2):
            i0, j0 = i / nk1, j / nk2
            loop = [ks + i0 * d1 + j0 * d2, ks + (i0 + dx) * d1 + j0 * d2, ks + (i0 + dx) * d1 + (j0 + dy) * d2,
                    ks + i0 * d1 + (j0 + dy) * d2, ks + i0 * d1 + j0 * d2]
            out[i, j] = wilson_loop(model, np.array(loop), occ)
    return out


def wannier_centre(model, occ, k_start, dir_1, dir_2, nk1, nk2):
    """``wannier_centre`` (geometry.rs:360-420): (n_occ, nk1), sorted per loop."""
    ks, d1, d2 = (np.asarray(v, dtype=np.float64) for v in (k_start, dir_1, dir_2))
    out = np.empty((nk1, len(occ)))
    for i in range(nk1):
        loop = np.array([ks + d1 * float(i) / float(nk1 - 1) + d2 * float(j) / float(nk2 - 1) for j in range(nk2)])
        out[i] = wilson_loop(model, loop, occ)
    return out.T


# --------------------------------------------------------------------------
# Energy-cut Hall integration (src/response/linear/mod.rs:226-268,
# primitives.rs:33-137, tracking.rs, energy_cut.rs, quadrature.rs)
# --------------------------------------------------------------------------

EC_EPS = 1e-12                                   # energy_cut.rs:47
FERMI_X_CUT, FERMI_X_STEPS = 18.0, 72            # energy_cut.rs:48-49
TRI_Q = [[2 / 3, 1 / 6, 1 / 6], [1 / 6, 2 / 3, 1 / 6], [1 / 6, 1 / 6, 2 / 3]]      # quadrature.rs:10-14
TET_Q = [[0.5854101966249685, 0.1381966011250105, 0.1381966011250105, 0.1381966011250105],
         [0.1381966011250105, 0.5854101966249685, 0.1381966011250105, 0.1381966011250105],
         [0.1381966011250105, 0.1381966011250105, 0.5854101966249685, 0.1381966011250105],
         [0.1381966011250105, 0.1381966011250105, 0.1381966011250105, 0.5854101966249685]]
CUBE_TETS = [[0, 1, 2, 4], [3, 1, 2, 7], [5, 1, 4, 7], [6, 2, 4, 7], [1, 2, 4, 7]]  # tracking.rs:8-14
TET_VOL_FACTOR = [1 / 6, 1 / 6, 1 / 6, 1 / 6, 1 / 3]


def vertex_kernels(model, kmesh, directions, spin=-1):
    """compute_velocity_kernel at every mesh point (primitives.rs:33-137):
    energies E (nk, N), eigenvectors W (nk, N, N) in columns, and
    K_nm = va_nm vb_mn (va spin-dressed)."""
    k = gen_kmesh(kmesh)
    nk, N = k.shape[0], model.nsta
    E = np.empty((nk, N))
    Wv = np.empty((nk, N, N), dtype=np.complex128)
    K = np.empty((nk, N, N), dtype=np.complex128)
    for i, kk in enumerate(k):
        V, H = gen_v_projected(model, kk, 1, directions)
        e, w = eigh(H)
        J = V[0]
        if model.spin and spin is not None and spin >= 0:
            S = spin_matrix(model.norb, spin)
            J = 0.5 * (S @ J + J @ S)
        va = w.conj().T @ J @ w
        vb = w.conj().T @ V[1] @ w
        E[i], Wv[i], K[i] = e, w, va * vb.T
    return E, Wv, K


def neighbour_indices(i, kmesh):
    """tracking.rs:177-240 (non-periodic, in the order +x, -x, +y, -y, +z, -z)."""
    dim = len(kmesh)
    out = []
    if dim == 1:
        for d in (1, -1):
            j = i + d
            if 0 <= j < kmesh[0]:
                out.append(j)
    elif dim == 2:
        nx, ny = kmesh
        ix, iy = divmod(i, ny)
        for dx, dy in ((1, 0), (-1, 0), (0, 1), (0, -1)):
            jx, jy = ix + dx, iy + dy
            if 0 <= jx < nx and 0 <= jy < ny:
                out.append(jx * ny + jy)
    else:
        nx, ny, nz = kmesh
        ix, rem = divmod(i, ny * nz)
        iy, iz = divmod(rem, nz)
        for dx, dy, dz in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
            jx, jy, jz = ix + dx, iy + dy, iz + dz
            if 0 <= jx < nx and 0 <= jy < ny and 0 <= jz < nz:
                out.append(jx * ny * nz + jy * nz + jz)
    return out


def greedy_assign(ov):
    """tracking.rs:43-68: rows by their best overlap (descending, stable), each
    takes its best still-free column (the first on ties)."""
    n = ov.shape[0]
    rows = sorted(range(n), key=lambda i: -np.max(ov[i]))
    taken = [False] * n
    perm = [0] * n
    for i in rows:
        best_j, best = 0, -1.0
        for j in range(n):
            if not taken[j] and ov[i, j] > best:
                best, best_j = ov[i, j], j
        taken[best_j] = True
        perm[i] = best_j
    return perm


def global_band_track(E, Wv, K, kmesh):
    """tracking.rs:123-175: breadth-first from vertex 0; each new vertex is
    permuted by the greedy assignment of its averaged overlaps with the
    already-visited neighbours.  Returns the permutation of every vertex."""
    nk = E.shape[0]
    perms = [list(range(E.shape[1])) for _ in range(nk)]
    if nk <= 1:
        return perms
    from collections import deque
    visited = [False] * nk
    visited[0] = True
    q = deque([0])
    while q:
        cur = q.popleft()
        for nb in neighbour_indices(cur, kmesh):
            if visited[nb]:
                continue
            ov_sum, cnt = None, 0
            for vn in neighbour_indices(nb, kmesh):
                if not visited[vn]:
                    continue
                A = Wv[vn][:, perms[vn]]
                ov = np.abs(A.conj().T @ Wv[nb]) ** 2
                ov_sum = ov if ov_sum is None else ov_sum + ov
                cnt += 1
            if ov_sum is not None:
                perms[nb] = greedy_assign(ov_sum / cnt)
            visited[nb] = True
            q.append(nb)
    return perms


def eval_berry_kernel(e, K, eta):
    """kernel.rs:54-80 (Omega part): terms with denominator < 1e-30 skipped."""
    N = len(e)
    om = np.zeros(N)
    eta2 = eta * eta
    for n in range(N):
        g = 0j
        for m in range(N):
            if m == n:
                continue
            de = e[n] - e[m]
            den = de * de + eta2
            if den < 1e-30:
                continue
            g += K[n, m] / den
        om[n] = -2.0 * g.imag
    return om


def _eval_band_at_lam(n, bands, krows, lam, eta):
    """eval_berry_band_at_lam_buf (kernel.rs:138-182): barycentric E_m and K_nm."""
    N = len(bands[0])
    e = np.zeros(N)
    for v in range(len(bands)):
        if lam[v] != 0.0:
            e = e + bands[v] * lam[v]
    kr = np.zeros(N, dtype=np.complex128)
    for v in range(len(krows)):
        if lam[v] != 0.0:
            kr = kr + krows[v] * lam[v]
    eta2 = eta * eta
    g = 0j
    for m in range(N):
        if m == n:
            continue
        de = e[n] - e[m]
        den = de * de + eta2
        if den < 1e-30:
            continue
        g += kr[m] / den
    return -2.0 * g.imag


def _tri_area(c):
    return 0.5 * abs((c[1][0] - c[0][0]) * (c[2][1] - c[0][1]) - (c[2][0] - c[0][0]) * (c[1][1] - c[0][1]))


def _clip_triangle(ev, mu):
    """energy_cut.rs:1120-1170."""
    eps = 1e-12
    if mu <= min(ev) + eps:
        return []
    if mu >= max(ev) - eps:
        return [[[1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]]]
    a, b, c = sorted(range(3), key=lambda i: ev[i])

    def unit(i):
        l = [0.0, 0.0, 0.0]
        l[i] = 1.0
        return l

    def cut(i, j):
        de = ev[j] - ev[i]
        t = 0.5 if abs(de) < eps else min(max((mu - ev[i]) / de, 0.0), 1.0)
        l = [0.0, 0.0, 0.0]
        l[i] = 1.0 - t
        l[j] = t
        return l

    if mu <= ev[b] + eps:
        return [[unit(a), cut(a, b), cut(a, c)]]
    return [[unit(a), unit(b), cut(a, c)], [unit(b), cut(a, c), cut(b, c)]]


def _tri_partial(coords, ev, bands, krows, mu, eta, n):
    """triangle_occupied_hybrid's partial branch (energy_cut.rs:1205-1228)."""
    total = 0.0
    for sub in _clip_triangle(ev, mu):
        pts = [[sum(l[i] * coords[i][0] for i in range(3)), sum(l[i] * coords[i][1] for i in range(3))] for l in sub]
        p0 = [sub[0][0] * coords[0][0] + sub[0][1] * coords[1][0] + sub[0][2] * coords[2][0],
              sub[0][0] * coords[0][1] + sub[0][1] * coords[1][1] + sub[0][2] * coords[2][1]]
        p1 = [sub[1][0] * coords[0][0] + sub[1][1] * coords[1][0] + sub[1][2] * coords[2][0],
              sub[1][0] * coords[0][1] + sub[1][1] * coords[1][1] + sub[1][2] * coords[2][1]]
        p2 = [sub[2][0] * coords[0][0] + sub[2][1] * coords[1][0] + sub[2][2] * coords[2][0],
              sub[2][0] * coords[0][1] + sub[2][1] * coords[1][1] + sub[2][2] * coords[2][1]]
        del pts
        sub_area = 0.5 * abs((p1[0] - p0[0]) * (p2[1] - p0[1]) - (p2[0] - p0[0]) * (p1[1] - p0[1]))
        if sub_area < 1e-30:
            continue
        for q in range(3):
            al = TRI_Q[q]
            lam = [al[0] * sub[0][i] + al[1] * sub[1][i] + al[2] * sub[2][i] for i in range(3)]
            total += sub_area * (1.0 / 3.0) * _eval_band_at_lam(n, bands, krows, lam, eta)
    return total


def _mu_ranges(mu, e_min, e_max):
    i_partial = int(np.searchsorted(mu, e_min + EC_EPS, side="right"))   # partition_point(x <= e_min + eps)
    i_full = int(np.searchsorted(mu, e_max - EC_EPS, side="left"))       # partition_point(x < e_max - eps)
    return i_partial, i_full


def integrate_fermi_cut_2d_t0(E, K, perms, kmesh, mu, eta):
    """energy_cut.rs:1231-1352 with the diagonal-averaged triangles of
    tracking.rs:278-341."""
    nx, ny = kmesh
    inx, iny = 1.0 / nx, 1.0 / ny
    mu = np.asarray(mu, dtype=np.float64)
    acc = np.zeros(len(mu))
    N = E.shape[1]
    Ep = [E[v][perms[v]] for v in range(E.shape[0])]
    Kp = [K[v][np.ix_(perms[v], perms[v])] for v in range(E.shape[0])]
    Om = [eval_berry_kernel(Ep[v], Kp[v], eta) for v in range(E.shape[0])]
    for idx in range(nx * ny):
        iy, ix = idx % ny, idx // ny
        ixp, iyp = (ix + 1) % nx, (iy + 1) % ny
        i00, i10, i11, i01 = ix * ny + iy, ixp * ny + iy, ixp * ny + iyp, ix * ny + iyp

        def coord_of(i):
            if i == i00:
                return (ix * inx, iy * iny)
            if i == i10:
                return ((ix + 1) * inx, iy * iny)
            if i == i11:
                return ((ix + 1) * inx, (iy + 1) * iny)
            return (ix * inx, (iy + 1) * iny)

        for vs in ((i00, i10, i01), (i11, i10, i01), (i00, i10, i11), (i00, i11, i01)):
            coords = [coord_of(v) for v in vs]
            area = _tri_area(coords)
            if area < EC_EPS:
                continue
            scale = (inx * iny / 4.0) / area
            bands = [Ep[v] for v in vs]
            for n in range(N):
                ev = [Ep[v][n] for v in vs]
                ov = [Om[v][n] for v in vs]
                krows = [Kp[v][n] for v in vs]
                full = area * (ov[0] + ov[1] + ov[2]) / 3.0
                ip, iff = _mu_ranges(mu, min(ev), max(ev))
                for im in range(ip, iff):
                    if mu[im] <= min(ev) + EC_EPS:
                        val = 0.0
                    elif mu[im] >= max(ev) - EC_EPS:
                        val = full
                    else:
                        val = _tri_partial(coords, ev, bands, krows, mu[im], eta, n)
                    acc[im] += scale * val
                if iff < len(mu):
                    acc[iff:] += scale * full
    return acc


def _tet_vol(p0, p1, p2, p3):
    """tet_vol_from_pts (energy_cut.rs:1449-1459)."""
    x0, y0, z0 = p0
    x1, y1, z1 = p1
    x2, y2, z2 = p2
    x3, y3, z3 = p3
    det = ((x1 - x0) * ((y2 - y0) * (z3 - z0) - (z2 - z0) * (y3 - y0))
           - (y1 - y0) * ((x2 - x0) * (z3 - z0) - (z2 - z0) * (x3 - x0))
           + (z1 - z0) * ((x2 - x0) * (y3 - y0) - (y2 - y0) * (x3 - x0)))
    return abs(det) / 6.0


def _b2p3(coords, lam):
    return [lam[0] * coords[0][d] + lam[1] * coords[1][d] + lam[2] * coords[2][d] + lam[3] * coords[3][d]
            for d in range(3)]


def _sub_tet(sub, coords, bands, krows, n, eta):
    """sub_tet_k_quad (energy_cut.rs:1501-1527)."""
    vol = _tet_vol(*[_b2p3(coords, l) for l in sub])
    if vol < 1e-30:
        return 0.0
    total = 0.0
    for q in range(4):
        al = TET_Q[q]
        lam = [0.0] * 4
        for k in range(4):
            for i in range(4):
                lam[i] += al[k] * sub[k][i]
        total += vol * 0.25 * _eval_band_at_lam(n, bands, krows, lam, eta)
    return total


def _tet_hybrid(coords, ev, ov, bands, krows, mu, eta, n):
    """tetrahedron_occupied_hybrid (energy_cut.rs:1529-1648)."""
    eps = EC_EPS
    full_vol = _tet_vol(*coords)
    if full_vol < eps:
        return 0.0
    if mu <= min(ev) + eps:
        return 0.0
    if mu >= max(ev) - eps:
        return full_vol * (ov[0] + ov[1] + ov[2] + ov[3]) / 4.0
    a, b, c, d = sorted(range(4), key=lambda i: ev[i])

    def unit(i):
        l = [0.0] * 4
        l[i] = 1.0
        return l

    def cut(i, j):
        de = ev[j] - ev[i]
        t = 0.5 if abs(de) < eps else min(max((mu - ev[i]) / de, 0.0), 1.0)
        l = [0.0] * 4
        l[i] = 1.0 - t
        l[j] = t
        return l

    args = (coords, bands, krows, n, eta)
    if mu <= ev[b] + eps:
        return _sub_tet([unit(a), cut(a, b), cut(a, c), cut(a, d)], *args)
    if mu <= ev[c] + eps:
        return (_sub_tet([unit(a), unit(b), cut(a, c), cut(b, d)], *args)
                + _sub_tet([unit(a), cut(a, c), cut(a, d), cut(b, d)], *args)
                + _sub_tet([unit(b), cut(b, c), cut(b, d), cut(a, c)], *args))
    full_val = full_vol * (ov[0] + ov[1] + ov[2] + ov[3]) / 4.0
    return full_val - _sub_tet([unit(d), cut(a, d), cut(b, d), cut(c, d)], *args)


def integrate_fermi_cut_3d_t0(E, K, perms, kmesh, mu, eta):
    """energy_cut.rs:1651-1795 with build_tetrahedra_3d (tracking.rs:343-405)."""
    nx, ny, nz = kmesh
    inx, iny, inz = 1.0 / nx, 1.0 / ny, 1.0 / nz
    mu = np.asarray(mu, dtype=np.float64)
    acc = np.zeros(len(mu))
    N = E.shape[1]
    Ep = [E[v][perms[v]] for v in range(E.shape[0])]
    Kp = [K[v][np.ix_(perms[v], perms[v])] for v in range(E.shape[0])]
    Om = [eval_berry_kernel(Ep[v], Kp[v], eta) for v in range(E.shape[0])]
    cube_vol = inx * iny * inz
    for idx in range(nx * ny * nz):
        iz = idx % nz
        iy = (idx // nz) % ny
        ix = idx // (ny * nz)
        ixp, iyp, izp = (ix + 1) % nx, (iy + 1) % ny, (iz + 1) % nz
        i3 = lambda x, y, z: x * ny * nz + y * nz + z  # noqa: E731
        c = [i3(ix, iy, iz), i3(ixp, iy, iz), i3(ix, iyp, iz), i3(ixp, iyp, iz),
             i3(ix, iy, izp), i3(ixp, iy, izp), i3(ix, iyp, izp), i3(ixp, iyp, izp)]
        f = lambda a, b, cc: (a * inx, b * iny, cc * inz)  # noqa: E731
        corners = [f(ix, iy, iz), f(ix + 1, iy, iz), f(ix, iy + 1, iz), f(ix + 1, iy + 1, iz),
                   f(ix, iy, iz + 1), f(ix + 1, iy, iz + 1), f(ix, iy + 1, iz + 1), f(ix + 1, iy + 1, iz + 1)]
        for t, tet in enumerate(CUBE_TETS):
            coords = [corners[l] for l in tet]
            vs = [c[l] for l in tet]
            vol = _tet_vol(*coords)
            if vol < EC_EPS:
                continue
            scale = (cube_vol * TET_VOL_FACTOR[t]) / vol
            bands = [Ep[v] for v in vs]
            for n in range(N):
                ev = [Ep[v][n] for v in vs]
                ov = [Om[v][n] for v in vs]
                krows = [Kp[v][n] for v in vs]
                full = vol * (ov[0] + ov[1] + ov[2] + ov[3]) / 4.0
                ip, iff = _mu_ranges(mu, min(ev), max(ev))
                for im in range(ip, iff):
                    acc[im] += scale * _tet_hybrid(coords, ev, ov, bands, krows, mu[im], eta, n)
                if iff < len(mu):
                    acc[iff:] += scale * full
    return acc


def _fermi_window_x(x):
    if abs(x) > 50.0:
        return 0.0
    ex = np.exp(x)
    return ex / ((1.0 + ex) * (1.0 + ex))


def integrate_fermi_cut(E, K, perms, kmesh, mu, width, eta):
    """integrate_fermi_cut_2d / _3d (energy_cut.rs:1355-1428, 1797-1849): the
    T = 0 sweep, or its thermal convolution on an extended fine mu grid."""
    t0 = integrate_fermi_cut_2d_t0 if len(kmesh) == 2 else integrate_fermi_cut_3d_t0
    mu = np.asarray(mu, dtype=np.float64)
    if width == 0.0:
        return t0(E, K, perms, kmesh, mu, eta)
    beta = 1.0 / width
    x_max = 12.0
    mu_lo = float(mu.min()) - x_max / beta
    mu_hi = float(mu.max()) + x_max / beta
    dmu = 0.1 / beta
    n_ext = int(np.ceil((mu_hi - mu_lo) / dmu)) + 1
    step = (mu_hi - mu_lo) / (n_ext - 1) if n_ext > 1 else 0.0
    mu_ext = mu_lo + step * np.arange(n_ext, dtype=np.float64)
    s0 = t0(E, K, perms, kmesh, mu_ext, eta)
    dx = 2.0 * FERMI_X_CUT / FERMI_X_STEPS
    out = np.empty(len(mu))
    for j, m in enumerate(mu):
        s = 0.0
        for iq in range(FERMI_X_STEPS):
            x = -FERMI_X_CUT + (iq + 0.5) * dx
            w = _fermi_window_x(x)
            i_f = (m + x / beta - mu_lo) / dmu
            i_lo = max(int(np.floor(i_f)), 0)
            i_hi = min(i_lo + 1, n_ext - 1)
            if i_hi > i_lo:
                t = i_f - i_lo
                s += dx * w * (s0[i_lo] + t * (s0[i_hi] - s0[i_lo]))
        out[j] = s
    return out


def hall_energy_cut(model, kmesh, directions, mu_list, T=0.0, eta=1e-3, spin=-1):
    """``hall_conductivity`` with Integration::EnergyCut (linear/mod.rs:226-268)."""
    E, Wv, K = vertex_kernels(model, kmesh, directions, spin)
    perms = global_band_track(E, Wv, K, list(kmesh))
    width = occupation_width(T)
    s = integrate_fermi_cut(E, K, perms, list(kmesh), mu_list, width, eta)
    return s / float(np.linalg.det(model.lat))
