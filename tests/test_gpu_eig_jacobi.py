"""The warp-per-matrix Jacobi solver (FP64, 8 < N <= 32) against the oracle's
eigenvalues and against the Householder solver, through the internal hook that
runs either one on a device copy of the matrices (GPU)."""

import ctypes

import numpy as np
import pytest

from oracle import tb_oracle as O
from rustb_gb300 import _lib

pytestmark = pytest.mark.gpu


def eig_f64(H, method):
    lib = _lib.load()
    nk, n = H.shape[0], H.shape[1]
    E = np.zeros((nk, n))
    U = np.zeros((nk, n, n), dtype=np.complex128)
    dp = ctypes.POINTER(ctypes.c_double)
    fn = lib.tbg_internal_eig_f64
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.c_int64, dp, dp, dp, ctypes.c_int, ctypes.c_int,
                   ctypes.POINTER(ctypes.c_float)]
    H = np.ascontiguousarray(H, dtype=np.complex128)
    ms = ctypes.c_float(0.0)
    _lib.check(fn(n, nk, H.view(np.float64).ctypes.data_as(dp), E.ctypes.data_as(dp),
                  U.view(np.float64).ctypes.data_as(dp), method, 1, ctypes.byref(ms)), lib)
    return E, U


def random_hermitian(nk, n, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((nk, n, n)) + 1j * rng.standard_normal((nk, n, n))
    return 0.5 * (X + np.conj(np.transpose(X, (0, 2, 1))))


def check(H, E, U, tol=1e-12):
    nrm = np.linalg.norm(H, 2, axis=(1, 2))
    for i in range(H.shape[0]):
        assert np.max(np.abs(E[i] - O.eigvalsh(H[i]))) <= tol * nrm[i]
    res = np.abs(H @ U - U * E[:, None, :]).max(axis=(1, 2)) / nrm
    orth = np.abs(np.conj(np.transpose(U, (0, 2, 1))) @ U - np.eye(H.shape[1])).max(axis=(1, 2))
    assert res.max() <= tol and orth.max() <= 1e-12
    assert np.all(np.diff(E, axis=1) >= 0)


@pytest.mark.parametrize("n", [9, 12, 15, 16, 17, 24, 31, 32])
def test_jacobi_random_hermitian(n):
    H = random_hermitian(70, n, 900 + n)  # 70 matrices: odd CTA tail with two warps per CTA
    E, U = eig_f64(H, 1)
    check(H, E, U)
    Eh, _ = eig_f64(H, 0)
    assert np.max(np.abs(E - Eh)) <= 1e-12 * np.max(np.abs(Eh))


def test_jacobi_degenerate_and_diagonal():
    """Repeated eigenvalues (two copies of one block, rotated), a diagonal
    matrix (no rotation at all) and a zero matrix."""
    n = 20
    rng = np.random.default_rng(5)
    b = random_hermitian(1, n // 2, 6)[0]
    D = np.zeros((n, n), dtype=np.complex128)
    D[: n // 2, : n // 2] = b
    D[n // 2:, n // 2:] = b
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    H = np.stack([Q @ D @ np.conj(Q.T), np.diag(rng.standard_normal(n)).astype(np.complex128),
                  np.zeros((n, n), dtype=np.complex128)])
    H[0] = 0.5 * (H[0] + np.conj(H[0].T))
    E, U = eig_f64(H, 1)
    check(H[:2], E[:2], U[:2])
    assert np.all(E[2] == 0.0)
    assert np.abs(U[2] - np.eye(n)).max() == 0.0


def test_driver_takes_jacobi_when_selected():
    """TBG_JACOBI_MAX_N=32 sends the FP64 driver's 9-32-band solves to the Jacobi
    solver (read once per process, so a child process runs it)."""
    import os
    import subprocess
    import sys

    code = (
        "import numpy as np\n"
        "from oracle import tb_oracle as O\n"
        "from rustb_gb300 import _lib, workloads as W\n"
        "from rustb_gb300.params import Precision\n"
        "lib = _lib.load()\n"
        "lib.tbg_kernel_timing_enable(1)\n"
        "_lib.kernel_timing(reset=True)\n"
        "m = W.random_model(2, 12, False, 1, seed=31)\n"
        "k = np.random.default_rng(2).uniform(0, 1, (50, 2))\n"
        "E = m.solve_band_all_parallel(k, Precision.FP64)\n"
        "H = O.gen_ham_batch(m, k, 1)\n"
        "err = max(np.max(np.abs(E[i] - O.eigvalsh(H[i]))) / np.linalg.norm(H[i], 2) for i in range(50))\n"
        "assert err <= 1e-12, err\n"
        "assert 'jacobi_warp_kernel' in _lib.kernel_timing(), _lib.kernel_timing()\n"
        "print('ok', err)\n")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, TBG_JACOBI_MAX_N="32")
    r = subprocess.run([sys.executable, "-c", code], cwd=root, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ok" in r.stdout
