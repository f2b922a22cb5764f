"""Accuracy of the FP32 eigensolver that starts the mixed path, on its own:
orthogonality and residual of the eigenpairs before refinement (GPU).

Measured on GB300 (128 bands): orthogonality ~1.5e-4 (eigenvalue pairs just
outside the 1e-3 ||T|| cluster threshold, error ~ eps ||T|| / gap), residual
~8e-7 ||H||, eigenvalues ~2.6e-7 ||H|| with the reduction on the CUDA cores;
from 65 bands the reduction's rank-2 updates (of the whole matrix up to 128
bands, of the last 128 steps up to 320) accumulate into the TMEM-resident
matrix on the tensor cores, whose FP32 accumulation rounds less well
(eigenvalues ~2-4e-6 ||H||, residual and orthogonality unchanged).
The Ogita-Aishima sweep that follows takes these to ~1e-12.  The bounds leave
margin and catch a broken stage."""


def eig_bound(n):
    """Eigenvalue bound (relative to ||H||) of the FP32 stage at order n (the
    TMEM-resident reduction runs the whole matrix up to 128 bands and the last
    128 steps up to 320)."""
    return 2e-5 if 64 < n <= 320 else 1e-6

import ctypes

import numpy as np
import pytest

from rustb_gb300 import _lib, workloads as W

pytestmark = pytest.mark.gpu


def eig_f32(H):
    lib = _lib.load()
    nk, n = H.shape[0], H.shape[1]
    E = np.zeros((nk, n))
    U = np.zeros((nk, n, n), dtype=np.complex128)
    dp = ctypes.POINTER(ctypes.c_double)
    fn = lib.tbg_internal_eig_f32
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.c_int64, dp, dp, dp]
    H = np.ascontiguousarray(H, dtype=np.complex128)
    _lib.check(fn(n, nk, H.view(np.float64).ctypes.data_as(dp), E.ctypes.data_as(dp),
                  U.view(np.float64).ctypes.data_as(dp)), lib)
    return E, U


def quality(H, E, U):
    nrm = np.abs(np.linalg.eigvalsh(H)).max(axis=1)
    orth = np.abs(np.conj(np.transpose(U, (0, 2, 1))) @ U - np.eye(H.shape[1])).max(axis=(1, 2))
    res = np.abs(H @ U - U * E[:, None, :]).max(axis=(1, 2)) / nrm
    eerr = np.abs(E - np.linalg.eigvalsh(H)).max(axis=1) / nrm
    return orth.max(), res.max(), eerr.max()


# Sizes cover each layout of the solver: two matrices per SM with the
# register-tiled back-transformation (<= 144 bands, including N not a multiple
# of 4), one matrix per SM with the panel back-transformation (150, 200, 220),
# the hybrid layout with the first rows in global memory (251, 300: rows below
# 22 and 72), the matrix in global memory (330), the TMEM-resident reduction
# and back-transformation (65-128: both ends, and sizes that are not multiples
# of the 8-column chunks), the small-matrix thread counts (9, 12, 17), and the
# fused one-pass reduction (up to 129 bands: 129, 2, 3, 5).
@pytest.mark.parametrize("n", [330, 300, 251, 220, 200, 150, 144, 131, 129, 128, 127, 100, 97, 65, 64, 40, 17, 12, 9, 5, 3,
                               2])
def test_fp32_eigenpairs_random_hermitian(n):
    rng = np.random.default_rng(n)
    X = rng.standard_normal((16, n, n)) + 1j * rng.standard_normal((16, n, n))
    H = 0.5 * (X + np.conj(np.transpose(X, (0, 2, 1))))
    E, U = eig_f32(H)
    orth, res, eerr = quality(H, E, U)
    print(f"n={n}: orthogonality {orth:.2e}, residual {res:.2e}, eigenvalues {eerr:.2e}")
    assert orth < 1e-3 and res < 1e-5 and eerr < eig_bound(n)


def test_fp32_eigenpairs_benchmark_model():
    m = W.random_spinful_3d()
    k = np.random.default_rng(1).uniform(0, 1, (32, 3))
    H = m.gen_ham_batch(k)
    E, U = eig_f32(H)
    orth, res, eerr = quality(H, E, U)
    print(f"128-band model: orthogonality {orth:.2e}, residual {res:.2e}, eigenvalues {eerr:.2e}")
    assert orth < 1e-3 and res < 1e-5 and eerr < eig_bound(128)


@pytest.mark.parametrize("n", [64, 128, 100])
def test_fp32_eigenpairs_many_waves_and_clusters(n):
    """More matrices than resident CTAs (the persistent loop: the tensor-core
    reduction's mbarrier phases run on across a CTA's matrices), and spectra
    with exact multiplicities (block-diagonal copies: the cluster path)."""
    rng = np.random.default_rng(5 + n)
    nk, hn = 700, n // 2
    X = rng.standard_normal((nk, n, n)) + 1j * rng.standard_normal((nk, n, n))
    H = 0.5 * (X + np.conj(np.transpose(X, (0, 2, 1))))
    h = H[:64, :hn, :hn].copy()
    H[:64] = 0
    H[:64, :hn, :hn] = h
    H[:64, hn:2 * hn, hn:2 * hn] = h  # every eigenvalue twice (plus a zero when n is odd)
    E, U = eig_f32(H)
    orth, res, eerr = quality(H, E, U)
    print(f"n={n}, {nk} matrices: orthogonality {orth:.2e}, residual {res:.2e}, eigenvalues {eerr:.2e}")
    assert orth < 1e-3 and res < 1e-5 and eerr < eig_bound(n)
