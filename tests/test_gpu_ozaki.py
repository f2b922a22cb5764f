"""Exact-slice BF16 tensor-core complex GEMM against numpy FP64 (GPU).

The HIGH class must reach 1e-12 of the natural product scale
(max|row of op(A)| * max|column of B| * K); the MID class (five digits,
used for the rotation into the eigenbasis) 1e-10; the LOW class 1e-5."""

import ctypes

import numpy as np
import pytest

from rustb_gb300 import _lib

pytestmark = pytest.mark.gpu


def ozaki(lib, A, B, conj_a, high, use_tc=0):
    batch = A.shape[0]
    if conj_a:
        K, M = A.shape[1], A.shape[2]
    else:
        M, K = A.shape[1], A.shape[2]
    Nc = B.shape[2]
    C = np.zeros((batch, M, Nc), dtype=np.complex128)
    dp = ctypes.POINTER(ctypes.c_double)
    fn = lib.tbg_internal_ozaki_zgemm
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, dp,
                   ctypes.c_int]
    A = np.ascontiguousarray(A)
    B = np.ascontiguousarray(B)
    st = fn(int(high), int(conj_a), batch, M, Nc, K, A.view(np.float64).ctypes.data_as(dp),
            B.view(np.float64).ctypes.data_as(dp), C.view(np.float64).ctypes.data_as(dp), int(use_tc))
    _lib.check(st, lib)
    return C


@pytest.mark.parametrize("use_tc", [0, 1], ids=["mma_sync", "tcgen05"])
@pytest.mark.parametrize("conj_a", [False, True])
@pytest.mark.parametrize("M,Nc,K", [(128, 128, 128), (70, 40, 100), (256, 64, 256), (1, 3, 2), (200, 130, 48)])
def test_ozaki_high_precision(conj_a, M, Nc, K, use_tc):
    lib = _lib.load()
    rng = np.random.default_rng(M + Nc + K)
    batch = 3
    shapeA = (batch, K, M) if conj_a else (batch, M, K)
    A = rng.standard_normal(shapeA) + 1j * rng.standard_normal(shapeA)
    B = rng.standard_normal((batch, K, Nc)) + 1j * rng.standard_normal((batch, K, Nc))
    # rows/columns of very different magnitude
    if conj_a:
        A *= 10.0 ** rng.uniform(-3, 3, (batch, 1, M))
    else:
        A *= 10.0 ** rng.uniform(-3, 3, (batch, M, 1))
    B *= 10.0 ** rng.uniform(-3, 3, (batch, 1, Nc))
    opA = np.conj(np.transpose(A, (0, 2, 1))) if conj_a else A
    ref = opA @ B
    C = ozaki(lib, A, B, conj_a, True, use_tc)
    scale = (np.abs(opA).max(axis=2)[:, :, None] * np.abs(B).max(axis=1)[:, None, :]) * K
    err = np.abs(C - ref) / scale
    assert err.max() < 1e-12, err.max()


@pytest.mark.parametrize("use_tc", [0, 1], ids=["mma_sync", "tcgen05"])
def test_ozaki_low_precision_and_zeros(use_tc):
    lib = _lib.load()
    rng = np.random.default_rng(3)
    A = rng.standard_normal((2, 64, 64)) + 1j * rng.standard_normal((2, 64, 64))
    B = rng.standard_normal((2, 64, 64)) + 1j * rng.standard_normal((2, 64, 64))
    A[0, 5, :] = 0.0  # an all-zero row
    ref = A @ B
    C = ozaki(lib, A, B, False, False, use_tc)
    scale = np.abs(A).max() * np.abs(B).max() * 64
    assert np.abs(C - ref).max() / scale < 1e-5
    assert np.all(C[0, 5, :] == 0.0)


@pytest.mark.parametrize("conj_a", [False, True])
@pytest.mark.parametrize("M,Nc,K", [(128, 64, 600), (70, 130, 257), (256, 128, 1024)])
def test_ozaki_tc_long_contractions(conj_a, M, Nc, K):
    """K > 256: exact chunks of 256 whose float pairs are added in the epilogue."""
    lib = _lib.load()
    rng = np.random.default_rng(M + Nc + K + 1)
    batch = 2
    shapeA = (batch, K, M) if conj_a else (batch, M, K)
    A = rng.standard_normal(shapeA) + 1j * rng.standard_normal(shapeA)
    B = rng.standard_normal((batch, K, Nc)) + 1j * rng.standard_normal((batch, K, Nc))
    if conj_a:
        A *= 10.0 ** rng.uniform(-3, 3, (batch, 1, M))
    else:
        A *= 10.0 ** rng.uniform(-3, 3, (batch, M, 1))
    B *= 10.0 ** rng.uniform(-3, 3, (batch, 1, Nc))
    opA = np.conj(np.transpose(A, (0, 2, 1))) if conj_a else A
    ref = opA @ B
    C = ozaki(lib, A, B, conj_a, True, 1)
    scale = (np.abs(opA).max(axis=2)[:, :, None] * np.abs(B).max(axis=1)[:, None, :]) * K
    assert (np.abs(C - ref) / scale).max() < 1e-12


def test_ozaki_tc_low_long_contraction():
    lib = _lib.load()
    rng = np.random.default_rng(11)
    A = rng.standard_normal((2, 64, 700)) + 1j * rng.standard_normal((2, 64, 700))
    B = rng.standard_normal((2, 700, 48)) + 1j * rng.standard_normal((2, 700, 48))
    C = ozaki(lib, A, B, False, False, 1)
    assert np.abs(C - A @ B).max() / (np.abs(A).max() * np.abs(B).max() * 700) < 1e-5


@pytest.mark.parametrize("conj_a", [False, True])
def test_ozaki_tc_many_tiles_per_cta(conj_a):
    """More tiles than SMs: every persistent CTA runs several tiles back to
    back (ragged edges in rows, columns and k), HIGH class within 1e-12."""
    lib = _lib.load()
    rng = np.random.default_rng(77 + conj_a)
    batch, M, Nc, K = 200, 200, 130, 100
    shapeA = (batch, K, M) if conj_a else (batch, M, K)
    A = rng.standard_normal(shapeA) + 1j * rng.standard_normal(shapeA)
    B = rng.standard_normal((batch, K, Nc)) + 1j * rng.standard_normal((batch, K, Nc))
    B *= 10.0 ** rng.uniform(-3, 3, (batch, 1, Nc))
    opA = np.conj(np.transpose(A, (0, 2, 1))) if conj_a else A
    ref = opA @ B
    C = ozaki(lib, A, B, conj_a, True, 1)
    scale = (np.abs(opA).max(axis=2)[:, :, None] * np.abs(B).max(axis=1)[:, None, :]) * K
    assert (np.abs(C - ref) / scale).max() < 1e-12


@pytest.mark.parametrize("conj_a", [False, True])
@pytest.mark.parametrize("M,Nc,K", [(128, 128, 128), (70, 40, 100), (200, 130, 300)])
def test_ozaki_tc_mid_precision(conj_a, M, Nc, K):
    """MID class on tcgen05: about 2^-35 of the natural scale (bound 1e-10),
    with rows and columns of very different magnitude and a contraction
    longer than one exact chunk (K = 300)."""
    lib = _lib.load()
    rng = np.random.default_rng(7 * M + Nc + K)
    batch = 3
    shapeA = (batch, K, M) if conj_a else (batch, M, K)
    A = rng.standard_normal(shapeA) + 1j * rng.standard_normal(shapeA)
    B = rng.standard_normal((batch, K, Nc)) + 1j * rng.standard_normal((batch, K, Nc))
    if conj_a:
        A *= 10.0 ** rng.uniform(-3, 3, (batch, 1, M))
    else:
        A *= 10.0 ** rng.uniform(-3, 3, (batch, M, 1))
    B *= 10.0 ** rng.uniform(-3, 3, (batch, 1, Nc))
    opA = np.conj(np.transpose(A, (0, 2, 1))) if conj_a else A
    ref = opA @ B
    C = ozaki(lib, A, B, conj_a, 2, 1)
    scale = (np.abs(opA).max(axis=2)[:, :, None] * np.abs(B).max(axis=1)[:, None, :]) * K
    err = (np.abs(C - ref) / scale).max()
    print(f"MID class {M}x{Nc}x{K}: {err:.2e}")
    assert err < 1e-10, err


@pytest.mark.parametrize("conj_a", [False, True])
def test_ozaki_tc_mid_many_tiles_long_contraction(conj_a):
    """MID class, more tiles than SMs and a contraction of two exact chunks:
    the persistent CTAs run several tiles each and the second chunk adds its
    float pairs to the first chunk's output (bound 1e-10)."""
    lib = _lib.load()
    rng = np.random.default_rng(91 + conj_a)
    batch, M, Nc, K = 120, 200, 130, 300
    shapeA = (batch, K, M) if conj_a else (batch, M, K)
    A = rng.standard_normal(shapeA) + 1j * rng.standard_normal(shapeA)
    B = rng.standard_normal((batch, K, Nc)) + 1j * rng.standard_normal((batch, K, Nc))
    B *= 10.0 ** rng.uniform(-3, 3, (batch, 1, Nc))
    opA = np.conj(np.transpose(A, (0, 2, 1))) if conj_a else A
    ref = opA @ B
    C = ozaki(lib, A, B, conj_a, 2, 1)
    scale = (np.abs(opA).max(axis=2)[:, :, None] * np.abs(B).max(axis=1)[:, None, :]) * K
    err = (np.abs(C - ref) / scale).max()
    assert err < 1e-10, err
