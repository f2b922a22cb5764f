"""tbg_eigvalsh_noalloc against the allocating band solver, through the C-ABI.

The no-allocation entry point exists for callers that cannot call cudaMalloc
(their own allocator owns the device memory, or a device-synchronising
cudaMalloc would stall a latency-critical loop).  They hand it device
pointers; the solver works in a fixed static device array.  Two calls in a row
must each agree with tbg_solve_band on the same Hamiltonians.
"""

import ctypes

import numpy as np
import pytest

from oracle import tb_oracle as O
from rustb_gb300 import _lib, errors, workloads as W

pytestmark = pytest.mark.gpu

SCRATCH_BYTES = 32 * 1024 * 1024


def _noalloc_bands(lib, torch, H):
    """Copy H (nk, n, n) complex to the device, solve there, return E."""
    nk, n, _ = H.shape
    Hd = torch.from_numpy(np.ascontiguousarray(H).view(np.float64).reshape(-1)).cuda()
    Ed = torch.empty(nk * n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    st = lib.tbg_eigvalsh_noalloc(n, nk, ctypes.c_void_p(Hd.data_ptr()), ctypes.c_void_p(Ed.data_ptr()),
                                  ctypes.c_void_p(stream))
    _lib.check(st, lib)
    torch.cuda.synchronize()
    return Ed.cpu().numpy().reshape(nk, n), Hd


@pytest.mark.parametrize("norb,spin,nk", [(64, True, 40), (5, False, 300)])
def test_noalloc_matches_solve_band_twice(norb, spin, nk):
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    model = W.random_model(3, norb, spin, 1, seed=norb)
    rng = np.random.default_rng(norb)
    for call in range(2):  # two calls in a row share the static array
        k = rng.uniform(0, 1, (nk - 7 * call, 3))
        H = model.gen_ham_batch(k)
        E_ref = model.solve_band_all_parallel(k)
        E, Hd = _noalloc_bands(lib, torch, H)
        nrm = max(np.linalg.norm(h, 2) for h in H[:4])
        assert np.max(np.abs(E - E_ref)) <= 1e-10 * nrm
        # the caller's input is left untouched
        assert np.array_equal(Hd.cpu().numpy(), np.ascontiguousarray(H).view(np.float64).reshape(-1))
    Ez = O.eigvalsh(H[0])
    assert np.max(np.abs(E[0] - Ez)) <= 1e-10 * nrm


def _random_hermitian(rng, nk, n):
    a = rng.standard_normal((nk, n, n)) + 1j * rng.standard_normal((nk, n, n))
    return 0.5 * (a + np.conj(np.swapaxes(a, 1, 2)))


@pytest.mark.parametrize("n,nk", [(1, 7), (2, 33), (128, SCRATCH_BYTES // (16 * 128 * 128))])
def test_noalloc_edges_and_exact_capacity(n, nk):
    """The smallest orders, and a call that fills the array exactly
    (nk * 16 n^2 == 32 MiB), against LAPACK."""
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    H = _random_hermitian(np.random.default_rng(n), nk, n)
    for _ in range(2):
        E, _ = _noalloc_bands(lib, torch, H)
        for i in range(0, nk, max(1, nk // 16)):
            nrm = max(np.linalg.norm(H[i], 2), 1e-300)
            assert np.max(np.abs(E[i] - O.eigvalsh(H[i]))) <= 1e-10 * nrm


def test_noalloc_rejects_oversized_request():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    n = 128
    too_many = SCRATCH_BYTES // (16 * n * n) + 1
    Hd = torch.empty(16, dtype=torch.float64, device="cuda")
    Ed = torch.empty(16, dtype=torch.float64, device="cuda")
    st = lib.tbg_eigvalsh_noalloc(n, too_many, ctypes.c_void_p(Hd.data_ptr()), ctypes.c_void_p(Ed.data_ptr()),
                                  None)
    assert st == errors.TBG_E_UNSUPPORTED
    assert "scratch" in _lib.last_error(lib)
    # one matrix beyond the array's largest order
    st = lib.tbg_eigvalsh_noalloc(1449, 1, ctypes.c_void_p(Hd.data_ptr()), ctypes.c_void_p(Ed.data_ptr()), None)
    assert st == errors.TBG_E_UNSUPPORTED
    assert "1448" in _lib.last_error(lib)
