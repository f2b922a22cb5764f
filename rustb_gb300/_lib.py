"""ctypes binding of ``libtbgpu.so`` (the C-ABI declared in include/tbgpu.h).

The library is built in-tree by :func:`rustb_gb300.build.build_library`.  There
is no fallback: if the shared object is missing or fails to load, every
device entry point raises :class:`LibraryMissing`.
"""

from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import errors

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "_build", "libtbgpu.so")

_c_double_p = ctypes.POINTER(ctypes.c_double)
_c_int64_p = ctypes.POINTER(ctypes.c_int64)


class LibraryMissing(RuntimeError):
    pass


class TbgReport(ctypes.Structure):
    _fields_ = [
        ("nk", ctypes.c_int64),
        ("nsta", ctypes.c_int64),
        ("precision", ctypes.c_int32),
        ("fourier_mode", ctypes.c_int32),
        ("kernel_launches", ctypes.c_int64),
        ("device_ms", ctypes.c_double),
        ("eig_ms", ctypes.c_double),
        ("refine_clusters", ctypes.c_int64),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class TbgJob(ctypes.Structure):
    """``tbg_job`` of the asynchronous batch queue."""
    _fields_ = [
        ("kind", ctypes.c_int),
        ("model", ctypes.c_void_p),
        ("kmesh", _c_int64_p),
        ("nk", ctypes.c_int64),
        ("k", _c_double_p),
        ("dirs2", _c_double_p),
        ("nmu", ctypes.c_int64),
        ("mu", _c_double_p),
        ("T", ctypes.c_double),
        ("eta", ctypes.c_double),
        ("spin", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("out0", _c_double_p),
        ("out1", _c_double_p),
    ]


JOB_HALL, JOB_BANDS, JOB_BERRY, JOB_OCCUPIED = 0, 1, 2, 3

# (name, restype, argtypes) for every symbol include/tbgpu.h declares.
SIGNATURES = [
    ("tbg_model_create", ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_int64,
                                        _c_int64_p, _c_double_p, _c_double_p, _c_double_p,
                                        ctypes.POINTER(ctypes.c_void_p)]),
    ("tbg_model_set_rmatrix", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, _c_double_p]),
    ("tbg_model_destroy", ctypes.c_int, [ctypes.c_void_p]),
    ("tbg_model_info", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                      _c_int64_p, _c_int64_p, _c_int64_p]),
    ("tbg_gen_ham", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, _c_double_p, ctypes.c_int, _c_double_p]),
    ("tbg_gen_v", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, _c_double_p, ctypes.c_int,
                                 _c_double_p, _c_double_p]),
    ("tbg_gen_v_projected", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, _c_double_p, ctypes.c_int,
                                           ctypes.c_int64, _c_double_p, _c_double_p, _c_double_p]),
    ("tbg_solve_band", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, _c_double_p, _c_double_p]),
    ("tbg_solve_band_prec", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, _c_double_p, ctypes.c_int, _c_double_p]),
    ("tbg_solve", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, _c_double_p, _c_double_p, _c_double_p,
                                 ctypes.c_int]),
    ("tbg_berry_curvature", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, _c_double_p, _c_double_p,
                                           ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                           _c_double_p, _c_double_p]),
    ("tbg_berry_curvature_multi", ctypes.c_int, [ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p), _c_int64_p,
                                                 _c_double_p, _c_double_p, ctypes.c_int, ctypes.c_double,
                                                 ctypes.c_int, _c_double_p, _c_double_p]),
    ("tbg_occupied_berry_curvature", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, _c_double_p, _c_double_p,
                                                    ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                                    ctypes.c_double, ctypes.c_int, _c_double_p]),
    ("tbg_hall_conductivity", ctypes.c_int, [ctypes.c_void_p, _c_int64_p, _c_double_p, ctypes.c_int64,
                                             _c_double_p, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                             ctypes.c_int, _c_double_p, ctypes.POINTER(TbgReport)]),
    ("tbg_hall_sums_range", ctypes.c_int, [ctypes.c_void_p, _c_int64_p, ctypes.c_int64, ctypes.c_int64,
                                           _c_double_p, ctypes.c_int64, _c_double_p, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_int, ctypes.c_int, _c_double_p,
                                           ctypes.POINTER(TbgReport)]),
    ("tbg_quantum_geometry", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, _c_double_p, _c_double_p,
                                            ctypes.c_double, ctypes.c_int, _c_double_p, _c_double_p,
                                            _c_double_p]),
    ("tbg_quantum_geometry_mesh", ctypes.c_int, [ctypes.c_void_p, _c_int64_p, _c_double_p, ctypes.c_int64,
                                                 _c_double_p, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                                 _c_double_p, _c_double_p, ctypes.POINTER(TbgReport)]),
    ("tbg_bands_mesh", ctypes.c_int, [ctypes.c_void_p, _c_int64_p, _c_double_p]),
    ("tbg_dos", ctypes.c_int, [ctypes.c_void_p, _c_int64_p, ctypes.c_double, ctypes.c_double, ctypes.c_int64,
                               ctypes.c_double, _c_double_p, _c_double_p]),
    ("tbg_hall_energy_cut", ctypes.c_int, [ctypes.c_void_p, _c_int64_p, _c_double_p, ctypes.c_int64, _c_double_p,
                                           ctypes.c_double, ctypes.c_double, ctypes.c_int, _c_double_p]),
    ("tbg_wilson_loops", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, _c_double_p,
                                        ctypes.c_int64, _c_int64_p, ctypes.c_int, ctypes.c_int, _c_double_p]),
    ("tbg_w90_read_hr", ctypes.c_int, [ctypes.c_char_p, ctypes.c_double, ctypes.POINTER(ctypes.c_void_p)]),
    ("tbg_w90_read_r", ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    ("tbg_w90_apply_wsvec", ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]),
    ("tbg_w90_hermitize_rmatrix", ctypes.c_int, [ctypes.c_void_p]),
    ("tbg_w90_info", ctypes.c_int, [ctypes.c_void_p, _c_int64_p, _c_int64_p, ctypes.POINTER(ctypes.c_int)]),
    ("tbg_w90_copy", ctypes.c_int, [ctypes.c_void_p, _c_double_p, _c_int64_p, _c_double_p]),
    ("tbg_w90_free", ctypes.c_int, [ctypes.c_void_p]),
    ("tbg_measure_fma_peaks", ctypes.c_int, [_c_double_p, _c_double_p]),
    ("tbg_set_device", ctypes.c_int, [ctypes.c_int]),
    ("tbg_kernel_timing_enable", ctypes.c_int, [ctypes.c_int]),
    ("tbg_chunk_budget_bytes", ctypes.c_int64, []),
    ("tbg_kernel_timing_read", ctypes.c_int, [ctypes.c_char_p, _c_int64_p, _c_double_p, _c_double_p,
                                              ctypes.c_int, ctypes.c_int]),
    ("tbg_eigvalsh_noalloc", ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_void_p]),
    ("tbg_batch_submit", ctypes.c_int, [ctypes.POINTER(TbgJob), _c_int64_p]),
    ("tbg_batch_poll", ctypes.c_int, [ctypes.c_int64, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    ("tbg_batch_wait", ctypes.c_int, [ctypes.c_int64, ctypes.POINTER(ctypes.c_int)]),
    ("tbg_batch_set_workers", ctypes.c_int, [ctypes.c_int]),
    ("tbg_last_error", ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    ("tbg_set_jacobi_max_n", ctypes.c_int, [ctypes.c_int]),
    ("tbg_version", ctypes.c_char_p, []),
    ("tbg_kernel_launch_count", ctypes.c_int64, [ctypes.c_int]),
]

_lock = threading.Lock()
_lib = None


def load(path: str | None = None):
    """Load (once) and return the ctypes library handle."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise LibraryMissing(
                f"{p} not found: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        lib = ctypes.CDLL(p)
        for name, restype, argtypes in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = restype
            fn.argtypes = argtypes
        if path is None:
            _lib = lib
        return lib


def last_error(lib=None) -> str:
    lib = lib or load()
    buf = ctypes.create_string_buffer(1024)
    lib.tbg_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int, lib=None) -> None:
    if status != errors.TBG_OK:
        raise errors.error_for(status, last_error(lib))


def dptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags.c_contiguous
    return a.ctypes.data_as(_c_double_p)


def iptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags.c_contiguous and a.dtype == np.int64
    return a.ctypes.data_as(_c_int64_p)


def as_f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def as_c128_view(a) -> np.ndarray:
    """complex128 array as a contiguous float64 view (re, im interleaved)."""
    a = np.ascontiguousarray(np.asarray(a, dtype=np.complex128))
    return a.view(np.float64)


def kernel_timing(reset: bool = True, lib=None) -> dict:
    """{kernel family: (launches, total_ms, total_flops)} accumulated while timing is enabled."""
    lib = lib or load()
    n = 64
    names = ctypes.create_string_buffer(64 * n)
    launches = np.zeros(n, dtype=np.int64)
    ms = np.zeros(n, dtype=np.float64)
    work = np.zeros(n, dtype=np.float64)
    cnt = lib.tbg_kernel_timing_read(names, launches.ctypes.data_as(_c_int64_p), ms.ctypes.data_as(_c_double_p),
                                     work.ctypes.data_as(_c_double_p), n, int(reset))
    out = {}
    raw = names.raw
    for i in range(cnt):
        name = raw[64 * i:64 * (i + 1)].split(b"\0", 1)[0].decode()
        out[name] = (int(launches[i]), float(ms[i]), float(work[i]))
    return out
