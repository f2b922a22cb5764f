"""Build recipe and ctypes wrapper for the C oracle port (oracle/cpu_port.c).

TEST INFRASTRUCTURE / CPU BASELINE ONLY.  The port dlopens the OpenBLAS that
scipy bundles (``scipy.libs/libscipy_openblas-*.so``) for zaxpy, zheev and
zgemm.  Built with gcc -O3 -fopenmp into oracle/_build/.
"""

from __future__ import annotations

import ctypes
import glob
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libtbport.so")


def scipy_openblas() -> str:
    import scipy

    base = os.path.dirname(scipy.__file__)
    cands = sorted(glob.glob(os.path.join(base + ".libs", "libscipy_openblas*.so*")))
    cands += sorted(glob.glob(os.path.join(base, ".dylibs", "libscipy_openblas*")))
    if not cands:
        raise FileNotFoundError("scipy's bundled OpenBLAS not found")
    return cands[0]


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    cmd = ["gcc", "-O3", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", os.path.join(HERE, "cpu_port.c"), "-o", LIB, "-ldl", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"gcc failed:\n{r.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


_port = None


def load():
    global _port
    if _port is None:
        if not os.path.exists(LIB):
            build()
        lib = ctypes.CDLL(LIB)
        lib.port_init.argtypes = [ctypes.c_char_p]
        lib.port_init.restype = ctypes.c_int
        rc = lib.port_init(scipy_openblas().encode())
        if rc != 0:
            raise RuntimeError(f"port_init failed ({rc})")
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int64)
        lib.port_hall_sums.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, ip, dp, dp, ip,
                                       ctypes.c_int64, ctypes.c_int64, dp, dp, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_int, dp, ctypes.c_double, ctypes.c_int, dp, dp, dp]
        lib.port_hall_sums.restype = ctypes.c_int
        lib.port_dos.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, ip, dp, ip,
                                 ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_int, dp]
        lib.port_dos.restype = ctypes.c_int
        lib.port_read_hr.argtypes = [ctypes.c_char_p, ctypes.c_double, dp, ctypes.c_int64]
        lib.port_read_hr.restype = ctypes.c_int64
        _port = lib
    return _port


def _dp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def hall_sums(model, directions, mu, T=0.0, eta=1e-3, spin=-1, kmesh=None, k0=0, nk=None, klist=None,
              threads=None, want_bands=False):
    """Per-k occupation sums S (nk, nmu) (and optionally Omega, E) from the C port."""
    lib = load()
    mu = np.ascontiguousarray(np.atleast_1d(mu), dtype=np.float64)
    dirs = np.ascontiguousarray(directions, dtype=np.float64)
    ham = np.ascontiguousarray(model.ham).view(np.float64)
    hamR = np.ascontiguousarray(model.hamR, dtype=np.int64)
    orb = np.ascontiguousarray(model.orb, dtype=np.float64)
    lat = np.ascontiguousarray(model.lat, dtype=np.float64)
    if klist is not None:
        klist = np.ascontiguousarray(klist, dtype=np.float64)
        nk = klist.shape[0]
    km = np.ascontiguousarray(kmesh if kmesh is not None else [1, 1, 1], dtype=np.int64)
    S = np.empty((nk, len(mu)))
    Om = np.empty((nk, model.nsta)) if want_bands else None
    E = np.empty((nk, model.nsta)) if want_bands else None
    width = 0.0 if T <= 0 else T * 8.617333262145e-5
    threads = threads or os.cpu_count() or 1
    rc = lib.port_hall_sums(model.dim, int(model.spin), model.norb, model.nR, _dp(ham),
                            hamR.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), _dp(orb), _dp(lat),
                            km.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), int(k0), int(nk), _dp(klist),
                            _dp(dirs), int(spin), float(eta), len(mu), _dp(mu), float(width), int(threads),
                            _dp(S), _dp(Om), _dp(E))
    if rc != 0:
        raise RuntimeError(f"zheev info={rc}")
    return (S, Om, E) if want_bands else S


def dos_sums(model, kmesh, E_min, E_max, E_n, sigma, k0=0, nk=None, threads=None):
    """Unnormalised DOS sums (E_n) over mesh points [k0, k0 + nk) from the C port."""
    lib = load()
    ham = np.ascontiguousarray(model.ham).view(np.float64)
    hamR = np.ascontiguousarray(model.hamR, dtype=np.int64)
    orb = np.ascontiguousarray(model.orb, dtype=np.float64)
    km = np.ascontiguousarray(kmesh, dtype=np.int64)
    if nk is None:
        nk = int(np.prod(km))
    acc = np.zeros(int(E_n))
    threads = threads or os.cpu_count() or 1
    rc = lib.port_dos(model.dim, int(model.spin), model.norb, model.nR, _dp(ham),
                      hamR.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), _dp(orb),
                      km.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), int(k0), int(nk), int(E_n),
                      float(E_min), float(E_max), float(sigma), int(threads), _dp(acc))
    if rc != 0:
        raise RuntimeError(f"zheev info={rc}")
    return acc


def read_hr(path, nvalues):
    """The reference's line-by-line _hr.dat reading on one thread (timing baseline)."""
    lib = load()
    out = np.empty(2 * int(nvalues))
    n = lib.port_read_hr(path.encode(), 0.0, _dp(out), out.size)
    if n < 0:
        raise RuntimeError("malformed _hr.dat")
    return out[: 2 * n].view(np.complex128)
