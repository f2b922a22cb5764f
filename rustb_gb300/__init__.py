"""rustb_gb300 -- GB300 (sm_103a) k-mesh engine for Rustb tight-binding models.

The device work (Fourier sum, batched Hermitian eigensolve, velocity rotation,
Berry curvature and the Hall k-sum, quantum geometry and the density of
states) runs in ``_build/libtbgpu.so`` behind the
C-ABI of ``include/tbgpu.h``; this package is the host-side mirror of Rustb's
``Model`` / ``Parameters`` interface over that library.
"""

from .errors import TbError
from .fermi import write_spin_frmsf
from .model import Model
from .params import (BandBerryCurvature, BandQuantumGeometry, Gauge, HallConductivityResult, Integration,
                     Parameters, Precision, QuantumGeometryMap, QuantumGeometryResult, SpinDirection)

__all__ = ["Model", "Parameters", "Gauge", "SpinDirection", "Integration", "Precision",
           "BandBerryCurvature", "HallConductivityResult", "BandQuantumGeometry", "QuantumGeometryMap",
           "QuantumGeometryResult", "TbError", "write_spin_frmsf"]
__version__ = "0.1.0"
