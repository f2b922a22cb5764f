"""Error classes mirroring Rustb's ``TbError`` variants on the k-mesh path.

The C-ABI returns an ``int`` status; :func:`raise_for_status` turns it into the
exception class that matches the Rust variant the reference raises at the same
point (``src/error.rs:83-185``).  Panics in the reference (``assert!`` on the
k-vector length in ``src/model_physics.rs:48-51``, LAPACK ``info != 0`` in
``src/ndarray_lapack.rs:446``) map to :class:`TbPanic`.
"""

from __future__ import annotations

# Status codes returned by every tbg_* entry point (include/tbgpu.h).
TBG_OK = 0
TBG_E_KVECTOR_LENGTH = 1
TBG_E_DIMENSION_MISMATCH = 2
TBG_E_INVALID_RESPONSE_PARAMETER = 3
TBG_E_SPIN_NOT_ALLOWED = 4
TBG_E_INVALID_KMESH = 5
TBG_E_LINALG = 6
TBG_E_INVALID_DIMENSION = 7
TBG_E_INVALID_MODEL = 8
TBG_E_INVALID_ARGUMENT = 9
TBG_E_INVALID_ENERGY_RANGE = 10
TBG_E_INVALID_DOS_PARAMETER = 11
TBG_E_FILE_PARSE = 12
TBG_E_FILE_OPEN = 13
TBG_E_CUDA = 20
TBG_E_NOCONV = 21
TBG_E_TIMEOUT = 22
TBG_E_OOM = 23
TBG_E_UNSUPPORTED = 24


class TbError(Exception):
    """Base class; ``code`` is the C-ABI status."""

    code = -1

    def __init__(self, message: str = ""):
        super().__init__(message)
        self.message = message


class KVectorLengthMismatch(TbError):
    """``TbError::KVectorLengthMismatch`` (error.rs; traits.rs:65-70)."""

    code = TBG_E_KVECTOR_LENGTH


class DimensionMismatch(TbError):
    """``TbError::DimensionMismatch`` (config.rs:207-219, traits.rs:109-115)."""

    code = TBG_E_DIMENSION_MISMATCH


class InvalidResponseParameter(TbError):
    """``TbError::InvalidResponseParameter`` (config.rs:183-303)."""

    code = TBG_E_INVALID_RESPONSE_PARAMETER


class SpinNotAllowed(TbError):
    """``TbError::SpinNotAllowed`` (traits.rs:73-75, linear/mod.rs:163-165)."""

    code = TBG_E_SPIN_NOT_ALLOWED


class InvalidKmeshDimensions(TbError):
    """``TbError::InvalidKmeshDimensions`` (config.rs:251-255, kpoints.rs:40-46)."""

    code = TBG_E_INVALID_KMESH


class Linalg(TbError):
    """``TbError::Linalg`` (singular lattice in ``det``, eigh failure)."""

    code = TBG_E_LINALG


class InvalidDimension(TbError):
    """``TbError::InvalidDimension`` (config.rs:246-250)."""

    code = TBG_E_INVALID_DIMENSION


class InvalidModel(TbError):
    """``TbError::InvalidModelInvariant`` / ``MissingHermitianConjugateHopping``."""

    code = TBG_E_INVALID_MODEL


class InvalidEnergyRange(TbError):
    """``TbError::InvalidEnergyRange`` (model_physics.rs:187-192)."""

    code = TBG_E_INVALID_ENERGY_RANGE


class InvalidDosParameter(TbError):
    """``TbError::InvalidDosParameter`` (model_physics.rs:193-204)."""

    code = TBG_E_INVALID_DOS_PARAMETER


class FileParse(TbError):
    """``TbError::FileParse`` (error.rs:63-64): malformed Wannier90 input."""

    code = TBG_E_FILE_PARSE


class FileCreation(TbError):
    """``TbError::FileCreation`` (error.rs:78-79): an input file cannot be opened."""

    code = TBG_E_FILE_OPEN


class InvalidOrbitalProjection(TbError):
    """``TbError::InvalidOrbitalProjection`` (error.rs:66-67), raised by the host .win parser."""


class Other(TbError):
    """``TbError::Other`` (e.g. the Wannier90 spin mismatch, wannier90.rs:538-544)."""


class TbPanic(TbError):
    """A condition on which the reference panics (assert!/todo!)."""

    code = TBG_E_INVALID_ARGUMENT


class DeviceError(TbError):
    """CUDA failure, non-convergence, timeout or allocation failure."""

    code = TBG_E_CUDA


_BY_CODE = {
    TBG_E_KVECTOR_LENGTH: KVectorLengthMismatch,
    TBG_E_DIMENSION_MISMATCH: DimensionMismatch,
    TBG_E_INVALID_RESPONSE_PARAMETER: InvalidResponseParameter,
    TBG_E_SPIN_NOT_ALLOWED: SpinNotAllowed,
    TBG_E_INVALID_KMESH: InvalidKmeshDimensions,
    TBG_E_LINALG: Linalg,
    TBG_E_INVALID_DIMENSION: InvalidDimension,
    TBG_E_INVALID_MODEL: InvalidModel,
    TBG_E_INVALID_ARGUMENT: TbPanic,
    TBG_E_INVALID_ENERGY_RANGE: InvalidEnergyRange,
    TBG_E_INVALID_DOS_PARAMETER: InvalidDosParameter,
    TBG_E_FILE_PARSE: FileParse,
    TBG_E_FILE_OPEN: FileCreation,
    TBG_E_CUDA: DeviceError,
    TBG_E_NOCONV: DeviceError,
    TBG_E_TIMEOUT: DeviceError,
    TBG_E_OOM: DeviceError,
    TBG_E_UNSUPPORTED: TbPanic,
}


def error_for(code: int, message: str) -> TbError:
    cls = _BY_CODE.get(code, DeviceError)
    err = cls(message)
    err.code = code
    return err


def raise_for_status(code: int, message: str) -> None:
    if code != TBG_OK:
        raise error_for(code, message)
