"""Host-side mirror of Rustb's response-parameter types.

``Parameters`` follows ``src/response/config.rs:41-102`` (field names, the
``eta = 1e-3`` default, ``rank2``), and the validators follow
``config.rs:141-147, 183-303`` so that invalid input raises the same error
class before anything reaches the device.  ``Gauge`` / ``SpinDirection``
follow ``src/model.rs:449-474``; ``Integration`` follows ``config.rs:14-28``.
"""

from __future__ import annotations

import enum
import math
from dataclasses import dataclass, field

import numpy as np

from . import errors

BOLTZMANN_CONSTANT_EV_PER_K = 8.617333262145e-5  # thermodynamics.rs:10


class Gauge(enum.IntEnum):
    """``Gauge::Lattice`` / ``Gauge::Atom`` (model.rs:449-452)."""

    Lattice = 0
    Atom = 1


class SpinDirection(enum.IntEnum):
    """``SpinDirection::{X,Y,Z}`` (model.rs:470-474)."""

    X = 0
    Y = 1
    Z = 2


SPIN_NONE = -1  # C-ABI encoding of ``Option::<SpinDirection>::None``


class Integration(enum.IntEnum):
    Direct = 0
    EnergyCut = 1
    Simplex = 2


class Precision(enum.IntEnum):
    """Arithmetic of the device path: plain FP64, or the mixed path
    (FP32 eigensolve + FP64 refinement)."""

    FP64 = 0
    MIXED = 1


def spin_code(spin) -> int:
    return SPIN_NONE if spin is None else int(SpinDirection(spin))


@dataclass
class Parameters:
    """``Parameters<DIM>`` (config.rs:41-70)."""

    kmesh: tuple
    direction: np.ndarray
    mu: np.ndarray
    T: np.ndarray = field(default_factory=lambda: np.array([0.0]))
    eta: float = 1e-3
    omega: np.ndarray = field(default_factory=lambda: np.array([0.0]))
    spin: SpinDirection | None = None
    integration: Integration = Integration.Direct

    def __post_init__(self):
        self.kmesh = tuple(int(n) for n in self.kmesh)
        self.direction = np.atleast_2d(np.asarray(self.direction, dtype=np.float64))
        self.mu = np.atleast_1d(np.asarray(self.mu, dtype=np.float64))
        self.T = np.atleast_1d(np.asarray(self.T, dtype=np.float64))

    @property
    def dim(self) -> int:
        return len(self.kmesh)

    @classmethod
    def new(cls, kmesh, direction, mu):
        """``Parameters::new`` (config.rs:75-87): T=0, eta=1e-3, Direct."""
        return cls(kmesh=kmesh, direction=direction, mu=mu)

    @classmethod
    def at_mu(cls, kmesh, direction, mu: float):
        return cls(kmesh=kmesh, direction=direction, mu=np.array([mu]))

    @classmethod
    def rank2(cls, kmesh, direction_a, direction_b, mu):
        """``Parameters::rank2`` (config.rs:95-102)."""
        return cls(kmesh=kmesh, direction=np.array([direction_a, direction_b], dtype=np.float64), mu=mu)

    def with_temperature(self, kelvin: float):
        self.T = np.array([kelvin], dtype=np.float64)
        return self

    def with_spin(self, spin: SpinDirection):
        self.spin = SpinDirection(spin)
        return self

    def with_integration(self, integration: Integration):
        self.integration = Integration(integration)
        return self

    def validate_rank2(self, dim: int) -> None:
        """``validate_rank2`` (config.rs:141-147)."""
        validate_k_mesh(self.kmesh, dim)
        validate_direction_matrix(self.direction, 2, dim)
        validate_chemical_potentials(self.mu)
        validate_broadening(self.eta)
        validate_temperature(self.T)

    def occupation_width(self) -> float:
        """``parameters_occupation`` (config.rs:173-181) reduced to the energy
        width the Fermi function uses (thermodynamics.rs:86-95)."""
        t0 = float(self.T[0])
        return 0.0 if t0 <= 0.0 else t0 * BOLTZMANN_CONSTANT_EV_PER_K


def validate_k_mesh(kmesh, dim: int) -> None:
    if not 1 <= dim <= 3:
        raise errors.InvalidDimension(f"dim {dim} not in [1, 2, 3]")
    if len(kmesh) != dim:
        raise errors.DimensionMismatch(f"kmesh: expected {dim}, found {len(kmesh)}")
    if any(int(n) == 0 for n in kmesh) or any(int(n) < 0 for n in kmesh):
        raise errors.InvalidKmeshDimensions(f"invalid k-mesh {list(kmesh)}")


def validate_direction_matrix(direction: np.ndarray, rank: int, dim: int) -> None:
    """``validate_direction_matrix`` (config.rs:202-233)."""
    direction = np.atleast_2d(np.asarray(direction, dtype=np.float64))
    if direction.shape[0] != rank:
        raise errors.DimensionMismatch(f"direction: expected {rank}, found {direction.shape[0]}")
    if direction.shape[1] != dim:
        raise errors.DimensionMismatch(f"direction: expected {dim}, found {direction.shape[1]}")
    for row in direction:
        if not np.all(np.isfinite(row)):
            raise errors.InvalidResponseParameter("direction: all components must be finite")
        if np.all(row == 0.0):
            raise errors.InvalidResponseParameter("direction: each direction row must not be the zero vector")


def validate_broadening(eta: float) -> None:
    if not math.isfinite(eta) or eta < 0.0:
        raise errors.InvalidResponseParameter("broadening: must be finite and non-negative")


def validate_chemical_potentials(mu: np.ndarray) -> None:
    if len(mu) == 0:
        raise errors.InvalidResponseParameter("chemical_potentials: must contain at least one value")
    if not np.all(np.isfinite(mu)):
        raise errors.InvalidResponseParameter("chemical_potentials: all values must be finite")


def validate_temperature(T: np.ndarray) -> None:
    if len(T) == 0:
        raise errors.InvalidResponseParameter("T: must contain at least one value")
    if not np.all(np.isfinite(T)) or np.any(T < 0.0):
        raise errors.InvalidResponseParameter("T: all values must be finite and non-negative")


@dataclass
class BandBerryCurvature:
    """``BandBerryCurvature`` (traits.rs:20-27)."""

    berry_curvature: np.ndarray
    energies: np.ndarray


@dataclass
class HallConductivityResult:
    """``HallConductivityResult`` (linear/mod.rs:51-63)."""

    chemical_potentials: np.ndarray
    conductivity: np.ndarray


@dataclass
class BandQuantumGeometry:
    """``BandQuantumGeometry`` (src/quantum_geometry.rs:30-39)."""

    metric: np.ndarray
    berry_curvature: np.ndarray
    energies: np.ndarray


@dataclass
class QuantumGeometryMap:
    """``QuantumGeometryMap`` (src/quantum_geometry.rs:41-50): each (nk, nsta)."""

    metric: np.ndarray
    berry_curvature: np.ndarray
    energies: np.ndarray


@dataclass
class QuantumGeometryResult:
    """``QuantumGeometryResult`` (src/quantum_geometry.rs:52-63); ``diagnostics``
    is set by Simplex integration only, which this library does not provide."""

    chemical_potentials: np.ndarray
    metric: np.ndarray
    berry_curvature: np.ndarray
    diagnostics: object = None
