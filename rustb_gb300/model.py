"""``Model`` -- host-side mirror of Rustb's ``Model<SPIN, DIM, R>``.

Model construction (``tb_model``, ``set_hop``, ``add_hop``, ``set_onsite``,
``add_onsite``, ``del_hop``) follows ``src/model_build.rs`` on the host: the
R = 0 block sits at index 0 (model_build.rs:244-245), every hopping also
stores its Hermitian partner at -R (model_build.rs:430-440, 546-556), and the
spin decoration follows ``update_hamiltonian!`` / ``add_hamiltonian!``
(model_build.rs:43-118: sigma_y writes +i t to [i+N, j] and -i t to [i, j+N]).

The k-mesh methods (``gen_ham``, ``gen_v``, ``gen_v_projected``, the ``Solve``
family, the ``BerryCurvature`` family, ``hall_conductivity``, the
``QuantumGeometry`` family and ``dos``) run on the GPU through ``libtbgpu.so``; the model's arrays are uploaded once and kept
resident until the model is modified.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib, errors
from .params import (Gauge, HallConductivityResult, BandBerryCurvature, BandQuantumGeometry, Integration,
                     Parameters, Precision, QuantumGeometryMap, QuantumGeometryResult, SpinDirection,
                     spin_code, validate_broadening,
                     validate_chemical_potentials, validate_direction_matrix, validate_temperature)


class Model:
    def __init__(self, lat, orb, spin: bool, ham=None, hamR=None):
        self.lat = np.ascontiguousarray(np.asarray(lat, dtype=np.float64))
        self.orb = np.ascontiguousarray(np.atleast_2d(np.asarray(orb, dtype=np.float64)))
        self.spin = bool(spin)
        dim = self.lat.shape[1]
        if ham is None:
            ham = np.zeros((1, self.nsta, self.nsta), dtype=np.complex128)
            hamR = np.zeros((1, dim), dtype=np.int64)
        self.ham = np.ascontiguousarray(np.asarray(ham, dtype=np.complex128))
        self.hamR = np.ascontiguousarray(np.asarray(hamR, dtype=np.int64))
        self.rmatrix = None
        self._handle = None

    # ---------------------------------------------------------------- shape
    @property
    def dim(self) -> int:
        return self.lat.shape[1]

    def dim_r(self) -> int:
        return self.dim

    @property
    def norb(self) -> int:
        return self.orb.shape[0]

    @property
    def nsta(self) -> int:
        """``nsta`` (src/model.rs:701-707)."""
        return 2 * self.norb if self.spin else self.norb

    @property
    def nR(self) -> int:
        return self.hamR.shape[0]

    # ------------------------------------------------------------ building
    @classmethod
    def tb_model(cls, lat, orb, spin: bool = False):
        """``tb_model`` (src/model_build.rs:212-257)."""
        lat = np.asarray(lat, dtype=np.float64)
        orb = np.atleast_2d(np.asarray(orb, dtype=np.float64))
        if lat.ndim != 2 or lat.shape[0] != lat.shape[1]:
            raise errors.InvalidModel("lattice_shape: lattice must be square (DIM x DIM)")
        if orb.shape[1] != lat.shape[1]:
            raise errors.InvalidModel(f"orbital_position_shape: expected {lat.shape[1]} columns, found {orb.shape[1]}")
        if orb.shape[0] == 0:
            raise errors.InvalidModel("model has no orbitals")
        if not (np.all(np.isfinite(lat)) and np.all(np.isfinite(orb))):
            raise errors.InvalidModel("finite_geometry: lattice and orbital positions must be finite")
        return cls(lat, orb, spin)

    def _find_R(self, R) -> int | None:
        """``find_R`` (src/model_utils.rs:17-34)."""
        hits = np.nonzero(np.all(self.hamR == np.asarray(R, dtype=np.int64)[None, :], axis=1))[0]
        return int(hits[0]) if len(hits) else None

    def _decorate(self, block, tmp, i, j, pauli, accumulate: bool):
        """``update_hamiltonian!`` / ``add_hamiltonian!`` (model_build.rs:43-118)."""
        n = self.norb
        if self.spin:
            if pauli is None:
                entries = [((i, j), tmp), ((i + n, j + n), tmp)]
            elif pauli == SpinDirection.X:
                entries = [((i + n, j), tmp), ((i, j + n), tmp)]
            elif pauli == SpinDirection.Y:
                entries = [((i + n, j), tmp * 1j), ((i, j + n), -tmp * 1j)]
            else:
                entries = [((i, j), tmp), ((i + n, j + n), -tmp)]
        else:
            entries = [((i, j), tmp)]
        for (a, b), v in entries:
            if accumulate:
                block[a, b] += v
            else:
                block[a, b] = v

    def _hop(self, tmp, ind_i, ind_j, R, pauli, accumulate: bool):
        tmp = complex(tmp)
        R = np.asarray(R, dtype=np.int64).reshape(-1)
        if pauli is not None:
            pauli = SpinDirection(pauli)
        if len(R) != self.dim:
            raise errors.TbPanic("Wrong, the R length should equal to dim_r")
        if not (0 <= ind_i < self.norb and 0 <= ind_j < self.norb):
            raise errors.TbPanic("Wrong, ind_i and ind_j must be less than norb")
        if ind_i == ind_j and np.all(R == 0) and tmp.imag != 0.0:
            raise errors.TbPanic(f"Wrong, the onsite hopping must be real, but here is {tmp}")
        index = self._find_R(R)
        if index is not None:
            index_inv = self._find_R(-R)
            if index_inv is None:
                raise errors.TbPanic("Negative R not found in hamR")
            self._decorate(self.ham[index], tmp, ind_i, ind_j, pauli, accumulate)
            if index != 0 or ind_i != ind_j:
                self._decorate(self.ham[index_inv], tmp.conjugate(), ind_j, ind_i, pauli, accumulate)
        else:
            new = np.zeros((2, self.nsta, self.nsta), dtype=np.complex128)
            self._decorate(new[0], tmp, ind_i, ind_j, pauli, False)
            self._decorate(new[1], tmp.conjugate(), ind_j, ind_i, pauli, False)
            self.ham = np.ascontiguousarray(np.concatenate([self.ham, new], axis=0))
            self.hamR = np.ascontiguousarray(np.concatenate([self.hamR, R[None, :], -R[None, :]], axis=0))
        self._invalidate()

    def set_hop(self, tmp, ind_i, ind_j, R, pauli=None):
        """``set_hop`` (src/model_build.rs:354-455)."""
        self._hop(tmp, ind_i, ind_j, R, pauli, accumulate=False)

    def add_hop(self, tmp, ind_i, ind_j, R, pauli=None):
        """``add_hop`` (src/model_build.rs:477-558)."""
        self._hop(tmp, ind_i, ind_j, R, pauli, accumulate=True)

    def set_onsite(self, tmp, pauli=None):
        """``set_onsite`` (src/model_build.rs:689-700)."""
        tmp = np.asarray(tmp, dtype=np.float64)
        if len(tmp) != self.norb:
            raise errors.TbPanic(f"Wrong, the norb is {self.norb}, however, the onsite input's length is {len(tmp)}")
        for i, v in enumerate(tmp):
            self.set_hop(complex(v, 0.0), i, i, np.zeros(self.dim, dtype=np.int64), pauli)

    def add_onsite(self, tmp, pauli=None):
        """``add_onsite`` (src/model_build.rs:737-751)."""
        tmp = np.asarray(tmp, dtype=np.float64)
        if len(tmp) != self.norb:
            raise errors.TbPanic(f"Wrong, the norb is {self.norb}, however, the onsite input's length is {len(tmp)}")
        for i, v in enumerate(tmp):
            self.add_hop(complex(v, 0.0), i, i, np.zeros(self.dim, dtype=np.int64), pauli)

    def del_hop(self, ind_i, ind_j, R, pauli=None):
        """``del_hop``: set_hop with amplitude 0."""
        self.set_hop(0.0, ind_i, ind_j, R, pauli)

    def set_rmatrix(self, rmatrix):
        """Attach a position matrix (n_rmat, dim, nsta, nsta) (HasRMatrix)."""
        rm = np.ascontiguousarray(np.asarray(rmatrix, dtype=np.complex128))
        if rm.ndim != 4 or rm.shape[1] != self.dim or rm.shape[2:] != (self.nsta, self.nsta) or rm.shape[0] > self.nR:
            raise errors.InvalidModel("rmatrix must have shape (n_rmat <= nR, dim, nsta, nsta)")
        self.rmatrix = rm
        self._invalidate()

    # ---------------------------------------------------------- device side
    def _invalidate(self):
        if self._handle is not None:
            try:
                _lib.load().tbg_model_destroy(self._handle)
            finally:
                self._handle = None

    def __del__(self):
        try:
            self._invalidate()
        except Exception:
            pass

    def device_handle(self):
        """Upload the model (once) and return the opaque ``tbg_model*``."""
        if self._handle is None:
            lib = _lib.load()
            h = ctypes.c_void_p()
            hamR = np.ascontiguousarray(self.hamR, dtype=np.int64)
            ham = _lib.as_c128_view(self.ham)
            st = lib.tbg_model_create(self.dim, int(self.spin), self.norb, self.nR, _lib.iptr(hamR),
                                      _lib.dptr(ham), _lib.dptr(_lib.as_f64(self.orb)),
                                      _lib.dptr(_lib.as_f64(self.lat)), ctypes.byref(h))
            _lib.check(st, lib)
            if self.rmatrix is not None:
                rm = _lib.as_c128_view(self.rmatrix)
                st = lib.tbg_model_set_rmatrix(h, self.rmatrix.shape[0], _lib.dptr(rm))
                if st != errors.TBG_OK:
                    lib.tbg_model_destroy(h)
                    _lib.check(st, lib)
            self._handle = h
        return self._handle

    def _klist(self, k) -> np.ndarray:
        k = np.asarray(k, dtype=np.float64)
        if k.ndim == 1:
            k = k[None, :]
        if k.shape[1] != self.dim:
            raise errors.TbPanic(f"Wrong, the k-vector's length {k.shape[1]} must equal to the dimension of model {self.dim}.")
        return np.ascontiguousarray(k)

    # ------------------------------------------------ Hamiltonian, velocity
    def gen_ham_batch(self, k, gauge=Gauge.Atom) -> np.ndarray:
        k = self._klist(k)
        out = np.empty((k.shape[0], self.nsta, self.nsta), dtype=np.complex128)
        lib = _lib.load()
        _lib.check(lib.tbg_gen_ham(self.device_handle(), k.shape[0], _lib.dptr(k), int(gauge),
                                   _lib.dptr(out.view(np.float64))), lib)
        return out

    def gen_ham(self, kvec, gauge=Gauge.Atom) -> np.ndarray:
        """``gen_ham`` (src/model_physics.rs:43-148)."""
        return self.gen_ham_batch(np.asarray(kvec, dtype=np.float64).reshape(1, -1), gauge)[0]

    def gen_v_batch(self, k, gauge=Gauge.Atom):
        k = self._klist(k)
        nk = k.shape[0]
        V = np.empty((nk, self.dim, self.nsta, self.nsta), dtype=np.complex128)
        H = np.empty((nk, self.nsta, self.nsta), dtype=np.complex128)
        lib = _lib.load()
        _lib.check(lib.tbg_gen_v(self.device_handle(), nk, _lib.dptr(k), int(gauge),
                                 _lib.dptr(V.view(np.float64)), _lib.dptr(H.view(np.float64))), lib)
        return V, H

    def gen_v(self, kvec, gauge=Gauge.Atom):
        """``Velocity::gen_v`` (src/velocity.rs:236-441) -> (v (dim,N,N), H)."""
        V, H = self.gen_v_batch(np.asarray(kvec, dtype=np.float64).reshape(1, -1), gauge)
        return V[0], H[0]

    def gen_v_projected_batch(self, k, gauge, directions):
        k = self._klist(k)
        d = np.ascontiguousarray(np.atleast_2d(np.asarray(directions, dtype=np.float64)))
        if d.shape[1] != self.dim:
            raise errors.TbPanic(f"directions has {d.shape[1]} columns, expected dim_r={self.dim}")
        nk = k.shape[0]
        V = np.empty((nk, d.shape[0], self.nsta, self.nsta), dtype=np.complex128)
        H = np.empty((nk, self.nsta, self.nsta), dtype=np.complex128)
        lib = _lib.load()
        _lib.check(lib.tbg_gen_v_projected(self.device_handle(), nk, _lib.dptr(k), int(gauge), d.shape[0],
                                           _lib.dptr(d), _lib.dptr(V.view(np.float64)),
                                           _lib.dptr(H.view(np.float64))), lib)
        return V, H

    def gen_v_projected(self, kvec, gauge, directions):
        """``gen_v_projected`` (src/velocity.rs:470-731)."""
        V, H = self.gen_v_projected_batch(np.asarray(kvec, dtype=np.float64).reshape(1, -1), gauge, directions)
        return V[0], H[0]

    # ---------------------------------------------------------------- Solve
    def solve_band_all_parallel(self, kvec, precision: Precision = Precision.FP64) -> np.ndarray:
        """``solve_band_all_parallel`` (src/solve_ham.rs:94-107).  ``precision``
        (not in the reference) selects the mixed-precision band energies
        (FP32 eigensolve + FP64-class eigenvalue refinement, <= 1e-9 ||H||)."""
        k = self._klist(kvec)
        E = np.empty((k.shape[0], self.nsta))
        lib = _lib.load()
        if int(precision) == int(Precision.FP64):
            _lib.check(lib.tbg_solve_band(self.device_handle(), k.shape[0], _lib.dptr(k), _lib.dptr(E)), lib)
        else:
            _lib.check(lib.tbg_solve_band_prec(self.device_handle(), k.shape[0], _lib.dptr(k), int(precision),
                                               _lib.dptr(E)), lib)
        return E

    solve_band_all = solve_band_all_parallel

    def solve_band_onek(self, kvec) -> np.ndarray:
        """``solve_band_onek`` (src/solve_ham.rs:52-62)."""
        return self.solve_band_all_parallel(np.asarray(kvec, dtype=np.float64).reshape(1, -1))[0]

    def solve_all_parallel(self, kvec):
        """``solve_all_parallel`` (src/solve_ham.rs:168-184): eigenvectors as rows."""
        k = self._klist(kvec)
        nk = k.shape[0]
        E = np.empty((nk, self.nsta))
        U = np.empty((nk, self.nsta, self.nsta), dtype=np.complex128)
        lib = _lib.load()
        _lib.check(lib.tbg_solve(self.device_handle(), nk, _lib.dptr(k), _lib.dptr(E),
                                 _lib.dptr(U.view(np.float64)), 1), lib)
        return E, U

    solve_all = solve_all_parallel

    def solve_onek(self, kvec):
        """``solve_onek`` (src/solve_ham.rs:110-129)."""
        E, U = self.solve_all_parallel(np.asarray(kvec, dtype=np.float64).reshape(1, -1))
        return E[0], U[0]

    # -------------------------------------------------------- BerryCurvature
    def _check_berry_params(self, params: Parameters):
        validate_direction_matrix(params.direction, 2, self.dim)
        validate_broadening(params.eta)
        if not self.spin and params.spin is not None:
            raise errors.SpinNotAllowed(f"Spin direction '{params.spin!r}' is invalid for a model without spin.")

    def berry_curvature_on(self, k_list, params: Parameters, precision=Precision.FP64):
        """Band-resolved Berry curvature and energies at many k-points
        (``berry_curvature_at`` applied per k, traits.rs:60-78)."""
        k = self._klist(k_list)
        self._check_berry_params(params)
        nk = k.shape[0]
        Om = np.empty((nk, self.nsta))
        E = np.empty((nk, self.nsta))
        d = _lib.as_f64(params.direction)
        lib = _lib.load()
        _lib.check(lib.tbg_berry_curvature(self.device_handle(), nk, _lib.dptr(k), _lib.dptr(d),
                                           spin_code(params.spin), float(params.eta), int(precision),
                                           _lib.dptr(Om), _lib.dptr(E)), lib)
        return Om, E

    def berry_curvature_at(self, k, params: Parameters, precision=Precision.FP64) -> BandBerryCurvature:
        """``BerryCurvature::berry_curvature_at`` (src/response/traits.rs:60-78)."""
        k = np.asarray(k, dtype=np.float64).reshape(-1)
        if len(k) != self.dim:
            raise errors.KVectorLengthMismatch(f"expected {self.dim}, actual {len(k)}")
        Om, E = self.berry_curvature_on(k[None, :], params, precision)
        return BandBerryCurvature(berry_curvature=Om[0], energies=E[0])

    def occupied_berry_curvature_on(self, k_points, params: Parameters, precision=Precision.FP64) -> np.ndarray:
        """``occupied_berry_curvature_on`` (src/response/traits.rs:104-150)."""
        k = np.asarray(k_points, dtype=np.float64)
        if k.ndim != 2 or k.shape[1] != self.dim:
            raise errors.DimensionMismatch(
                f"Berry-curvature k-points: expected {self.dim}, got {k.shape[-1] if k.ndim else 0}")
        validate_chemical_potentials(params.mu)
        if len(params.mu) != 1:
            raise errors.InvalidResponseParameter("mu: occupied_berry_curvature_on expects a single chemical potential")
        validate_temperature(params.T)
        self._check_berry_params(params)
        k = np.ascontiguousarray(k)
        out = np.empty(k.shape[0])
        d = _lib.as_f64(params.direction)
        lib = _lib.load()
        _lib.check(lib.tbg_occupied_berry_curvature(
            self.device_handle(), k.shape[0], _lib.dptr(k), _lib.dptr(d), spin_code(params.spin),
            float(params.eta), float(params.T[0]), float(params.mu[0]), int(precision), _lib.dptr(out)), lib)
        return out

    def occupied_berry_curvature_at(self, k, params: Parameters, precision=Precision.FP64) -> float:
        """``occupied_berry_curvature_at`` (src/response/traits.rs:80-102)."""
        validate_chemical_potentials(params.mu)
        if len(params.mu) != 1:
            raise errors.InvalidResponseParameter("mu: occupied_berry_curvature_at expects a single chemical potential")
        k = np.asarray(k, dtype=np.float64).reshape(-1)
        if len(k) != self.dim:
            raise errors.KVectorLengthMismatch(f"expected {self.dim}, actual {len(k)}")
        return float(self.occupied_berry_curvature_on(k[None, :], params, precision)[0])

    # ------------------------------------------------------------------ Hall
    def hall_conductivity(self, params: Parameters, precision=Precision.FP64,
                          report: dict | None = None) -> HallConductivityResult:
        """``hall_conductivity`` (src/response/linear/mod.rs:160-268): Direct
        integration, or EnergyCut (band tracking + simplex occupancy cut, FP64;
        ``precision`` applies to Direct only); Simplex is rejected as in the
        reference (:166-176)."""
        params.validate_rank2(self.dim)
        if not self.spin and params.spin is not None:
            raise errors.SpinNotAllowed(f"Spin direction '{params.spin!r}' is invalid for a model without spin.")
        if params.integration == Integration.Simplex:
            raise errors.InvalidResponseParameter(
                "integration: hall_conductivity supports Integration::Direct or EnergyCut, not Simplex")
        kmesh = np.ascontiguousarray(np.asarray(params.kmesh, dtype=np.int64))
        mu = _lib.as_f64(params.mu)
        d = _lib.as_f64(params.direction)
        sigma = np.empty(len(mu))
        if params.integration == Integration.EnergyCut:
            # linear/mod.rs:177-185: sorted mu, dimension 2 or 3; FP64 path
            if np.any(np.diff(mu) < 0):
                raise errors.InvalidResponseParameter("mu: must be sorted in ascending order")
            if self.dim not in (2, 3):
                raise errors.InvalidDimension(f"dimension {self.dim} is not supported; supported: [2, 3]")
            lib = _lib.load()
            _lib.check(lib.tbg_hall_energy_cut(self.device_handle(), _lib.iptr(kmesh), _lib.dptr(d), len(mu),
                                               _lib.dptr(mu), float(params.T[0]), float(params.eta),
                                               spin_code(params.spin), _lib.dptr(sigma)), lib)
            return HallConductivityResult(chemical_potentials=params.mu.copy(), conductivity=sigma)
        rep = _lib.TbgReport()
        lib = _lib.load()
        _lib.check(lib.tbg_hall_conductivity(self.device_handle(), _lib.iptr(kmesh), _lib.dptr(d), len(mu),
                                             _lib.dptr(mu), float(params.T[0]), float(params.eta),
                                             spin_code(params.spin), int(precision), _lib.dptr(sigma),
                                             ctypes.byref(rep)), lib)
        if report is not None:
            report.update(rep.as_dict())
        return HallConductivityResult(chemical_potentials=params.mu.copy(), conductivity=sigma)

    # ------------------------------------------------------- QuantumGeometry
    def quantum_geometry_on(self, k_points, params: Parameters, precision=Precision.FP64) -> QuantumGeometryMap:
        """``QuantumGeometry::quantum_geometry_on`` (src/quantum_geometry.rs:104-138):
        band-resolved metric, Berry curvature and energies, each (nk, nsta)."""
        k = np.asarray(k_points, dtype=np.float64)
        if k.ndim != 2 or k.shape[1] != self.dim:
            raise errors.DimensionMismatch(
                f"quantum geometry k-points: expected {self.dim}, got {k.shape[-1] if k.ndim else 0}")
        validate_direction_matrix(params.direction, 2, self.dim)
        validate_broadening(params.eta)
        k = np.ascontiguousarray(k)
        nk = k.shape[0]
        g = np.empty((nk, self.nsta))
        om = np.empty((nk, self.nsta))
        E = np.empty((nk, self.nsta))
        d = _lib.as_f64(params.direction)
        lib = _lib.load()
        _lib.check(lib.tbg_quantum_geometry(self.device_handle(), nk, _lib.dptr(k), _lib.dptr(d),
                                            float(params.eta), int(precision), _lib.dptr(g), _lib.dptr(om),
                                            _lib.dptr(E)), lib)
        return QuantumGeometryMap(metric=g, berry_curvature=om, energies=E)

    def quantum_geometry_at(self, k, params: Parameters, precision=Precision.FP64) -> BandQuantumGeometry:
        """``QuantumGeometry::quantum_geometry_at`` (src/quantum_geometry.rs:88-102)."""
        k = np.asarray(k, dtype=np.float64).reshape(-1)
        if len(k) != self.dim:
            raise errors.KVectorLengthMismatch(f"expected {self.dim}, actual {len(k)}")
        r = self.quantum_geometry_on(k[None, :], params, precision)
        return BandQuantumGeometry(metric=r.metric[0], berry_curvature=r.berry_curvature[0], energies=r.energies[0])

    def quantum_geometry(self, params: Parameters, precision=Precision.FP64,
                         report: dict | None = None) -> QuantumGeometryResult:
        """``Model::quantum_geometry`` (src/quantum_geometry.rs:196-240), Direct
        integration; EnergyCut is rejected as in the reference, Simplex is not
        provided by the GPU library."""
        params.validate_rank2(self.dim)
        if params.integration == Integration.EnergyCut:
            raise errors.InvalidResponseParameter(
                "integration: quantum_geometry supports Integration::Direct or Simplex, not EnergyCut")
        if params.integration == Integration.Simplex:
            if self.dim == 1:
                raise errors.InvalidDimension(f"dimension {self.dim} is not supported; supported: [2, 3]")
            raise errors.TbPanic("Integration::Simplex is not provided by the GPU library")
        kmesh = np.ascontiguousarray(np.asarray(params.kmesh, dtype=np.int64))
        mu = _lib.as_f64(params.mu)
        d = _lib.as_f64(params.direction)
        g = np.empty(len(mu))
        om = np.empty(len(mu))
        rep = _lib.TbgReport()
        lib = _lib.load()
        _lib.check(lib.tbg_quantum_geometry_mesh(self.device_handle(), _lib.iptr(kmesh), _lib.dptr(d), len(mu),
                                                 _lib.dptr(mu), float(params.T[0]), float(params.eta),
                                                 int(precision), _lib.dptr(g), _lib.dptr(om), ctypes.byref(rep)),
                   lib)
        if report is not None:
            report.update(rep.as_dict())
        return QuantumGeometryResult(chemical_potentials=params.mu.copy(), metric=g, berry_curvature=om)

    # ------------------------------------------------------------------- DOS
    def dos(self, k_mesh, E_min: float, E_max: float, E_n: int, sigma: float):
        """``Model::dos`` (src/model_physics.rs:179-230): Gaussian-smeared
        density of states on the uniform mesh; returns ``(energies, dos)``."""
        E_min = float(E_min)
        E_max = float(E_max)
        sigma = float(sigma)
        if E_min >= E_max:
            raise errors.InvalidEnergyRange(f"Invalid energy range: min={E_min}, max={E_max}")
        if int(E_n) <= 0:
            raise errors.InvalidDosParameter("E_n: number of energy bins must be at least 1")
        if not np.isfinite(sigma) or sigma <= 0.0:
            raise errors.InvalidDosParameter("sigma: Gaussian smearing width must be finite and positive")
        kmesh = np.ascontiguousarray(np.asarray(k_mesh, dtype=np.int64).reshape(-1))
        if kmesh.size == 0 or np.any(kmesh <= 0):
            raise errors.InvalidKmeshDimensions(f"Invalid k-point mesh dimensions: {kmesh.tolist()}")
        if kmesh.size != self.dim:
            raise errors.TbPanic(f"k-mesh has {kmesh.size} entries, the model has dimension {self.dim}")
        E = np.empty(int(E_n))
        out = np.empty(int(E_n))
        lib = _lib.load()
        _lib.check(lib.tbg_dos(self.device_handle(), _lib.iptr(kmesh), E_min, E_max, int(E_n), sigma,
                               _lib.dptr(E), _lib.dptr(out)), lib)
        return E, out

    # ----------------------------------------------------------- band meshes
    def solve_band_mesh(self, k_mesh) -> np.ndarray:
        """``solve_band_all_parallel(&gen_kmesh(k_mesh))`` (src/solve_ham.rs:94-107,
        src/kpoints.rs:49-87) in one device call: energies (nk, nsta)."""
        from . import fermi

        return fermi.bands_mesh(self, k_mesh)

    def write_bxsf(self, k_mesh, e_fermi: float, filename: str) -> str:
        """``BxsfExport::write_bxsf`` (src/fermi_surface.rs:454-546)."""
        from . import fermi

        return fermi.write_bxsf(self, k_mesh, e_fermi, filename)

    def rec_lat(self) -> np.ndarray:
        """``Model::rec_lat`` (src/model.rs:679-687)."""
        from . import fermi

        return fermi.rec_lat(self.lat)

    # ------------------------------------------------------------- Wannier90
    @classmethod
    def from_hr(cls, path: str, file_name: str, zero_energy: float = 0.0, spin: bool | None = None,
                with_rmatrix: bool = False) -> "Model":
        """``Wannier90::from_hr`` (src/wannier90.rs:49-1203); see ``rustb_gb300.wannier90``."""
        from . import wannier90

        return wannier90.from_hr(path, file_name, zero_energy, spin, with_rmatrix)

    @classmethod
    def from_hr_with_rmatrix(cls, path: str, file_name: str, zero_energy: float = 0.0,
                             spin: bool | None = None) -> "Model":
        """``Model::from_hr_with_rmatrix`` (src/wannier90.rs:1208-1219)."""
        from . import wannier90

        return wannier90.from_hr_with_rmatrix(path, file_name, zero_energy, spin)

    def natom(self) -> int:
        """Number of atoms (set by the Wannier90 loader; 0 for hand-built models)."""
        return len(getattr(self, "atoms", []) or [])

    # ----------------------------------------------------------- Wilson loops
    def _wilson(self, kvec3: np.ndarray, occ, mode: int, precision=Precision.FP64) -> np.ndarray:
        kv = np.ascontiguousarray(np.asarray(kvec3, dtype=np.float64))
        n_loops, n_k = kv.shape[0], kv.shape[1]
        occ_a = np.ascontiguousarray(np.asarray(list(occ), dtype=np.int64).reshape(-1))
        out = np.empty((n_loops, occ_a.size) if mode == 0 else (n_loops,))
        lib = _lib.load()
        _lib.check(lib.tbg_wilson_loops(self.device_handle(), n_loops, n_k, _lib.dptr(kv), occ_a.size,
                                        _lib.iptr(occ_a) if occ_a.size else None, int(mode), int(precision),
                                        _lib.dptr(out)), lib)
        return out

    def _check_loop(self, kvec):
        k = np.asarray(kvec, dtype=np.float64)
        if k.ndim != 2 or k.shape[1] != self.dim or k.shape[0] < 1:
            raise errors.TbPanic(f"k-loop must have shape (n_k, {self.dim})")
        return k

    def berry_loop(self, kvec, occ, precision=Precision.FP64) -> np.ndarray:
        """``Berry::berry_loop`` (src/geometry.rs:156-215): -arg of the eigenvalues
        of the product of the unitary parts of the overlap matrices along the
        closed loop ``kvec`` (n_k, dim); ascending (the reference's order is
        LAPACK zgeev's)."""
        k = self._check_loop(kvec)
        return self._wilson(k[None], occ, 0, precision)[0]

    def berry_loop_det(self, kvec, occ, precision=Precision.FP64) -> float:
        """``Berry::berry_loop_det`` (src/geometry.rs:217-270)."""
        k = self._check_loop(kvec)
        return float(self._wilson(k[None], occ, 1, precision)[0])

    def berry_flux(self, occ, k_start, dir_1, dir_2, nk1: int, nk2: int, precision=Precision.FP64) -> np.ndarray:
        """``Berry::berry_flux`` (src/geometry.rs:272-339): Wilson loop around
        every plaquette of the (nk1, nk2) mesh spanned by dir_1, dir_2 from
        k_start; (nk1, nk2, n_occ), each plaquette's phases ascending."""
        ks, d1, d2 = (np.asarray(v, dtype=np.float64).reshape(-1) for v in (k_start, dir_1, dir_2))
        for name, v in (("k_start", ks), ("dir_1", d1), ("dir_2", d2)):
            if v.size != self.dim:
                raise errors.TbPanic(f"Wrong!, the {name}'s length is {v.size} but dim_r is {self.dim}, it's not equal!")
        if nk1 < 1 or nk2 < 1:
            raise errors.TbPanic(f"Wrong!, nk1 and nk2 must be at least 1, but nk1={nk1} and nk2={nk2}")
        # element-wise the same operations in the same order as geometry.rs:309-326
        dx, dy = 1.0 / nk1, 1.0 / nk2
        i0 = (np.arange(nk1, dtype=np.float64) / nk1)[:, None, None]
        j0 = (np.arange(nk2, dtype=np.float64) / nk2)[None, :, None]
        loops = np.empty((nk1, nk2, 5, self.dim))
        loops[:, :, 0] = ks + i0 * d1 + j0 * d2
        loops[:, :, 1] = ks + (i0 + dx) * d1 + j0 * d2
        loops[:, :, 2] = ks + (i0 + dx) * d1 + (j0 + dy) * d2
        loops[:, :, 3] = ks + i0 * d1 + (j0 + dy) * d2
        loops[:, :, 4] = ks + i0 * d1 + j0 * d2
        loops = loops.reshape(nk1 * nk2, 5, self.dim)
        occ = list(occ)
        return self._wilson(loops, occ, 0, precision).reshape(nk1, nk2, len(occ))

    def berry_phase(self, occ, kvec, precision=Precision.FP64) -> np.ndarray:
        """``Berry::berry_phase`` (src/geometry.rs:341-358): one loop per
        ``kvec[i]`` (nk1, nk2, dim); returns (n_occ, nk1), each column sorted."""
        kv = np.asarray(kvec, dtype=np.float64)
        return self._wilson(kv, occ, 0, precision).T.copy()

    def wannier_centre(self, occ, k_start, dir_1, dir_2, nk1: int, nk2: int, precision=Precision.FP64) -> np.ndarray:
        """``Berry::wannier_centre`` (src/geometry.rs:360-420): loops along dir_2
        at nk1 positions along dir_1 (both ends included); (n_occ, nk1)."""
        ks, d1, d2 = (np.asarray(v, dtype=np.float64).reshape(-1) for v in (k_start, dir_1, dir_2))
        for name, v in (("k_start", ks), ("dir_1", d1), ("dir_2", d2)):
            if v.size != self.dim:
                raise errors.TbPanic(f"Wrong!, the {name}'s length is {v.size} but dim_r is {self.dim}, it's not equal!")
        if nk1 < 2 or nk2 < 2:
            raise errors.TbPanic(f"Wrong!, nk1 and nk2 must be at least 2 for a finite-difference k-mesh, but "
                                 f"nk1={nk1} and nk2={nk2}")
        # element-wise as geometry.rs:398-403: k_start + dir_1 * i / (nk1 - 1) + dir_2 * j / (nk2 - 1)
        fi = np.arange(nk1, dtype=np.float64)[:, None, None]
        fj = np.arange(nk2, dtype=np.float64)[None, :, None]
        kv = ks + d1 * fi / float(nk1 - 1) + d2 * fj / float(nk2 - 1)
        return self._wilson(kv, occ, 0, precision).T.copy()
