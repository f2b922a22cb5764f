"""Seeded synthetic models for the k-mesh workloads.

* :func:`haldane_200` -- Haldane model ``Model<false,2>`` (lattice rows
  [sqrt3,-1], [sqrt3,1]; orbitals (0,0), (1/3,1/3); NN t1 = -1 on R = (0,0),
  (-1,0), (0,-1); NNN 0.15 i on the A-sublattice triple (1,0), (-1,1), (0,-1)
  and the B-sublattice triple (-1,0), (1,-1), (0,1); onsite +0.2/-0.2), built
  with ``add_hop`` exactly as Rustb's tests build it (src/lib.rs:902-925).
* :func:`random_spinful_3d` -- random 3D spinful model: cubic lattice, 64
  orbitals at uniform fractional positions, all R with |R_i| <= 3 (343
  vectors), spatial block (N(0,1)+iN(0,1))/sqrt2 * exp(-|R|/1.2)/sqrt(64), and
  sigma_x/y/z spin-orbit blocks of relative amplitude 0.1, placed with Rustb's
  Pauli conventions (model_build.rs:43-71).  numpy ``default_rng(20260101)``.
* :func:`random_model` -- the same statistics for any (dim, norb, spin, rmax);
  the batched uneven workload draws its models from it.
* :func:`supercell_2d` -- 1024-orbital square supercell, R in {-1,0,1}^2,
  t_ij(R) = exp(-d_ij/0.8) (N(0,1)+iN(0,1))/sqrt2, onsite U(-0.5, 0.5).
* :func:`honeycomb_small` -- the two-band honeycomb model Rustb's benchmarks
  use for ``dos`` (benches/bench_main.rs:15-25): lattice [1,0],[1/2,sqrt3/2],
  orbitals (1/3,1/3),(2/3,2/3), onsite -0.7/+0.7, t = -1 on R = (0,0),(-1,0),(0,-1).

Hopping tables are stored the way ``add_hop`` stores them: R = 0 first, then
each R immediately followed by -R with H(-R) = H(R)^dagger.
"""

from __future__ import annotations

import itertools
import math

import numpy as np

from .model import Model

SEED_SPINFUL_3D = 20260101


def honeycomb_small() -> Model:
    s3 = math.sqrt(3.0)
    model = Model.tb_model([[1.0, 0.0], [0.5, s3 / 2.0]], [[1.0 / 3.0, 1.0 / 3.0], [2.0 / 3.0, 2.0 / 3.0]],
                           spin=False)
    model.set_onsite([-0.7, 0.7])
    for R in [(0, 0), (-1, 0), (0, -1)]:
        model.add_hop(-1.0, 0, 1, R)
    return model


def haldane_200(t1=-1.0, t2=0.15, m=0.2) -> Model:
    s3 = math.sqrt(3.0)
    model = Model.tb_model([[s3, -1.0], [s3, 1.0]], [[0.0, 0.0], [1.0 / 3.0, 1.0 / 3.0]], spin=False)
    model.set_onsite([m, -m])
    for R in [(0, 0), (-1, 0), (0, -1)]:
        model.add_hop(t1, 0, 1, R)
    for R in [(1, 0), (-1, 1), (0, -1)]:
        model.add_hop(t2 * 1j, 0, 0, R)
    for R in [(-1, 0), (1, -1), (0, 1)]:
        model.add_hop(t2 * 1j, 1, 1, R)
    return model


def _half_vectors(dim: int, rmax: int):
    """R != 0 in the box |R_i| <= rmax whose first non-zero component is > 0."""
    out = []
    for R in itertools.product(range(-rmax, rmax + 1), repeat=dim):
        nz = [c for c in R if c != 0]
        if nz and nz[0] > 0:
            out.append(R)
    return out


def _cn(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / math.sqrt(2.0)


def random_model(dim: int, norb: int, spin: bool, rmax: int, seed: int, decay: float = 1.2,
                 soc: float = 0.1) -> Model:
    """Random Hermitian-closed model with cfg2 hopping statistics."""
    rng = np.random.default_rng(seed)
    lat = np.eye(dim)
    orb = rng.uniform(0.0, 1.0, (norb, dim))
    nsta = 2 * norb if spin else norb
    half = _half_vectors(dim, rmax)
    nR = 1 + 2 * len(half)
    ham = np.empty((nR, nsta, nsta), dtype=np.complex128)
    hamR = np.zeros((nR, dim), dtype=np.int64)
    norm = 1.0 / math.sqrt(norb)

    def block(R, hermitise: bool):
        amp = math.exp(-math.sqrt(sum(c * c for c in R)) / decay) * norm
        a0 = amp * _cn(rng, (norb, norb))
        if hermitise:
            a0 = 0.5 * (a0 + a0.conj().T)
        if not spin:
            return a0
        ax, ay, az = (soc * amp * _cn(rng, (norb, norb)) for _ in range(3))
        if hermitise:
            ax, ay, az = (0.5 * (a + a.conj().T) for a in (ax, ay, az))
        # sigma_0 a0 + sigma_x ax + sigma_y ay + sigma_z az with Rustb's
        # decoration: X -> [i+N,j], [i,j+N]; Y -> +i t at [i+N,j], -i t at [i,j+N].
        return np.block([[a0 + az, ax - 1j * ay], [ax + 1j * ay, a0 - az]])

    ham[0] = block((0,) * dim, True)
    for idx, R in enumerate(half):
        b = block(R, False)
        ham[1 + 2 * idx] = b
        ham[2 + 2 * idx] = b.conj().T
        hamR[1 + 2 * idx] = R
        hamR[2 + 2 * idx] = [-c for c in R]
    return Model(lat, orb, spin, ham=ham, hamR=hamR)


def random_spinful_3d(seed: int = SEED_SPINFUL_3D, norb: int = 64, rmax: int = 3) -> Model:
    return random_model(3, norb, True, rmax, seed)


def supercell_2d(norb: int = 1024, seed: int = 20260104, decay: float = 0.8) -> Model:
    """Large 2D supercell-like model with distance-decaying random hoppings."""
    rng = np.random.default_rng(seed)
    lat = np.eye(2)
    orb = rng.uniform(0.0, 1.0, (norb, 2))
    half = _half_vectors(2, 1)
    nR = 1 + 2 * len(half)
    ham = np.empty((nR, norb, norb), dtype=np.complex128)
    hamR = np.zeros((nR, 2), dtype=np.int64)

    def block(R):
        d = orb[None, :, :] + np.asarray(R, dtype=np.float64)[None, None, :] - orb[:, None, :]
        dist = np.sqrt((d * d).sum(-1))
        return np.exp(-dist / decay) * _cn(rng, (norb, norb))

    b0 = block((0, 0))
    b0 = 0.5 * (b0 + b0.conj().T)
    np.fill_diagonal(b0, rng.uniform(-0.5, 0.5, norb))
    ham[0] = b0
    for idx, R in enumerate(half):
        b = block(R)
        ham[1 + 2 * idx] = b
        ham[2 + 2 * idx] = b.conj().T
        hamR[1 + 2 * idx] = R
        hamR[2 + 2 * idx] = [-c for c in R]
    return Model(lat, orb, False, ham=ham, hamR=hamR)


def batched_uneven_specs(n_models: int = 512, seed: int = 20260103, mesh_scale: float = 1.0):
    """(dim, norb, kmesh, seed) for the batched uneven workload: half 2D square,
    half 3D cubic; norb log-uniform in [4, 256]; 2D meshes uniform in
    32^2..128^2, 3D in 16^3..48^3 (scaled by ``mesh_scale``)."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n_models):
        dim = 2 if i < n_models // 2 else 3
        norb = int(round(math.exp(rng.uniform(math.log(4), math.log(256)))))
        if dim == 2:
            n = int(rng.integers(32, 129))
        else:
            n = int(rng.integers(16, 49))
        n = max(1, int(round(n * mesh_scale)))
        specs.append((dim, norb, (n,) * dim, int(rng.integers(1 << 31))))
    return specs
