"""Models used by Rustb's own tests (src/lib.rs), rebuilt with the host-side
``Model`` builder so that the same known answers can be checked here."""

import math

import numpy as np

from rustb_gb300.model import Model
from rustb_gb300.params import SpinDirection

S3 = math.sqrt(3.0)
HEX_LAT = [[1.0, 0.0], [0.5, S3 / 2.0]]
HEX_ORB = [[1.0 / 3.0, 1.0 / 3.0], [2.0 / 3.0, 2.0 / 3.0]]


def graphene(t=1.0, delta=0.0) -> Model:
    """test_gen_v (src/lib.rs:692-700)."""
    m = Model.tb_model(HEX_LAT, HEX_ORB)
    m.set_onsite([-delta, delta])
    for R in [(0, 0), (-1, 0), (0, -1)]:
        m.set_hop(t, 0, 1, R)
    return m


def haldane(t2_imag=-1.0, t=-1.0, delta=0.7) -> Model:
    """conductivity_test / Haldan_model / build_haldane_2d (src/lib.rs:757-780, 2356-2375)."""
    m = Model.tb_model(HEX_LAT, HEX_ORB)
    m.set_onsite([-delta, delta])
    for R in [(0, 0), (-1, 0), (0, -1)]:
        m.add_hop(t, 0, 1, R)
    for R in [(1, 0), (-1, 1), (0, -1)]:
        m.add_hop(t2_imag * 1j, 0, 0, R)
    for R in [(-1, 0), (1, -1), (0, 1)]:
        m.add_hop(t2_imag * 1j, 1, 1, R)
    return m


def qwz_stacked_3d(mass=-1.0) -> Model:
    """build_qwz_stacked_3d (src/lib.rs:3196-3218)."""
    m = Model.tb_model(np.eye(3), [[0.0, 0.0, 0.0], [0.0, 0.0, 0.0]])
    m.add_onsite([mass, -mass])
    m.add_hop(-0.5j, 0, 1, (1, 0, 0))
    m.add_hop(0.5j, 0, 1, (-1, 0, 0))
    m.add_hop(-0.5, 0, 1, (0, 1, 0))
    m.add_hop(0.5, 0, 1, (0, -1, 0))
    for R in [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0)]:
        m.add_hop(0.5, 0, 0, R)
        m.add_hop(-0.5, 1, 1, R)
    return m


def kane_mele(t=-1.0, soc=-0.06, rashba=0.0) -> Model:
    """kane_mele (src/lib.rs:1410-1460): spinful honeycomb with sigma_z SOC."""
    m = Model.tb_model(HEX_LAT, HEX_ORB, spin=True)
    m.set_onsite([0.0, 0.0])
    for R in [(0, 0), (-1, 0), (0, -1)]:
        m.set_hop(t, 0, 1, R)
    for R in [(1, 0), (-1, 1), (0, -1)]:
        m.set_hop(soc * 1j, 0, 0, R, SpinDirection.Z)
    for R in [(-1, 0), (1, -1), (0, 1)]:
        m.set_hop(soc * 1j, 1, 1, R, SpinDirection.Z)
    lat = np.asarray(HEX_LAT)
    for R in [(1, 0), (-1, 1), (0, -1)]:
        r0 = np.asarray(R, float) @ lat
        m.add_hop(rashba * 1j * r0[1], 0, 0, R, SpinDirection.X)
        m.add_hop(rashba * 1j * r0[0], 0, 0, R, SpinDirection.Y)
    for R in [(-1, 0), (1, -1), (0, 1)]:
        r0 = np.asarray(R, float) @ lat
        m.add_hop(-rashba * 1j * r0[1], 1, 1, R, SpinDirection.X)
        m.add_hop(-rashba * 1j * r0[0], 1, 1, R, SpinDirection.Y)
    return m


def qwz_2d(mass=-1.0) -> Model:
    """qwz_model (src/quantum_geometry.rs:298-315)."""
    m = Model.tb_model(np.eye(2), [[0.0, 0.0], [0.0, 0.0]])
    m.add_onsite([mass, -mass])
    m.add_hop(-0.5j, 0, 1, (1, 0))
    m.add_hop(0.5j, 0, 1, (-1, 0))
    m.add_hop(-0.5, 0, 1, (0, 1))
    m.add_hop(0.5, 0, 1, (0, -1))
    for R in [(1, 0), (-1, 0), (0, 1), (0, -1)]:
        m.add_hop(0.5, 0, 0, R)
        m.add_hop(-0.5, 1, 1, R)
    return m


def massive_dirac() -> Model:
    """massive_dirac_model (src/quantum_geometry.rs:287-296): onsite -0.5, 0.5, no hopping."""
    m = Model.tb_model(np.eye(2), [[0.0, 0.0], [0.0, 0.0]])
    m.set_onsite([-0.5, 0.5])
    return m


def bench_small() -> Model:
    """build_small (benches/bench_main.rs:15-25): honeycomb, onsite -0.7 / 0.7, t = -1."""
    m = Model.tb_model(HEX_LAT, HEX_ORB)
    m.set_onsite([-0.7, 0.7])
    for R in [(0, 0), (-1, 0), (0, -1)]:
        m.add_hop(-1.0, 0, 1, R)
    return m


def flat_bands(energies, dim=2) -> Model:
    """Orbitals with on-site energies only: k-independent bands at ``energies``."""
    n = len(energies)
    m = Model.tb_model(np.eye(dim), np.zeros((n, dim)))
    m.set_onsite(list(energies))
    return m


def haldane_2d(t2_imag: float) -> Model:
    """build_haldane_2d (src/lib.rs:2356-2375): NNN amplitude t2_imag * i."""
    m = Model.tb_model(HEX_LAT, HEX_ORB)
    m.set_onsite([-0.7, 0.7])
    for R in [(0, 0), (-1, 0), (0, -1)]:
        m.add_hop(-1.0, 0, 1, R)
    for R in [(1, 0), (-1, 1), (0, -1)]:
        m.add_hop(t2_imag * 1j, 0, 0, R)
    for R in [(-1, 0), (1, -1), (0, 1)]:
        m.add_hop(t2_imag * 1j, 1, 1, R)
    return m
