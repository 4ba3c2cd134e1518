"""Named workloads: pyrochlore cubic supercells and their seeded Hamiltonians.

Lattices (package data, written by the reference's scripts/make_latfile.py
--A1 8 0 0 --A2 0 16 0 --A3 0 0 {8,16,24}):
  pyro_1x2x1  32 spins, 32 hexagons, 16 tetrahedra
  pyro_1x2x2  64 spins
  pyro_1x2x3  96 spins
Hamiltonian family: H = -sum_hex g_type (O + O^dagger) - sum_i (B . z_a) S^z_i
(hamiltonian.build_ring_zeeman), parameters drawn from numpy default_rng(seed).
"""
from __future__ import annotations

from dataclasses import dataclass
from pathlib import Path

import numpy as np

from .core import ZBasis, enumerate_basis
from .hamiltonian import build_ring_zeeman
from .lattice import Lattice

LATTICE_DIR = Path(__file__).resolve().parent / "lattices"


def lattice(name: str) -> Lattice:
    return Lattice.load(LATTICE_DIR / f"{name}.json")


def equal_sector(lat: Lattice) -> list[int]:
    """Equal sublattice polarisation (the zero-winding sector): N/8 up spins per sublattice."""
    n_sl = int(lat.sublattice.max()) + 1
    per = lat.n_spins // n_sl
    return [per // 2] * n_sl


@dataclass
class Workload:
    name: str
    lattice: Lattice
    basis_lohi: np.ndarray
    g: list
    B: list
    Jpm: float = 0.0

    def hamiltonian(self):
        return build_ring_zeeman(self.lattice, self.g, self.B, self.Jpm)


def ring_zeeman_params(seed: int, g_range=None, b_amp=0.2):
    rng = np.random.default_rng(seed)
    g = [1.0, 0.8, 0.6, 0.4] if g_range is None else list(rng.uniform(g_range[0], g_range[1], 4))
    B = list(rng.uniform(-b_amp, b_amp, 3))
    return g, B


def q0_32spin(seed: int = 1) -> Workload:
    """32 spins, full Q=0 basis (3,618 states), g=(1,0.8,0.6,0.4), B ~ U[-0.2,0.2]^3."""
    lat = lattice("pyro_1x2x1")
    g, B = ring_zeeman_params(seed)
    return Workload("pyro_1x2x1.Q0", lat, enumerate_basis(lat), g, B)


def sector_workload(name: str, seed: int = 3, g_range=(0.2, 1.0), b_amp=0.5, lat_name=None, gpu: bool = False) -> Workload:
    """Equal-polarisation sector basis of a lattice with g ~ U[g_range]^4, B ~ U[-b_amp, b_amp]^3.

    gpu=True enumerates on the GPU (enumerate_basis_gpu), which is how large sectors are built."""
    from .core import enumerate_basis_gpu

    lat = lattice(lat_name or name)
    g, B = ring_zeeman_params(seed, g_range, b_amp)
    enum = enumerate_basis_gpu if gpu else enumerate_basis
    return Workload(f"{lat.name()[:-5]}.s{'.'.join(map(str, equal_sector(lat)))}", lat,
                    enum(lat, sector=equal_sector(lat)), g, B)


def sector_96spin(seed: int = 3) -> Workload:
    """96 spins, 12.12.12.12 sector, g ~ U[0.2,1]^4, B ~ U[-0.5,0.5]^3."""
    return sector_workload("pyro_1x2x3", seed)


def build(w: Workload, bucket_bits: int = 0):
    """Device basis and operator for a workload."""
    from .core import LazyOpSum

    b = ZBasis(w.basis_lohi, bucket_bits)
    return b, LazyOpSum(b, w.hamiltonian())
