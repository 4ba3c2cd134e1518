"""Lattice JSON files of qsi_subspace_ED (scripts/pyrochlore.py export_json).

Fields used on this path: atoms[{xyz, sl}], bonds[{from_idx, to_idx}],
tetrahedra[{member_spin_idx}], rings[{sl, member_spin_idx, signs}],
__version__ (include/hamiltonian_setup.hpp:18-25).
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np


@dataclass
class Lattice:
    data: dict
    path: str = ""
    n_spins: int = 0
    sublattice: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    tetrahedra: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.int32))

    @classmethod
    def load(cls, path) -> "Lattice":
        p = Path(path)
        with open(p) as f:
            d = json.load(f)
        return cls.from_dict(d, str(p))

    @classmethod
    def from_dict(cls, d: dict, path: str = "") -> "Lattice":
        L = cls(d, path)
        L.n_spins = len(d["atoms"])
        L.sublattice = np.array([int(a["sl"]) for a in d["atoms"]], dtype=np.int32)
        L.tetrahedra = np.array([t["member_spin_idx"] for t in d["tetrahedra"]], dtype=np.int32)
        return L

    @property
    def rings(self):
        return self.data.get("rings", [])

    @property
    def bonds(self):
        return self.data.get("bonds", [])

    @property
    def version(self) -> float:
        return float(self.data["__version__"])

    def name(self) -> str:
        return Path(self.path).name
