"""Shared helpers for the tests (fixture loading, cases)."""
import hashlib
import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def golden_json(name):
    return json.load(open(GOLDEN / name))


def cases():
    """name -> (basis lohi, SymbolicOpSum), matching tests/golden/make_fixtures.py."""
    import qsi_subspace_ed_gb300 as q
    from qsi_subspace_ed_gb300 import workloads

    lat48 = q.Lattice.load(GOLDEN / "lattices" / "golden48.json")
    lat32 = q.Lattice.load(GOLDEN / "lattices" / "ref32.json")
    b32 = np.load(GOLDEN / "basis_ref32.npy")
    q0_32 = workloads.q0_32spin()
    sec4 = workloads.sector_workload("pyro_1x2x1", seed=3)
    return {
        "golden48_JpmB": (q.enumerate_basis(lat48), q.build_hamiltonian(lat48, 0.02, [0.1, 0.1, 0.1])),
        "ref32_g": (b32, q.build_hamiltonian_g(lat32, [1.0, -0.2, -0.2, -0.2])),
        "ref32_JpmB": (b32, q.build_hamiltonian(lat32, 0.05, [0.3, -0.1, 0.2])),
        "q0_32": (q0_32.basis_lohi, q0_32.hamiltonian()),
        "s4444": (sec4.basis_lohi, sec4.hamiltonian()),
    }
