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


def wide_case():
    """The 32-spin Q=0 basis and ring/Zeeman Hamiltonian with spin i moved to bit 4i+3 (states up to 128 bits,
    beyond the 96 bits the hash index takes): (basis lohi, SymbolicOpSum, specs), matching
    tests/golden/make_fixtures.py."""
    import qsi_subspace_ed_gb300 as q
    from qsi_subspace_ed_gb300 import workloads

    w = workloads.q0_32spin()
    wide = []
    for lo, hi in w.basis_lohi:
        s = int(lo) | (int(hi) << 64)
        v = 0
        for i in range(32):
            if (s >> i) & 1:
                v |= 1 << (4 * i + 3)
        wide.append(v)
    wide.sort()
    lohi = np.array([[v & (2**64 - 1), v >> 64] for v in wide], dtype=np.uint64)
    specs = [(c, ops, [4 * i + 3 for i in ids]) for c, ops, ids in w.hamiltonian().specs()]
    H = q.SymbolicOpSum()
    for c, ops, ids in specs:
        H.add_term(c, q.SymbolicPMROperator(ops, ids))
    return lohi, H, specs
