"""Ring-exchange / Zeeman Hamiltonians from a lattice file.

Mirrors include/hamiltonian_setup.hpp:14-121, include/physics/geometry.hpp:29-62
and include/physics/Jring.hpp:6-54 of qsi_subspace_ED.  Term order follows the
reference (it fixes the order of the exported connectivity).
"""
from __future__ import annotations

import math

import numpy as np

from .core import SymbolicOpSum, SymbolicPMROperator
from .lattice import Lattice

_SQRT3 = math.sqrt(3.0)
# local easy axes of the four pyrochlore sublattices (rows), unnormalised
_LOCAL_Z_RAW = np.array([[1.0, 1.0, 1.0], [1.0, -1.0, -1.0], [-1.0, 1.0, -1.0], [-1.0, -1.0, 1.0]])


def get_loc_z() -> np.ndarray:
    """Unit local z axes z_a (physics/Jring.hpp:6-14)."""
    return _LOCAL_Z_RAW / _SQRT3


def _dot3(a, b) -> float:
    return (float(a[0]) * float(b[0]) + float(a[1]) * float(b[1])) + float(a[2]) * float(b[2])


def g_vals(Jpm: float, B) -> list[float]:
    """Perturbative ring couplings g_a(Jpm, B) (physics/Jring.hpp:17-54).

    With h_a = B . (unnormalised z_a):
      g_a = ( -21/4 prod_{b!=a} h_b^2 - 35/2 Jpm prod_b h_b - 15 Jpm^2 h_a^2 + 54 Jpm^3 ) / 36
    """
    h = [_dot3(B, _LOCAL_Z_RAW[a]) for a in range(4)]
    prod_all = h[0] * h[1] * h[2] * h[3]
    out = []
    for a in range(4):
        others = 1.0
        for b in range(4):
            if b != a:
                others *= h[b] * h[b]
        out.append((-21.0 / 4 * others + (-35.0 / 2 * prod_all * Jpm + (-15.0 * h[a] * h[a] * Jpm * Jpm
                                                                         + 54.0 * Jpm * Jpm * Jpm))) / 36.0)
    return out


def get_ring_ops(lat: Lattice, incl_partial: bool = False):
    """(O, O_dagger, sublattice) per hexagon (geometry.hpp:29-62): sign +1 -> '+', -1 -> '-'."""
    O, Oh, sls = [], [], []
    for ring in lat.rings:
        spins = list(ring["member_spin_idx"])
        if not incl_partial and len(spins) != 6:
            continue
        ops = "".join("+" if s == 1 else "-" for s in ring["signs"])
        conj = "".join("-" if s == 1 else "+" for s in ring["signs"])
        O.append(SymbolicPMROperator(ops, spins))
        Oh.append(SymbolicPMROperator(conj, spins))
        sls.append(int(ring["sl"]))
    return O, Oh, sls


def build_hamiltonian(lat: Lattice, Jpm: float, B) -> SymbolicOpSum:
    """The --Jpm/--B Hamiltonian of diag_DOQSI_ham (hamiltonian_setup.hpp:14-101)."""
    try:
        version = lat.data["__version__"]
    except KeyError:
        raise RuntimeError("__version__ field missing, suspect an old file")
    if float(version) < 1.1 - 2e-5:
        raise RuntimeError("JSON file is old, API version 1.1 is required")
    H = SymbolicOpSum()
    g = g_vals(Jpm, B)
    lz = get_loc_z()
    ringL, ringR, sls = get_ring_ops(lat)
    for L, R, sl in zip(ringL, ringR, sls):
        H.add_term(g[sl], R)
        H.add_term(g[sl], L)
    atoms = lat.data["atoms"]
    for bond in lat.bonds:
        i, j = int(bond["from_idx"]), int(bond["to_idx"])
        si, sj = int(atoms[i]["sl"]), int(atoms[j]["sl"])
        zi, zj = _dot3(B, lz[si]), _dot3(B, lz[sj])
        H.add_term(-4.0 * Jpm * zi * zj, SymbolicPMROperator("zz", [i, j]))
    for s in lat.data.get("neighbour2", []):
        H.add_term(Jpm / 2, SymbolicPMROperator("+-", [s[0], s[1]]))
        H.add_term(Jpm / 2, SymbolicPMROperator("-+", [s[0], s[1]]))
    h4 = Jpm * Jpm / 4
    for s in lat.data.get("neighbour4", []):
        # the reference adds this product twice (hamiltonian_setup.hpp:85-91)
        H.add_term(h4, SymbolicPMROperator("+-+-", [s[0], s[1], s[2], s[3]]))
        H.add_term(h4, SymbolicPMROperator("+-+-", [s[0], s[1], s[2], s[3]]))
    return H


def build_hamiltonian_g(lat: Lattice, g) -> SymbolicOpSum:
    """The --g Hamiltonian: raw ring exchange g[sl] (O + O^dagger) (hamiltonian_setup.hpp:105-121)."""
    H = SymbolicOpSum()
    ringL, ringR, sls = get_ring_ops(lat)
    for L, R, sl in zip(ringL, ringR, sls):
        H.add_term(float(g[sl]), R)
        H.add_term(float(g[sl]), L)
    return H


KAPPA = 0.5  # S^z = sigma^z / 2 (the reference's 'z' operator is sigma^z, operator.hpp:246-253)


def build_ring_zeeman(lat: Lattice, g, B, Jpm: float = 0.0, kappa: float = KAPPA) -> SymbolicOpSum:
    """H = -sum_hex g_type (O + O^dagger) - sum_i (B . z_a(i)) S^z_i  [- Jpm sum_<ij> (S+_i S-_j + h.c.)].

    Ring terms: add_term(-g[sl], O^dagger), add_term(-g[sl], O); Zeeman:
    add_term(-(B . z_a) * kappa, z_i) with kappa = 1/2; optional nearest-neighbour
    hopping on every bond as add_term(-Jpm, '+-') + add_term(-Jpm, '-+').
    """
    H = SymbolicOpSum()
    ringL, ringR, sls = get_ring_ops(lat)
    for L, R, sl in zip(ringL, ringR, sls):
        H.add_term(-float(g[sl]), R)
        H.add_term(-float(g[sl]), L)
    if Jpm:
        for bond in lat.bonds:
            i, j = int(bond["from_idx"]), int(bond["to_idx"])
            H.add_term(-float(Jpm), SymbolicPMROperator("+-", [i, j]))
            H.add_term(-float(Jpm), SymbolicPMROperator("-+", [i, j]))
    lz = get_loc_z()
    for i, a in enumerate(lat.data["atoms"]):
        h = _dot3(B, lz[int(a["sl"])])
        H.add_term(-h * kappa, SymbolicPMROperator("z", [i]))
    return H


def ring_zeeman_classes(lat: Lattice, Jpm: float = 0.0):
    """Class of every term of build_ring_zeeman (in its to_terms() order) for an operator family: the ring terms
    of hexagon type sl are class sl (0..3), the Zeeman term of a spin on sublattice a is class 4 + a, bond hopping
    (Jpm != 0) is class 8.  Returns (classes, n_classes)."""
    off, diag = [], []
    for ring in lat.rings:
        if len(ring["member_spin_idx"]) != 6:
            continue
        off += [int(ring["sl"])] * 2
    if Jpm:
        off += [8] * (2 * len(lat.bonds))
    diag = [4 + int(a["sl"]) for a in lat.data["atoms"]]
    return off + diag, 9 if Jpm else 8


def ring_zeeman_class_coefficients(g, B, Jpm: float = 0.0, kappa: float = KAPPA):
    """Class coefficients p of H(g, B) for ring_zeeman_classes: -g[sl] for the rings, -(B . z_a) kappa for the
    Zeeman terms (the same arithmetic as build_ring_zeeman, so a family member equals build_ring_zeeman's
    operator term by term), -Jpm for the hopping."""
    lz = get_loc_z()
    p = [-float(g[k]) for k in range(4)] + [-_dot3(B, lz[a]) * kappa for a in range(4)]
    if Jpm:
        p.append(-float(Jpm))
    return p
