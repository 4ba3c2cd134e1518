"""Ring, ring-ring and partial-volume expectation values of eigenvectors (the eval_observables step).

  get_partial_vol_ops   geometry.hpp:107-145 (three rings of a volume, multiplied in six orders and summed)
  expectations          compute_all_expectations / compute_cross_correlation (src/expectation_eval.cpp:27-110)
  eval_observables      src/eval_observables.cpp:134-208 (ring, ring_ring, partial_vol_sl0..3)
  write_observables_h5  the .out.h5 file eval_observables writes (eigenvalues, latfile_json, the datasets above)

All operator applications and dot products run on the GPU through qsi_expectations.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import _lib
from ._lib import Term, call, ptr
from .core import SymbolicOpSum, SymbolicPMROperator, ZBasis
from .hamiltonian import get_ring_ops
from .lattice import Lattice

_PERM3 = ((0, 1, 2), (1, 2, 0), (2, 0, 1), (0, 2, 1), (2, 1, 0), (1, 0, 2))


def get_partial_vol_ops(lat: Lattice, rings: list, missing_plaq_sl: int) -> list:
    """Per volume of the lattice file ("vols", member_plaq_idx), the rings of the three plaquettes other than
    the one at position `missing_plaq_sl`, multiplied in the six orders of perm3 and summed, coefficient 1."""
    out = []
    for vol in lat.data["vols"]:
        plaq = vol["member_plaq_idx"]
        ops = [rings[plaq[i]] for i in range(4) if i != missing_plaq_sl]
        assert len(ops) == 3
        ooo = SymbolicOpSum()
        for p in _PERM3:
            v = SymbolicPMROperator("")
            for j in range(3):
                v *= ops[p[j]]
            ooo += v
        out.append(ooo)
    return out


def _as_sum(op) -> SymbolicOpSum:
    return op if isinstance(op, SymbolicOpSum) else SymbolicOpSum(op)


def expectations(basis: ZBasis, ops: list, psi: np.ndarray, cross: bool = False):
    """expect[l, i, j] = psi_j . (O_l psi_i) and, with cross, cross[l, m, i, j] = (O_l psi_i) . (O_m psi_j).

    ops: SymbolicOpSum or SymbolicPMROperator items; psi: (dim,) or (dim, nvec)."""
    psi = np.asarray(psi, dtype=np.float64)
    if psi.ndim == 1:
        psi = psi[:, None]
    n, nv = psi.shape
    if n != basis.dim():
        raise ValueError("psi rows must match the basis dimension")
    sums = [_as_sum(o) for o in ops]
    counts = [len(s) for s in sums]
    total = max(1, sum(counts))
    arr = (Term * total)()
    k = 0
    for s in sums:
        a, m = s.to_terms()
        for t in range(m):
            C.memmove(C.byref(arr[k]), C.byref(a[t]), C.sizeof(Term))
            k += 1
    offsets = np.zeros(len(sums) + 1, dtype=np.int32)
    offsets[1:] = np.cumsum(counts)
    colmajor = np.ascontiguousarray(psi.T)  # column i contiguous
    expect = np.zeros((len(sums), nv, nv))
    cr = np.zeros((len(sums), len(sums), nv, nv)) if cross else None
    call("qsi_expectations", basis._h, C.cast(arr, C.c_void_p), ptr(offsets), len(sums), ptr(colmajor), nv,
         ptr(expect), ptr(cr) if cross else None)
    return expect, cr


def eval_observables(lat: Lattice, basis: ZBasis, eigvecs: np.ndarray, ring: bool = True, ring_ring: bool = True,
                     partial_vol: bool = True) -> dict:
    """The datasets eval_observables computes for the given eigenvectors (columns of eigvecs)."""
    rings, _, _ = get_ring_ops(lat)
    out = {}
    if ring or ring_ring:
        e, c = expectations(basis, rings, eigvecs, cross=ring_ring)
        if ring:
            out["ring"] = e
        if ring_ring:
            out["ring_ring"] = c
    if partial_vol:
        for sl in range(4):
            out[f"partial_vol_sl{sl}"], _ = expectations(basis, get_partial_vol_ops(lat, rings, sl), eigvecs)
    return out


def write_observables_h5(path, obs: dict, eigenvalues, latfile_name: str) -> None:
    """eval_observables' output file: latfile_json (the lattice file name), eigenvalues, then each dataset."""
    path = str(path)
    call("qsi_h5_write_string", path.encode(), b"latfile_json", str(latfile_name).encode(), 0)
    ev = np.ascontiguousarray(eigenvalues, dtype=np.float64).reshape(-1)
    dims = np.array([len(ev)], dtype=np.int64)
    call("qsi_h5_write_f64", path.encode(), b"eigenvalues", ptr(ev), ptr(dims), 1, 1)
    for name, a in obs.items():
        a = np.ascontiguousarray(a, dtype=np.float64)
        dims = np.array(a.shape, dtype=np.int64)
        call("qsi_h5_write_f64", path.encode(), name.encode(), ptr(a), ptr(dims), a.ndim, 1)


def read_observables_h5(path) -> dict:
    from .core import read_f64_h5

    out = {}
    for name in ["eigenvalues", "ring", "ring_ring"] + [f"partial_vol_sl{k}" for k in range(4)]:
        try:
            out[name] = read_f64_h5(Path(path), name)
        except _lib.QsiError:
            pass
    return out
