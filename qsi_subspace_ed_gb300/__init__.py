"""GB300 (sm_103a) matrix-free Hamiltonian apply and Lanczos/FTLM engine for
projected exact diagonalisation of quantum-spin-ice ring-exchange models.

The compute path is libqsi_ed.so (CUDA C++ behind the C-ABI of
include/qsi_ed.h); this package mirrors qsi_subspace_ED's operator/basis API
on top of it.
"""
from ._lib import QsiError, load
from .core import (LazyOpSum, LazyOpSumProd, OperatorFamily, SymbolicOpSum, SymbolicPMROperator, ZBasis, enumerate_basis, enumerate_basis_gpu,
                   partition_basis, partition_basis_h5, sector_name, sublattice_masks,
                   read_basis_csv, read_basis_h5, read_f64_h5, real_apply_fn, states_to_lohi, write_basis_h5,
                   write_eigs_h5)
from .hamiltonian import build_hamiltonian, build_hamiltonian_g, build_ring_zeeman, g_vals, get_loc_z, get_ring_ops
from .lattice import Lattice
from .solvers import diagonalise, eigval0, ftlm, ftlm_thermo, tridiag_ritz
from .observables import eval_observables, expectations, get_partial_vol_ops, read_observables_h5, write_observables_h5

__all__ = [
    "QsiError", "load", "LazyOpSum", "LazyOpSumProd", "OperatorFamily", "SymbolicOpSum", "SymbolicPMROperator", "ZBasis",
    "enumerate_basis", "enumerate_basis_gpu", "partition_basis", "partition_basis_h5", "sector_name", "sublattice_masks", "read_basis_csv", "read_basis_h5", "read_f64_h5", "real_apply_fn", "states_to_lohi",
    "write_basis_h5", "write_eigs_h5", "build_hamiltonian", "build_hamiltonian_g", "build_ring_zeeman", "g_vals",
    "get_loc_z", "get_ring_ops", "Lattice", "diagonalise", "eigval0", "ftlm", "ftlm_thermo", "tridiag_ritz",
    "eval_observables", "expectations", "get_partial_vol_ops", "read_observables_h5", "write_observables_h5",
]
