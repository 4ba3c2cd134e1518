"""Eigen-solvers and FTLM over a LazyOpSum (all Krylov work on the GPU).

  diagonalise      mfsparse: compute_spectrum_iterative (include/matrix_diag_bits.hpp:51-95)
  eigval0          mfeig0:   projED::lanczos::eigval0 (components/linalg_routines/src/lanczos.cpp:184-227)
  ftlm / ftlm_thermo         finite-temperature Lanczos over several sectors in one batch
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import Eigval0Cfg, LanczosCfg, Report, call, ptr
from .core import LazyOpSum


@dataclass
class SolveReport:
    converged: int
    restarts: int
    applies: int
    residual: np.ndarray
    seconds: float


def diagonalise(op: LazyOpSum, nev: int = 1, ncv: int = 15, tol: float = 1e-10, max_iter: int = 1000,
                seed: int = 0, precision: str = "f64", polish_steps: int | None = None, want_vectors: bool = True,
                block: int = 0):
    """nev smallest eigenpairs by thick-restart Lanczos with full reorthogonalisation.

    ncv is clamped to the dimension and nev to ncv-1 (matrix_diag_bits.hpp:64-66).
    precision 'mixed' stores Krylov vectors in FP32 and polishes with FP64 Rayleigh-Ritz; polish_steps (None: 3
    rounds for 'mixed', none for 'f64'): with two rounds the FP32 phase runs to a 1e-7 relative residual, with three
    to 1e-6 (on the 96-spin sector three rounds give the ten lowest eigenvalues within 3e-11 of FP64 with half the
    FP32 restarts of two); block (mixed only): 16 = block Lanczos on FP32 blocks of 16 vectors through the batched
    apply, 0 or 1 = single-vector.
    Returns (evals, evecs (dim x nev) or None, SolveReport).
    """
    if polish_steps is None:
        polish_steps = 3 if precision == "mixed" else 0
    n = op.rows()
    ncv_e = min(ncv, n)
    nev_e = min(nev, max(1, ncv_e - 1))
    cfg = LanczosCfg(nev=nev_e, ncv=ncv_e, max_iter=max_iter,
                     precision=_lib.QSI_F32 if precision == "mixed" else _lib.QSI_F64,
                     tol=tol, seed=seed, polish_steps=polish_steps, want_vectors=int(want_vectors), block=int(block))
    evals = np.zeros(nev_e)
    evecs = np.zeros((nev_e, n)) if want_vectors else None
    rep = Report()
    call("qsi_lanczos_solve", op._h, C.byref(cfg), ptr(evals), ptr(evecs) if want_vectors else None, C.byref(rep))
    r = SolveReport(rep.converged, rep.restarts, rep.applies, np.array(rep.residual[:nev_e]), rep.seconds)
    return evals, (evecs.T if want_vectors else None), r


def eigval0(op: LazyOpSum, seed: int = 10, abs_tol: float = 1e-8, rel_tol: float = 1e-8, min_iterations: int = 10,
            max_iterations: int = 5000, calc_eigenvector: bool = True, checkpoint: str | None = None,
            checkpoint_every: int = 0, stop_after: int = 0, wall_limit_s: float = 0.0):
    """Lowest eigenvalue by plain Lanczos (no reorthogonalisation), two-pass eigenvector.

    Defaults follow lanczos::Settings (components/linalg_routines/include/lanczos.hpp:9-20);
    diag_DOQSI_ham sets min_iterations=10 and calc_eigenvector=true (include/lanczos_cli.hpp:29-38).
    With `checkpoint` (an HDF5 path) the first pass resumes from that file when it holds a checkpoint of
    this run, and writes it every `checkpoint_every` iterations and on an early stop (`stop_after`
    iterations of this call, or `wall_limit_s` seconds), which raises QsiError with status QSI_TIMEOUT.
    Returns (E0, eigvec or None, iterations).
    """
    n = op.rows()
    cfg = Eigval0Cfg(max_iterations=max_iterations, min_iterations=min_iterations, abs_tol=abs_tol, rel_tol=rel_tol,
                     seed=seed, calc_eigenvector=int(calc_eigenvector))
    e0 = C.c_double()
    its = C.c_int32()
    vec = np.zeros(n) if calc_eigenvector else None
    if checkpoint is None:
        call("qsi_eigval0", op._h, C.byref(cfg), C.byref(e0), ptr(vec) if calc_eigenvector else None, C.byref(its))
    else:
        call("qsi_eigval0_checkpointed", op._h, C.byref(cfg), str(checkpoint).encode(), int(checkpoint_every),
             int(stop_after), float(wall_limit_s), C.byref(e0), ptr(vec) if calc_eigenvector else None,
             C.byref(its))
    return e0.value, vec, its.value


def ftlm(ops, R, M: int = 100, seed: int = 0, precision: str = "mixed", blocks: int = 0):
    """Batched FTLM Lanczos recurrences: R[s] Rademacher vectors per sector, M steps.

    blocks: R-vector blocks kept per sector, 3 (H q in its own block) or 2 (in-place recurrence, R can double at
    the same device memory); 0 = three when they fit in free device memory, else two.
    Returns a list of (alphas (R[s], M), betas (R[s], M)) per sector.
    """
    ops = list(ops)
    R = [int(r) for r in R]
    handles = (C.c_void_p * len(ops))(*[o._h.value for o in ops])
    Rs = np.array(R, dtype=np.int32)
    tot = int(sum(R)) * M
    a = np.zeros(tot)
    b = np.zeros(tot)
    call("qsi_ftlm_run_blocks", C.cast(handles, C.c_void_p), len(ops), ptr(Rs), M, seed,
         _lib.QSI_F32 if precision == "mixed" else _lib.QSI_F64, int(blocks), ptr(a), ptr(b))
    out, off = [], 0
    for r in R:
        out.append((a[off:off + r * M].reshape(r, M), b[off:off + r * M].reshape(r, M)))
        off += r * M
    return out


def tridiag_ritz(alphas: np.ndarray, betas: np.ndarray):
    """Ritz values and first eigenvector components of each tridiagonal (rows of alphas/betas)."""
    a = np.ascontiguousarray(alphas, dtype=np.float64)
    b = np.ascontiguousarray(betas, dtype=np.float64)
    k, m = a.shape
    ev = np.zeros((k, m))
    first = np.zeros((k, m))
    call("qsi_tridiag_ritz", ptr(a), ptr(b), m, k, ptr(ev), ptr(first))
    return ev, first


def ftlm_thermo(alphas: np.ndarray, betas: np.ndarray, dim: int, temps: np.ndarray, e_ref: float | None = None):
    """Energy, specific heat and partition function from FTLM recurrences.

    Z(T) = dim/R sum_r sum_j w_rj exp(-(e_rj - e_ref)/T), w_rj = first component^2;
    C(T) = (<E^2> - <E>^2) / T^2.
    """
    ev, first = tridiag_ritz(alphas, betas)
    return thermo_from_ritz(ev, first ** 2, dim, temps, e_ref)


def thermo_from_ritz(ev: np.ndarray, w: np.ndarray, dim: int, temps, e_ref: float | None = None):
    temps = np.asarray(temps, dtype=np.float64)
    R = ev.shape[0]
    if e_ref is None:
        e_ref = float(ev.min())
    x = (ev - e_ref).reshape(-1)
    ww = w.reshape(-1) * (dim / R)
    bf = np.exp(-np.outer(1.0 / temps, x))  # (nT, R*M)
    Z = bf @ ww
    E1 = (bf @ (ww * x)) / Z
    E2 = (bf @ (ww * x * x)) / Z
    Cv = (E2 - E1 * E1) / temps ** 2
    return {"T": temps, "E": E1 + e_ref, "C": Cv, "Z_shifted": Z, "e_ref": e_ref}
