"""Command-line front ends with the flags of the reference's executables, running on the GPU engine.

  python -m qsi_subspace_ed_gb300.cli diag_DOQSI_ham LATTICE.json [flags]     -> <out>/<params>.eigs.h5
  python -m qsi_subspace_ed_gb300.cli ftlm_DOQSI_ham LATTICE.json [flags]     -> <out>/<params>.ftlm.h5
  python -m qsi_subspace_ed_gb300.cli eval_observables FILE.eigs.h5 [flags]   -> FILE.eigs.out.h5
  python -m qsi_subspace_ed_gb300.cli build_hamiltonian LATTICE.json [flags]  -> <out>/<params>.mat.mtx
  python -m qsi_subspace_ed_gb300.cli partition_basis STEM.N.basis.h5         -> STEM.N.basis.partitioned.h5

Flags, defaults, basis-file naming and output layouts follow src/diag_DOQSI_ham.cpp:14-173,
include/lanczos_cli.hpp:5-40, include/basis_format_bits.hpp:8-48, src/ftlm_DOQSI_ham.cpp:14-72,
src/eval_observables.cpp:44-130, src/build_hamiltonian.cpp and components/build_basis/partition_basis.cpp.  Every algorithm choice runs on the GPU:
mfeig0 is the reference's plain Lanczos (qsi_eigval0); dense, sparse and mfsparse use the thick-restart
Lanczos solver on the matrix-free apply (qsi_lanczos_solve).
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np

from .core import LazyOpSum, ZBasis, read_basis_h5, read_f64_h5, write_eigs_h5
from .hamiltonian import build_hamiltonian, build_hamiltonian_g
from .lattice import Lattice


def get_basis_file(lattice_file, n_spinons: int, subspace: bool = False) -> Path:
    """basis_format_bits.hpp:8-29: LATTICE.json -> LATTICE.<n>.basis[.partitioned].h5."""
    ext = f".{n_spinons}.basis" + (".partitioned" if subspace else "") + ".h5"
    p = Path(lattice_file)
    return p.with_suffix(ext) if p.suffix == ".json" else Path(str(p) + ext)


def _hamiltonian_args(p: argparse.ArgumentParser) -> None:
    g = p.add_mutually_exclusive_group(required=True)
    g.add_argument("--B", nargs=3, type=float, help="magnetic field, units of Jzz")
    g.add_argument("--g", nargs=4, type=float, help="raw ring exchange, units of Jzz")
    p.add_argument("--Jpm", type=float, help="Jpm, units of Jzz")


def _hamiltonian(lat: Lattice, a):
    """(H, output stem) as the executables name their results."""
    if a.g is not None:
        g = a.g
        return build_hamiltonian_g(lat, g), "g0=%.4f%%g1=%.4f%%g2=%.4f%%g3=%.4f%%" % tuple(g)
    if a.Jpm is None:
        raise SystemExit("--Jpm is required with --B")
    B = a.B
    return build_hamiltonian(lat, a.Jpm, B), "Jpm=%.4f%%Bx=%.4f%%By=%.4f%%Bz=%.4f%%" % (a.Jpm, B[0], B[1], B[2])


def _load_basis(a) -> tuple[np.ndarray, str]:
    """load_basis (basis_format_bits.hpp:32-48): --basis_file, else the default name; dataset --sector or 'basis'."""
    path = a.basis_file or get_basis_file(a.lattice_file, a.n_spinons, a.sector is not None)
    dset = a.sector if a.sector is not None else "basis"
    return read_basis_h5(path, dset), dset


def _lanczos_args(p: argparse.ArgumentParser) -> None:
    """provide_lanczos_options (include/lanczos_cli.hpp:5-30)."""
    p.add_argument("--ncv", "-k", type=int, default=15, help="Krylov dimension, should be > 2*n_eigvals")
    p.add_argument("--atol", type=int, default=-8, help="absolute tolerance exponent, e.g. -8 = 10^-8")
    p.add_argument("--rtol", type=int, default=-8, help="relative tolerance exponent")
    p.add_argument("--rng_seed", type=int, default=0, help="seed of the random Lanczos start vector")
    p.add_argument("--verify", action="store_true", help="check the answer (reported residuals)")


def diag_parser() -> argparse.ArgumentParser:
    p = argparse.ArgumentParser(prog="diag_DOQSI_ham")
    p.add_argument("lattice_file")
    p.add_argument("-s", "--sector")
    p.add_argument("--basis_file", "-b", help="basis file (HDF5); default ${lattice_file%%.json}.<n>.basis.h5")
    _hamiltonian_args(p)
    p.add_argument("-o", "--output_dir", required=True)
    p.add_argument("--n_eigvals", "-n", type=int, default=1)
    p.add_argument("--n_eigvecs", "-N", type=int, default=1)
    p.add_argument("--n_spinons", type=int, default=0)
    p.add_argument("--save_matrix", action="store_true")
    p.add_argument("--max_iters", type=int, default=1000)
    p.add_argument("--algorithm", "-a", choices=["dense", "sparse", "mfsparse", "mfeig0"])
    _lanczos_args(p)
    return p


def diag_main(argv=None) -> Path:
    from .solvers import diagonalise, eigval0

    a = diag_parser().parse_args(argv)
    lat = Lattice.load(a.lattice_file)
    basis, dset = _load_basis(a)
    H, stem = _hamiltonian(lat, a)
    op = LazyOpSum(ZBasis(basis), H)
    n = len(basis)
    algo = a.algorithm or ("dense" if n < 100 else "sparse" if n < 10_000_000 else "mfsparse")
    if algo == "mfeig0":  # matrix_diag_bits.hpp:138-166
        if a.n_eigvals != 1 or a.n_eigvecs != 1:
            raise SystemExit("n_eigvals and n_eigvecs must be 1 for mfeig0")
        e0, vec, its = eigval0(op, seed=a.rng_seed, abs_tol=10.0 ** a.atol, rel_tol=10.0 ** a.rtol, min_iterations=10)
        evals, evecs = np.array([e0]), vec[:, None]
        print(f"eigval0: E0 = {e0!r} after {its} iterations")
    else:  # compute_spectrum_iterative (matrix_diag_bits.hpp:51-95)
        if algo in ("dense", "sparse"):  # the reference materialises H first (matrix_diag_bits.hpp:174-189)
            _materialise_if_it_fits(op)
        evals, evecs, rep = diagonalise(op, nev=a.n_eigvals, ncv=a.ncv, tol=10.0 ** a.atol, max_iter=a.max_iters,
                                        seed=a.rng_seed)
        evecs = evecs[:, : a.n_eigvecs]
        print(f"lanczos: {rep.converged} converged, {rep.applies} applies, residuals {rep.residual}")
        if a.save_matrix and algo == "sparse":
            op.saveMarket("H.mtx")
            print("Saved to H.mtx")
    print("Eigenvalues:\n" + "\n".join(repr(float(v)) for v in evals))
    out = Path(a.output_dir) / (stem + ".eigs.h5")
    out.parent.mkdir(parents=True, exist_ok=True)
    write_eigs_h5(out, evals, evecs, Path(a.lattice_file).name, dset)
    op.close()
    print(f"Writing to\n{out}")
    return out


def _materialise_if_it_fits(op) -> None:
    """Materialises the operator (qsi_op_materialise) unless the device is out of memory for its cache: the
    matrix-free apply gives the same results, only slower."""
    from ._lib import QsiError

    try:
        op.materialise(True)
    except QsiError as e:
        print(f"not materialised ({e}); applying matrix-free")


def ftlm_parser() -> argparse.ArgumentParser:
    p = argparse.ArgumentParser(prog="ftlm_DOQSI_ham")
    p.add_argument("lattice_file")
    p.add_argument("-s", "--sector")
    p.add_argument("--basis_file", "-b")
    _hamiltonian_args(p)
    p.add_argument("-o", "--output_dir", required=True)
    p.add_argument("--ncv", "-k", type=int, default=15, help="Lanczos steps per random vector")
    p.add_argument("--n_randvecs", "-R", type=int, default=20)
    p.add_argument("--n_temps", "-S", type=int, default=100)
    p.add_argument("--T_min", type=float, required=True)
    p.add_argument("--T_max", type=float, required=True)
    p.add_argument("--n_spinons", type=int, default=0)
    p.add_argument("--tol", type=float, default=1e-10)
    p.add_argument("--rng_seed", type=int, default=0)
    p.add_argument("--precision", choices=["f64", "mixed"], default="f64")
    return p


def ftlm_main(argv=None) -> Path:
    from .core import _lib as lib_mod  # noqa: F401
    from .solvers import ftlm, tridiag_ritz, thermo_from_ritz
    from ._lib import call, ptr

    a = ftlm_parser().parse_args(argv)
    lat = Lattice.load(a.lattice_file)
    basis, _ = _load_basis(a)
    H, stem = _hamiltonian(lat, a)
    op = LazyOpSum(ZBasis(basis), H)
    R = 1 << max(0, int(np.ceil(np.log2(max(1, a.n_randvecs)))))  # batched runs take a power of two
    _materialise_if_it_fits(op)  # as the reference materialises H (src/ftlm_DOQSI_ham.cpp:150-153)
    (al, be), = ftlm([op], [R], M=a.ncv, seed=a.rng_seed, precision=a.precision)
    al, be = al[: a.n_randvecs], be[: a.n_randvecs]
    temps = np.logspace(np.log10(a.T_min), np.log10(a.T_max), a.n_temps)
    ev, first = tridiag_ritz(al, be)
    th = thermo_from_ritz(ev, first ** 2, len(basis), temps)
    out = Path(a.output_dir) / (stem + ".ftlm.h5")
    out.parent.mkdir(parents=True, exist_ok=True)
    ds = {"beta": 1.0 / temps, "T": temps, "H": th["E"], "C": th["C"], "Z_shifted": th["Z_shifted"],
          "e_ref": np.array([th["e_ref"]]), "alphas": al, "betas": be,
          "num_samples": np.array([float(a.n_randvecs)])}
    first_ds = True
    for name, arr in ds.items():
        arr = np.ascontiguousarray(arr, dtype=np.float64)
        dims = np.array(arr.shape, dtype=np.int64)
        call("qsi_h5_write_f64", str(out).encode(), name.encode(), ptr(arr), ptr(dims), arr.ndim, 0 if first_ds else 1)
        first_ds = False
    op.close()
    print(f"Writing FTLM output to {out}")
    return out


def eval_parser() -> argparse.ArgumentParser:
    p = argparse.ArgumentParser(prog="eval_observables")
    p.add_argument("output_file")
    p.add_argument("--latfile_dir", default="../lattice_files")
    p.add_argument("-s", "--n_spinons", type=int, default=0)
    p.add_argument("--calculate", nargs="+", choices=["ring", "ring_ring", "partial_vol"])
    p.add_argument("--n_eigvecs", "-N", type=int, default=2)
    return p


def eval_main(argv=None) -> Path:
    from .core import _read_string_h5
    from .observables import eval_observables, write_observables_h5

    a = eval_parser().parse_args(argv)
    calc = set(a.calculate) if a.calculate else {"ring", "ring_ring", "partial_vol"}
    eigfile = Path(a.output_file)
    evals = read_f64_h5(eigfile, "eigenvalues").reshape(-1)
    vecs = read_f64_h5(eigfile, "eigenvectors")
    nvec_file = vecs.shape[1] if vecs.ndim == 2 else 1
    evecs = vecs.reshape(-1).reshape(nvec_file, -1).T  # Eigen's column-major bytes under a (dim, nvec) shape
    latname = _read_string_h5(eigfile, "latfile_json")
    dset = _read_string_h5(eigfile, "dset_name")
    latfile = Path(a.latfile_dir) / latname
    lat = Lattice.load(latfile)
    basis = read_basis_h5(get_basis_file(latfile, a.n_spinons, dset != "basis"), dset)
    nv = min(evecs.shape[1], a.n_eigvecs)
    obs = eval_observables(lat, ZBasis(basis), evecs[:, :nv], ring="ring" in calc, ring_ring="ring_ring" in calc,
                           partial_vol="partial_vol" in calc)
    out = eigfile.with_suffix(".out.h5")
    write_observables_h5(out, obs, evals, latname)
    print(f"Wrote {out}")
    return out


def build_parser() -> argparse.ArgumentParser:
    p = argparse.ArgumentParser(prog="build_hamiltonian")
    p.add_argument("lattice_file")
    p.add_argument("-s", "--sector")
    p.add_argument("--basis_file", "-b")
    _hamiltonian_args(p)
    p.add_argument("-o", "--output_dir", required=True)
    p.add_argument("--n_spinons", type=int, default=0)
    return p


def build_main(argv=None) -> Path:
    a = build_parser().parse_args(argv)
    lat = Lattice.load(a.lattice_file)
    basis, _ = _load_basis(a)
    H, stem = _hamiltonian(lat, a)
    op = LazyOpSum(ZBasis(basis), H)
    out = Path(a.output_dir) / (stem + ".mat.mtx")
    out.parent.mkdir(parents=True, exist_ok=True)
    op.saveMarket(out)
    op.close()
    print(f"Saved to {out}")
    return out


def lattice_of_basis_file(basis_file) -> Path:
    """replace_filename of partition_basis.cpp:235-256: STEM.N.basis.h5 -> STEM.json."""
    name = str(basis_file)
    k = name.rfind(".basis.h5")
    j = k
    while j > 0 and name[j - 1].isdigit():
        j -= 1
    if k < 0 or j == k or j == 0 or name[j - 1] != ".":
        raise SystemExit("Mangled basis name: expects .n.basis.h5 for some int n")
    return Path(name[: j - 1] + ".json")


def partition_main(argv=None) -> Path:
    """partition_basis STEM.N.basis.h5 (components/build_basis/partition_basis.cpp:258-269): the basis split into
    one dataset per sublattice-polarisation sector in STEM.N.basis.partitioned.h5, the sublattice masks read from
    STEM.json."""
    p = argparse.ArgumentParser(prog="partition_basis")
    p.add_argument("basis_file", help="<latfile_stem>.N.basis.h5")
    a = p.parse_args(argv)
    from .core import partition_basis_h5

    out = partition_basis_h5(a.basis_file, Lattice.load(lattice_of_basis_file(a.basis_file)))
    print(f"Wrote {out}")
    return out


COMMANDS = {"diag_DOQSI_ham": diag_main, "ftlm_DOQSI_ham": ftlm_main, "eval_observables": eval_main,
            "build_hamiltonian": build_main, "partition_basis": partition_main}


def main(argv=None) -> None:
    argv = list(sys.argv[1:] if argv is None else argv)
    if not argv or argv[0] not in COMMANDS:
        raise SystemExit("usage: python -m qsi_subspace_ed_gb300.cli {" + ",".join(COMMANDS) + "} ...")
    COMMANDS[argv[0]](argv[1:])


if __name__ == "__main__":
    main()
