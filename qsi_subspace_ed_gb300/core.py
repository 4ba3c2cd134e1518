"""Host-side mirror of the reference's operator and basis API on top of the C-ABI.

Names follow qsi_subspace_ED:
  SymbolicPMROperator  components/operator/include/operator.hpp:215-467
  SymbolicOpSum        operator.hpp:476-503
  ZBasis               ZBasisBase/ZBasisBST/ZBasisInterp, operator.hpp:153-204
  LazyOpSum            components/operator/include/operator_matrix.hpp:10-118
  LazyOpSumProd        operator_matrix.hpp:120-139
All arithmetic runs in libqsi_ed.so on the GPU (term compilation and basis
enumeration are host C++ in the same library).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path
from typing import Iterable, Sequence

import numpy as np

from . import _lib
from ._lib import Term, call, ptr


# ---------------------------------------------------------------- operators
def _parse_spec(spec: str):
    """Token rule of parseSpec (operator.hpp:349-381): leading digits, then the op character."""
    ops, ids = [], []
    for tok in spec.split():
        i = 0
        while i < len(tok) - 1 and tok[i].isdigit():
            i += 1
        ops.append(tok[i])
        ids.append(int(tok[:i]) if i else 0)
    return "".join(ops), ids


class SymbolicPMROperator:
    """One permutation-matrix-representation operator: sign * Z X P."""

    __slots__ = ("t", "spec")

    def __init__(self, ops=None, spin_ids=None):
        self.t = Term()
        self.t.sign = 1
        self.spec = ("", [])  # (op characters, spin ids) it was built from; None after products
        if ops is None:
            return
        if spin_ids is None:  # spec string "0+ 1- 12z"
            call("qsi_term_parse", str(ops).encode(), 1.0, C.byref(self.t))
            self.spec = _parse_spec(str(ops))
        else:
            ops = "".join(ops)
            ids = np.ascontiguousarray(spin_ids, dtype=np.int32)
            call("qsi_term_compile", ops.encode(), ptr(ids), len(ops), 1.0, C.byref(self.t))
            self.spec = (ops, [int(i) for i in ids])

    @staticmethod
    def _mask(pair) -> int:
        return int(pair[0]) | (int(pair[1]) << 64)

    @property
    def X_mask(self) -> int:
        return self._mask(self.t.x)

    @property
    def Z_mask(self) -> int:
        return self._mask(self.t.z)

    @property
    def up_mask(self) -> int:
        return self._mask(self.t.up)

    @property
    def down_mask(self) -> int:
        return self._mask(self.t.down)

    @property
    def sign(self) -> int:
        return int(self.t.sign)

    def is_diagonal(self) -> bool:
        return self.X_mask == 0

    def applyState(self, state: int):
        """Returns (new_state, sign) as SymbolicPMROperator::applyState."""
        s = (C.c_uint64 * 2)(state & (2**64 - 1), state >> 64)
        sg = C.c_int32()
        call("qsi_term_apply_state", C.byref(self.t), C.cast(s, C.c_void_p), C.byref(sg))
        return int(s[0]) | (int(s[1]) << 64), int(sg.value)

    def __imul__(self, other):
        if isinstance(other, int):
            self.t.sign *= other
            return self
        call("qsi_term_mul", C.byref(self.t), C.byref(other.t))
        self.spec = None
        return self

    def __mul__(self, other):
        r = self.copy()
        r *= other
        return r

    def __rmul__(self, m: int):
        r = self.copy()
        r.t.sign *= m
        return r

    def copy(self):
        r = SymbolicPMROperator()
        C.memmove(C.byref(r.t), C.byref(self.t), C.sizeof(Term))
        r.spec = self.spec
        return r

    def __eq__(self, o):
        return (self.X_mask, self.Z_mask, self.up_mask, self.down_mask, self.sign) == (
            o.X_mask, o.Z_mask, o.up_mask, o.down_mask, o.sign)

    def __repr__(self):
        return (f"SymbolicPMROperator(X={self.X_mask:#x}, Z={self.Z_mask:#x}, up={self.up_mask:#x}, "
                f"down={self.down_mask:#x}, sign={self.sign})")


class SymbolicOpSum:
    """Sum of c * operator; add_term splits diagonal and off-diagonal terms."""

    def __init__(self, op: SymbolicPMROperator | None = None):
        self.diagonal_terms: list[tuple[float, SymbolicPMROperator]] = []
        self.off_diag_terms: list[tuple[float, SymbolicPMROperator]] = []
        if op is not None:
            self.add_term(1.0, op)

    def add_term(self, c: float, op: SymbolicPMROperator) -> None:
        (self.diagonal_terms if op.is_diagonal() else self.off_diag_terms).append((float(c), op.copy()))

    def __iadd__(self, op):
        self.add_term(1.0, op)
        return self

    def to_terms(self) -> C.Array:
        """Packed qsi_term array: off-diagonal terms then diagonal terms (each in insertion order)."""
        items = self.off_diag_terms + self.diagonal_terms
        arr = (Term * max(1, len(items)))()
        for k, (c, op) in enumerate(items):
            C.memmove(C.byref(arr[k]), C.byref(op.t), C.sizeof(Term))
            arr[k].c = c
        return arr, len(items)

    def __len__(self):
        return len(self.off_diag_terms) + len(self.diagonal_terms)

    def specs(self):
        """[(c, op characters, spin ids)] in to_terms() order (for the checkers)."""
        return [(c, op.spec[0], op.spec[1]) for c, op in self.off_diag_terms + self.diagonal_terms]


# ---------------------------------------------------------------- basis
def states_to_lohi(states: Iterable[int]) -> np.ndarray:
    s = list(states)
    a = np.zeros((len(s), 2), dtype=np.uint64)
    for k, v in enumerate(s):
        a[k, 0] = v & (2**64 - 1)
        a[k, 1] = v >> 64
    return a


def read_basis_h5(path, dataset: str = "basis") -> np.ndarray:
    n = C.c_int64()
    call("qsi_h5_read_basis", str(path).encode(), dataset.encode(), None, 0, C.byref(n))
    a = np.zeros((n.value, 2), dtype=np.uint64)
    call("qsi_h5_read_basis", str(path).encode(), dataset.encode(), ptr(a), n.value, C.byref(n))
    return a


def read_f64_h5(path, dataset: str) -> np.ndarray:
    n = C.c_int64()
    dims = np.zeros(4, dtype=np.int64)
    rank = C.c_int32()
    call("qsi_h5_read_f64", str(path).encode(), dataset.encode(), None, 0, C.byref(n), ptr(dims), C.byref(rank))
    a = np.zeros(n.value, dtype=np.float64)
    call("qsi_h5_read_f64", str(path).encode(), dataset.encode(), ptr(a), n.value, C.byref(n), ptr(dims),
         C.byref(rank))
    return a.reshape(tuple(int(d) for d in dims[: rank.value])) if rank.value else a


def _read_string_h5(path, dataset: str) -> str:
    buf = C.create_string_buffer(65536)
    call("qsi_h5_read_string", str(path).encode(), dataset.encode(), buf, len(buf))
    return buf.value.decode()


def read_basis_csv(path) -> np.ndarray:
    n = C.c_int64()
    call("qsi_csv_read_basis", str(path).encode(), None, 0, C.byref(n))
    a = np.zeros((n.value, 2), dtype=np.uint64)
    call("qsi_csv_read_basis", str(path).encode(), ptr(a), n.value, C.byref(n))
    return a


def write_basis_h5(path, lohi: np.ndarray, dataset: str = "basis", append: bool = False) -> None:
    a = np.ascontiguousarray(lohi, dtype=np.uint64)
    call("qsi_h5_write_basis", str(path).encode(), dataset.encode(), ptr(a), len(a), int(append))


def write_eigs_h5(path, evals, evecs, latfile_json: str, dset_name: str) -> None:
    """The .eigs.h5 layout of diag_DOQSI_ham: evecs is (dim, nvec) in Eigen column-major bytes."""
    e = np.ascontiguousarray(evals, dtype=np.float64)
    v = np.asarray(evecs, dtype=np.float64)
    dim, nvec = v.shape
    colmajor = np.ascontiguousarray(v.T)  # Eigen stores columns contiguously
    call("qsi_h5_write_eigs", str(path).encode(), ptr(e), len(e), ptr(colmajor), dim, nvec,
         latfile_json.encode(), dset_name.encode())


def enumerate_basis(lattice, n_spinon_pairs: int = 0, sector=None, ordering: str = "greedy",
                    n_threads: int = 0) -> np.ndarray:
    """Sorted spin-ice basis of a lattice (see qsi_enumerate_basis)."""
    from .lattice import Lattice

    L = lattice if isinstance(lattice, Lattice) else Lattice.load(lattice)
    tets = np.ascontiguousarray(L.tetrahedra, dtype=np.int32)
    sl = np.ascontiguousarray(L.sublattice, dtype=np.int32)
    sec = None if sector is None else np.ascontiguousarray(sector, dtype=np.int32)
    out = C.POINTER(C.c_uint64)()
    n = C.c_int64()
    call("qsi_enumerate_basis", L.n_spins, ptr(tets), tets.shape[0], tets.shape[1], ptr(sl), int(sl.max()) + 1,
         int(n_spinon_pairs), ptr(sec) if sec is not None else None, 1 if ordering == "greedy" else 0,
         int(n_threads), C.byref(out), C.byref(n))
    try:
        a = np.ctypeslib.as_array(out, shape=(max(1, n.value) * 2,))[: n.value * 2].reshape(-1, 2).copy()
    finally:
        _lib.load().qsi_free_host(C.cast(out, C.c_void_p))
    return a


def enumerate_basis_gpu(lattice, sector=None, n_spinon_pairs: int = 0) -> np.ndarray:
    """Sorted spin-ice basis enumerated on the GPU (same set as enumerate_basis, spinon pairs included)."""
    from .lattice import Lattice

    L = lattice if isinstance(lattice, Lattice) else Lattice.load(lattice)
    tets = np.ascontiguousarray(L.tetrahedra, dtype=np.int32)
    sl = np.ascontiguousarray(L.sublattice, dtype=np.int32)
    sec = None if sector is None else np.ascontiguousarray(sector, dtype=np.int32)
    out = C.POINTER(C.c_uint64)()
    n = C.c_int64()
    call("qsi_enumerate_basis_gpu", L.n_spins, ptr(tets), tets.shape[0], tets.shape[1], ptr(sl), int(sl.max()) + 1,
         ptr(sec) if sec is not None else None, int(n_spinon_pairs), C.byref(out), C.byref(n))
    try:
        a = np.ctypeslib.as_array(out, shape=(max(1, n.value) * 2,))[: n.value * 2].reshape(-1, 2).copy()
    finally:
        _lib.load().qsi_free_host(C.cast(out, C.c_void_p))
    return a


def sublattice_masks(lattice) -> np.ndarray:
    """(n_sl, 2) uint64 (lo, hi) masks of the spins of each sublattice (partition_basis.cpp:256-260)."""
    from .lattice import Lattice

    L = lattice if isinstance(lattice, Lattice) else Lattice.load(lattice)
    n_sl = int(L.sublattice.max()) + 1
    m = np.zeros((n_sl, 2), dtype=np.uint64)
    for i, a in enumerate(L.sublattice.tolist()):
        m[a, i // 64] |= np.uint64(1) << np.uint64(i % 64)
    return m


def partition_basis(lohi: np.ndarray, lattice):
    """Splits a sorted basis into its sublattice-polarisation sectors on the GPU.

    Returns {sector counts (tuple): sorted (n_s, 2) uint64 states}, the sectors in ascending order of their counts;
    the dataset name of a sector is sector_name(counts)."""
    a = np.ascontiguousarray(lohi, dtype=np.uint64)
    m = np.ascontiguousarray(sublattice_masks(lattice))
    ns = C.c_int32()
    call("qsi_partition_basis", ptr(a), len(a), ptr(m), len(m), None, None, None, 0, C.byref(ns))
    out = np.zeros_like(a)
    counts = np.zeros((ns.value, len(m)), dtype=np.int32)
    starts = np.zeros(ns.value + 1, dtype=np.int64)
    call("qsi_partition_basis", ptr(a), len(a), ptr(m), len(m), ptr(out), ptr(counts), ptr(starts), ns.value,
         C.byref(ns))
    return {tuple(int(v) for v in counts[k]): out[starts[k]:starts[k + 1]] for k in range(ns.value)}


def sector_name(counts) -> str:
    """make_sector_string (components/common/include/basis_io_h5.hpp:77-87): basis_s<n0>.<n1>.<n2>.<n3>."""
    return "basis_s" + ".".join(str(int(c)) for c in counts)


def partition_basis_h5(infile, lattice, outfile=None, dataset: str = "basis") -> Path:
    """The partition_basis tool: INFILE's basis split into one dataset per sector in OUTFILE (default: INFILE with
    its last extension replaced by .partitioned.h5, partition_basis.cpp:50-56)."""
    infile = Path(infile)
    if outfile is None:
        outfile = infile.with_suffix(".partitioned.h5") if infile.suffix else Path(str(infile) + ".partitioned.h5")
    m = np.ascontiguousarray(sublattice_masks(lattice))
    call("qsi_partition_basis_h5", str(infile).encode(), dataset.encode(), str(outfile).encode(), ptr(m), len(m))
    return Path(outfile)


class ZBasis:
    """Sorted 128-bit basis resident on the GPU with its bucket table."""

    def __init__(self, lohi: np.ndarray, bucket_bits: int = 0):
        self.states = np.ascontiguousarray(lohi, dtype=np.uint64).reshape(-1, 2)
        self._h = C.c_void_p()
        call("qsi_basis_create", ptr(self.states), len(self.states), int(bucket_bits), C.byref(self._h))

    @classmethod
    def load_from_file(cls, path, dataset: str = "basis", bucket_bits: int = 0):
        """ZBasisBase::load_from_file (operator.cpp:138-159): .h5 (dataset) or .csv."""
        p = Path(path)
        if p.suffix == ".h5":
            return cls(read_basis_h5(p, dataset), bucket_bits)
        if p.suffix == ".csv":
            return cls(read_basis_csv(p), bucket_bits)
        raise ValueError("Bad basis format: file must end with .csv or .h5")

    def dim(self) -> int:
        return len(self.states)

    size = dim

    def __len__(self):
        return len(self.states)

    def __getitem__(self, i) -> int:
        return int(self.states[i, 0]) | (int(self.states[i, 1]) << 64)

    def set_index(self, use_hash: bool = True, bucket_bits: int = 0) -> None:
        """Rebuilds the lookup index (top-bits table with bucket_bits bits; optional hash index)."""
        call("qsi_basis_index", self._h, int(use_hash), int(bucket_bits))

    def index_info(self) -> dict:
        b, h, nb = C.c_int32(), C.c_int32(), C.c_int64()
        call("qsi_basis_info", self._h, C.byref(b), C.byref(h), C.byref(nb))
        return {"bucket_bits": b.value, "hash": bool(h.value), "index_bytes": nb.value}

    def search(self, lohi: np.ndarray) -> np.ndarray:
        """Exact indices (or -1) of many states."""
        q = np.ascontiguousarray(lohi, dtype=np.uint64).reshape(-1, 2)
        idx = np.zeros(len(q), dtype=np.int64)
        call("qsi_basis_search", self._h, ptr(q), len(q), ptr(idx), _lib.QSI_PTR_HOST, None)
        return idx

    def close(self):
        if self._h:
            _lib.load().qsi_basis_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LazyOpSum:
    """Matrix-free H on a ZBasis (non-owning basis reference, copied term list)."""

    def __init__(self, basis: ZBasis, ops: SymbolicOpSum):
        self.basis = basis
        self.ops = ops
        self._terms, n = ops.to_terms()
        self._h = C.c_void_p()
        call("qsi_op_create", basis._h, C.cast(self._terms, C.c_void_p), n, C.byref(self._h))

    @classmethod
    def _from_handle(cls, basis: ZBasis, handle: C.c_void_p) -> "LazyOpSum":
        """An operator the library created (a family member)."""
        op = cls.__new__(cls)
        op.basis = basis
        op.ops = None
        op._terms = None
        op._h = handle
        return op

    def rows(self):
        return self.basis.dim()

    cols = rows

    def materialise(self, enable: bool = True) -> int:
        """Stores the column of every admitted term (the reference's toSparseMatrix before its sparse solvers);
        applies then read columns instead of looking them up, with bitwise the same results.  Returns the cache's
        size in bytes (0 after enable=False)."""
        nb = C.c_int64()
        call("qsi_op_materialise", self._h, int(bool(enable)), C.byref(nb))
        return nb.value

    def set_kernel(self, kernel: int = 1, use_hash: bool = True, list_cap: int = 0) -> None:
        """kernel 0: row per thread / warp per row; 1: bit-sliced 32-row tiles (default).  use_hash bit 0: hash
        index lookups; bit 1: FP64 instead of double-float accumulation of FP32 batched applies."""
        call("qsi_op_set_kernel", self._h, int(kernel), int(use_hash), int(list_cap))

    def info(self) -> dict:
        """Off-diagonal terms applied and pruned (never landing in the basis), diagonal classes and others."""
        v = [C.c_int32() for _ in range(4)]
        call("qsi_op_info", self._h, *[C.byref(a) for a in v])
        return dict(zip(("offdiag", "pruned", "diag_classes", "diag_generic"), (a.value for a in v)))

    def set_tuning(self, grid_bps: int = 0, vec_chunk: int = 0, which: int = -1, vec_width: int = 0) -> None:
        """Blocks per SM of the tile kernels, vectors per pass and vectors per lane (4 or 8) of the FP32 batched
        kernel (0 = built-in) for single-vector (which=0), batched (1) or both (-1) applies."""
        call("qsi_op_set_tuning", self._h, int(which), int(grid_bps), int(vec_chunk), int(vec_width))

    def tuning(self, which: int = 0) -> dict:
        """Launch settings of single-vector (which=0) or batched (1) applies."""
        v = [C.c_int32() for _ in range(6)]
        call("qsi_op_get_tuning", self._h, int(which), *[C.byref(a) for a in v])
        k, h, cap, g, vc, vw = (a.value for a in v)
        return {"kernel": k, "use_hash": h & 1, "fp64_accumulate": bool(h & 2), "list_cap": cap, "grid_bps": g,
                "vec_chunk": vc, "vec_width": vw, "bucket_bits": self.basis.index_info()["bucket_bits"]}

    def autotune(self, R: int = 1, dtype: str = "f64", X=None, Y=None, tune_index: bool = False,
                 tune_lookup: bool = False, reps: int = 2) -> str:
        """Times applies of R vectors (device tensors X, Y of shape (dim, R) or scratch) and keeps the
        fastest launch settings; returns the trial log.  tune_index also tries the bucket table at several
        widths (the basis keeps the best), tune_lookup the hash against the table at its current width.
        Results of applies do not depend on the settings."""
        buf = C.create_string_buffer(8192)
        dt = _lib.QSI_F32 if dtype in ("f32", "mixed", "float32") else _lib.QSI_F64
        xp = C.c_void_p(X.data_ptr()) if X is not None else None
        yp = C.c_void_p(Y.data_ptr()) if Y is not None else None
        flags = (_lib.QSI_TUNE_INDEX if tune_index else 0) | (_lib.QSI_TUNE_LOOKUP if tune_lookup else 0)
        call("qsi_op_autotune", self._h, xp, yp, int(R), dt, flags, int(reps), buf, len(buf))
        return buf.value.decode()

    @staticmethod
    def _kind(a):
        return _lib.QSI_PTR_DEVICE if hasattr(a, "is_cuda") and a.is_cuda else _lib.QSI_PTR_HOST

    def _stream(self, a):
        """torch's current stream; its legacy default stream (handle 0) is passed as cudaStreamLegacy,
        since NULL selects the operator's own stream in the C-ABI."""
        if self._kind(a) == _lib.QSI_PTR_DEVICE:
            import torch

            h = torch.cuda.current_stream(a.device).cuda_stream
            return C.c_void_p(h if h else _lib.CUDA_STREAM_LEGACY)
        return None

    def evaluate_add(self, x, y) -> None:
        """y += H x (FP64; numpy arrays or CUDA tensors)."""
        call("qsi_op_apply", self._h, ptr(x), ptr(y), 1, self._kind(x), self._stream(x))

    def evaluate(self, x, y) -> None:
        """y = H x."""
        call("qsi_op_apply", self._h, ptr(x), ptr(y), 0, self._kind(x), self._stream(x))

    def evaluate_static(self, x, y, accumulate: bool = False) -> None:
        """y (+)= H x for host numpy vectors without any device allocation (bases of at most
        262,144 states; see qsi_op_apply_static).  x and y must be C-contiguous float64 numpy arrays of
        shape (rows(),): the library copies rows() doubles in and out through raw host pointers."""
        n = self.rows()
        for name, a in (("x", x), ("y", y)):
            if not isinstance(a, np.ndarray):
                raise ValueError(f"evaluate_static: {name} must be a host numpy array, not {type(a).__name__}")
            if a.dtype != np.float64 or a.shape != (n,) or not a.flags.c_contiguous:
                raise ValueError(f"evaluate_static: {name} must be a C-contiguous float64 array of shape ({n},), "
                                 f"got {a.dtype} {a.shape}{'' if a.flags.c_contiguous else ' (strided)'}")
        if not y.flags.writeable:
            raise ValueError("evaluate_static: y is read-only")
        call("qsi_op_apply_static", self._h, ptr(x), ptr(y), int(accumulate))

    def __matmul__(self, x):
        y = np.zeros_like(x) if not hasattr(x, "is_cuda") else x.new_zeros(x.shape)
        self.evaluate(x, y)
        return y

    def apply_batched(self, X, Y, accumulate: bool = False) -> None:
        """Y (+)= H X for X of shape (dim, R), float64 or float32 (FP64 row accumulation)."""
        R = X.shape[1]
        dt = str(X.dtype)
        dtype = _lib.QSI_F32 if "float32" in dt else _lib.QSI_F64
        call("qsi_op_apply_batched", self._h, ptr(X), ptr(Y), R, dtype, int(accumulate), self._kind(X),
             self._stream(X))

    def triplets(self, tol: float = 1e-14):
        """(rows, cols, vals) in LazyOpSum::toSparseMatrix order."""
        n = C.c_int64()
        call("qsi_op_triplets", self._h, tol, None, None, None, 0, C.byref(n))
        r = np.zeros(n.value, dtype=np.int64)
        c = np.zeros(n.value, dtype=np.int64)
        v = np.zeros(n.value, dtype=np.float64)
        call("qsi_op_triplets", self._h, tol, ptr(r), ptr(c), ptr(v), n.value, C.byref(n))
        return r, c, v

    def toSparseMatrix(self, tol: float = 1e-14):
        import scipy.sparse as sp

        r, c, v = self.triplets(tol)
        N = self.basis.dim()
        return sp.csr_matrix((v, (r, c)), shape=(N, N))

    def saveMarket(self, path, tol: float = 1e-14) -> int:
        """Writes toSparseMatrix as a MatrixMarket file (Eigen::saveMarket layout); returns the entry count."""
        nnz = C.c_int64()
        call("qsi_op_write_mtx", self._h, str(path).encode(), float(tol), C.byref(nnz))
        return nnz.value

    def connectivity(self):
        """(hits, misses): off-diagonal terms over all rows landing in / leaving the basis."""
        h, m = C.c_int64(), C.c_int64()
        call("qsi_op_connectivity", self._h, C.byref(h), C.byref(m))
        return h.value, m.value

    def count_misses(self) -> int:
        n = C.c_int64()
        call("qsi_op_count_misses", self._h, C.byref(n))
        return n.value

    def close(self):
        if self._h:
            _lib.load().qsi_op_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class OperatorFamily:
    """H(p) = sum_t p[class(t)] term_t over one basis: the terms of `ops` with a class per term (in to_terms()
    order); members H(p) are LazyOpSum operators whose FP64 single-vector applies run batched with those of the
    family's other members waiting at the same time (qsi_family_create / qsi_family_member)."""

    def __init__(self, basis: ZBasis, ops: SymbolicOpSum, term_class: Sequence[int], n_classes: int,
                 max_cols: int = 8):
        self.basis = basis
        self.n_classes = int(n_classes)
        self._terms, n = ops.to_terms()
        cls = np.ascontiguousarray(term_class, dtype=np.int32)
        if len(cls) != n:
            raise ValueError(f"{len(cls)} classes for {n} terms")
        self._h = C.c_void_p()
        call("qsi_family_create", basis._h, C.cast(self._terms, C.c_void_p), n, ptr(cls), self.n_classes,
             int(max_cols), C.byref(self._h))

    def member(self, p) -> "LazyOpSum":
        """The operator H(p) (p: one coefficient per class)."""
        pa = np.ascontiguousarray(p, dtype=np.float64)
        if pa.shape != (self.n_classes,):
            raise ValueError(f"need {self.n_classes} class coefficients")
        h = C.c_void_p()
        call("qsi_family_member", self._h, ptr(pa), C.byref(h))
        op = LazyOpSum._from_handle(self.basis, h)
        op._family = self  # the family outlives its members
        return op

    def set_min_rows(self, min_rows: int) -> None:
        """Bases below min_rows states run each member's apply at once instead of batching (0: always batch)."""
        call("qsi_family_set_min_rows", self._h, int(min_rows))

    def stats(self) -> dict:
        b, a = C.c_int64(), C.c_int64()
        call("qsi_family_stats", self._h, C.byref(b), C.byref(a))
        return {"batches": b.value, "applies": a.value, "mean_columns": a.value / max(1, b.value)}

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            _lib.load().qsi_family_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LazyOpSumProd:
    """Spectra adaptor: perform_op(x, y) computes y = H x."""

    def __init__(self, op: LazyOpSum):
        self.op = op

    def perform_op(self, x_in, y_out) -> None:
        self.op.evaluate(x_in, y_out)

    def rows(self):
        return self.op.rows()

    cols = rows


def real_apply_fn(op: LazyOpSum):
    """projED::RealApplyFn adaptor: f(in, out) performs out += H in."""
    return lambda x, y: op.evaluate_add(x, y)
