"""ORACLE — test infrastructure, never product code.

Python access to the two CPU checkers of the hot path:
  * the plain-C restatement oracle/qsi_oracle.c  -> oracle/libqsi_oracle.so ("port")
  * the reference's own operator.cpp + oracle/ref_harness.cpp -> oracle/_ref/libqsi_ref.so
    (built only where the reference checkout exists)
plus the FP64 eigen-oracle (scipy ARPACK eigsh / numpy eigh on the oracle's
triplets, the same implicitly-restarted-Lanczos family as the Spectra solver
behind mfsparse, include/matrix_diag_bits.hpp:51-95) and an exact
thermodynamics oracle from the full spectrum (the dense branch of the
reference's FTLM study, jl/calc_Cv_ftlm.jl:114-139: Boltzmann weights with
the ground state subtracted, C = beta^2 (<E^2> - <E>^2)).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_SO = HERE / "libqsi_oracle.so"
REF_SO = HERE / "_ref" / "libqsi_ref.so"


def build_port() -> Path:
    srcs = [HERE / "qsi_oracle.c", HERE / "enumerate_oracle.c", HERE / "start_vector.cpp"]
    if not PORT_SO.exists() or PORT_SO.stat().st_mtime < max(s.stat().st_mtime for s in srcs):
        tmp = PORT_SO.with_suffix(".tmp.so")
        objs = []
        for src in srcs:
            obj = HERE / (src.stem + ".o")
            cc = ["gcc", "-O3", "-fopenmp"] if src.suffix == ".c" else ["g++", "-O2"]
            subprocess.run([*cc, "-fPIC", "-c", str(src), "-o", str(obj)], check=True)
            objs.append(str(obj))
        subprocess.run(["g++", "-shared", "-fopenmp", *objs, "-o", str(tmp)], check=True)
        os.replace(tmp, PORT_SO)
    return PORT_SO


def reference_root() -> str | None:
    """The qsi_subspace_ED checkout the reference-built checker compiles from: $QSI_REFERENCE_ROOT, else a
    directory named `reference` beside this repository, else None (GPU hosts have no checkout)."""
    env = os.environ.get("QSI_REFERENCE_ROOT")
    if env:
        return env if Path(env).exists() else None
    sib = HERE.parent.parent / "reference"
    return str(sib) if (sib / "components" / "operator").exists() else None


def build_ref(root: str | None = None) -> Path | None:
    """Builds the reference-built checker from the checkout at `root` (default: reference_root()); None where
    there is no checkout."""
    root = root or reference_root()
    if not root or not Path(root).exists():
        return None
    deps = [HERE / "ref_harness.cpp", HERE / "build_ref.sh", HERE / "ref_shim" / "hdf5.h"]
    if not REF_SO.exists() or REF_SO.stat().st_mtime < max(d.stat().st_mtime for d in deps):
        subprocess.run(["sh", str(HERE / "build_ref.sh"), root], check=True, capture_output=True)
    return REF_SO


_port = None
_ref = None


def port():
    global _port
    if _port is None:
        lib = C.CDLL(str(build_port()))
        lib.oracle_apply_state.restype = C.c_int
        lib.oracle_search.restype = C.c_int
        lib.oracle_evaluate_add.restype = C.c_int
        lib.oracle_triplets.restype = C.c_int64
        lib.oracle_term_compile.restype = C.c_int
        lib.oracle_dot.restype = C.c_double
        lib.oracle_dot.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
        lib.oracle_axpby.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int64]
        lib.oracle_triplets.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int, C.c_double, C.c_void_p,
                                        C.c_void_p, C.c_void_p]
        lib.oracle_evaluate_add.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                            C.c_int]
        lib.oracle_term_compile.argtypes = [C.c_char_p, C.c_void_p, C.c_int, C.c_double, C.c_void_p]
        lib.oracle_apply_state.argtypes = [C.c_void_p, C.c_void_p]
        lib.oracle_term_mul.restype = None
        lib.oracle_term_mul.argtypes = [C.c_void_p, C.c_void_p]
        lib.oracle_set_random_unit.restype = None
        lib.oracle_set_random_unit.argtypes = [C.c_void_p, C.c_int64, C.c_uint]
        lib.oracle_evaluate_add_rows.restype = C.c_int
        lib.oracle_evaluate_add_rows.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_void_p, C.c_int,
                                                 C.c_void_p, C.c_void_p, C.c_int]
        lib.oracle_interp_build.restype = C.c_void_p
        lib.oracle_interp_build.argtypes = [C.c_void_p, C.c_int64]
        lib.oracle_interp_free.restype = None
        lib.oracle_interp_free.argtypes = [C.c_void_p]
        lib.oracle_interp_search_many.restype = None
        lib.oracle_interp_search_many.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
        lib.oracle_evaluate_add_rows_interp.restype = C.c_int
        lib.oracle_evaluate_add_rows_interp.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_void_p,
                                                        C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                                        C.c_void_p]
        lib.oracle_enumerate.restype = C.c_int64
        lib.oracle_enumerate.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                         C.c_int, C.c_int, C.POINTER(C.POINTER(C.c_uint64))]
        lib.oracle_free.restype = None
        lib.oracle_free.argtypes = [C.c_void_p]
        _port = lib
    return _port


def ref():
    """The reference-built checker, or None where the reference is absent."""
    global _ref
    if _ref is None:
        p = build_ref()
        if p is None or not p.exists():
            return None
        lib = C.CDLL(str(p))
        lib.ref_term_masks.restype = C.c_int
        lib.ref_apply_state.restype = C.c_int
        lib.ref_triplets.restype = C.c_int64
        _ref = lib
    return _ref


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


# ------------------------------------------------------------------ port wrappers
def terms_array(specs):
    """specs: list of (c, ops, ids) -> numpy structured bytes in qsi_term layout, compiled by the port."""
    lib = port()
    buf = np.zeros((max(1, len(specs)), 80), dtype=np.uint8)
    for k, (c, ops, ids) in enumerate(specs):
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        rc = lib.oracle_term_compile(ops.encode(), _p(ids), len(ops), float(c), buf[k].ctypes.data_as(C.c_void_p))
        if rc != 0:
            raise ValueError(f"bad operator spec {ops!r}")
    return buf[: len(specs)].copy()


def apply_terms_port(basis: np.ndarray, terms: np.ndarray, x: np.ndarray, threads: int = 0) -> np.ndarray:
    """y = O x by the restated push loop for a compiled term array (qsi_term layout rows)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros_like(x)
    t = np.ascontiguousarray(terms)
    port().oracle_evaluate_add(_p(basis), len(basis), _p(t), len(t), _p(x), _p(y), threads)
    return y


def term_product_port(factors: np.ndarray) -> np.ndarray:
    """The product factors[0] * factors[1] * ... (SymbolicPMROperator::operator*=, restated), one term row."""
    out = np.ascontiguousarray(factors[0:1]).copy()
    for k in range(1, len(factors)):
        f = np.ascontiguousarray(factors[k:k + 1])
        port().oracle_term_mul(_p(out), _p(f))
    return out


def ring_terms_port(lat: dict) -> list:
    """One term array per hexagon ring (get_ring_ops, geometry.hpp:29-62: sign +1 -> '+', -1 -> '-')."""
    out = []
    for ring in lat["rings"]:
        ids = list(ring["member_spin_idx"])
        if len(ids) != 6:
            continue
        ops = "".join("+" if v == 1 else "-" for v in ring["signs"])
        out.append(terms_array([(1.0, ops, ids)]))
    return out


_PERM3 = ((0, 1, 2), (1, 2, 0), (2, 0, 1), (0, 2, 1), (2, 1, 0), (1, 0, 2))


def partial_vol_terms_port(lat: dict, rings: list, missing_sl: int) -> list:
    """get_partial_vol_ops (geometry.hpp:107-145): per volume, the three rings other than the one of
    sublattice `missing_sl`, multiplied in the six orders and summed (coefficient 1 each)."""
    out = []
    for vol in lat["vols"]:
        plaq = vol["member_plaq_idx"]
        three = [rings[plaq[i]][0] for i in range(4) if i != missing_sl]
        terms = [term_product_port(np.stack([three[p[0]], three[p[1]], three[p[2]]]))[0] for p in _PERM3]
        out.append(np.stack(terms))
    return out


def expectations_port(basis: np.ndarray, ops: list, psi: np.ndarray, cross: bool = False):
    """compute_all_expectations / compute_cross_correlation (src/expectation_eval.cpp:27-110), FP64:
    expect[l, i, j] = psi_j . (O_l psi_i), cross[l, m, i, j] = (O_l psi_i) . (O_m psi_j)."""
    psi = np.asarray(psi, dtype=np.float64).reshape(len(basis), -1)
    nv = psi.shape[1]
    W = np.stack([np.stack([apply_terms_port(basis, t, psi[:, i]) for i in range(nv)]) for t in ops])  # (L, nv, N)
    expect = np.einsum("lin,nj->lij", W, psi)
    if not cross:
        return expect, None
    return expect, np.einsum("lin,mjn->lmij", W, W)


def apply_port(basis: np.ndarray, specs, x: np.ndarray, y: np.ndarray | None = None, threads: int = 0):
    """y += H x by the restated push loop (y = H x when y is None)."""
    t = terms_array(specs)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros_like(x) if y is None else y
    port().oracle_evaluate_add(_p(basis), len(basis), _p(t), len(specs), _p(x), _p(y), threads)
    return y


def apply_rows_port(basis: np.ndarray, terms: np.ndarray, x: np.ndarray, y: np.ndarray, row_begin: int,
                    row_end: int, threads: int = 0) -> None:
    """Push loop over source rows [row_begin, row_end) only (CPU-baseline sample)."""
    port().oracle_evaluate_add_rows(_p(basis), len(basis), row_begin, row_end, _p(terms), len(terms), _p(x), _p(y),
                                    threads)


class InterpIndex:
    """ZBasisInterp's high-word bounds over a sorted basis (restated; the basis array must outlive it)."""

    def __init__(self, basis: np.ndarray):
        self.basis = np.ascontiguousarray(basis, dtype=np.uint64)
        self.h = port().oracle_interp_build(_p(self.basis), len(self.basis))
        if not self.h:
            raise MemoryError("interp index")

    def search(self, queries: np.ndarray) -> np.ndarray:
        """Index per query, -1 when absent, -2 for an unseen high word (where the reference throws)."""
        q = np.ascontiguousarray(queries, dtype=np.uint64)
        idx = np.zeros(len(q), np.int64)
        port().oracle_interp_search_many(self.h, _p(self.basis), _p(q), len(q), _p(idx))
        return idx

    def apply_rows(self, terms: np.ndarray, x: np.ndarray, y: np.ndarray, row_begin: int, row_end: int,
                   threads: int = 0) -> int:
        """The push loop with ZBasisInterp lookups over source rows [row_begin, row_end); returns the number of
        lookups with an unseen high word."""
        unseen = C.c_int64(0)
        rc = port().oracle_evaluate_add_rows_interp(_p(self.basis), len(self.basis), row_begin, row_end, _p(terms),
                                                    len(terms), _p(x), _p(y), threads, self.h, C.byref(unseen))
        if rc != 0:
            raise RuntimeError("oracle_evaluate_add_rows_interp failed")
        return unseen.value

    def __del__(self):
        if getattr(self, "h", None):
            port().oracle_interp_free(self.h)
            self.h = None


def search_interp_ref(basis: np.ndarray, queries: np.ndarray) -> np.ndarray:
    """The reference's ZBasisInterp::search: index, -1 absent, -2 where it throws (unseen high word)."""
    lib = ref()
    q = np.ascontiguousarray(queries, dtype=np.uint64)
    idx = np.zeros(len(q), np.int64)
    lib.ref_search_interp(_p(basis), C.c_int64(len(basis)), _p(q), C.c_int64(len(q)), _p(idx))
    return idx


def triplets_port(basis: np.ndarray, specs, tol: float = 1e-14):
    t = terms_array(specs)
    n = port().oracle_triplets(_p(basis), len(basis), _p(t), len(specs), tol, None, None, None)
    r = np.zeros(n, np.int64)
    c = np.zeros(n, np.int64)
    v = np.zeros(n, np.float64)
    port().oracle_triplets(_p(basis), len(basis), _p(t), len(specs), tol, _p(r), _p(c), _p(v))
    return r, c, v


# ------------------------------------------------------------------ reference-built wrappers
def _spec_args(specs):
    ops = (C.c_char_p * len(specs))(*[s[1].encode() for s in specs])
    idarrs = [np.ascontiguousarray(s[2], dtype=np.int32) for s in specs]
    ids = (C.c_void_p * len(specs))(*[a.ctypes.data for a in idarrs])
    lens = np.array([len(s[1]) for s in specs], dtype=np.int32)
    coef = np.array([s[0] for s in specs], dtype=np.float64)
    return ops, ids, lens, coef, idarrs


def term_masks_ref(ops: str, ids):
    lib = ref()
    ids = np.ascontiguousarray(ids, dtype=np.int32)
    m = np.zeros(8, np.uint64)
    sg = C.c_int()
    rc = lib.ref_term_masks(ops.encode(), _p(ids), len(ops), _p(m), C.byref(sg))
    if rc != 0:
        raise ValueError("bad operator spec")
    return m, sg.value


def apply_state_ref(ops: str, ids, state: int):
    """(new state, sign) of the reference's SymbolicPMROperator::applyState on a 128-bit state."""
    lib = ref()
    ids = np.ascontiguousarray(ids, dtype=np.int32)
    st = np.array([state & (2**64 - 1), state >> 64], dtype=np.uint64)
    sg = lib.ref_apply_state(ops.encode(), _p(ids), len(ops), _p(st))
    return int(st[0]) | (int(st[1]) << 64), int(sg)


def triplets_ref(basis: np.ndarray, specs, tol: float = 1e-14):
    lib = ref()
    ops, ids, lens, coef, keep = _spec_args(specs)
    args = (_p(basis), C.c_int64(len(basis)), ops, ids, _p(lens), _p(coef), C.c_int(len(specs)), C.c_double(tol))
    n = lib.ref_triplets(*args, None, None, None)
    r = np.zeros(n, np.int64)
    c = np.zeros(n, np.int64)
    v = np.zeros(n, np.float64)
    lib.ref_triplets(*args, _p(r), _p(c), _p(v))
    return r, c, v


def apply_ref(basis: np.ndarray, specs, x: np.ndarray, threads: int = 0):
    lib = ref()
    ops, ids, lens, coef, keep = _spec_args(specs)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros_like(x)
    lib.ref_evaluate_add(_p(basis), C.c_int64(len(basis)), ops, ids, _p(lens), _p(coef), C.c_int(len(specs)), _p(x),
                         _p(y), C.c_int(threads))
    return y


def search_ref(basis: np.ndarray, queries: np.ndarray):
    lib = ref()
    q = np.ascontiguousarray(queries, dtype=np.uint64)
    idx = np.zeros(len(q), np.int64)
    lib.ref_search(_p(basis), C.c_int64(len(basis)), _p(q), C.c_int64(len(q)), _p(idx))
    return idx


# ------------------------------------------------------------------ checksums and eigen-oracles
def triplet_digest(r, c, v) -> str:
    h = hashlib.sha256()
    for a in (r, c, v):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def save_market_port(r, c, v, n: int, path) -> int:
    """The MatrixMarket text Eigen::saveMarket writes for SparseMatrix::setFromTriplets(r, c, v)
    (src/build_hamiltonian.cpp:104-111; Eigen's MarketIO writer restated): duplicates summed in triplet
    order, column-major with rows ascending, explicit zeros kept, 1-based indices, values '%.17e'."""
    order = np.lexsort((r, c))  # stable: by column, then row, ties in triplet order
    rr, cc, vv = r[order], c[order], v[order]
    er, ec, ev = [], [], []
    for a, b, x in zip(rr.tolist(), cc.tolist(), vv.tolist()):
        if er and er[-1] == a and ec[-1] == b:
            ev[-1] += x
        else:
            er.append(a), ec.append(b), ev.append(x)
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate  real general\n")
        f.write(f"{n} {n} {len(ev)}\n")
        f.writelines("%d %d %.17e\n" % (a + 1, b + 1, x) for a, b, x in zip(er, ec, ev))
    return len(ev)


def csr_from_triplets(r, c, v, n):
    import scipy.sparse as sp

    return sp.csr_matrix((v, (r, c)), shape=(n, n))


def lowest_eigs(r, c, v, n, k=1, tol=1e-13, v0_seed=0):
    """FP64 eigen-oracle: numpy eigh (n <= 4000) or scipy eigsh(which='SA')."""
    H = csr_from_triplets(r, c, v, n)
    if n <= 4000:
        w, V = np.linalg.eigh(H.toarray())
        return w[:k], V[:, :k]
    from scipy.sparse.linalg import eigsh

    rng = np.random.default_rng(v0_seed)
    w, V = eigsh(H, k=k, which="SA", tol=tol, v0=rng.standard_normal(n), ncv=max(2 * k + 1, 30))
    o = np.argsort(w)
    return w[o], V[:, o]


def exact_thermo(evals: np.ndarray, temps: np.ndarray):
    """E(T), C(T) from a full spectrum with the ground state subtracted."""
    e = np.asarray(evals, np.float64)
    e0 = e.min()
    x = e - e0
    bf = np.exp(-np.outer(1.0 / np.asarray(temps), x))
    Z = bf.sum(1)
    E1 = (bf @ x) / Z
    E2 = (bf @ (x * x)) / Z
    return {"T": np.asarray(temps), "E": E1 + e0, "C": (E2 - E1 * E1) / np.asarray(temps) ** 2}


def ftlm_oracle(r, c, v, n, R, M, seed, temps):
    """Per-vector FP64 FTLM (plain Lanczos, M steps) over R Rademacher vectors, numpy on the CPU."""
    H = csr_from_triplets(r, c, v, n)
    rng = np.random.default_rng(seed)
    ev_all, w_all = [], []
    for _ in range(R):
        q = rng.choice([-1.0, 1.0], size=n) / np.sqrt(n)
        qp = np.zeros(n)
        a, b = [], []
        beta = 0.0
        for j in range(M):
            w = H @ q
            al = q @ w
            w = w - al * q - beta * qp
            beta = np.linalg.norm(w)
            a.append(al)
            b.append(beta)
            qp, q = q, w / beta
        T = np.diag(a) + np.diag(b[:-1], 1) + np.diag(b[:-1], -1)
        ew, Y = np.linalg.eigh(T)
        ev_all.append(ew)
        w_all.append(Y[0] ** 2)
    ev = np.array(ev_all)
    w = np.array(w_all)
    e0 = ev.min()
    x = (ev - e0).reshape(-1)
    ww = w.reshape(-1) * (n / R)
    bf = np.exp(-np.outer(1.0 / np.asarray(temps), x))
    Z = bf @ ww
    E1 = (bf @ (ww * x)) / Z
    E2 = (bf @ (ww * x * x)) / Z
    return {"T": np.asarray(temps), "E": E1 + e0, "C": (E2 - E1 * E1) / np.asarray(temps) ** 2, "ritz": ev,
            "weights": w}


def _splitmix64(z: np.ndarray) -> np.ndarray:
    """SplitMix64 finaliser (Steele, Lea, Flood 2014), elementwise on uint64 (wrapping arithmetic)."""
    z = (z + np.uint64(0x9E3779B97F4A7C15)).astype(np.uint64)
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)).astype(np.uint64)
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)).astype(np.uint64)
    return z ^ (z >> np.uint64(31))


def ftlm_start_vectors(n: int, R: int, seed: int) -> np.ndarray:
    """The engine's FTLM start block for one sector, restated: element (i, r) is +1/sqrt(n) when the top bit of
    splitmix64(seed ^ splitmix64((r << 40) ^ i)) is set, else -1/sqrt(n).  Returns (n, R) FP64 (the
    Rademacher start vectors of the FTLM workload; a sector s of a multi-sector run uses seed + s)."""
    i = np.arange(n, dtype=np.uint64)
    inv = 1.0 / np.sqrt(float(n))
    out = np.empty((n, R))
    with np.errstate(over="ignore"):
        for r in range(R):
            h = _splitmix64(np.uint64(seed) ^ _splitmix64((np.uint64(r) << np.uint64(40)) ^ i))
            out[:, r] = np.where((h >> np.uint64(63)) != 0, inv, -inv)
    return out


def ftlm_recurrences(r, c, v, n, Q0: np.ndarray, M: int):
    """Per-vector FP64 three-term Lanczos from the given start vectors (columns of Q0), M steps each:
    w = H q; alpha = <q, w>; w -= alpha q + beta_prev q_prev; beta = |w|; q_prev, q = q, w / beta.
    Returns (alphas, betas), each (R, M) -- the standard FTLM recurrence the ftlm workload defines (the
    reference's own C++ FTLM, include/ftlm.hpp:19-142, is unbuilt)."""
    H = csr_from_triplets(r, c, v, n)
    R = Q0.shape[1]
    A = np.zeros((R, M))
    B = np.zeros((R, M))
    for k in range(R):
        q = Q0[:, k].copy()
        qp = np.zeros(n)
        beta = 0.0
        for j in range(M):
            w = H @ q
            al = float(q @ w)
            w -= al * q + beta * qp
            beta = float(np.sqrt(w @ w))
            A[k, j], B[k, j] = al, beta
            qp, q = q, w / beta
    return A, B


def ftlm_thermo_oracle(alphas, betas, n: int, temps, e_ref: float | None = None):
    """E(T) and C(T) from FTLM recurrences: Ritz values e_rj and weights (first eigenvector component)^2 of each
    tridiagonal by numpy eigh, Z = n/R sum exp(-(e - e_ref)/T) w, C = (<E^2> - <E>^2) / T^2."""
    R, M = alphas.shape
    ev, ww = [], []
    for k in range(R):
        T = np.diag(alphas[k]) + np.diag(betas[k, :-1], 1) + np.diag(betas[k, :-1], -1)
        w, Y = np.linalg.eigh(T)
        ev.append(w)
        ww.append(Y[0] ** 2)
    ev = np.array(ev)
    e0 = float(ev.min()) if e_ref is None else e_ref
    x = (ev - e0).reshape(-1)
    wt = np.array(ww).reshape(-1) * (n / R)
    temps = np.asarray(temps, np.float64)
    bf = np.exp(-np.outer(1.0 / temps, x))
    Z = bf @ wt
    E1 = (bf @ (wt * x)) / Z
    E2 = (bf @ (wt * x * x)) / Z
    return {"T": temps, "E": E1 + e0, "C": (E2 - E1 * E1) / temps ** 2, "e_ref": e0}


def ring_zeeman_specs(lat: dict, g, B, Jpm: float = 0.0, kappa: float = 0.5):
    """Term list [(c, op characters, spin ids)] of H = -sum_hex g[sl] (O + O^dagger) - sum_i (B . z_a(i)) kappa
    z_i [- Jpm sum_bonds (S+_i S-_j + h.c.)], off-diagonal terms first, each group in insertion order
    (SymbolicOpSum::add_term's split, components/operator/include/operator.hpp:489-495).  Ring operators follow
    get_ring_ops (include/physics/geometry.hpp:29-62: six-member rings only, sign +1 -> '+', -1 -> '-', O^dagger
    with the signs flipped) and are added as (-g, O^dagger) then (-g, O) per hexagon, as
    include/hamiltonian_setup.hpp:36-43 adds them with its coupling; z_a are the rows of get_loc_z
    (include/physics/Jring.hpp:6-14), B . z_a summed as (B0 z0 + B1 z1) + B2 z2."""
    off, diag = [], []
    for ring in lat.get("rings", []):
        ids = [int(i) for i in ring["member_spin_idx"]]
        if len(ids) != 6:
            continue
        ops = "".join("+" if v == 1 else "-" for v in ring["signs"])
        conj = "".join("-" if v == 1 else "+" for v in ring["signs"])
        off.append((-float(g[int(ring["sl"])]), conj, ids))
        off.append((-float(g[int(ring["sl"])]), ops, ids))
    if Jpm:
        for bond in lat.get("bonds", []):
            i, j = int(bond["from_idx"]), int(bond["to_idx"])
            off.append((-float(Jpm), "+-", [i, j]))
            off.append((-float(Jpm), "-+", [i, j]))
    lz = np.array([[1.0, 1.0, 1.0], [1.0, -1.0, -1.0], [-1.0, 1.0, -1.0], [-1.0, -1.0, 1.0]]) / np.sqrt(3.0)
    for i, a in enumerate(lat["atoms"]):
        z = lz[int(a["sl"])]
        h = (float(B[0]) * float(z[0]) + float(B[1]) * float(z[1])) + float(B[2]) * float(z[2])
        diag.append((-h * kappa, "z", [i]))
    return off + diag


def enumerate_basis_oracle(lat: dict, sector=None, n_spinon_pairs: int = 0, threads: int = 0) -> np.ndarray:
    """The reference's basis enumeration restated (oracle/enumerate_oracle.c): sorted (n, 2) uint64 (lo, hi)
    rows for a lattice dict (atoms[{sl}], tetrahedra[{member_spin_idx}]); sector = per-sublattice up counts."""
    sl = np.array([int(a["sl"]) for a in lat["atoms"]], dtype=np.int32)
    mem = [list(t["member_spin_idx"]) for t in lat["tetrahedra"]]
    off = np.zeros(len(mem) + 1, dtype=np.int32)
    off[1:] = np.cumsum([len(m) for m in mem])
    flat = np.array([i for m in mem for i in m], dtype=np.int32)
    sec = None if sector is None else np.ascontiguousarray(sector, dtype=np.int32)
    out = C.POINTER(C.c_uint64)()
    n = port().oracle_enumerate(len(sl), _p(sl), len(mem), _p(off), _p(flat), None if sec is None else _p(sec),
                                0 if sec is None else len(sec), int(n_spinon_pairs), int(threads), C.byref(out))
    if n < 0:
        raise MemoryError("oracle_enumerate failed (bad lattice or out of memory)")
    try:
        a = np.ctypeslib.as_array(out, shape=(max(int(n), 1) * 2,))[: 2 * int(n)].copy()
    finally:
        port().oracle_free(out)
    return a.reshape(-1, 2)


def set_random_unit(n: int, seed: int) -> np.ndarray:
    v = np.zeros(n)
    port().oracle_set_random_unit(_p(v), n, seed)
    return v


def eigval0_oracle(r, c, v, n, seed, abs_tol=1e-8, rel_tol=1e-8, min_iterations=10, max_iterations=5000):
    """projED::lanczos::eigval0 restated in numpy (components/linalg_routines/src/lanczos.cpp:67-227):
    first pass to max_iterations (or beta < abs_tol) without stopping on convergence, lowest
    Ritz pair of the full tridiagonal, second pass accumulating the Ritz vector until the
    lowest Ritz value changes by less than abs_tol / rel_tol.  Returns (E0, eigvec, iterations)."""
    from scipy.linalg import eigh_tridiagonal

    A = csr_from_triplets(r, c, v, n)
    v0 = set_random_unit(n, seed)

    def run(ritz):
        vv, u = v0.copy(), np.zeros(n)
        al, be = [], []
        beta, eig = 0.0, np.inf
        ev = np.zeros(n) if ritz is not None else None
        it = 0
        for it in range(max_iterations + 1):
            if it == max_iterations:  # loop ran out: n_iterations == max_iterations, as in C
                break
            if ritz is not None and it < len(ritz):
                ev += ritz[it] * vv
            if it > 0:
                u *= -beta
            u += A @ vv
            a = vv @ u
            u -= a * vv
            beta = np.sqrt(u @ u)
            if beta < abs_tol:
                break
            vv, u = u, vv
            vv *= 1 / beta
            al.append(a)
            be.append(beta)
            if ritz is not None and it >= min_iterations:
                e = eigh_tridiagonal(np.array(al), np.array(be[:-1]), eigvals_only=True, select="i",
                                     select_range=(0, 0))[0]
                err = abs(e - eig)
                eig = e
                if err < abs_tol or err / max(abs(e), 1e-10) < rel_tol:
                    break
        return al, be, ev, it

    al, be, _, its = run(None)
    w, Y = eigh_tridiagonal(np.array(al), np.array(be[:-1]), select="i", select_range=(0, 0))
    _, _, ev, _ = run(Y[:, 0])
    return float(w[0]), ev, its


def cpu_threads() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
