"""GPU apply, lookup and connectivity through the C-ABI against the oracle."""
import ctypes as C

import numpy as np
import pytest

import qsi_subspace_ed_gb300 as q
from helpers import GOLDEN, cases, golden_json, wide_case
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = ["golden48_JpmB", "ref32_g", "ref32_JpmB", "q0_32", "s4444"]


@pytest.fixture(scope="module")
def built():
    out = {}
    for name, (basis, H) in cases().items():
        b = q.ZBasis(basis)
        out[name] = (basis, H, b, q.LazyOpSum(b, H))
    return out


@pytest.mark.parametrize("name", CASES)
def test_triplets_bit_exact(built, name):
    basis, H, b, op = built[name]
    r, c, v = op.triplets()
    ref = golden_json("triplets.json")[name]
    assert len(r) == ref["n_triplets"]
    assert O.triplet_digest(r, c, v) == ref["sha256"]
    ro, co, vo = O.triplets_port(basis, H.specs())
    assert np.array_equal(r, ro) and np.array_equal(c, co) and np.array_equal(v, vo)


@pytest.mark.parametrize("name", CASES)
def test_search_exact(built, name):
    basis, H, b, op = built[name]
    idx = b.search(basis)
    assert np.array_equal(idx, np.arange(len(basis)))
    # flipped non-members: not found
    rng = np.random.default_rng(1)
    probe = basis[rng.integers(0, len(basis), 500)].copy()
    probe[:, 0] ^= np.uint64(1)
    member = {tuple(x) for x in basis.tolist()}
    expect = np.array([(-1 if tuple(p) not in member else None) for p in probe.tolist()], dtype=object)
    got = b.search(probe)
    for e, g, p in zip(expect, got, probe.tolist()):
        if e is None:
            assert basis[g].tolist() == p
        else:
            assert g == -1
    # beyond the top bucket and the empty state
    assert b.search(np.array([[0, 2**63]], np.uint64))[0] == -1
    assert q.ZBasis(basis[:1]).search(basis[:2]).tolist() == [0, -1]


@pytest.mark.parametrize("name", CASES)
def test_apply_fp64_matches_oracle(built, name):
    basis, H, b, op = built[name]
    x = np.random.default_rng(7).standard_normal(len(basis))
    y_ref = O.apply_port(basis, H.specs(), x, threads=1)
    y = np.zeros_like(x)
    op.evaluate(x, y)
    np.testing.assert_allclose(y, y_ref, rtol=0, atol=1e-12 * np.abs(y_ref).max())
    # deterministic (pull form, fixed summation order)
    y2 = np.zeros_like(x)
    op.evaluate(x, y2)
    assert np.array_equal(y, y2)
    # accumulate: y += H x
    y3 = x.copy()
    op.evaluate_add(x, y3)
    np.testing.assert_allclose(y3, x + y_ref, rtol=0, atol=1e-12 * np.abs(y_ref).max())


def test_apply_matches_reference_stored_applies(built):
    for fname, name in [("apply_ref32.npy", "ref32_g"), ("apply_q0_32.npy", "q0_32")]:
        x, y_ref = np.load(GOLDEN / fname)
        y = np.zeros_like(x)
        built[name][3].evaluate(x, y)
        np.testing.assert_allclose(y, y_ref, rtol=0, atol=1e-12 * np.abs(y_ref).max())


def test_apply_tol_skips_tiny_sources(built):
    basis, H, b, op = built["q0_32"]
    x = np.zeros(len(basis))
    x[5] = 1.0
    x[17] = 5e-16  # below APPLY_TOL: its off-diagonal pushes are dropped
    y = np.zeros_like(x)
    op.evaluate(x, y)
    np.testing.assert_allclose(y, O.apply_port(basis, H.specs(), x, threads=1), rtol=0, atol=1e-15)


@pytest.mark.parametrize("R", [1, 3, 32, 64, 100])
def test_batched_apply(built, R):
    basis, H, b, op = built["golden48_JpmB"]
    n = len(basis)
    X = np.random.default_rng(R).standard_normal((n, R))
    Y = np.zeros_like(X)
    op.apply_batched(X, Y)
    cols = [0, R - 1, R // 2]
    for c in cols:
        y = np.zeros(n)
        op.evaluate(np.ascontiguousarray(X[:, c]), y)
        np.testing.assert_allclose(Y[:, c], y, rtol=0, atol=1e-12 * np.abs(y).max())
    X32 = X.astype(np.float32)
    Y32 = np.zeros_like(X32)
    op.apply_batched(X32, Y32)
    Yd = np.zeros_like(X)
    op.apply_batched(X32.astype(np.float64), Yd)
    np.testing.assert_allclose(Y32, Yd, rtol=2e-6, atol=2e-6 * np.abs(Yd).max())


def test_device_pointers_and_stream(built):
    torch = pytest.importorskip("torch")
    basis, H, b, op = built["q0_32"]
    x = torch.randn(len(basis), dtype=torch.float64, device="cuda")
    y = torch.zeros_like(x)
    op.evaluate(x, y)
    torch.cuda.synchronize()
    y_ref = O.apply_port(basis, H.specs(), x.cpu().numpy(), threads=1)
    np.testing.assert_allclose(y.cpu().numpy(), y_ref, rtol=0, atol=1e-12 * np.abs(y_ref).max())


def test_pinned_host_result_buffers(built):
    """Host pointers into page-locked buffers: the result is written straight into the host buffer (no staging
    copy) and equals the staged and the device-pointer applies bitwise; accumulation still adds to it."""
    torch = pytest.importorskip("torch")
    basis, H, b, op = built["q0_32"]
    n, R = len(basis), 32
    xh = torch.randn(n, dtype=torch.float64).pin_memory()
    yh = torch.full((n,), 3.0, dtype=torch.float64).pin_memory()
    lib = q.load()
    assert lib.qsi_op_apply(op._h, C.c_void_p(xh.data_ptr()), C.c_void_p(yh.data_ptr()), 0, 0, None) == 0
    y_staged = np.zeros(n)
    op.evaluate(xh.numpy(), y_staged)
    assert np.array_equal(yh.numpy(), y_staged)
    assert lib.qsi_op_apply(op._h, C.c_void_p(xh.data_ptr()), C.c_void_p(yh.data_ptr()), 1, 0, None) == 0
    assert np.array_equal(yh.numpy(), 2 * y_staged)
    Xh = torch.randn(n, R, dtype=torch.float32).pin_memory()
    Yh = torch.zeros(n, R, dtype=torch.float32).pin_memory()
    assert lib.qsi_op_apply_batched(op._h, C.c_void_p(Xh.data_ptr()), C.c_void_p(Yh.data_ptr()), R, 1, 0, 0,
                                    None) == 0
    Xd = Xh.cuda()
    Yd = torch.zeros_like(Xd)
    op.apply_batched(Xd, Yd)
    torch.cuda.synchronize()
    assert np.array_equal(Yh.numpy(), Yd.cpu().numpy())


def test_projected_hopping_drops_misses():
    """Bond hopping leaves the ice manifold: misses are dropped, as the reference's push loop does."""
    from qsi_subspace_ed_gb300 import workloads

    lat = workloads.lattice("pyro_1x2x1")
    basis = q.enumerate_basis(lat)
    H = q.build_ring_zeeman(lat, [1, .8, .6, .4], [0.1, 0.2, -0.1], Jpm=0.05)
    b = q.ZBasis(basis)
    op = q.LazyOpSum(b, H)
    assert op.count_misses() > 0
    x = np.random.default_rng(3).standard_normal(len(basis))
    y = np.zeros_like(x)
    op.evaluate(x, y)
    y_ref = O.apply_port(basis, H.specs(), x, threads=1)
    np.testing.assert_allclose(y, y_ref, rtol=0, atol=1e-12 * np.abs(y_ref).max())
    r, c, v = op.triplets()
    assert O.triplet_digest(r, c, v) == O.triplet_digest(*O.triplets_port(basis, H.specs()))


def test_basis_errors():
    with pytest.raises(q.QsiError):
        q.ZBasis(np.array([[5, 0], [3, 0]], np.uint64))  # not increasing
    with pytest.raises(q.QsiError):
        q.ZBasis(np.zeros((0, 2), np.uint64))


@pytest.mark.parametrize("name", CASES)
def test_kernel_variants_bit_identical(built, name):
    """Row-per-thread, bit-sliced tiles, table and hash lookups: same sums in the same order."""
    basis, H, b, op = built[name]
    x = np.random.default_rng(11).standard_normal(len(basis))
    X = np.random.default_rng(12).standard_normal((len(basis), 40))
    outs, bouts = [], []
    for kernel, use_hash in [(0, 0), (1, 0), (1, 1), (0, 1)]:
        op.set_kernel(kernel, use_hash)
        y = np.zeros_like(x)
        op.evaluate(x, y)
        outs.append(y)
        Y = np.zeros_like(X)
        op.apply_batched(X, Y)
        bouts.append(Y)
    # narrow and wide bucket tables (buckets of thousands of states, and bucket numbers in every position of the
    # table's groups of four), with the bisection and with the regional hash, whose regions are the table's buckets
    # and are rebuilt with it
    bits0 = b.index_info()["bucket_bits"]
    for bits in (8, 12, 31):
        b.set_index(use_hash=True, bucket_bits=bits)
        assert b.index_info()["hash"]
        for use_hash in (0, 1):
            op.set_kernel(1, use_hash)
            y = np.zeros_like(x)
            op.evaluate(x, y)
            outs.append(y)
            Y = np.zeros_like(X)
            op.apply_batched(X, Y)
            bouts.append(Y)
    b.set_index(use_hash=True, bucket_bits=bits0)
    op.set_kernel(1, 1)
    for y in outs[1:]:
        assert np.array_equal(y, outs[0])
    for Y in bouts[1:]:
        assert np.array_equal(Y, bouts[0])


def test_hash_index_and_table_sizes(built):
    basis, H, b, op = built["golden48_JpmB"]
    info = b.index_info()
    assert info["hash"]
    for bits in (8, 12, 20):
        b.set_index(use_hash=False, bucket_bits=bits)
        assert b.index_info()["bucket_bits"] == bits and not b.index_info()["hash"]
        assert np.array_equal(b.search(basis[::97]), np.arange(0, len(basis), 97))
    b.set_index(use_hash=True, bucket_bits=0)
    assert b.index_info()["hash"]


def test_batched_hit_list_overflow_chunks(built):
    """A small hit list forces the batched tile kernel to split tiles into row chunks."""
    basis, H, b, op = built["golden48_JpmB"]
    X = np.random.default_rng(5).standard_normal((len(basis), 8))
    Y1, Y2 = np.zeros_like(X), np.zeros_like(X)
    op.set_kernel(1, 1, list_cap=512)
    op.apply_batched(X, Y1)
    op.set_kernel(1, 1, list_cap=8)  # raised to the term count internally
    op.apply_batched(X, Y2)
    op.set_kernel(1, 1, list_cap=512)
    assert np.array_equal(Y1, Y2)


def test_double_float_accumulation_matches_fp64(built):
    """FP32 batched applies: double-float row accumulation agrees with FP64 accumulation to FP32 output rounding."""
    basis, H, b, op = built["golden48_JpmB"]
    X = np.random.default_rng(21).standard_normal((len(basis), 64)).astype(np.float32)
    Yff, Y64 = np.zeros_like(X), np.zeros_like(X)
    op.set_kernel(1, 1)
    op.apply_batched(X, Yff)
    op.set_kernel(1, 1 | 2)
    op.apply_batched(X, Y64)
    op.set_kernel(1, 1)
    ulp = np.spacing(np.abs(Y64).astype(np.float32))
    assert np.all(np.abs(Yff - Y64) <= ulp)
    Yacc = Y64.copy()
    op.apply_batched(X, Yacc, accumulate=True)
    np.testing.assert_allclose(Yacc, 2 * Y64, rtol=1e-6, atol=1e-6 * np.abs(Y64).max())


@pytest.mark.parametrize("vw", [4, 8, 16])
@pytest.mark.parametrize("R", [16, 24, 32, 64, 128, 256, 512])
def test_fp32_batched_widths(built, R, vw):
    """FP32 batched applies at vector counts that take 16-byte gathers (16..128, multiples of 128) and one that
    does not (24): each within one FP32 ulp of FP64 accumulation, equal to the oracle's FP64 apply to FP32
    rounding, and bitwise independent of the hit-list size."""
    basis, H, b, op = built["ref32_JpmB"]
    X = np.random.default_rng(R).standard_normal((len(basis), R)).astype(np.float32)
    Yff, Y64, Ysmall = np.zeros_like(X), np.zeros_like(X), np.zeros_like(X)
    op.set_tuning(0, 0, which=1, vec_width=vw)
    op.set_kernel(1, 1)
    op.apply_batched(X, Yff)
    op.set_kernel(1, 1, list_cap=8)
    op.apply_batched(X, Ysmall)
    op.set_kernel(1, 1 | 2)
    op.apply_batched(X, Y64)
    op.set_kernel(1, 1)
    op.set_tuning(0, 0, which=1)
    assert np.array_equal(Yff, Ysmall)
    assert np.all(np.abs(Yff - Y64) <= np.spacing(np.abs(Y64).astype(np.float32)))
    for col in (0, R - 1):
        ref = O.apply_port(basis, H.specs(), X[:, col].astype(np.float64))
        np.testing.assert_allclose(Yff[:, col], ref, rtol=0, atol=4e-6 * np.abs(ref).max())


def test_fp32_batched_unaligned_device_vectors(built):
    """Device vectors that are not 16-byte aligned take the one-column-per-load path: same values to FP32 rounding."""
    torch = pytest.importorskip("torch")
    basis, H, b, op = built["ref32_JpmB"]
    n, R = len(basis), 32
    X = np.random.default_rng(3).standard_normal((n, R)).astype(np.float32)
    Y = np.zeros_like(X)
    op.apply_batched(X, Y)
    xb = torch.zeros(n * R + 1, dtype=torch.float32, device="cuda")
    yb = torch.zeros(n * R + 1, dtype=torch.float32, device="cuda")
    xd, yd = xb[1:].view(n, R), yb[1:].view(n, R)
    xd.copy_(torch.from_numpy(X))
    op.apply_batched(xd, yd)
    torch.cuda.synchronize()
    Yd = yd.cpu().numpy()
    assert np.all(np.abs(Yd - Y) <= np.spacing(np.abs(Y)))


def test_autotune_keeps_results(built):
    """The autotuner changes launch settings only: applies before and after are bitwise equal."""
    basis, H, b, op = built["q0_32"]
    x = np.random.default_rng(31).standard_normal(len(basis))
    X = np.random.default_rng(32).standard_normal((len(basis), 64)).astype(np.float32)
    y0, Y0 = np.zeros_like(x), np.zeros_like(X)
    op.evaluate(x, y0)
    op.apply_batched(X, Y0)
    log1 = op.autotune(R=1, dtype="f64", tune_index=True, reps=1)
    log64 = op.autotune(R=64, dtype="f32", reps=1)
    assert "best" in log1 and "vec_chunk" in log64
    t = op.tuning(1)
    y1, Y1 = np.zeros_like(x), np.zeros_like(X)
    op.evaluate(x, y1)
    op.apply_batched(X, Y1)
    assert np.array_equal(y0, y1) and np.array_equal(Y0, Y1)
    for vw, vc in ((4, 16), (4, 32), (4, 64), (8, 16), (8, 32), (8, 64), (16, 16), (16, 64)):
        op.set_tuning(t["grid_bps"], vc, which=1, vec_width=vw)
        Y2 = np.zeros_like(X)
        op.apply_batched(X, Y2)
        assert np.array_equal(Y0, Y2), (vw, vc)
    with pytest.raises(q.QsiError):
        op.set_tuning(0, 48)
    op.set_tuning(0, 0)
    op.set_kernel(1, 1, list_cap=256)
    b.set_index(use_hash=True, bucket_bits=0)


def test_terms_never_landing_in_the_basis_are_pruned(built):
    """Bond hopping on an ice-rule (Q=0) basis always leaves it: those terms are removed at creation, and the
    apply (single and batched) still equals the oracle's push loop over all terms; with two spinon pairs some
    hops stay in the basis and are kept."""
    from qsi_subspace_ed_gb300 import workloads

    lat = workloads.lattice("pyro_1x2x1")
    H = q.build_ring_zeeman(lat, [1, .8, .6, .4], [0.1, 0.2, -0.1], Jpm=0.05)
    n_hop = sum(1 for c, ops, ids in H.specs() if ops in ("+-", "-+"))
    for pairs, all_pruned in ((0, True), (2, False)):
        basis = q.enumerate_basis(lat, n_spinon_pairs=pairs)
        op = q.LazyOpSum(q.ZBasis(basis), H)
        info = op.info()
        assert (info["pruned"] == n_hop) if all_pruned else (info["pruned"] < n_hop), (pairs, info, n_hop)
        x = np.random.default_rng(41).standard_normal(len(basis))
        y = np.zeros_like(x)
        op.evaluate(x, y)
        ref = O.apply_port(basis, H.specs(), x, threads=1)
        np.testing.assert_allclose(y, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
        X = np.random.default_rng(42).standard_normal((len(basis), 32)).astype(np.float32)
        Y = np.zeros_like(X)
        op.apply_batched(X, Y)
        ref0 = O.apply_port(basis, H.specs(), X[:, 0].astype(np.float64), threads=1)
        np.testing.assert_allclose(Y[:, 0], ref0, rtol=0, atol=4e-6 * np.abs(ref0).max())
    # the ring-only Hamiltonian on its sector keeps every term
    assert built["s4444"][3].info()["pruned"] == 0


@pytest.mark.parametrize("name", ["ref32_g", "s4444"])
def test_matrix_market_export(built, name, tmp_path):
    """saveMarket of the GPU triplets is byte-identical to the oracle's restatement of Eigen's writer over the
    oracle's triplets, and reads back (scipy) as the same matrix."""
    import scipy.io

    basis, H, b, op = built[name]
    p_gpu, p_ora = tmp_path / "gpu.mtx", tmp_path / "oracle.mtx"
    nnz = op.saveMarket(p_gpu)
    r, c, v = O.triplets_port(basis, H.specs())
    assert O.save_market_port(r, c, v, len(basis), p_ora) == nnz
    assert p_gpu.read_bytes() == p_ora.read_bytes()
    M = scipy.io.mmread(str(p_gpu)).tocsr()
    ref = O.csr_from_triplets(r, c, v, len(basis))
    assert abs(M - ref).max() == 0


def test_states_up_to_128_bits():
    """The 32-spin Q=0 basis and ring/Zeeman Hamiltonian with spin i moved to bit 4i+3 (states up to 128 bits,
    beyond the 96 bits the hash index takes): lookups go through the bucket table; connectivity and applies
    equal the reference code's (fixtures) and the oracle's."""
    lohi, Hw, specs = wide_case()
    assert int(lohi[:, 1].max()) >> 62  # bits above 96 are in use
    b = q.ZBasis(lohi)
    assert not b.index_info()["hash"]
    op = q.LazyOpSum(b, Hw)
    r, c, v = op.triplets()
    assert O.triplet_digest(r, c, v) == golden_json("wide128.json")["sha256"]
    x, y_ref = np.load(GOLDEN / "apply_wide128.npy")
    y = np.zeros_like(x)
    op.evaluate(x, y)
    np.testing.assert_allclose(y, y_ref, rtol=0, atol=1e-12 * np.abs(y_ref).max())
    x = np.random.default_rng(8).standard_normal(len(lohi))
    op.evaluate(x, y)
    ref = O.apply_port(lohi, specs, x, threads=1)
    np.testing.assert_allclose(y, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
    for bits in (12, 31):  # other table widths, bitwise the same
        b.set_index(use_hash=False, bucket_bits=bits)
        y2 = np.zeros_like(x)
        op.evaluate(x, y2)
        assert np.array_equal(y2, y)
    X = np.random.default_rng(9).standard_normal((len(lohi), 64)).astype(np.float32)
    for vw in (4, 8, 16):
        op.set_tuning(0, 0, which=1, vec_width=vw)
        Y = np.zeros_like(X)
        op.apply_batched(X, Y)
        ref0 = O.apply_port(lohi, specs, X[:, 5].astype(np.float64), threads=1)
        np.testing.assert_allclose(Y[:, 5], ref0, rtol=0, atol=4e-6 * np.abs(ref0).max())
    # materialised without a hash index (the cache filled through the bucket table): bitwise the same applies
    assert op.materialise(True) > 0
    y3 = np.zeros_like(x)
    op.evaluate(x, y3)
    assert np.array_equal(y3, y)
    Y3 = np.zeros_like(X)
    op.apply_batched(X, Y3)
    assert np.array_equal(Y3, Y)
    op.materialise(False)


def test_degenerate_sizes():
    """One-state basis, an operator without terms, and vector counts of 1 and 3 (no 16-byte path)."""
    one = np.array([[5, 0]], dtype=np.uint64)
    op = q.LazyOpSum(q.ZBasis(one), q.SymbolicOpSum())
    y = np.ones(1)
    op.evaluate(np.array([2.0]), y)
    assert y[0] == 0.0
    basis, H = cases()["s4444"]
    op2 = q.LazyOpSum(q.ZBasis(basis), H)
    for R in (1, 3):
        X = np.random.default_rng(R).standard_normal((len(basis), R))
        Y = np.zeros_like(X)
        op2.apply_batched(X, Y)
        for col in range(R):
            ref = O.apply_port(basis, H.specs(), X[:, col], threads=1)
            np.testing.assert_allclose(Y[:, col], ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def _materialised_case_ops():
    """The fixture cases, and a one-spinon-pair basis with bond hopping, whose hops land in the basis for some
    rows and leave it for others (cached misses)."""
    from qsi_subspace_ed_gb300 import workloads

    lat = workloads.lattice("pyro_1x2x1")
    basis = q.enumerate_basis(lat, n_spinon_pairs=1)
    H = q.build_ring_zeeman(lat, [1, .8, .6, .4], [0.1, 0.2, -0.1], Jpm=0.05)
    return basis, H


@pytest.mark.parametrize("name", CASES + ["pair1_hop"])
def test_materialised_applies_are_bitwise_matrix_free(built, name):
    """qsi_op_materialise: single-vector FP64/FP32, batched FP64 and double-float FP32 applies, plain and
    accumulating, bitwise equal to the matrix-free ones; freeing the cache restores the lookups."""
    if name == "pair1_hop":
        basis, H = _materialised_case_ops()
        b = q.ZBasis(basis)
        op = q.LazyOpSum(b, H)
        assert op.count_misses() > 0
    else:
        basis, H, b, op = built[name]
    n = len(basis)
    rng = np.random.default_rng(21)
    x = rng.standard_normal(n)
    X = rng.standard_normal((n, 24))
    X32 = rng.standard_normal((n, 64)).astype(np.float32)
    y0 = rng.standard_normal(n)

    def run():
        y = np.zeros_like(x)
        op.evaluate(x, y)
        ya = y0.copy()
        op.evaluate_add(x, ya)
        Y = np.zeros_like(X)
        op.apply_batched(X, Y)
        Y32 = np.zeros_like(X32)
        op.apply_batched(X32, Y32)
        return y, ya, Y, Y32

    ref = run()
    nb = op.materialise(True)
    assert nb >= 4 * n  # at least one column per row of the widest tile rows
    got = run()
    for a, g in zip(ref, got):
        assert np.array_equal(a, g)
    assert op.materialise(False) == 0
    for a, g in zip(ref, run()):
        assert np.array_equal(a, g)
