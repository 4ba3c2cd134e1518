"""GPU Lanczos / FTLM against the FP64 oracles and the reference's golden answer."""
import numpy as np
import pytest

import qsi_subspace_ed_gb300 as q
from helpers import GOLDEN, cases, golden_json
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_golden_e0_through_eigval0():
    """test/test_correct.sh: 48 spins, Jpm=0.02, B=(0.1,0.1,0.1), mfeig0, seed 11, atol/rtol 1e-9."""
    g = golden_json("golden48.json")
    basis, H = cases()["golden48_JpmB"]
    b = q.ZBasis(basis)
    op = q.LazyOpSum(b, H)
    e0, vec, its = q.eigval0(op, seed=g["rng_seed"], abs_tol=g["atol"], rel_tol=g["rtol"], min_iterations=10)
    assert abs(e0 - g["E0"]) <= g["eigval_tol"]
    # E0 and the iteration count equal the oracle restatement of eigval0 (same std::mt19937 start).
    # Its eigenvector is a Ritz vector of the full first-pass tridiagonal, accumulated over the second
    # pass only up to that pass's convergence step; with no reorthogonalisation the tridiagonal holds
    # many rounding-level copies of E0, so which copy is "lowest" (and the scale of the truncated sum)
    # differs between any two floating-point implementations, the reference's included.  Only its
    # direction is compared.
    r, c, v = O.triplets_port(basis, H.specs())
    e_o, vec_o, its_o = O.eigval0_oracle(r, c, v, len(basis), g["rng_seed"], g["atol"], g["rtol"])
    assert abs(e0 - e_o) < 1e-12 and its == its_o
    # the stored file holds a unit vector of the same direction
    ref = np.load(GOLDEN / "golden48_evec.npy").astype(np.float64)
    ov = abs(vec @ ref) / (np.linalg.norm(vec) * np.linalg.norm(ref))
    assert ov > 1 - 1e-4


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_q0_32spin_lowest_five(precision):
    """32-spin Q=0 basis (3,618 states): ncv=15, 5 eigenvalues, tol 1e-10, against the FP64 dense oracle."""
    basis, H = cases()["q0_32"]
    ref = golden_json("eigs_q0_32.json")["evals"]
    op = q.LazyOpSum(q.ZBasis(basis), H)
    w, V, rep = q.diagonalise(op, nev=5, ncv=15, tol=1e-10, seed=1, precision=precision,
                              polish_steps=2 if precision == "mixed" else 0)
    np.testing.assert_allclose(w, ref[:5], atol=1e-9)
    assert np.all(rep.residual[:5] < 1e-6)
    # eigenvectors: H v = lambda v
    for k in range(5):
        y = np.zeros(len(basis))
        op.evaluate(np.ascontiguousarray(V[:, k]), y)
        assert np.linalg.norm(y - w[k] * V[:, k]) < 1e-6 * np.linalg.norm(V[:, k])


def test_lanczos_small_dimension_exhausts_krylov_space():
    basis, H = cases()["s4444"]
    op = q.LazyOpSum(q.ZBasis(basis[:40]), H)
    w, V, rep = q.diagonalise(op, nev=3, ncv=60, tol=1e-12)
    r, c, v = O.triplets_port(basis[:40], H.specs())
    ref = np.linalg.eigvalsh(O.csr_from_triplets(r, c, v, 40).toarray())
    np.testing.assert_allclose(w, ref[:3], atol=1e-10)


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_ftlm_against_exact_thermodynamics(precision):
    basis, H = cases()["s4444"]
    th = np.load(GOLDEN / "thermo_s4444.npz")
    op = q.LazyOpSum(q.ZBasis(basis), H)
    (al, be), = q.ftlm([op], [64], M=60, seed=5, precision=precision)
    assert al.shape == (64, 60)
    out = q.ftlm_thermo(al, be, len(basis), th["T"])
    hi = th["T"] > 0.5
    np.testing.assert_allclose(out["C"][hi], th["C"][hi], rtol=0.15, atol=0.02)
    # the FTLM ground-state estimate is the exact one (FP32 vectors: to ~1e-7 relative)
    r, c, v = O.triplets_port(basis, H.specs())
    e_exact = np.linalg.eigvalsh(O.csr_from_triplets(r, c, v, len(basis)).toarray())[0]
    assert abs(out["e_ref"] - e_exact) < (1e-8 if precision == "f64" else 1e-6 * abs(e_exact))


def test_ftlm_mixed_matches_fp64():
    basis, H = cases()["q0_32"]
    op = q.LazyOpSum(q.ZBasis(basis), H)
    T = np.logspace(-2, 1, 200)
    (a64, b64), = q.ftlm([op], [32], M=50, seed=9, precision="f64")
    (a32, b32), = q.ftlm([op], [32], M=50, seed=9, precision="mixed")
    t64 = q.ftlm_thermo(a64, b64, len(basis), T)
    t32 = q.ftlm_thermo(a32, b32, len(basis), T)
    np.testing.assert_allclose(a32[:, :10], a64[:, :10], atol=1e-5)
    np.testing.assert_allclose(t32["C"], t64["C"], rtol=1e-3, atol=1e-4)


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_ftlm_two_block_recurrence(precision):
    """The in-place two-block recurrence (H q accumulated into the previous vector block) gives the three-block
    recurrences up to rounding and the same thermodynamics, in single- and multi-sector launches."""
    cs = cases()
    names = ["q0_32", "s4444"]
    ops = [q.LazyOpSum(q.ZBasis(cs[n][0]), cs[n][1]) for n in names]
    three = q.ftlm(ops, [32, 16], M=40, seed=6, precision=precision, blocks=3)
    two = q.ftlm(ops, [32, 16], M=40, seed=6, precision=precision, blocks=2)
    alone = q.ftlm(ops[:1], [32], M=40, seed=6, precision=precision, blocks=2)
    T = np.logspace(-2, 1, 100)
    tol = 1e-10 if precision == "f64" else 1e-5
    for (a3, b3), (a2, b2), name in zip(three, two, names):
        np.testing.assert_allclose(a2[:, :10], a3[:, :10], rtol=0, atol=tol)
        np.testing.assert_allclose(b2[:, :10], b3[:, :10], rtol=0, atol=tol)
        t3 = q.ftlm_thermo(a3, b3, len(cs[name][0]), T)
        t2 = q.ftlm_thermo(a2, b2, len(cs[name][0]), T)
        np.testing.assert_allclose(t2["C"], t3["C"], rtol=1e-3, atol=1e-4)
    np.testing.assert_allclose(alone[0][0][:, :10], two[0][0][:, :10], rtol=0, atol=tol)
    with pytest.raises(q.QsiError):
        q.ftlm(ops[:1], [8], M=5, blocks=4)


def test_ftlm_multi_sector_batch():
    cs = cases()
    ops = [q.LazyOpSum(q.ZBasis(cs[n][0]), cs[n][1]) for n in ["q0_32", "s4444"]]
    res = q.ftlm(ops, [32, 16], M=30, seed=2, precision="mixed")
    assert [r[0].shape for r in res] == [(32, 30), (16, 30)]
    # each sector alone (seed + sector index) gives bit-identical recurrences
    alone = q.ftlm([ops[1]], [16], M=30, seed=3, precision="mixed")
    assert np.array_equal(alone[0][0], res[1][0]) and np.array_equal(alone[0][1], res[1][1])


def test_ftlm_sector_launch_lookup_and_tuning_independent():
    """The one-launch sector apply gives the same recurrences with hash or bucket-table lookups and under any
    launch settings."""
    cs = cases()
    ops = [q.LazyOpSum(q.ZBasis(cs[n][0]), cs[n][1]) for n in ["q0_32", "s4444"]]
    ref = q.ftlm(ops, [64, 64], M=20, seed=4, precision="mixed")
    for vw in (4, 8, 16):
        for op in ops:
            op.set_kernel(1, 0)  # bucket table
            op.set_tuning(4, 16, which=1, vec_width=vw)
        other = q.ftlm(ops, [64, 64], M=20, seed=4, precision="mixed")
        for (a, b), (c, d) in zip(ref, other):
            assert np.array_equal(a, c) and np.array_equal(b, d)
    for op in ops:
        op.set_kernel(1, 1)
        op.set_tuning(0, 0)
    # materialised sectors (the lookup caches in the same one-launch apply): bitwise the same recurrences
    for op in ops:
        assert op.materialise(True) > 0
    other = q.ftlm(ops, [64, 64], M=20, seed=4, precision="mixed")
    for (a, b), (c, d) in zip(ref, other):
        assert np.array_equal(a, c) and np.array_equal(b, d)
    for op in ops:
        op.materialise(False)


def test_tridiag_ritz_matches_numpy():
    rng = np.random.default_rng(4)
    a = rng.standard_normal((5, 40))
    b = np.abs(rng.standard_normal((5, 40))) + 0.1
    ev, first = q.tridiag_ritz(a, b)
    for k in range(5):
        T = np.diag(a[k]) + np.diag(b[k, :-1], 1) + np.diag(b[k, :-1], -1)
        w, Y = np.linalg.eigh(T)
        np.testing.assert_allclose(ev[k], w, atol=1e-12)
        np.testing.assert_allclose(first[k] ** 2, Y[0] ** 2, atol=1e-10)


def test_eigval0_checkpoint_resume_is_bitwise(tmp_path):
    """A run stopped at an iteration limit and resumed from its checkpoint gives the uninterrupted result bitwise;
    the checkpoint file holds the reference's checkpoint datasets."""
    basis, H = cases()["q0_32"]
    op = q.LazyOpSum(q.ZBasis(basis), H)
    kw = dict(seed=5, max_iterations=150, min_iterations=10, abs_tol=1e-10, rel_tol=1e-10)
    e_ref, v_ref, it_ref = q.eigval0(op, **kw)
    path = tmp_path / "ckpt.h5"
    with pytest.raises(q.QsiError) as ex:
        q.eigval0(op, checkpoint=path, checkpoint_every=20, stop_after=57, **kw)
    assert ex.value.status == 5  # QSI_TIMEOUT
    al = q.read_f64_h5(path, "alphas")
    v = q.read_f64_h5(path, "v")
    assert len(al) == 57 and len(v) == len(basis) and abs(np.linalg.norm(v) - 1) < 1e-12
    assert np.isfinite(q.read_f64_h5(path, "eigval")).all()
    with pytest.raises(q.QsiError):  # a second interruption, resumed from the first checkpoint
        q.eigval0(op, checkpoint=path, stop_after=40, **kw)
    assert len(q.read_f64_h5(path, "alphas")) == 97
    e, vec, its = q.eigval0(op, checkpoint=path, checkpoint_every=20, **kw)
    assert e == e_ref and its == it_ref and np.array_equal(vec, v_ref)
    # a checkpoint of another seed is refused
    with pytest.raises(q.QsiError):
        q.eigval0(op, checkpoint=path, **{**kw, "seed": 6})


@pytest.mark.parametrize("nev", [5, 10])
def test_block_mixed_solver_matches_dense_oracle(nev):
    """Block Lanczos on FP32 blocks of 16 vectors through the batched apply (kept Ritz blocks 1 and 2), then the
    FP64 polish: the lowest eigenvalues of the 32-spin Q=0 basis within 1e-9 of the dense FP64 oracle."""
    basis, H = cases()["q0_32"]
    ref = golden_json("eigs_q0_32.json")["evals"]
    op = q.LazyOpSum(q.ZBasis(basis), H)
    w, V, rep = q.diagonalise(op, nev=nev, ncv=24, tol=1e-10, seed=3, precision="mixed", polish_steps=2, block=16)
    np.testing.assert_allclose(w, ref[:nev], atol=1e-9)
    assert np.all(rep.residual[:nev] < 1e-6)
    for k in range(nev):
        y = np.zeros(len(basis))
        op.evaluate(np.ascontiguousarray(V[:, k]), y)
        assert np.linalg.norm(y - w[k] * V[:, k]) < 1e-6 * np.linalg.norm(V[:, k])


@pytest.mark.parametrize("block, polish", [(16, 2), (0, 2), (0, 3)])
def test_mixed_solvers_match_fp64_on_a_larger_sector(block, polish):
    """The 64-spin 8.8.8.8 sector (221,628 states): ten lowest eigenvalues of the FP32 solves with FP64 polish
    (block Lanczos, and single-vector Lanczos with double-float sums over the FP32 vectors, its FP32 phase stopped
    at 1e-7 or, with three polish rounds, at 1e-6) against the plain FP64 thick-restart solve, within 1e-9; a
    second run is bitwise the same (fixed reduction orders)."""
    from qsi_subspace_ed_gb300 import workloads

    w_ = workloads.sector_workload("pyro_1x2x2", seed=3, gpu=True)
    op = q.LazyOpSum(q.ZBasis(w_.basis_lohi), w_.hamiltonian())
    e64, _, _ = q.diagonalise(op, nev=10, ncv=24, tol=1e-10, seed=1, precision="f64", want_vectors=False)
    eb, _, rep = q.diagonalise(op, nev=10, ncv=24, tol=1e-10, seed=1, precision="mixed", polish_steps=polish,
                               want_vectors=False, block=block)
    top = min(eb.max(), e64.max())
    err = [np.abs(e64 - v).min() for v in eb if v <= top + 1e-8]
    assert len(err) >= 8 and max(err) <= 1e-9, err
    eb2, _, _ = q.diagonalise(op, nev=10, ncv=24, tol=1e-10, seed=1, precision="mixed", polish_steps=polish,
                              want_vectors=False, block=block)
    assert np.array_equal(eb, eb2)


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_solves_on_the_materialised_operator_are_bitwise(precision):
    """Eigen-solves through the materialised operator (its single-vector applies read the lookup cache alone) give
    bitwise the eigenvalues and residuals of the matrix-free solve."""
    basis, H = cases()["q0_32"]
    op = q.LazyOpSum(q.ZBasis(basis), H)
    kw = dict(nev=5, ncv=15, tol=1e-10, seed=2, precision=precision, polish_steps=2 if precision == "mixed" else 0)
    e0, v0, r0 = q.diagonalise(op, **kw)
    assert op.materialise(True) > 0
    e1, v1, r1 = q.diagonalise(op, **kw)
    op.materialise(False)
    assert np.array_equal(e0, e1) and np.array_equal(v0, v1) and np.array_equal(r0.residual, r1.residual)
