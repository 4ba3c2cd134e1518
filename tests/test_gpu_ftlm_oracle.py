"""GPU FTLM against the FP64 oracle on identical start vectors.

The oracle restates the engine's Rademacher start block (oracle.ftlm_start_vectors) and runs the plain
per-vector three-term recurrence in numpy (oracle.ftlm_recurrences), so the GPU recurrences and the oracle's
start from the same vectors.

What is compared, and why at these points:
  * alpha_j, beta_j over the first K steps, at 1e-10 relative.  Without reorthogonalisation a Lanczos run
    loses orthogonality once its extreme Ritz values converge; from then on rounding differences of any two
    FP64 implementations (summation order of the row sums and dot products) grow until the recurrences
    differ at O(1).  Two oracle runs that differ only in summation order agree to 1e-14 before that point,
    and K is placed before it for each case.
  * E(T) and C(T) over all M steps, at 1e-10 relative to their largest magnitude: the Ritz values and
    weights that the thermodynamics use are unaffected by where the copies of converged levels appear.
"""
import numpy as np
import pytest

import qsi_subspace_ed_gb300 as q
from helpers import cases
from oracle import oracle as O

pytestmark = pytest.mark.gpu

T_GRID = np.logspace(-2, 1, 200)


def _sector_64spin_8888():
    from qsi_subspace_ed_gb300 import workloads

    w = workloads.sector_workload("pyro_1x2x2", seed=3, gpu=True)
    return w.basis_lohi, w.hamiltonian()


def _relmax(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("case, R, M, K", [("q0_32", 16, 60, 30), ("s8888", 8, 100, 50)])
def test_ftlm_fp64_matches_oracle_on_same_start_vectors(case, R, M, K):
    basis, H = _sector_64spin_8888() if case == "s8888" else cases()[case]
    n = len(basis)
    seed = 11
    op = q.LazyOpSum(q.ZBasis(basis), H)
    (a_gpu, b_gpu), = q.ftlm([op], [R], M=M, seed=seed, precision="f64")
    r, c, v = O.triplets_port(basis, H.specs())
    a_o, b_o = O.ftlm_recurrences(r, c, v, n, O.ftlm_start_vectors(n, R, seed), M)
    assert _relmax(a_gpu[:, :K], a_o[:, :K]) < 1e-10
    assert _relmax(b_gpu[:, :K], b_o[:, :K]) < 1e-10
    t_gpu = O.ftlm_thermo_oracle(a_gpu, b_gpu, n, T_GRID)
    t_o = O.ftlm_thermo_oracle(a_o, b_o, n, T_GRID, e_ref=t_gpu["e_ref"])
    assert _relmax(t_gpu["E"], t_o["E"]) < 1e-10
    assert _relmax(t_gpu["C"], t_o["C"]) < 1e-10
    # the engine's own thermodynamics (device Ritz data) agree with the oracle's as well
    t_eng = q.ftlm_thermo(a_gpu, b_gpu, n, T_GRID, e_ref=t_gpu["e_ref"])
    assert _relmax(t_eng["C"], t_o["C"]) < 1e-10


def test_ftlm_fp64_two_sectors_match_oracle():
    """Several sectors in one call: sector s starts from the oracle's vectors of seed + s."""
    cs = cases()
    names = ["q0_32", "s4444"]
    ops = [q.LazyOpSum(q.ZBasis(cs[nm][0]), cs[nm][1]) for nm in names]
    seed, R, M, K = 21, 8, 40, 25
    res = q.ftlm(ops, [R, R], M=M, seed=seed, precision="f64")
    for s, nm in enumerate(names):
        basis, H = cs[nm]
        n = len(basis)
        r, c, v = O.triplets_port(basis, H.specs())
        a_o, b_o = O.ftlm_recurrences(r, c, v, n, O.ftlm_start_vectors(n, R, seed + s), M)
        assert _relmax(res[s][0][:, :K], a_o[:, :K]) < 1e-10
        assert _relmax(res[s][1][:, :K], b_o[:, :K]) < 1e-10


def test_ftlm_mixed_against_fp64_oracle():
    """FP32 vector blocks with FP64 recurrence coefficients against the FP64 oracle on the same start vectors:
    the specific heat to 1e-5 of its largest value."""
    basis, H = _sector_64spin_8888()
    n, R, M, seed = len(basis), 8, 100, 13
    op = q.LazyOpSum(q.ZBasis(basis), H)
    (a32, b32), = q.ftlm([op], [R], M=M, seed=seed, precision="mixed")
    r, c, v = O.triplets_port(basis, H.specs())
    a_o, b_o = O.ftlm_recurrences(r, c, v, n, O.ftlm_start_vectors(n, R, seed), M)
    assert _relmax(a32[:, :10], a_o[:, :10]) < 1e-5
    t32 = O.ftlm_thermo_oracle(a32, b32, n, T_GRID)
    t_o = O.ftlm_thermo_oracle(a_o, b_o, n, T_GRID, e_ref=t32["e_ref"])
    assert _relmax(t32["C"], t_o["C"]) < 1e-5
