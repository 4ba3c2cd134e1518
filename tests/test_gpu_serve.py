"""Request loop: concurrent solves on resident bases give the same results as solves run alone."""
import numpy as np
import pytest

import qsi_subspace_ed_gb300 as q
from qsi_subspace_ed_gb300 import serve, workloads
from helpers import GOLDEN

pytestmark = pytest.mark.gpu


def _sectors():
    l32 = workloads.lattice("pyro_1x2x1")
    l48 = q.Lattice.load(GOLDEN / "lattices" / "golden48.json")
    return {
        "q32": serve.Sector("q32", l32, q.enumerate_basis(l32)),
        "s32": serve.Sector("s32", l32, q.enumerate_basis(l32, sector=[4, 4, 4, 4])),
        "q48": serve.Sector("q48", l48, q.enumerate_basis(l48)),
    }


def _requests(n=14):
    arr = serve.poisson_requests(n, rate=1e6, sector_weights={"q32": 0.4, "s32": 0.3, "q48": 0.3}, seed=3)
    return [r for _, r in arr]


def test_family_members_batch_bitwise_and_match_their_operators():
    """Operator-family members H(p): a member's apply equals the plain operator of the same H to rounding, and
    its results are bitwise the same whether its applies ran alone or batched with other members' (several host
    threads applying at once)."""
    import threading

    from qsi_subspace_ed_gb300.hamiltonian import ring_zeeman_class_coefficients, ring_zeeman_classes

    lat = workloads.lattice("pyro_1x2x1")
    lohi = q.enumerate_basis(lat)
    b = q.ZBasis(lohi)
    cls, ncls = ring_zeeman_classes(lat)
    fam = q.OperatorFamily(b, q.build_ring_zeeman(lat, [1.0] * 4, [0.0] * 3), cls, ncls, max_cols=4)
    fam.set_min_rows(0)  # batch this small basis too
    rng = np.random.default_rng(5)
    params = [(list(rng.uniform(0, 1, 4)), list(rng.uniform(-1, 1, 3))) for _ in range(4)]
    members = [fam.member(ring_zeeman_class_coefficients(g, B)) for g, B in params]
    x = rng.standard_normal(len(lohi))
    alone = []
    for (g, B), m in zip(params, members):
        y = np.zeros_like(x)
        m.evaluate(x, y)
        alone.append(y)
        ref = np.zeros_like(x)
        q.LazyOpSum(b, q.build_ring_zeeman(lat, g, B)).evaluate(x, ref)
        np.testing.assert_allclose(y, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
    assert fam.stats()["mean_columns"] == 1.0
    out = [[None] * 20 for _ in members]
    gate = threading.Barrier(len(members))

    def run(k):
        gate.wait()
        for rep in range(20):
            y = np.zeros_like(x)
            members[k].evaluate(x, y)
            out[k][rep] = y

    ts = [threading.Thread(target=run, args=(k,)) for k in range(len(members))]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    for k in range(len(members)):
        for y in out[k]:
            assert np.array_equal(y, alone[k])
    st = fam.stats()
    assert st["mean_columns"] > 1.0, st  # concurrent applies ran as batched columns


def test_family_small_basis_runs_applies_directly():
    """Below the family's row threshold (by default 131072) members' applies run at once, one column each, with
    the results of batched runs."""
    from qsi_subspace_ed_gb300.hamiltonian import ring_zeeman_class_coefficients, ring_zeeman_classes

    lat = workloads.lattice("pyro_1x2x1")
    lohi = q.enumerate_basis(lat)
    b = q.ZBasis(lohi)
    cls, ncls = ring_zeeman_classes(lat)
    fam = q.OperatorFamily(b, q.build_ring_zeeman(lat, [1.0] * 4, [0.0] * 3), cls, ncls, max_cols=4)
    m = fam.member(ring_zeeman_class_coefficients([0.3, 0.5, 0.7, 0.9], [0.1, -0.2, 0.3]))
    x = np.random.default_rng(2).standard_normal(len(lohi))
    y_direct = np.zeros_like(x)
    m.evaluate(x, y_direct)
    st = fam.stats()
    assert st["batches"] == st["applies"] == 1
    fam.set_min_rows(0)
    y_queued = np.zeros_like(x)
    m.evaluate(x, y_queued)
    assert np.array_equal(y_direct, y_queued)
    with pytest.raises(q.QsiError):
        fam.set_min_rows(-1)


def test_results_identical_alone_and_in_the_mix():
    sectors = _sectors()
    alone = {}
    solo = serve.RequestLoop(sectors, slots=1)
    try:
        for r in _requests():
            solo.submit(r)
            r.event.wait(120)
            assert r.error is None, r.error
            alone[r.rid] = r.evals
    finally:
        solo.close()
    mix = serve.RequestLoop(sectors, slots=4, min_batch_rows=0)  # batch the small test bases too
    try:
        reqs = [mix.submit(r) for r in _requests()]
        mix.drain(timeout=300)
        st = mix.stats()
        fam = mix.family_stats()
    finally:
        mix.close()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    for r in reqs:
        assert np.array_equal(r.evals, alone[r.rid]), r.rid
    assert st["p99_s"] >= st["p50_s"] > 0
    # same-sector requests shared batched applies (continuous batching, not a queue alone)
    assert max(f["mean_columns"] for f in fam.values()) > 1.0, fam


def test_batched_results_match_unbatched_solves():
    """A request served through its sector's operator family gives the eigenvalues of a plain solve of the same
    H(g, B) to 1e-9."""
    sectors = _sectors()
    reqs = _requests(6)
    loop = serve.RequestLoop(sectors, slots=3, min_batch_rows=0)
    try:
        for r in reqs:
            loop.submit(r)
        loop.drain(timeout=300)
    finally:
        loop.close()
    for r in reqs:
        sec = sectors[r.sector]
        op = q.LazyOpSum(q.ZBasis(sec.basis_lohi), q.build_ring_zeeman(sec.lattice, r.g, r.B))
        ev, _, _ = q.diagonalise(op, nev=r.nev, ncv=r.ncv, tol=r.tol, seed=r.rid + 1, want_vectors=False)
        np.testing.assert_allclose(r.evals, ev, atol=1e-9)


def test_admission_respects_the_memory_budget():
    sectors = _sectors()
    # a budget below two concurrent q48 solves admits them one at a time (never rejects outright)
    one = serve.solve_footprint(sectors["q48"].dim, 5, 20) + serve.basis_footprint(sectors["q48"].dim)
    loop = serve.RequestLoop(sectors, slots=4, hbm_budget=int(1.5 * one))
    try:
        reqs = [loop.submit(serve.Request(rid=k, sector="q48", g=[1, .8, .6, .4], B=[0.1, 0.2, 0.3])) for k in range(3)]
        loop.drain(timeout=300)
    finally:
        loop.close()
    assert all(r.error is None for r in reqs)
    spans = sorted((r.start, r.done) for r in reqs)
    for (s0, d0), (s1, d1) in zip(spans, spans[1:]):
        assert s1 >= d0 - 1e-3  # no overlap under this budget
