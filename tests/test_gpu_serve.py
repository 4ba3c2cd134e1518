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
    mix = serve.RequestLoop(sectors, slots=4)
    try:
        reqs = [mix.submit(r) for r in _requests()]
        mix.drain(timeout=300)
        st = mix.stats()
    finally:
        mix.close()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    for r in reqs:
        assert np.array_equal(r.evals, alone[r.rid]), r.rid
    assert st["p99_s"] >= st["p50_s"] > 0


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
