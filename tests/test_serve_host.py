"""Host logic of the request loop (admission, continuous batching, same-sector preference, failures) with a
host-side fake solver and basis, on the CPU."""
import threading
import time

import numpy as np

from qsi_subspace_ed_gb300 import serve


class FakeSolver:
    """Sleeps a per-request time and records how many solves ran at once."""

    def __init__(self, durations=None, fail=()):
        self.durations = durations or {}
        self.fail = set(fail)
        self.lock = threading.Lock()
        self.active = 0
        self.max_active = 0
        self.bases = []

    def make_basis(self, lohi):
        self.bases.append(len(lohi))
        return ("basis", len(lohi))

    def __call__(self, req, basis, sec):
        with self.lock:
            self.active += 1
            self.max_active = max(self.max_active, self.active)
        try:
            time.sleep(self.durations.get(req.rid, 0.05))
            if req.rid in self.fail:
                raise RuntimeError("planted failure")
            return np.array([float(req.rid), float(sec.dim)])
        finally:
            with self.lock:
                self.active -= 1


def sectors(dims):
    return {k: serve.Sector(k, None, np.zeros((d, 2), np.uint64)) for k, d in dims.items()}


def test_continuous_batching_runs_solves_together():
    fake = FakeSolver()
    loop = serve.RequestLoop(sectors({"a": 1000, "b": 2000}), slots=3, solve=fake, make_basis=fake.make_basis)
    try:
        reqs = [loop.submit(serve.Request(rid=k, sector="ab"[k % 2], g=[1] * 4, B=[0] * 3)) for k in range(6)]
        loop.drain(timeout=30)
    finally:
        loop.close()
    assert fake.max_active >= 2
    for r in reqs:
        assert r.error is None and r.evals[0] == r.rid and r.evals[1] == {"a": 1000, "b": 2000}[r.sector]
    assert sorted(fake.bases) == [1000, 2000]  # each basis made once and kept resident
    st = loop.stats()
    assert st["completed"] == 6 and st["failed"] == 0 and st["p99_s"] >= st["p50_s"] > 0


def test_device_memory_budget_serialises_solves():
    fake = FakeSolver()
    dim = 10_000
    one = serve.solve_footprint(dim, 5, 20) + serve.basis_footprint(dim)
    loop = serve.RequestLoop(sectors({"a": dim}), slots=4, hbm_budget=one, solve=fake, make_basis=fake.make_basis)
    try:
        for k in range(4):
            loop.submit(serve.Request(rid=k, sector="a", g=[1] * 4, B=[0] * 3))
        loop.drain(timeout=30)
    finally:
        loop.close()
    assert fake.max_active == 1 and len(loop.completed) == 4


def test_waiting_request_of_a_running_sector_goes_first():
    # x runs long; z frees its slot early; then y (older) and x2 (newer) wait: x2 shares x's resident sector
    fake = FakeSolver(durations={0: 0.8, 1: 0.1})
    loop = serve.RequestLoop(sectors({"x": 100, "y": 100, "z": 100}), slots=2, solve=fake,
                             make_basis=fake.make_basis)
    try:
        loop.submit(serve.Request(rid=0, sector="x", g=[1] * 4, B=[0] * 3))
        loop.submit(serve.Request(rid=1, sector="z", g=[1] * 4, B=[0] * 3))
        time.sleep(0.03)
        y = loop.submit(serve.Request(rid=2, sector="y", g=[1] * 4, B=[0] * 3))
        x2 = loop.submit(serve.Request(rid=3, sector="x", g=[1] * 4, B=[0] * 3))
        loop.drain(timeout=30)
    finally:
        loop.close()
    assert y.arrival < x2.arrival and x2.start < y.start


def test_failed_solve_is_reported_and_the_loop_goes_on():
    fake = FakeSolver(fail={1})
    loop = serve.RequestLoop(sectors({"a": 100}), slots=2, solve=fake, make_basis=fake.make_basis)
    try:
        reqs = [loop.submit(serve.Request(rid=k, sector="a", g=[1] * 4, B=[0] * 3)) for k in range(3)]
        loop.drain(timeout=30)
    finally:
        loop.close()
    assert "planted failure" in reqs[1].error and reqs[0].error is None and reqs[2].error is None
    assert loop.stats()["failed"] == 1


def test_poisson_arrivals():
    w = {"a": 0.5, "b": 0.35, "c": 0.15}
    arr = serve.poisson_requests(2000, 40.0, w, seed=7)
    again = serve.poisson_requests(2000, 40.0, w, seed=7)  # seeded: the same arrivals
    assert all(t1 == t2 and r1.sector == r2.sector and r1.g == r2.g and r1.B == r2.B
               for (t1, r1), (t2, r2) in zip(arr, again))
    t = np.array([a[0] for a in arr])
    assert np.all(np.diff(t) > 0) and abs(len(t) / t[-1] - 40.0) < 4.0
    share = {k: sum(r.sector == k for _, r in arr) / len(arr) for k in w}
    for k in w:
        assert abs(share[k] - w[k]) < 0.04
    for _, r in arr:
        assert all(0.0 <= v <= 1.0 for v in r.g) and np.linalg.norm(r.B) <= 1.0 + 1e-12
