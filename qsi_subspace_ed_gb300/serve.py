"""Request loop for phase-diagram points: resident bases, HBM admission, continuous batching.

A request is one ground-state-manifold solve (the nev lowest eigenvalues) of the ring/Zeeman Hamiltonian
H(g, B) on one named sector; it replaces the reference's static phase-diagram plans run by a process pool
(driver/ed_phasedia_plan.sh:21-25, driver/execute_asynchronous.sh:1-38).  The loop keeps every sector's basis
and lookup index resident on the device once loaded, and runs up to `slots` solves at a time, each on its own
worker thread and operator stream; a request that arrives while others run is admitted as soon as a slot and
enough device memory are free.  Among waiting requests, one whose sector already has a solve running is
preferred, then the oldest.

With batching (the default) every sector is an operator family (OperatorFamily: H(p) with per-class
coefficients p = ring couplings by hexagon type and Zeeman field by sublattice) and each request's operator
is a member of it: the single-vector applies of all same-sector solves that wait at the same moment run as one
batched apply, one column per request, so concurrent requests share every basis read and lookup while each
runs its own Lanczos (restarts, convergence) at its own pace; requests join at their first apply and leave
when their solve ends.  Every solve is deterministic and a member's results do not depend on the batch it ran
in, so a result is identical whether the request ran alone or in the mix.

Latency is completion minus arrival; the loop reports p50/p99 and completed solves per second.
"""
from __future__ import annotations

import threading
import time
from collections import deque
from dataclasses import dataclass, field
from typing import Callable

import numpy as np

from .core import LazyOpSum, OperatorFamily, ZBasis
from .hamiltonian import build_ring_zeeman, ring_zeeman_class_coefficients, ring_zeeman_classes
from .lattice import Lattice
from .solvers import diagonalise


@dataclass
class Sector:
    name: str
    lattice: Lattice
    basis_lohi: np.ndarray

    @property
    def dim(self) -> int:
        return len(self.basis_lohi)


@dataclass
class Request:
    rid: int
    sector: str
    g: list
    B: list
    nev: int = 5
    tol: float = 1e-9
    ncv: int = 20
    arrival: float = 0.0
    # filled by the loop
    start: float = 0.0
    done: float = 0.0
    evals: np.ndarray | None = None
    error: str | None = None
    event: threading.Event = field(default_factory=threading.Event, repr=False)

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def solve_footprint(dim: int, nev: int, ncv: int) -> int:
    """Device bytes one FP64 solve needs beyond the resident basis (Krylov basis, Ritz block, vectors, diagonal)."""
    return 8 * dim * (ncv + 1 + 2 * nev + 4) + (64 << 20)


def basis_footprint(dim: int, batch_cols: int = 0) -> int:
    """Resident bytes of a basis: states, bucket table (~4 B/state at the automatic size), hash index (<= 64 B/state),
    and with batching the family's two [dim][batch_cols] FP64 batch blocks."""
    return dim * (16 + 4 + 64 + 16 * batch_cols)


class RequestLoop:
    """slots worker threads; solve(req, basis, sector) -> eigenvalues and make_basis(basis_lohi) -> resident basis
    default to the device solve and ZBasis (both replaceable, e.g. by host-side fakes)."""

    def __init__(self, sectors: dict[str, Sector], slots: int = 4, hbm_budget: int = 200 << 30,
                 solve: Callable | None = None, make_basis: Callable | None = None, batching: bool = True,
                 min_batch_rows: int | None = None):
        self.sectors = sectors
        self.slots = slots
        self.budget = hbm_budget
        self.batching = batching and solve is None
        self.min_batch_rows = min_batch_rows  # None: the family's default (small bases run their applies at once)
        self._solve = solve or self._solve_default
        self._make_basis = make_basis or ZBasis
        self._families: dict[str, OperatorFamily] = {}
        self._lock = threading.Condition()
        self._waiting: deque[Request] = deque()
        self._running: dict[int, Request] = {}
        self._bases: dict[str, ZBasis] = {}
        self._in_use = 0
        self._stop = False
        self.completed: list[Request] = []
        self._threads = [threading.Thread(target=self._worker, daemon=True) for _ in range(slots)]
        for t in self._threads:
            t.start()

    # -------------------------------------------------------------- public
    def submit(self, req: Request) -> Request:
        if req.sector not in self.sectors:
            raise KeyError(f"unknown sector {req.sector}")
        with self._lock:
            if not req.arrival:
                req.arrival = time.perf_counter()
            self._waiting.append(req)
            self._lock.notify_all()
        return req

    def drain(self, timeout: float | None = None) -> None:
        deadline = None if timeout is None else time.perf_counter() + timeout
        with self._lock:
            while self._waiting or self._running:
                left = None if deadline is None else deadline - time.perf_counter()
                if left is not None and left <= 0:
                    raise TimeoutError("request loop did not drain in time")
                self._lock.wait(timeout=left if left is not None else 1.0)

    def close(self) -> None:
        with self._lock:
            self._stop = True
            self._lock.notify_all()
        for t in self._threads:
            t.join(timeout=30)

    def stats(self) -> dict:
        lat = np.array([r.latency for r in self.completed if r.error is None])
        if len(lat) == 0:
            return {"completed": 0}
        t0 = min(r.arrival for r in self.completed)
        t1 = max(r.done for r in self.completed)
        return {"completed": int(len(lat)), "failed": sum(r.error is not None for r in self.completed),
                "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                "mean_s": float(lat.mean()), "solves_per_s": float(len(lat) / max(t1 - t0, 1e-9)),
                "wall_s": float(t1 - t0)}

    # -------------------------------------------------------------- internals
    def _need(self, req: Request) -> int:
        sec = self.sectors[req.sector]
        need = solve_footprint(sec.dim, req.nev, req.ncv)
        if req.sector not in self._bases:
            need += basis_footprint(sec.dim, self.slots if self.batching else 0)
        return need

    def _pick(self) -> Request | None:
        """Next admissible request: a resident, running sector first, then the oldest that fits."""
        running_sectors = {r.sector for r in self._running.values()}
        order = sorted(range(len(self._waiting)),
                       key=lambda i: (self._waiting[i].sector not in running_sectors, self._waiting[i].arrival))
        for i in order:
            req = self._waiting[i]
            if self._in_use + self._need(req) <= self.budget or not self._running:
                del self._waiting[i]
                return req
        return None

    def _worker(self) -> None:
        while True:
            with self._lock:
                req = None
                while not self._stop:
                    req = self._pick()
                    if req is not None:
                        break
                    self._lock.wait(timeout=0.5)
                if self._stop and req is None:
                    return
                need = solve_footprint(self.sectors[req.sector].dim, req.nev, req.ncv)
                self._in_use += need
                self._running[req.rid] = req
                basis = self._bases.get(req.sector)
                if basis is None:
                    sec = self.sectors[req.sector]
                    basis = self._make_basis(sec.basis_lohi)
                    self._bases[req.sector] = basis
                    if self.batching:
                        cls, n_cls = ring_zeeman_classes(sec.lattice)
                        fam = OperatorFamily(basis, build_ring_zeeman(sec.lattice, [1.0] * 4, [0.0] * 3), cls, n_cls,
                                             self.slots)
                        if self.min_batch_rows is not None:
                            fam.set_min_rows(self.min_batch_rows)
                        self._families[req.sector] = fam
                    # stays resident and accounted for
                    self._in_use += basis_footprint(sec.dim, self.slots if self.batching else 0)
                family = self._families.get(req.sector)
            req.start = time.perf_counter()
            try:
                if family is not None:
                    req.evals = self._solve_member(req, family)
                else:
                    req.evals = self._solve(req, basis, self.sectors[req.sector])
            except Exception as e:  # a failed solve is reported with its request, the loop carries on
                req.error = f"{type(e).__name__}: {e}"
            req.done = time.perf_counter()
            with self._lock:
                self._in_use -= need
                del self._running[req.rid]
                self.completed.append(req)
                req.event.set()
                self._lock.notify_all()

    def family_stats(self) -> dict:
        """Per sector: batches run, member applies served and mean columns per batch."""
        return {k: f.stats() for k, f in self._families.items()}

    @staticmethod
    def _solve_member(req: Request, family: OperatorFamily) -> np.ndarray:
        op = family.member(ring_zeeman_class_coefficients(req.g, req.B))
        try:
            ev, _, _ = diagonalise(op, nev=req.nev, ncv=req.ncv, tol=req.tol, seed=req.rid + 1, want_vectors=False)
        finally:
            op.close()
        return ev

    @staticmethod
    def _solve_default(req: Request, basis: ZBasis, sec: Sector) -> np.ndarray:
        op = LazyOpSum(basis, build_ring_zeeman(sec.lattice, req.g, req.B))
        try:
            ev, _, _ = diagonalise(op, nev=req.nev, ncv=req.ncv, tol=req.tol, seed=req.rid + 1, want_vectors=False)
        finally:
            op.close()
        return ev


def poisson_requests(n: int, rate: float, sector_weights: dict[str, float], seed: int = 5, nev: int = 5,
                     tol: float = 1e-9) -> list[tuple[float, Request]]:
    """Phase-diagram arrivals: g ~ U[0,1]^4, B = |B| n with |B| ~ U[0,1] and n uniform on the sphere."""
    rng = np.random.default_rng(seed)
    names = list(sector_weights)
    p = np.array([sector_weights[k] for k in names], dtype=float)
    p /= p.sum()
    t = 0.0
    out = []
    for k in range(n):
        t += rng.exponential(1.0 / rate)
        g = list(rng.uniform(0.0, 1.0, 4))
        v = rng.standard_normal(3)
        B = list(rng.uniform(0.0, 1.0) * v / np.linalg.norm(v))
        out.append((t, Request(rid=k, sector=names[rng.choice(len(names), p=p)], g=g, B=B, nev=nev, tol=tol)))
    return out


def run_arrivals(loop: RequestLoop, arrivals: list[tuple[float, Request]]) -> dict:
    """Submits requests at their arrival offsets (seconds from now) and waits for all of them."""
    t0 = time.perf_counter()
    for offset, req in arrivals:
        dt = t0 + offset - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        req.arrival = t0 + offset
        loop.submit(req)
    loop.drain()
    return loop.stats()
