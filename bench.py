#!/usr/bin/env python
"""Benchmark of the matrix-free Hamiltonian apply (and its Krylov drivers).

Headline (`value`): plain FP64 single-vector H-apply throughput, basis
states per second, on the 96-spin pyrochlore 1x2x3 cubic supercell restricted
to the equal-polarisation (12.12.12.12, zero-winding) sector, H = ring exchange
+ Zeeman with seeded parameters.  One step = one y = H x over the whole sector.
Beside it: the batched mixed-precision apply (R FP32 vectors, FP64 row
accumulation) in state-vectors/s, FTLM vector-steps/s, the end-to-end rate
through the C-ABI with host buffers, the kernel's HBM roofline and the CPU
push loop of the reference (oracle restatement) on the host cores.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
Under torchrun (N>1) each rank runs an independent replica on its own GPU
(the apply does not shard across GPUs in this build); `value` sums the ranks'
states over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "H-apply states/s, FTLM vec-steps/s: batched mixed vs plain FP64 GPU, |dE|<=1e-9"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--lattice", default="pyro_1x2x3", help="pyro_1x2x1 | pyro_1x2x2 | pyro_1x2x3")
    p.add_argument("--full-basis", action="store_true", help="all Q=0 states instead of the equal sector")
    p.add_argument("--sector", default="", help="comma-separated sublattice up-counts (default: equal sector)")
    p.add_argument("--R", default="128,64",
                   help="vector counts of the batched mixed apply legs (the first is `batched_mixed`, as FTLM's R)")
    p.add_argument("--no-tune", action="store_true", help="skip the launch autotuner (built-in settings)")
    p.add_argument("--ftlm-steps", type=int, default=30, help="Lanczos steps of the timed FTLM runs")
    p.add_argument("--seed", type=int, default=3)
    p.add_argument("--ref-step-seconds", type=float, default=2.5,
                   help="target length of one reference-arm step (a sample of whole source rows)")
    p.add_argument("--no-extras", action="store_true", help="skip batched / FTLM / e2e / CPU legs")
    p.add_argument("--legs", default="e2e,batched,ftlm,lanczos,ftlm_sectors,serve,materialised,cpu",
                   help="extra legs after the FP64 headline: e2e, batched, ftlm, lanczos (FP64 vs mixed 10-eigenvalue "
                        "solves), ftlm_sectors (multi-sector FTLM), serve (request loop), materialised (the applies, "
                        "FTLM and, with lanczos, the solves on the materialised operator), cpu (whole oracle apply: "
                        "CPU baseline and parity)")
    p.add_argument("--nev", type=int, default=10)
    p.add_argument("--serve-n", type=int, default=200)
    p.add_argument("--ftlm-R", type=int, default=0,
                   help="FTLM vectors per sector (0: the first of --R; the ftlm_sectors leg: 64)")
    p.add_argument("--ftlm-M", type=int, default=100)
    p.add_argument("--serve-rate", type=float, default=40.0)
    p.add_argument("--serve-slots", type=int, default=8)
    p.add_argument("--serve-96", action="store_true",
                   help="serve leg: the request mix with the 96-spin sector (32-spin Q=0, 64-spin Q=0, 96-spin "
                        "12.12.12.12; weights 0.5/0.35/0.15) instead of the 64-spin 8.8.8.8 sector")
    p.add_argument("--ncv", type=int, default=24)
    return p.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def wait_first(self, timeout: float = 5.0) -> None:
        """Waits for the first sample, so that nvidia-smi's start-up is over before a timed region."""
        t0 = time.time()
        while self.proc and not self.lines and time.time() - t0 < timeout:
            time.sleep(0.02)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0: float | None = None, t1: float | None = None):
        """Median SM clock and throttle reasons of the samples taken in [t0, t1] (all samples without a window;
        the nearest sample when none fell inside it)."""
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines
        if t0 is not None and t1 is not None and lines:
            inside = [x for x in lines if t0 <= x[0] <= t1 + 0.25]
            lines = inside or [min(lines, key=lambda x: abs(x[0] - 0.5 * (t0 + t1)))]
        for _, ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def workload_spec(args):
    """The workload both arms run, derived from the command line alone (no engine call): lattice file, sector
    (None: the full Q=0 basis), ring couplings g ~ U[0.2, 1]^4 and field B ~ U[-0.5, 0.5]^3 from
    numpy default_rng(seed) (the draws of workloads.ring_zeeman_params)."""
    import numpy as np

    lat = json.load(open(ROOT / "qsi_subspace_ed_gb300" / "lattices" / f"{args.lattice}.json"))
    rng = np.random.default_rng(args.seed)
    g = [float(v) for v in rng.uniform(0.2, 1.0, 4)]
    B = [float(v) for v in rng.uniform(-0.5, 0.5, 3)]
    n_sl = max(int(a["sl"]) for a in lat["atoms"]) + 1
    if args.full_basis:
        sector, name = None, f"{args.lattice}.Q0"
    else:
        if args.sector:
            sector = [int(v) for v in args.sector.split(",")]
        else:  # equal sublattice polarisation (the zero-winding sector): N/8 up spins per sublattice
            sector = [len(lat["atoms"]) // n_sl // 2] * n_sl
        name = f"{args.lattice}.s{'.'.join(map(str, sector))}"
    return {"name": name, "lattice": lat, "sector": sector, "g": g, "B": B}


def workload_config(spec, n: int, n_terms: int) -> dict:
    """`config` of the JSON line, the same in both arms."""
    return {"workload": spec["name"], "n_states": int(n), "n_terms": int(n_terms), "vectors_per_apply": 1,
            "l2": "inputs larger than L2" if n * 24 > 2 * 129 * 2**20 else "L2 flushed between steps"}


def make_workload(args):
    """Our arm: the workload's basis enumerated on the GPU and its Hamiltonian built by the engine."""
    import qsi_subspace_ed_gb300 as q
    from qsi_subspace_ed_gb300 import workloads

    spec = workload_spec(args)
    lat = workloads.lattice(args.lattice)
    t0 = time.time()
    basis = q.enumerate_basis_gpu(lat, sector=spec["sector"])
    w = workloads.Workload(spec["name"], lat, basis, spec["g"], spec["B"])
    return spec, w, time.time() - t0


def measured_traffic(workload: str, kernel: str, n: int):
    """DRAM bytes of one full launch from the ncu summaries in profiles/apply_traffic.json, or None."""
    tp = ROOT / "profiles" / "apply_traffic.json"
    if not tp.exists():
        return None
    for e in json.load(open(tp)).get("entries", []):
        if e.get("workload") == workload and e.get("kernel") == kernel and e.get("bytes_per_row"):
            return e["bytes_per_row"] * n
    return None


def oracle_whole_apply(basis_lohi, specs, x):
    """One whole y = H x by the reference's push loop (oracle restatement: per-term OpenMP pass over all source
    rows, atomic scatter, ZBasisInterp lookups) on all host cores; returns (y, seconds, threads, lookups)."""
    import numpy as np

    from oracle import oracle as O

    threads = O.cpu_threads()
    terms = O.terms_array(specs)
    y = np.zeros(len(basis_lohi))
    try:
        ix = O.InterpIndex(basis_lohi)
    except MemoryError:  # no room for the high-word bounds: whole-basis bisection (ZBasisBST)
        ix = None
    t0 = time.time()
    if ix is not None:
        ix.apply_rows(terms, x, y, 0, len(basis_lohi), threads)
    else:
        O.apply_rows_port(basis_lohi, terms, x, y, 0, len(basis_lohi), threads)
    return y, time.time() - t0, threads, "ZBasisInterp" if ix is not None else "ZBasisBST"


def sample_blocks(n: int, rows: int, step: int, n_blocks: int = 16):
    """Source-row blocks of one reference-arm step: n_blocks blocks of rows / n_blocks rows, one in each of
    n_blocks equal slices of the basis, at an offset inside the slice that moves from step to step."""
    rows = min(n, rows)
    nb = max(1, min(n_blocks, rows))
    size = rows // nb
    slice_ = n // nb
    out = []
    for k in range(nb):
        room = max(0, slice_ - size)
        off = (step * 7919 * (k + 1)) % (room + 1)
        out.append((k * slice_ + off, k * slice_ + off + size))
    return out


def ftlm_sectors_leg(args):
    """Multi-sector FTLM: R Rademacher vectors, M steps, three sectors of uneven dimension advanced together
    (one apply launch per step for all sectors, the run captured in one CUDA graph), FP32 vectors with FP64
    recurrence coefficients, against the same run in plain FP64."""
    import numpy as np

    import qsi_subspace_ed_gb300 as q
    from qsi_subspace_ed_gb300 import workloads

    l32, l64 = workloads.lattice("pyro_1x2x1"), workloads.lattice("pyro_1x2x2")
    g, B = workloads.ring_zeeman_params(args.seed, (0.2, 1.0), 0.5)
    t0 = time.time()
    secs = [("pyro_1x2x2.n0", l64, q.enumerate_basis_gpu(l64)),
            ("pyro_1x2x2.n1", l64, q.enumerate_basis_gpu(l64, n_spinon_pairs=1)),
            ("pyro_1x2x1.n2", l32, q.enumerate_basis_gpu(l32, n_spinon_pairs=2))]
    t_enum = time.time() - t0
    ops = [q.LazyOpSum(q.ZBasis(b), q.build_ring_zeeman(lat, g, B, Jpm=0.05)) for _, lat, b in secs]
    R, M = args.ftlm_R or 64, args.ftlm_M
    T = np.logspace(-2, 1, 200)
    out = {"R": R, "M": M, "Jpm": 0.05, "g": g, "B": B, "sectors": {nm: int(len(b)) for nm, _, b in secs},
           "enumerate_s": round(t_enum, 2), "note": "the 2-spinon-pair sector is taken on the 32-spin cell "
           "(its 64-spin basis does not fit R=64 FP32 vectors in memory)"}
    res = {}
    for prec in ("mixed", "f64"):
        q.ftlm(ops, [R] * len(ops), M=3, seed=1, precision=prec)  # warm-up
        torch_sync()
        t0 = time.time()
        res[prec] = q.ftlm(ops, [R] * len(ops), M=M, seed=1, precision=prec)
        dt = time.time() - t0
        out[prec] = {"seconds": dt, "vec_steps_per_s": len(ops) * R * M / dt,
                     "state_vector_steps_per_s": sum(len(b) for _, _, b in secs) * R * M / dt}
    out["speedup_mixed_vs_f64"] = out["f64"]["seconds"] / out["mixed"]["seconds"]
    errs = {}
    for k, (nm, _, b) in enumerate(secs):
        th32 = q.ftlm_thermo(*res["mixed"][k], len(b), T)
        th64 = q.ftlm_thermo(*res["f64"][k], len(b), T)
        errs[nm] = {"max_abs_dC": float(np.abs(th32["C"] - th64["C"]).max()),
                    "max_C": float(np.abs(th64["C"]).max()), "e_ref_diff": abs(th32["e_ref"] - th64["e_ref"])}
    out["mixed_vs_f64"] = errs
    # the same runs on the materialised sectors, as the reference's ftlm_DOQSI_ham materialises H first
    mat = {"cache_bytes": sum(op.materialise(True) for op in ops)}
    for prec in ("mixed", "f64"):
        q.ftlm(ops, [R] * len(ops), M=3, seed=1, precision=prec)
        torch_sync()
        t0 = time.time()
        rm = q.ftlm(ops, [R] * len(ops), M=M, seed=1, precision=prec)
        dt = time.time() - t0
        mat[prec] = {"seconds": dt, "vec_steps_per_s": len(ops) * R * M / dt,
                     "bitwise_equal_to_matrix_free": all(np.array_equal(a[0], c[0]) and np.array_equal(a[1], c[1])
                                                         for a, c in zip(rm, res[prec]))}
    mat["speedup_mixed_vs_f64"] = mat["f64"]["seconds"] / mat["mixed"]["seconds"]
    for op in ops:
        op.materialise(False)
    out["materialised"] = mat
    return out


def torch_sync():
    import torch

    torch.cuda.synchronize()


def serve_leg(args):
    """Request loop (the phase-diagram request mix, scaled to the bench's time): Poisson points over three resident sectors,
    served with `slots` concurrent solves and same-sector continuous batching (operator families: concurrent
    requests' applies run as columns of one batched apply), against the same requests solved one after another
    without batching (plain FP64 GPU solves)."""
    import qsi_subspace_ed_gb300 as q
    from qsi_subspace_ed_gb300 import serve, workloads

    l32, l64 = workloads.lattice("pyro_1x2x1"), workloads.lattice("pyro_1x2x2")
    if args.serve_96:
        l96 = workloads.lattice("pyro_1x2x3")
        sectors = {"pyro_1x2x1.Q0": serve.Sector("pyro_1x2x1.Q0", l32, q.enumerate_basis(l32)),
                   "pyro_1x2x2.Q0": serve.Sector("pyro_1x2x2.Q0", l64, q.enumerate_basis_gpu(l64)),
                   "pyro_1x2x3.s12.12.12.12": serve.Sector("pyro_1x2x3.s12.12.12.12", l96,
                                                            q.enumerate_basis_gpu(l96, workloads.equal_sector(l96)))}
        weights = {"pyro_1x2x1.Q0": 0.5, "pyro_1x2x2.Q0": 0.35, "pyro_1x2x3.s12.12.12.12": 0.15}
        note = "the request mix with the 96-spin sector; admission by HBM footprint lets two or three of its solves run at once"
    else:
        sectors = {"pyro_1x2x1.Q0": serve.Sector("pyro_1x2x1.Q0", l32, q.enumerate_basis(l32)),
                   "pyro_1x2x2.s8.8.8.8": serve.Sector("pyro_1x2x2.s8.8.8.8", l64,
                                                        q.enumerate_basis_gpu(l64, [8, 8, 8, 8])),
                   "pyro_1x2x2.Q0": serve.Sector("pyro_1x2x2.Q0", l64, q.enumerate_basis_gpu(l64))}
        weights = {"pyro_1x2x1.Q0": 0.5, "pyro_1x2x2.s8.8.8.8": 0.35, "pyro_1x2x2.Q0": 0.15}
        note = ("the 96-spin sector of the request mix is replaced by the 64-spin Q=0 basis to keep the default run "
                "short (the mix with it: --serve-96)")
    out = {"requests": args.serve_n, "rate_per_s": args.serve_rate, "nev": 5, "tol": 1e-9, "slots": args.serve_slots,
           "sectors": {k: v.dim for k, v in sectors.items()}, "weights": weights, "note": note}
    for name, slots, batching in (("serial", 1, False), ("continuous", args.serve_slots, True)):
        loop = serve.RequestLoop(sectors, slots=slots, batching=batching)
        try:
            arr = serve.poisson_requests(args.serve_n, args.serve_rate if slots > 1 else 1e9, weights, seed=7)
            out[name] = serve.run_arrivals(loop, arr)
            if batching:
                out[name]["batching"] = loop.family_stats()
        finally:
            loop.close()
    out["throughput_ratio"] = out["continuous"]["solves_per_s"] / out["serial"]["solves_per_s"]
    return out


def run_reference(args):
    """The reference's CPU path on this workload: the oracle's restatement of its push loop (per term, an
    OpenMP loop over source rows scattering y[J] += c x[i] atomically, ZBasisInterp lookups) on all host cores.
    Its basis comes from the oracle's restatement of the reference's enumerator and its term list from the
    oracle's Hamiltonian builder, so nothing of the engine is loaded.  Each step is a bounded sample: whole
    source rows in 16 blocks spread over the basis (sample_blocks), sized to about --ref-step-seconds."""
    import numpy as np

    from oracle import oracle as O

    ws, rank, _ = dist_env()
    if rank != 0:
        return
    spec = workload_spec(args)
    t0 = time.time()
    basis = O.enumerate_basis_oracle(spec["lattice"], spec["sector"])
    t_enum = time.time() - t0
    specs = O.ring_zeeman_specs(spec["lattice"], spec["g"], spec["B"])
    terms = O.terms_array(specs)
    n = len(basis)
    threads = O.cpu_threads()
    t0 = time.time()
    try:
        ix = O.InterpIndex(basis)
    except MemoryError:
        ix = None
    t_index = time.time() - t0
    x = np.random.default_rng(0).standard_normal(n)
    y = np.zeros(n)

    def run(blocks):
        t = time.time()
        for a, b in blocks:
            if ix is not None:
                ix.apply_rows(terms, x, y, a, b, threads)
            else:
                O.apply_rows_port(basis, terms, x, y, a, b, threads)
        return time.time() - t

    # calibrate the sample to about --ref-step-seconds per step
    probe = min(n, 200_000)
    dt = run(sample_blocks(n, probe, 0))
    rows = int(min(n, max(probe, probe * args.ref_step_seconds / max(dt, 1e-3))))
    for k in range(max(1, args.warmup)):
        run(sample_blocks(n, rows, k + 1))
    per = []
    for k in range(args.steps):
        blocks = sample_blocks(n, rows, args.warmup + k + 1)
        per.append((sum(b - a for a, b in blocks), run(blocks)))
    total_rows = sum(r for r, _ in per)
    total_s = sum(t for _, t in per)
    v = total_rows / total_s
    sample = (f"per step {per[0][0]} source rows ({per[0][0] / n:.1%} of {n}) in 16 blocks spread over the basis, "
              f"whole rows: per-term OpenMP pass, atomic scatter, "
              f"{'ZBasisInterp' if ix is not None else 'ZBasisBST'} lookups")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "states/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total_s / len(per), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded ring/Zeeman parameters)",
            "config": workload_config(spec, n, len(specs)),
            "setup": {"enumerate_s": round(t_enum, 2), "index_s": round(t_index, 2), "parallelism": "host OpenMP",
                      "basis": "oracle restatement of the reference's enumerator"},
            "cpu_baseline": {"value": v, "unit": "states/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "states/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def ftlm_step_bytes(n: int, R: int, h: float, blocks: int, s: int = 4) -> float:
    """Algorithmic bytes of one FTLM step (one sector, R vectors of s bytes, h off-diagonal hits per row).
    Two blocks (the one-launch FP32 form): the apply P <- H C - beta P (16 + R s (h + 2) per row, plus the read of
    P it accumulates into), one pass of dots over C and P (2 R s) and P <- (P - alpha C) / beta (reads C, P and
    writes P: 3 R s).  Three blocks: the apply W = H C, the dots <C, W> (2 R s), the update P <- W - alpha C -
    beta P (4 R s) and the scale P /= beta (2 R s)."""
    apply_b = 16 + R * s * (h + 2)
    if blocks == 2:
        return n * (apply_b + R * s + 2 * R * s + 3 * R * s)
    return n * (apply_b + 2 * R * s + 4 * R * s + 2 * R * s)


def ftlm_rate(q, ops, R, prec, M1, blocks=0):
    """FTLM vector-steps/s of one sector: per-step time from the difference of an M1 and an M1/3 step run (setup,
    capture and readout cancel), after a 2-step warm-up run; the rate including setup beside it."""
    import torch

    M1 = max(3, M1)
    M0 = max(1, M1 // 3)
    q.ftlm(ops, [R], M=2, seed=1, precision=prec, blocks=blocks)
    t = {}
    for M in (M0, M1):
        torch.cuda.synchronize()
        t0 = time.time()
        if M == M1:
            torch.cuda.nvtx.range_push(f"timed_ftlm_{prec}")  # lets ncu list one run's launches
        q.ftlm(ops, [R], M=M, seed=1, precision=prec, blocks=blocks)
        if M == M1:
            torch.cuda.nvtx.range_pop()
        t[M] = time.time() - t0
    per = (t[M1] - t[M0]) / (M1 - M0)
    return {"R": R, "precision": prec, "ms_per_step": per * 1e3, "vec_steps_per_s": R / per,
            "vec_steps_per_s_incl_setup": R * M1 / t[M1], "seconds": {str(M0): t[M0], str(M1): t[M1]}}


def event_ms(fn, steps, warmup):
    """Mean milliseconds of fn over `steps` runs timed with CUDA events on the current stream, after `warmup`."""
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for a, b in ev:
        a.record()
        fn()
        b.record()
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev) / steps


def materialised_leg(args, q, op, n, h, x, y_host, peak, peak_kind, with_solves, workload):
    """The operator materialised (qsi_op_materialise: the column of every admitted term stored, as the reference
    materialises H with toSparseMatrix for diag_DOQSI_ham --algorithm sparse and ftlm_DOQSI_ham): the FP64
    single-vector apply (bitwise the matrix-free result), the batched FP32 applies, FTLM and optionally the
    eigen-solves, each as in the matrix-free legs."""
    import numpy as np
    import torch

    out = {}
    torch.cuda.synchronize()
    t0 = time.time()
    out["cache_bytes"] = op.materialise(True)
    out["build_s"] = time.time() - t0
    y = torch.zeros_like(x)
    torch.cuda.nvtx.range_push("timed_materialised")  # lets ncu capture these launches
    ms = event_ms(lambda: op.evaluate(x, y), args.steps, args.warmup)
    torch.cuda.nvtx.range_pop()
    bpr = 16 + 8 + 8 * h + 8 + 5 * h  # the matrix-free bytes plus each hit's cached column and term index
    ach = n * bpr / (ms * 1e-3) / 1e9
    out["apply_fp64"] = {"value": n / (ms * 1e-3), "unit": "states/s", "ms_per_apply": ms,
                         "bitwise_equal_to_matrix_free": bool(np.array_equal(y.cpu().numpy(), y_host)),
                         "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                                      "peak_kind": peak_kind, "bytes_per_row": bpr,
                                      "kernel": "k_apply_cached<double,double,uint8>",
                                      "traffic": measured_traffic(workload, "k_apply_cached<double,double,uint8>", n)}}
    del y
    for R in [int(v) for v in str(args.R).split(",") if v]:
        torch.cuda.empty_cache()
        try:
            X = torch.randn(n, R, dtype=torch.float32, device=x.device)
            Y = torch.zeros_like(X)
        except torch.cuda.OutOfMemoryError as e:
            out[f"batched_r{R}"] = {"skipped": str(e)[:160]}
            continue
        torch.cuda.nvtx.range_push(f"timed_materialised_r{R}")
        ms = event_ms(lambda: op.apply_batched(X, Y), max(3, args.steps // 3), 1)
        torch.cuda.nvtx.range_pop()
        bpr = 16 + R * 4 * (h + 2) + 4 * h
        ach = n * bpr / (ms * 1e-3) / 1e9
        kn = f"k_apply_tile_batched<float,LookupCache,FF,16-byte gathers x{op.tuning(1)['vec_width'] or 4}> R={R}"
        out[f"batched_r{R}"] = {"value": n * R / (ms * 1e-3), "unit": "state-vectors/s", "ms_per_apply": ms,
                                "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                                             "frac": ach / peak, "peak_kind": peak_kind, "bytes_per_row": bpr,
                                             "kernel": kn, "traffic": measured_traffic(workload, kn, n)}}
        del X, Y
    torch.cuda.empty_cache()
    if "ftlm" in args.legs:
        R = args.ftlm_R or int(str(args.R).split(",")[0])
        try:
            mixed = ftlm_rate(q, [op], R, "mixed", args.ftlm_steps, 2)
        except q.QsiError as e:
            mixed = {"R": R, "skipped": str(e)[:160]}
        torch.cuda.empty_cache()
        plain = ftlm_rate(q, [op], 1, "f64", args.ftlm_steps)
        out["ftlm"] = {"mixed": mixed, "plain_fp64": plain}
        if "vec_steps_per_s" in mixed:
            out["ftlm"]["speedup_vs_plain_fp64"] = mixed["vec_steps_per_s"] / plain["vec_steps_per_s"]
    if with_solves:
        sol = {}
        for prec, polish in (("f64", 0), ("mixed", 3)):
            torch.cuda.synchronize()
            t0 = time.time()
            ev, _, rep = q.diagonalise(op, nev=args.nev, ncv=args.ncv, tol=1e-10, max_iter=400, seed=1,
                                       precision=prec, polish_steps=polish, want_vectors=False)
            sol[prec] = {"seconds": time.time() - t0, "applies": rep.applies, "restarts": rep.restarts,
                         "evals": [float(v) for v in ev], "max_residual": float(np.max(rep.residual[:args.nev]))}
        e64, emx = np.array(sol["f64"]["evals"]), np.array(sol["mixed"]["evals"])
        top = min(emx.max(), e64.max())
        err = np.array([np.abs(e64 - v).min() for v in emx if v <= top + 1e-8])
        sol["max_abs_err"] = float(err.max())
        sol["within_1e-9"] = bool(err.max() <= 1e-9)
        sol["speedup_mixed_vs_f64"] = sol["f64"]["seconds"] / sol["mixed"]["seconds"]
        out["lanczos"] = sol
    op.materialise(False)
    torch.cuda.empty_cache()
    return out


def run_ours(args):
    import numpy as np
    import torch

    import qsi_subspace_ed_gb300 as q

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    spec, w, setup_s = make_workload(args)
    H = w.hamiltonian()
    n = len(w.basis_lohi)
    t0 = time.time()
    basis = q.ZBasis(w.basis_lohi)
    t_basis = time.time() - t0
    t0 = time.time()
    op = q.LazyOpSum(basis, H)
    t_op = time.time() - t0
    tuning = {}
    if not args.no_tune:
        # launch autotuner (single-vector FP64 applies): lookup structure, table width and mode, blocks per SM
        t0 = time.time()
        log = op.autotune(R=1, dtype="f64", tune_index=True)
        tuning["single"] = {"seconds": round(time.time() - t0, 2), "trials": len(log.splitlines()) - 2,
                            "settings": op.tuning(0)}
    hits, misses = op.connectivity()
    h = hits / n
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)  # the applies below are launched on this stream too
    x = torch.randn(n, dtype=torch.float64, device=dev, generator=torch.Generator(dev).manual_seed(1234 + rank))
    y = torch.zeros_like(x)
    l2_flush = torch.empty(256 * 2**20, dtype=torch.uint8, device=dev)
    inputs_exceed_l2 = (n * 16 + n * 8) > 2 * 129 * 2**20

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        # the sampler starts before the warm-up: its start-up (NVML initialisation) stays out of the timed steps
        for _ in range(args.warmup):
            op.evaluate(x, y)
        clk.wait_first()
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        t_wall = time.time()
        t_start = t_wall
        torch.cuda.nvtx.range_push("timed_single")  # lets ncu capture exactly the timed launches
        for s in range(args.steps):
            if not inputs_exceed_l2:
                l2_flush.fill_(s & 0xff)
            ev[s][0].record(stream)
            op.evaluate(x, y)
            ev[s][1].record(stream)
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        t_end = time.time()
        t_wall = t_end - t_wall
    barrier()
    per = [a.elapsed_time(b) for a, b in ev]
    from qsi_subspace_ed_gb300.replicas import aggregate

    units, ms = aggregate(float(n), sum(per) / len(per), dev)  # sum of states over ranks, slowest rank's time
    value = units / (ms * 1e-3)
    peak, peak_kind = measured_peaks()
    bytes_per_row = 16 + 8 + 8 * h + 8
    achieved = n * bytes_per_row / (ms * 1e-3) / 1e9
    lookup = "LookupHash" if op.tuning(0)["use_hash"] and basis.index_info()["hash"] else "LookupTable"
    kname = f"k_apply_tile<double,double,{lookup}>"
    traffic = measured_traffic(w.name, kname, n)
    # the timed steps' input and result, kept on the host for the whole-size parity check against the oracle
    x_host = x.cpu().numpy() if rank == 0 else None
    y_host = y.cpu().numpy() if rank == 0 else None
    line = {"metric": METRIC, "value": value, "unit": "states/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded ring/Zeeman parameters, N(0,1) vectors)",
            "config": workload_config(spec, n, len(H)),
            "setup": {"parallelism": f"replicas x{ws}", "offdiag_hits_per_row": round(h, 4), "misses": misses,
                      "seconds": {"enumerate": round(setup_s, 2), "basis_index": round(t_basis, 2),
                                  "operator": round(t_op, 2)},
                      "index": basis.index_info(), "tuning": tuning},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "bytes_per_row": bytes_per_row, "kernel": kname},
            "gpu_launches": args.steps, "clocks": clk.summary(t_start, t_end), "wall_s_timed": t_wall}
    legs = set() if args.no_extras else set(args.legs.split(","))
    col0 = None  # FP32 batched result column fed with x, for the parity check
    if "e2e" in legs and rank == 0:
        # end to end through the C-ABI with pinned host buffers (copies inside the timed region), measured
        # right after the headline, in the same device state
        xh = torch.from_numpy(x_host).pin_memory()
        yh = torch.zeros(n, dtype=torch.float64).pin_memory()
        lib = q.load()
        lib.qsi_op_apply(op._h, C.c_void_p(xh.data_ptr()), C.c_void_p(yh.data_ptr()), 0, 0, None)
        ke = max(3, args.steps // 2)
        t0 = time.time()
        for _ in range(ke):
            st = lib.qsi_op_apply(op._h, C.c_void_p(xh.data_ptr()), C.c_void_p(yh.data_ptr()), 0, 0, None)
            assert st == 0, q._lib.last_error()
        te = (time.time() - t0) / ke
        line["e2e"] = {"value": n / te, "unit": "states/s", "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n,
                       "api": "qsi_op_apply(host pointers)",
                       "bitwise_equal_to_device_apply": bool(np.array_equal(yh.numpy(), y_host))}
        del xh, yh
    if "batched" in legs and rank == 0:
        # batched mixed precision: R FP32 vectors [row][R], double-float row accumulation.  The first R of --R
        # is reported as `batched_mixed` and runs last, so that its tuned settings stay for the FTLM leg.  Its
        # column 0 holds the headline's x (rounded to FP32) for the parity check.
        Rs = [int(v) for v in str(args.R).split(",") if v]
        for R in Rs[1:] + Rs[:1]:
            tkey = "batched" if R == Rs[0] else f"batched_r{R}"
            X = Y = None
            try:
                X = torch.randn(n, R, dtype=torch.float32, device=dev)
                Y = torch.zeros_like(X)
            except torch.cuda.OutOfMemoryError as e:  # device memory taken by others: report, go on
                line["batched_mixed" if R == Rs[0] else f"batched_mixed_r{R}"] = {"R": R, "skipped": str(e)[:160]}
                X = Y = None
                torch.cuda.empty_cache()
                continue
            X[:, 0] = x.float()
            if not args.no_tune:
                t0 = time.time()
                log = op.autotune(R=R, dtype="f32", X=X, Y=Y, tune_lookup=True)
                tuning[tkey] = {"seconds": round(time.time() - t0, 2), "trials": len(log.splitlines()) - 2,
                                "settings": op.tuning(1)}
            for _ in range(2):
                op.apply_batched(X, Y)
            torch.cuda.synchronize()
            kb = max(3, args.steps // 2)
            ev_b = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(kb)]
            torch.cuda.nvtx.range_push("timed_batched")
            for a_, b_ in ev_b:
                a_.record(stream)
                op.apply_batched(X, Y)
                b_.record(stream)
            torch.cuda.nvtx.range_pop()
            torch.cuda.synchronize()
            if R == Rs[0]:
                col0 = Y[:, 0].double().cpu().numpy()
            bms = sum(a_.elapsed_time(b_) for a_, b_ in ev_b) / kb
            bval = n * R / (bms * 1e-3)
            bbytes = n * (16 + R * 4 * (h + 2))
            tb = op.tuning(1)
            blk = "LookupHash" if tb["use_hash"] and basis.index_info()["hash"] else "LookupTable"
            bk = f"k_apply_tile_batched<float,{blk},FF,16-byte gathers x{tb['vec_width'] or 4}> R={R}"
            bach = bbytes / (bms * 1e-3) / 1e9
            key = "batched_mixed" if R == Rs[0] else f"batched_mixed_r{R}"
            line[key] = {"value": bval, "unit": "state-vectors/s", "R": R, "ms_per_apply": bms,
                         "accumulation": "double-float (2xFP32) per row", "storage": "FP32 [row][R]",
                         "vs_plain_fp64": bval / value * ws,
                         "roofline": {"bound": "hbm", "achieved": bach, "peak": peak, "unit": "GB/s",
                                      "frac": bach / peak, "peak_kind": peak_kind,
                                      "bytes_per_row": 16 + R * 4 * (h + 2), "kernel": bk,
                                      "traffic": measured_traffic(w.name, bk, n)}}
            del X, Y
            torch.cuda.empty_cache()
    if "ftlm" in legs and rank == 0:
        # FTLM vector-steps/s on the same operator: batched mixed precision (ftlm-R FP32 vectors, one apply
        # launch per step, the run captured in one CUDA graph, the in-place two-block recurrence) against plain
        # FP64 single-vector Lanczos.
        # Per-step rates come from the difference of an M and an M/3 step run (setup, capture and readout
        # cancel); the rates including setup are given beside them (ftlm_rate).

        R_ftlm = args.ftlm_R or int(str(args.R).split(",")[0])
        note = None
        try:
            mixed = ftlm_rate(q, [op], R_ftlm, "mixed", args.ftlm_steps, 2)  # settings tuned for R = first of --R
        except q.QsiError as e:  # device memory taken by others: half the vectors
            if R_ftlm <= 16:
                raise
            note = f"R={R_ftlm} failed ({str(e)[:120]}); R={R_ftlm // 2} instead"
            R_ftlm //= 2
            torch.cuda.empty_cache()
            mixed = ftlm_rate(q, [op], R_ftlm, "mixed", args.ftlm_steps, 2)
        mixed["vector_blocks"] = 2
        step_b = ftlm_step_bytes(n, R_ftlm, h, mixed["vector_blocks"])
        fach = step_b / (mixed["ms_per_step"] * 1e-3) / 1e9
        mixed["roofline"] = {"bound": "hbm", "achieved": fach, "peak": peak, "unit": "GB/s", "frac": fach / peak,
                             "peak_kind": peak_kind, "bytes_per_step": step_b,
                             "counted": "apply (with the read of the block it accumulates into) + one dots pass + one update pass (ftlm_step_bytes)"}
        if note:
            mixed["note"] = note
        torch.cuda.empty_cache()
        plain = ftlm_rate(q, [op], 1, "f64", args.ftlm_steps)
        line["ftlm"] = {"value": mixed["vec_steps_per_s"], "unit": "vec-steps/s", "mixed": mixed, "plain_fp64": plain,
                        "speedup_vs_plain_fp64": mixed["vec_steps_per_s"] / plain["vec_steps_per_s"]}
    if "lanczos" in legs and rank == 0:
        # 96-spin eigen-solves: the nev lowest eigenpairs in plain FP64 and in
        # mixed precision (FP32 Krylov vectors and gathers, FP64 recurrences, FP64 Rayleigh-Ritz polish), and the
        # errors of the mixed eigenvalues against the FP64 ones
        del x, y
        torch.cuda.empty_cache()
        out = {"nev": args.nev, "ncv": args.ncv, "tol": 1e-10}
        res = {}
        for prec, polish in (("f64", 0), ("mixed", 3)):
            torch.cuda.synchronize()
            t0 = time.time()
            ev, _, rep = q.diagonalise(op, nev=args.nev, ncv=args.ncv, tol=1e-10, max_iter=400, seed=1,
                                       precision=prec, polish_steps=polish, want_vectors=False)
            dt = time.time() - t0
            res[prec] = ev
            out[prec] = {"seconds": dt, "applies": rep.applies, "restarts": rep.restarts, "converged": rep.converged,
                         "evals": [float(v) for v in ev], "max_residual": float(np.max(rep.residual[:args.nev]))}
        # Single-vector Krylov methods pick up copies of a degenerate level only through rounding, so the two
        # runs may list a degenerate level a different number of times: each mixed eigenvalue is compared
        # with the nearest FP64 eigenvalue, over the levels both runs reached (below the larger of their
        # highest values, the lists are complete in both).
        top = min(res["mixed"].max(), res["f64"].max())
        err = np.array([np.abs(res["f64"] - v).min() for v in res["mixed"] if v <= top + 1e-8])
        out["abs_err_mixed_vs_f64"] = [float(v) for v in err]
        out["max_abs_err"] = float(err.max())
        out["levels_compared"] = int(len(err))
        out["within_1e-9"] = bool(err.max() <= 1e-9)
        out["speedup_mixed_vs_f64"] = out["f64"]["seconds"] / out["mixed"]["seconds"]
        line["lanczos"] = out
    if "ftlm_sectors" in legs and rank == 0:
        line["ftlm_sectors"] = ftlm_sectors_leg(args)
    if "serve" in legs and rank == 0:
        line["serve"] = serve_leg(args)
    if "materialised" in legs and rank == 0:
        if "x" not in locals():  # the lanczos leg released the headline's vectors
            x = torch.from_numpy(x_host).to(dev)
        line["materialised"] = materialised_leg(args, q, op, n, h, x, y_host, peak, peak_kind, "lanczos" in legs,
                                                w.name)
    if "cpu" in legs and rank == 0:
        # One whole apply of the reference's push loop (oracle restatement) on all host cores, on the headline's
        # x: the CPU baseline (whole apply, no sample) and the full-size parity check of the GPU results.
        y_ref, dt, threads, lookups = oracle_whole_apply(w.basis_lohi, H.specs(), x_host)
        line["cpu_baseline"] = {"value": n / dt, "unit": "states/s", "cores": threads, "kind": "port",
                                "sample": f"one whole apply, all {n} source rows (per-term OpenMP pass, atomic "
                                          f"scatter, {lookups} lookups), {dt:.1f}s"}
        scale = float(np.abs(y_ref).max())
        par = {"reference": "oracle push-loop apply of the same x, whole basis",
               "apply_fp64": {"max_abs_err": float(np.abs(y_host - y_ref).max()),
                              "rel_err": float(np.abs(y_host - y_ref).max()) / scale, "tol_rel": 1e-12}}
        par["apply_fp64"]["pass"] = par["apply_fp64"]["rel_err"] <= 1e-12
        if col0 is not None:
            e = float(np.abs(col0 - y_ref).max()) / scale
            par["apply_fp32_batched_col0"] = {"rel_err": e, "tol_rel": 4e-6, "pass": e <= 4e-6,
                                              "note": "x rounded to FP32, double-float row accumulation"}
        line["parity"] = par
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
