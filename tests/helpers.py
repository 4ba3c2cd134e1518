"""Shared helpers for the tests (fixture loading, cases)."""
import hashlib
import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def golden_json(name):
    return json.load(open(GOLDEN / name))


def cases():
    """name -> (basis lohi, SymbolicOpSum), matching tests/golden/make_fixtures.py."""
    import qsi_subspace_ed_gb300 as q
    from qsi_subspace_ed_gb300 import workloads

    lat48 = q.Lattice.load(GOLDEN / "lattices" / "golden48.json")
    lat32 = q.Lattice.load(GOLDEN / "lattices" / "ref32.json")
    b32 = np.load(GOLDEN / "basis_ref32.npy")
    q0_32 = workloads.q0_32spin()
    sec4 = workloads.sector_workload("pyro_1x2x1", seed=3)
    return {
        "golden48_JpmB": (q.enumerate_basis(lat48), q.build_hamiltonian(lat48, 0.02, [0.1, 0.1, 0.1])),
        "ref32_g": (b32, q.build_hamiltonian_g(lat32, [1.0, -0.2, -0.2, -0.2])),
        "ref32_JpmB": (b32, q.build_hamiltonian(lat32, 0.05, [0.3, -0.1, 0.2])),
        "q0_32": (q0_32.basis_lohi, q0_32.hamiltonian()),
        "s4444": (sec4.basis_lohi, sec4.hamiltonian()),
    }


def wide_case():
    """The 32-spin Q=0 basis and ring/Zeeman Hamiltonian with spin i moved to bit 4i+3 (states up to 128 bits,
    beyond the 96 bits the hash index takes): (basis lohi, SymbolicOpSum, specs), matching
    tests/golden/make_fixtures.py."""
    import qsi_subspace_ed_gb300 as q
    from qsi_subspace_ed_gb300 import workloads

    w = workloads.q0_32spin()
    wide = []
    for lo, hi in w.basis_lohi:
        s = int(lo) | (int(hi) << 64)
        v = 0
        for i in range(32):
            if (s >> i) & 1:
                v |= 1 << (4 * i + 3)
        wide.append(v)
    wide.sort()
    lohi = np.array([[v & (2**64 - 1), v >> 64] for v in wide], dtype=np.uint64)
    specs = [(c, ops, [4 * i + 3 for i in ids]) for c, ops, ids in w.hamiltonian().specs()]
    H = q.SymbolicOpSum()
    for c, ops, ids in specs:
        H.add_term(c, q.SymbolicPMROperator(ops, ids))
    return lohi, H, specs


def run_adaptor(workdir, basis_lohi, specs, x, reference_root):
    """Builds tests/adaptor_main.cpp against the reference checkout's operator code and the engine's library, runs
    it on (basis, term specs, x) and returns (the qsi_term bytes the adaptor hands to the library, y = H x and
    y += H x as a (2, n) array, or the library's error text when its device path cannot run)."""
    import subprocess

    from qsi_subspace_ed_gb300 import _lib

    workdir = Path(workdir)
    ref = Path(reference_root)
    root = Path(__file__).resolve().parent.parent
    lib = Path(_lib.LIB_PATH)
    exe = workdir / "adaptor_main"
    cmd = ["g++", "-std=c++17", "-O1", "-fopenmp", f"-I{root / 'oracle' / 'ref_shim'}",
           f"-I{ref / 'components' / 'operator' / 'include'}", f"-I{ref / 'components' / 'common' / 'include'}",
           f"-I{root / 'include'}", str(root / "tests" / "adaptor_main.cpp"),
           str(ref / "components" / "operator" / "src" / "operator.cpp"),
           f"-L{lib.parent}", "-lqsi_ed", f"-Wl,-rpath,{lib.parent}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr[-3000:])
    with open(workdir / "basis.csv", "w") as f:  # basis_io::write_line (components/common/include/basis_io.hpp:16-18)
        f.writelines("0x%016x%016x\n" % (int(hi), int(lo)) for lo, hi in basis_lohi)
    with open(workdir / "terms.txt", "w") as f:
        f.writelines("%.17g %s %s\n" % (c, ops, " ".join(map(str, ids))) for c, ops, ids in specs)
    np.ascontiguousarray(x, dtype=np.float64).tofile(workdir / "x.bin")
    r = subprocess.run([str(exe), str(workdir / "basis.csv"), str(workdir / "terms.txt"), str(workdir / "x.bin"),
                        str(workdir / "terms_out.bin"), str(workdir / "y_out.bin")], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"adaptor_main exited {r.returncode}: {r.stderr[-2000:]}")
    terms = (workdir / "terms_out.bin").read_bytes()
    if r.stdout.startswith("library error:"):
        return terms, r.stdout.strip()
    return terms, np.fromfile(workdir / "y_out.bin", dtype=np.float64).reshape(2, -1)
