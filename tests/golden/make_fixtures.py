"""Generates the golden fixtures of tests/golden from the reference checkout.

Run where the reference exists (python tests/golden/make_fixtures.py
REFERENCE_ROOT).  It reads the reference's own test data and drives the
reference's own operator code (oracle/_ref, built by oracle/build_ref.sh), and
writes small files next to this script:

  lattices/*.json          reference test lattices (copied data)
  bases.json               counts + SHA-256 of the reference's stored bases
  basis_ref16.npy, basis_ref32.npy   the two small stored bases
  golden48.json            stored E0 of test/data/REFERENCE_...eigs.h5 + run settings
  golden48_evec.npy        its stored eigenvector (float32)
  term_kats.json           masks/signs/applications from the reference's SymbolicPMROperator
  triplets.json            connectivity counts + SHA-256 digests from the reference code
  apply_ref32.npy, apply_q0_32.npy   y = H x from the reference code (seeded x)
  eigs_q0_32.json           FP64 lowest eigenvalues of the 32-spin Q=0 ring/Zeeman Hamiltonian
  thermo_s4444.npz         exact E(T), C(T) of the 32-spin 4.4.4.4 sector
  observables48.npz        ring, ring_ring, partial_vol_sl0..3 of the reference's stored .eigs.out.h5
  wide128.json, apply_wide128.npy   connectivity digest and y = H x from the reference code for the 32-spin
                           Q=0 case with spin i at bit 4i+3 (states up to 128 bits)
  adaptor_terms_q0_32.bin  the qsi_term array include/gb300_lazy_op.hpp builds from the reference's own operator
                           objects for the 32-spin Q=0 Hamiltonian (tests/adaptor_main.cpp)

`python tests/golden/make_fixtures.py REFERENCE_ROOT observables` (or `wide`, `adaptor`) writes only those files.
"""
from __future__ import annotations

import hashlib
import json
import shutil
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import qsi_subspace_ed_gb300 as q  # noqa: E402
from qsi_subspace_ed_gb300 import workloads  # noqa: E402
from oracle import oracle as O  # noqa: E402

if len(sys.argv) < 2:
    sys.exit("usage: make_fixtures.py REFERENCE_ROOT  (the qsi_subspace_ED checkout the fixtures are made from)")
REF = Path(sys.argv[1])
T = REF / "test"
GOLDEN_EIGS = T / "data" / "REFERENCE_Jpm=0.0200%Bx=0.1000%By=0.1000%Bz=0.1000%.eigs.h5"
GOLDEN_OBS = T / "data" / "REFERENCE_Jpm=0.0200%Bx=0.1000%By=0.1000%Bz=0.1000%.eigs.out.h5"


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    assert O.build_ref(str(REF)) is not None, "reference checkout needed"
    (HERE / "lattices").mkdir(exist_ok=True)
    lat_src = {
        "ref16": T / "lattice_files" / "pyro_1,0,0_0,1,0_0,0,2.json",
        "ref32": T / "lattice_files" / "pyro_2,0,0_0,2,0_0,0,2.json",
        "golden48": T / "lattice_files" / "pyro_2,0,0_0,2,0_0,0,3.json",
    }
    for k, p in lat_src.items():
        shutil.copy(p, HERE / "lattices" / f"{k}.json")

    # stored bases of the reference's basis-generator regression tests
    bases = {
        "ref16": q.read_basis_h5(T / "data" / "pyro_1,0,0_0,1,0_0,0,2.reference.basis.h5"),
        "ref32": q.read_basis_h5(T / "data" / "pyro_2_2_2x0,4,4b4,0,4b4,4,0b1.reference.basis.h5"),
        "golden48": q.read_basis_h5(T / "lattice_files" / "pyro_2_2_3x0,4,4b4,0,4b4,4,0b1.0test.h5"),
    }
    csv = q.read_basis_csv(T / "data" / "pyro_2_2_2x0,4,4b4,0,4b4,4,0b1.reference.basis.csv")
    assert np.array_equal(csv, bases["ref32"])
    json.dump({k: {"n": int(len(v)), "sha256": sha(v)} for k, v in bases.items()},
              open(HERE / "bases.json", "w"), indent=1)
    np.save(HERE / "basis_ref16.npy", bases["ref16"])
    np.save(HERE / "basis_ref32.npy", bases["ref32"])

    # golden end-to-end eigen-answer (test/test_correct.sh)
    e0 = q.read_f64_h5(GOLDEN_EIGS, "eigenvalues")
    ev = q.read_f64_h5(GOLDEN_EIGS, "eigenvectors").reshape(-1)
    json.dump({"E0": float(e0[0]), "E0_repr": repr(float(e0[0])), "Jpm": 0.02, "B": [0.1, 0.1, 0.1],
               "ncv": 20, "rng_seed": 11, "atol": 1e-9, "rtol": 1e-9, "algorithm": "mfeig0",
               "eigval_tol": 1e-8, "eigvec_tol": 1e-4, "dim": int(len(ev))},
              open(HERE / "golden48.json", "w"), indent=1)
    np.save(HERE / "golden48_evec.npy", ev.astype(np.float32))

    # operator known answers from the reference's SymbolicPMROperator
    specs = ["0+", "0-", "64-", "64+", "0X", "0Z", "64Z", "1z 0z", "0+ 1- 2+ 3-", "0- 1+ 2- 3+", "0Z 1X", "1X 0Z",
             "0Z 0X", "0X 0Z", "1+ 1Z", "1Z 1+", "1- 1Z", "1Z 1-", "1+ 1X", "1+ 1-", "1- 1X", "1- 1+", "1X 1+",
             "1X 1-", "1+ 1+", "1- 1-", "0Z 0X 0Z", "0X 0Z 0X", "0+ 0X 0+", "0+ 0- 0+", "0- 0X 0-", "0- 0+ 0-",
             "0+ 0Z", "0Z 0+", "64+ 64Z", "64Z 64+", "0X 0+", "0X 0-", "0p", "0q", "0P 1+", "3q 3z", "127+ 0-",
             "95- 94+ 63+ 64-", "5p 5x", "2z 2z 2x"]
    states = [0, 1, 1 << 64, 0b111010, 0b110101, 1 | 7263729, (1 << 127) | 5, (1 << 95) | (1 << 63) | 0xF0]
    kats = []
    for spec in specs:
        toks = spec.split()
        ops = "".join(t[-1] for t in toks)
        ids = [int(t[:-1]) for t in toks]
        m, sg = O.term_masks_ref(ops, ids)
        apps = []
        lib = O.ref()
        for s in states:
            st = np.array([s & (2**64 - 1), s >> 64], np.uint64)
            sign = lib.ref_apply_state(ops.encode(), np.ascontiguousarray(ids, np.int32).ctypes.data_as(
                __import__("ctypes").c_void_p), len(ops), st.ctypes.data_as(__import__("ctypes").c_void_p))
            apps.append([str(s), str(int(st[0]) | (int(st[1]) << 64)), int(sign)])
        kats.append({"spec": spec, "masks": [str(int(x)) for x in m], "sign": sg, "apply": apps})
    json.dump(kats, open(HERE / "term_kats.json", "w"), indent=0)

    # connectivity digests and applies from the reference code
    lat48 = q.Lattice.load(HERE / "lattices" / "golden48.json")
    lat32 = q.Lattice.load(HERE / "lattices" / "ref32.json")
    q0_32 = workloads.q0_32spin()
    sec4 = workloads.sector_workload("pyro_1x2x1", seed=3)
    cases = {
        "golden48_JpmB": (bases["golden48"], q.build_hamiltonian(lat48, 0.02, [0.1, 0.1, 0.1])),
        "ref32_g": (bases["ref32"], q.build_hamiltonian_g(lat32, [1.0, -0.2, -0.2, -0.2])),
        "ref32_JpmB": (bases["ref32"], q.build_hamiltonian(lat32, 0.05, [0.3, -0.1, 0.2])),
        "q0_32": (q0_32.basis_lohi, q0_32.hamiltonian()),
        "s4444": (sec4.basis_lohi, sec4.hamiltonian()),
    }
    trip = {}
    for name, (basis, H) in cases.items():
        r, c, v = O.triplets_ref(basis, H.specs())
        assert O.triplet_digest(r, c, v) == O.triplet_digest(*O.triplets_port(basis, H.specs())), name
        trip[name] = {"n_basis": int(len(basis)), "basis_sha256": sha(basis), "n_terms": len(H),
                      "n_triplets": int(len(r)), "sha256": O.triplet_digest(r, c, v)}
    json.dump(trip, open(HERE / "triplets.json", "w"), indent=1)
    rng = np.random.default_rng(0)
    x32 = rng.standard_normal(len(bases["ref32"]))
    np.save(HERE / "apply_ref32.npy", np.stack([x32, O.apply_ref(bases["ref32"], cases["ref32_g"][1].specs(), x32,
                                                                 threads=1)]))
    x1 = rng.standard_normal(len(q0_32.basis_lohi))
    np.save(HERE / "apply_q0_32.npy", np.stack([x1, O.apply_ref(q0_32.basis_lohi, cases["q0_32"][1].specs(), x1,
                                                               threads=1)]))

    # FP64 eigen-oracle for the 32-spin Q=0 case (dense, n = 3618)
    r, c, v = O.triplets_port(q0_32.basis_lohi, cases["q0_32"][1].specs())
    w, _ = O.lowest_eigs(r, c, v, len(q0_32.basis_lohi), k=10)
    json.dump({"g": q0_32.g, "B": q0_32.B, "evals": [float(x) for x in w], "n": int(len(q0_32.basis_lohi))},
              open(HERE / "eigs_q0_32.json", "w"), indent=1)
    # exact thermodynamics of the 4.4.4.4 sector (n = 388)
    r, c, v = O.triplets_port(sec4.basis_lohi, cases["s4444"][1].specs())
    H = O.csr_from_triplets(r, c, v, len(sec4.basis_lohi)).toarray()
    temps = np.logspace(-2, 1, 200)
    th = O.exact_thermo(np.linalg.eigvalsh(H), temps)
    np.savez(HERE / "thermo_s4444.npz", T=temps, E=th["E"], C=th["C"], g=np.array(sec4.g), B=np.array(sec4.B))
    print("fixtures written to", HERE)


def observables():
    """The reference's eval_observables output for the golden eigenvector (test/data/...eigs.out.h5)."""
    names = ["ring", "ring_ring"] + [f"partial_vol_sl{k}" for k in range(4)]
    np.savez(HERE / "observables48.npz", **{k: q.read_f64_h5(GOLDEN_OBS, k) for k in names},
             eigenvalues=q.read_f64_h5(GOLDEN_OBS, "eigenvalues"))
    print("observables48.npz written to", HERE)


def wide():
    """Reference connectivity and apply for states up to 128 bits (tests/helpers.py wide_case)."""
    sys.path.insert(0, str(ROOT / "tests"))
    from helpers import wide_case

    lohi, H, specs = wide_case()
    r, c, v = O.triplets_ref(lohi, specs)
    assert O.triplet_digest(r, c, v) == O.triplet_digest(*O.triplets_port(lohi, specs))
    json.dump({"n_basis": int(len(lohi)), "basis_sha256": sha(lohi), "n_terms": len(specs), "n_triplets": int(len(r)),
               "sha256": O.triplet_digest(r, c, v)}, open(HERE / "wide128.json", "w"), indent=1)
    x = np.random.default_rng(128).standard_normal(len(lohi))
    np.save(HERE / "apply_wide128.npy", np.stack([x, O.apply_ref(lohi, specs, x, threads=1)]))
    print("wide128 fixtures written to", HERE)


def adaptor():
    """The qsi_term array the reference-side adaptor (include/gb300_lazy_op.hpp) hands to the library for the
    32-spin Q=0 ring/Zeeman Hamiltonian, produced by tests/adaptor_main.cpp from the reference's own
    SymbolicPMROperator objects (the GPU test makes the adaptor's C-ABI calls with it)."""
    import tempfile

    sys.path.insert(0, str(ROOT / "tests"))
    from helpers import run_adaptor

    w = workloads.q0_32spin()
    x, _ = np.load(HERE / "apply_q0_32.npy")
    with tempfile.TemporaryDirectory() as d:
        terms, _ = run_adaptor(d, w.basis_lohi, w.hamiltonian().specs(), x, str(REF))
    (HERE / "adaptor_terms_q0_32.bin").write_bytes(terms)
    print("adaptor_terms_q0_32.bin written to", HERE)


if __name__ == "__main__":
    if len(sys.argv) > 2 and sys.argv[2] == "observables":
        observables()
    elif len(sys.argv) > 2 and sys.argv[2] == "wide":
        wide()
    elif len(sys.argv) > 2 and sys.argv[2] == "adaptor":
        adaptor()
    else:
        main()
        observables()
        wide()
        adaptor()
