"""Host logic of libqsi_ed.so (no GPU): exports, term compiler, enumerator, file IO, builders."""
import re
from pathlib import Path

import numpy as np
import pytest

import qsi_subspace_ed_gb300 as q
from qsi_subspace_ed_gb300 import _lib, workloads
from helpers import GOLDEN, golden_json, sha

ROOT = Path(__file__).resolve().parent.parent


def test_library_exports_every_header_symbol():
    import ctypes

    header = (ROOT / "include" / "qsi_ed.h").read_text()
    declared = set(re.findall(r"^\s*(?:qsi_status|void|const char\*)\s+(qsi_\w+)\s*\(", header, re.M))
    assert declared, "no declarations parsed"
    lib = ctypes.CDLL(str(_lib.LIB_PATH))
    for name in sorted(declared):
        assert hasattr(lib, name), name
    assert declared == set(_lib.SIGNATURES), declared ^ set(_lib.SIGNATURES)


def _spec(spec):
    return q.SymbolicPMROperator(spec)


def test_term_compiler_matches_reference_kats():
    for kat in golden_json("term_kats.json"):
        op = _spec(kat["spec"])
        words = [op.t.x[0], op.t.x[1], op.t.z[0], op.t.z[1], op.t.up[0], op.t.up[1], op.t.down[0], op.t.down[1]]
        assert [str(int(w)) for w in words] == kat["masks"], kat["spec"]
        assert op.sign == kat["sign"]
        for s0, s1, sign in kat["apply"]:
            assert op.applyState(int(s0)) == (int(s1), sign), (kat["spec"], s0)


def test_operator_algebra_kats():
    # test/test_PMR_construct.cpp:164-191
    a, b = _spec("0Z 1X"), _spec("1Z")
    assert a * b == _spec("0Z 1X 1Z")
    assert (_spec("0+") * _spec("0-")).sign == 1
    assert (_spec("0+") * _spec("0+")).sign == 0
    assert (_spec("0-") * _spec("0-")).sign == 0
    assert _spec("0+ 1- 2+ 3-") * _spec("0- 1+ 4- 5+") == _spec("0+ 0- 1- 1+ 2+ 3- 4- 5+")
    assert _spec("0+ 1- 2+ 3-").applyState(0b111010) == (0b110101, 1)
    assert _spec("").applyState(12345) == (12345, 1)


def test_bad_operator_spec_raises():
    with pytest.raises(q.QsiError) as e:
        _spec("3y")
    assert e.value.status == _lib.QSI_INVALID_ARG
    with pytest.raises(q.QsiError):
        _spec("5")
    with pytest.raises(q.QsiError):
        _spec("4+ 3k")
    # the reference tokeniser reads "x+" as op 'x' on spin 0
    assert _spec("x+") == _spec("0x")


def test_enumerator_reproduces_reference_bases():
    ref = golden_json("bases.json")
    for name in ["ref16", "ref32", "golden48"]:
        b = q.enumerate_basis(q.Lattice.load(GOLDEN / "lattices" / f"{name}.json"))
        assert len(b) == ref[name]["n"] and sha(b) == ref[name]["sha256"], name
    assert np.array_equal(q.enumerate_basis(q.Lattice.load(GOLDEN / "lattices" / "ref32.json")),
                          np.load(GOLDEN / "basis_ref32.npy"))


def test_enumerator_counts_on_cubic_cells():
    l32, l64 = workloads.lattice("pyro_1x2x1"), workloads.lattice("pyro_1x2x2")
    assert len(q.enumerate_basis(l32)) == 3618
    assert len(q.enumerate_basis(l32, sector=[4, 4, 4, 4])) == 388
    assert len(q.enumerate_basis(l64, sector=[8, 8, 8, 8])) == 221628
    b = q.enumerate_basis(l64)
    assert len(b) == 2891562
    hi = b[:, 1].astype(object) * 2**64 + b[:, 0].astype(object)
    assert all(hi[1:] > hi[:-1])
    # every state obeys the ice rule
    tets = l64.tetrahedra
    for s in b[:: 9973]:
        v = int(s[0]) | (int(s[1]) << 64)
        assert all(sum((v >> int(k)) & 1 for k in t) == 2 for t in tets)


def test_enumerator_spinon_rule_and_orders():
    l32 = workloads.lattice("pyro_1x2x1")
    b0 = q.enumerate_basis(l32)
    b1 = q.enumerate_basis(l32, n_spinon_pairs=1)
    s0 = {tuple(r) for r in b0.tolist()}
    assert s0 <= {tuple(r) for r in b1.tolist()}
    # without spinon pairs the set does not depend on the visiting order
    assert np.array_equal(q.enumerate_basis(l32, ordering="none"), b0)


def test_h5_roundtrip_and_errors(tmp_path):
    b = np.load(GOLDEN / "basis_ref32.npy")
    p = tmp_path / "x.h5"
    q.write_basis_h5(p, b)
    assert np.array_equal(q.read_basis_h5(p), b)
    q.write_basis_h5(p, b[:10], dataset="basis_s1.1.1.1", append=True)
    assert np.array_equal(q.read_basis_h5(p, "basis_s1.1.1.1"), b[:10])
    assert np.array_equal(q.read_basis_h5(p), b)
    with pytest.raises(q.QsiError) as e:
        q.read_basis_h5(p, "nope")
    assert e.value.status == _lib.QSI_NOT_FOUND
    with pytest.raises(q.QsiError) as e:
        q.read_basis_h5(tmp_path / "missing.h5")
    assert e.value.status == _lib.QSI_IO_ERROR
    (tmp_path / "trunc.h5").write_bytes(p.read_bytes()[:700])
    with pytest.raises(q.QsiError):
        q.read_basis_h5(tmp_path / "trunc.h5")
    e = tmp_path / "o.eigs.h5"
    vecs = np.arange(12.0).reshape(6, 2)
    q.write_eigs_h5(e, [1.0, 2.0], vecs, "lat.json", "basis")
    assert np.array_equal(q.read_f64_h5(e, "eigenvalues"), [1.0, 2.0])
    assert np.array_equal(q.read_f64_h5(e, "eigenvectors").reshape(-1), vecs.T.reshape(-1))


def test_csv_reader(tmp_path):
    b = np.load(GOLDEN / "basis_ref32.npy")
    p = tmp_path / "b.csv"
    p.write_text("".join(f"0x{int(h):016x}{int(l):016x}\n" for l, h in b))
    assert np.array_equal(q.read_basis_csv(p), b)


def test_hamiltonian_builders():
    lat = q.Lattice.load(GOLDEN / "lattices" / "golden48.json")
    H = q.build_hamiltonian(lat, 0.02, [0.1, 0.1, 0.1])
    assert len(H.off_diag_terms) == 2 * 48 and len(H.diagonal_terms) == 144
    g = q.g_vals(0.02, [0.1, 0.1, 0.1])
    assert H.off_diag_terms[0][0] == g[lat.rings[0]["sl"]]
    # ring pairs are mutual conjugates: equal coefficient, swapped up/down masks
    for k in range(0, len(H.off_diag_terms), 2):
        (c1, a), (c2, b) = H.off_diag_terms[k], H.off_diag_terms[k + 1]
        assert c1 == c2 and a.X_mask == b.X_mask and a.up_mask == b.down_mask
    Hz = q.build_ring_zeeman(workloads.lattice("pyro_1x2x1"), [1, .8, .6, .4], [0.1, 0.0, 0.0])
    assert len(Hz.diagonal_terms) == 32 and len(Hz.off_diag_terms) == 64
    with pytest.raises(RuntimeError):
        q.build_hamiltonian(q.Lattice.from_dict({**lat.data, "__version__": "1.0"}), 0.02, [0, 0, 0])


def test_cli_names_and_flags():
    """Basis-file and output naming of the reference executables, and their flags."""
    from qsi_subspace_ed_gb300 import cli

    assert str(cli.get_basis_file("a/pyro_2,0,0_0,2,0_0,0,3.json", 0)) == "a/pyro_2,0,0_0,2,0_0,0,3.0.basis.h5"
    assert str(cli.get_basis_file("a/x.json", 1, True)) == "a/x.1.basis.partitioned.h5"
    assert str(cli.get_basis_file("a/x", 2)) == "a/x.2.basis.h5"
    a = cli.diag_parser().parse_args(["L.json", "--Jpm", "0.02", "--B", "0.1", "0.1", "0.1", "-n", "1", "-N", "1",
                                      "--algorithm", "mfeig0", "-k", "20", "--rng_seed", "11", "--atol", "-9",
                                      "--rtol", "-9", "-o", "out"])
    assert (a.ncv, a.rng_seed, a.atol, a.rtol, a.algorithm, a.max_iters) == (20, 11, -9, -9, "mfeig0", 1000)
    with pytest.raises(SystemExit):
        cli.diag_parser().parse_args(["L.json", "--g", "1", "1", "1", "1", "--B", "0", "0", "0", "-o", "o"])
    f = cli.ftlm_parser().parse_args(["L.json", "--g", "1", "2", "3", "4", "-o", "o", "--T_min", "0.1", "--T_max", "2"])
    assert (f.n_randvecs, f.n_temps, f.ncv) == (20, 100, 15)
    # partition_basis: STEM.N.basis.h5 -> lattice STEM.json (replace_filename, partition_basis.cpp:235-256)
    assert str(cli.lattice_of_basis_file("a/pyro_1x2x1.12.basis.h5")) == "a/pyro_1x2x1.json"
    with pytest.raises(SystemExit):
        cli.lattice_of_basis_file("a/x.basis.h5")


def test_h5_string_round_trip(tmp_path):
    from qsi_subspace_ed_gb300.core import _read_string_h5

    p = tmp_path / "s.h5"
    q._lib.call("qsi_h5_write_string", str(p).encode(), b"latfile_json", b"pyro_2,0,0_0,2,0_0,0,3.json", 0)
    q._lib.call("qsi_h5_write_string", str(p).encode(), b"dset_name", b"basis", 1)
    assert _read_string_h5(p, "latfile_json") == "pyro_2,0,0_0,2,0_0,0,3.json"
    assert _read_string_h5(p, "dset_name") == "basis"


def test_reference_side_adaptor_runs_with_the_reference_operator_code(tmp_path):
    """include/gb300_lazy_op.hpp driven by the reference's own code (tests/adaptor_main.cpp, built against the
    reference's operator.hpp/operator.cpp): the 32-spin Q=0 basis loaded into ZBasisBST from CSV, the Hamiltonian
    built with SymbolicPMROperator, then GB300LazyOpSum::evaluate and evaluate_add.  The terms it hands to the
    library equal the engine's own term compiler's bytes; on a machine without a GPU the adaptor surfaces the
    library's error as an exception (no host fallback), and with one its results equal the reference's stored
    apply.  tests/golden/adaptor_terms_q0_32.bin holds those terms for the GPU test of the same calls."""
    import shutil

    from helpers import run_adaptor
    from oracle import oracle as O

    root = O.reference_root()
    if not shutil.which("g++") or root is None:
        pytest.skip("needs g++ and the reference checkout")
    w = workloads.q0_32spin()
    H = w.hamiltonian()
    x, y_ref = np.load(GOLDEN / "apply_q0_32.npy")
    terms, y = run_adaptor(tmp_path, w.basis_lohi, H.specs(), x, root)
    arr, nt = H.to_terms()
    assert terms == bytes(arr)[: nt * 80]
    assert terms == (GOLDEN / "adaptor_terms_q0_32.bin").read_bytes()
    if isinstance(y, str):
        assert "QSI_CUDA_ERROR" in y or "CUDA" in y, y
    else:
        np.testing.assert_allclose(y[0], y_ref, rtol=0, atol=1e-12 * np.abs(y_ref).max())
        np.testing.assert_allclose(y[1], 2 * y_ref, rtol=0, atol=2e-12 * np.abs(y_ref).max())


def test_reference_arm_runs_on_the_host():
    """`bench.py --impl reference` (the restated push loop on the host cores) prints one contract line, builds its
    basis and terms with the oracle alone (the engine's library is never loaded) and reports the same config as
    the GPU arm would for that workload."""
    import json
    import subprocess
    import sys

    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--lattice', 'pyro_1x2x1', "
            "'--full-basis', '--steps', '2', '--warmup', '1', '--ref-step-seconds', '0.2']; "
            "runpy.run_path('bench.py', run_name='__main__'); "
            "print('LOADED_ENGINE', 'libqsi_ed' in open('/proc/self/maps').read())")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    assert "LOADED_ENGINE False" in r.stdout
    d = lines[0]
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "states/s"
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "states/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["ms_per_step"] > 0 and d["steps"] == 2
    # the GPU arm's config for this workload: same keys and values
    sys.path.insert(0, str(ROOT))
    import bench

    class A:
        lattice, full_basis, sector, seed = "pyro_1x2x1", True, "", 3

    spec = bench.workload_spec(A)
    w = workloads.q0_32spin()
    g, B = workloads.ring_zeeman_params(3, (0.2, 1.0), 0.5)
    assert spec["g"] == [float(v) for v in g] and spec["B"] == [float(v) for v in B]
    H = q.build_ring_zeeman(workloads.lattice("pyro_1x2x1"), spec["g"], spec["B"])
    assert d["config"] == bench.workload_config(spec, len(w.basis_lohi), len(H))
    assert d["config"]["workload"] == "pyro_1x2x1.Q0" and d["config"]["n_states"] == 3618


def test_reference_arm_samples_cover_the_basis():
    import bench

    n = 1_000_003
    for step in range(5):
        blocks = bench.sample_blocks(n, 100_000, step)
        assert len(blocks) == 16
        assert all(0 <= a < b <= n for a, b in blocks)
        assert all(blocks[k][1] <= blocks[k + 1][0] for k in range(15))  # disjoint, in order
        assert blocks[0][0] < n // 16 and blocks[-1][0] >= 15 * (n // 16)  # spread over the whole basis
    assert bench.sample_blocks(100, 1000, 0)[-1][1] <= 100


def test_device_path_fails_loudly_without_a_gpu():
    """No host fallback: without a usable GPU the device entry points return an error, never a CPU result."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    basis = workloads.q0_32spin().basis_lohi
    with pytest.raises(q.QsiError, match="QSI_CUDA_ERROR"):
        q.ZBasis(basis)


def test_new_entry_points_reject_null_handles():
    """qsi_op_materialise and qsi_family_set_min_rows return QSI_INVALID_ARG for a null handle (no GPU needed)."""
    import ctypes as C

    from qsi_subspace_ed_gb300 import _lib

    lib = q.load()
    nb = C.c_int64()
    assert lib.qsi_op_materialise(None, 1, C.byref(nb)) == _lib.QSI_INVALID_ARG
    assert lib.qsi_op_materialise(None, 0, None) == _lib.QSI_INVALID_ARG
    assert lib.qsi_family_set_min_rows(None, 0) == _lib.QSI_INVALID_ARG
