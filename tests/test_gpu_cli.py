"""The reference executables' command lines, run on the GPU engine (the flow of the reference's
test/test_correct.sh, then eval_observables, build_hamiltonian and an FTLM run)."""
import json
import shutil

import numpy as np
import pytest

import qsi_subspace_ed_gb300 as q
from helpers import GOLDEN, cases, golden_json
from qsi_subspace_ed_gb300 import cli

pytestmark = pytest.mark.gpu

LAT = "pyro_2,0,0_0,2,0_0,0,3.json"


@pytest.fixture(scope="module")
def golden_dir(tmp_path_factory):
    d = tmp_path_factory.mktemp("lat")
    shutil.copy(GOLDEN / "lattices" / "golden48.json", d / LAT)
    q.write_basis_h5(cli.get_basis_file(d / LAT, 0), cases()["golden48_JpmB"][0])
    return d


def test_diag_mfeig0_reproduces_reference_file(golden_dir, tmp_path):
    """bin/diag_DOQSI_ham LAT --Jpm 0.02 --B 0.1 0.1 0.1 -n 1 -N 1 --algorithm mfeig0 -k 20 --rng_seed 11
    --atol -9 --rtol -9 -o OUT, compared as test_correct.sh does (eigenvalue to 1e-8)."""
    out = cli.diag_main([str(golden_dir / LAT), "--Jpm", "0.02", "--B", "0.1", "0.1", "0.1", "-n", "1", "-N", "1",
                         "--algorithm", "mfeig0", "-k", "20", "--rng_seed", "11", "--atol", "-9", "--rtol", "-9",
                         "-o", str(tmp_path)])
    assert out.name == "Jpm=0.0200%Bx=0.1000%By=0.1000%Bz=0.1000%.eigs.h5"
    g = golden_json("golden48.json")
    e = q.read_f64_h5(out, "eigenvalues")
    assert abs(e[0] - g["E0"]) < 1e-8
    v = q.read_f64_h5(out, "eigenvectors").reshape(-1)
    stored = np.load(GOLDEN / "golden48_evec.npy").astype(np.float64)
    assert abs(v @ stored) / np.linalg.norm(v) / np.linalg.norm(stored) > 1 - 1e-4
    from qsi_subspace_ed_gb300.core import _read_string_h5
    assert _read_string_h5(out, "latfile_json") == LAT and _read_string_h5(out, "dset_name") == "basis"


def test_diag_mfsparse_and_matrix_export(golden_dir, tmp_path):
    out = cli.diag_main([str(golden_dir / LAT), "--Jpm", "0.02", "--B", "0.1", "0.1", "0.1", "-n", "3", "-N", "2",
                         "--algorithm", "mfsparse", "--ncv", "12", "--atol", "-10", "-o", str(tmp_path)])
    e = q.read_f64_h5(out, "eigenvalues")
    assert e.shape == (3,) and abs(e[0] - golden_json("golden48.json")["E0"]) < 1e-9
    assert q.read_f64_h5(out, "eigenvectors").shape == (len(cases()["golden48_JpmB"][0]), 2)
    # eval_observables on that file (its ground-state vector): the reference's stored output
    obs = q.read_observables_h5(cli.eval_main([str(out), "--latfile_dir", str(golden_dir), "-N", "1"]))
    ref = np.load(GOLDEN / "observables48.npz")
    for k in ("ring", "ring_ring") + tuple(f"partial_vol_sl{sl}" for sl in range(4)):
        np.testing.assert_allclose(obs[k], ref[k], rtol=0, atol=5e-5)
    mtx = cli.build_main([str(golden_dir / LAT), "--Jpm", "0.02", "--B", "0.1", "0.1", "0.1", "-o", str(tmp_path)])
    basis, H = cases()["golden48_JpmB"]
    op = q.LazyOpSum(q.ZBasis(basis), H)
    op.saveMarket(tmp_path / "direct.mtx")
    assert mtx.read_bytes() == (tmp_path / "direct.mtx").read_bytes()


def test_ftlm_cli(tmp_path):
    from qsi_subspace_ed_gb300 import workloads

    lat = workloads.lattice("pyro_1x2x1")
    shutil.copy(workloads.LATTICE_DIR / "pyro_1x2x1.json", tmp_path / "lat.json")
    q.write_basis_h5(cli.get_basis_file(tmp_path / "lat.json", 0), q.enumerate_basis(lat))
    out = cli.ftlm_main([str(tmp_path / "lat.json"), "--g", "1", "0.8", "0.6", "0.4", "-o", str(tmp_path), "-k", "40",
                         "-R", "16", "-S", "50", "--T_min", "0.05", "--T_max", "5", "--rng_seed", "2"])
    assert out.name == "g0=1.0000%g1=0.8000%g2=0.6000%g3=0.4000%.ftlm.h5"
    C = q.read_f64_h5(out, "C")
    T = q.read_f64_h5(out, "T")
    assert C.shape == (50,) and np.all(np.isfinite(C)) and np.all(C >= -1e-9) and T[0] == pytest.approx(0.05)
