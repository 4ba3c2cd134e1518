"""GPU basis enumeration against the host enumerator and the reference's stored bases."""
import numpy as np
import pytest

import qsi_subspace_ed_gb300 as q
from qsi_subspace_ed_gb300 import workloads
from helpers import GOLDEN, golden_json, sha

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["ref16", "ref32", "golden48"])
def test_gpu_enumeration_matches_reference_bases(name):
    ref = golden_json("bases.json")[name]
    b = q.enumerate_basis_gpu(q.Lattice.load(GOLDEN / "lattices" / f"{name}.json"))
    assert len(b) == ref["n"] and sha(b) == ref["sha256"]


@pytest.mark.parametrize("lat,sector", [("pyro_1x2x1", None), ("pyro_1x2x1", [4, 4, 4, 4]),
                                        ("pyro_1x2x2", None), ("pyro_1x2x2", [8, 8, 8, 8]),
                                        ("pyro_1x2x2", [7, 9, 8, 8])])
def test_gpu_enumeration_matches_host(lat, sector):
    L = workloads.lattice(lat)
    assert np.array_equal(q.enumerate_basis_gpu(L, sector=sector), q.enumerate_basis(L, sector=sector))


@pytest.mark.parametrize("lat,pairs,sector", [("pyro_1x2x1", 1, None), ("pyro_1x2x1", 2, None),
                                              ("pyro_1x2x1", 1, [4, 4, 4, 4]), ("pyro_1x2x1", 2, [4, 4, 4, 4]),
                                              ("pyro_1x2x2", 1, None)])
def test_gpu_enumeration_with_spinon_pairs(lat, pairs, sector):
    """Spinon-pair bases (the forking rule of the reference's enumerator) from the GPU walk equal the host
    enumerator's and the oracle's restatement of the reference's."""
    from oracle import oracle as O

    L = workloads.lattice(lat)
    b = q.enumerate_basis_gpu(L, sector=sector, n_spinon_pairs=pairs)
    assert np.array_equal(b, q.enumerate_basis(L, sector=sector, n_spinon_pairs=pairs))
    assert np.array_equal(b, O.enumerate_basis_oracle(L.data, sector, pairs))


def _sector_oracle(lohi, lat):
    """States grouped by sublattice up counts, restated in numpy (basis order inside a sector)."""
    out = {}
    sl = lat.sublattice
    for row in lohi:
        v = int(row[0]) | (int(row[1]) << 64)
        key = tuple(sum((v >> int(i)) & 1 for i in np.flatnonzero(sl == a)) for a in range(int(sl.max()) + 1))
        out.setdefault(key, []).append(row)
    return {k: np.array(v, dtype=np.uint64) for k, v in out.items()}


def test_partition_into_sectors_matches_sector_enumeration():
    """The GPU partition of the 32- and 64-spin Q=0 bases: every sector is the sector's own enumeration, sectors
    in ascending order of their counts, their union the whole basis."""
    for name in ("pyro_1x2x1", "pyro_1x2x2"):
        L = workloads.lattice(name)
        b = q.enumerate_basis_gpu(L)
        parts = q.partition_basis(b, L)
        assert list(parts) == sorted(parts)
        assert sum(len(v) for v in parts.values()) == len(b)
        for counts in list(parts)[:: max(1, len(parts) // 12)] + [max(parts, key=lambda k: len(parts[k]))]:
            assert np.array_equal(parts[counts], q.enumerate_basis(L, sector=list(counts))), (name, counts)
        if name == "pyro_1x2x1":
            ref = _sector_oracle(b, L)
            assert set(ref) == set(parts) and all(np.array_equal(ref[k], parts[k]) for k in ref)


def test_partition_basis_tool_writes_the_sector_datasets(tmp_path):
    """partition_basis STEM.0.basis.h5 -> STEM.0.basis.partitioned.h5 with one basis_s<n0>.<n1>.<n2>.<n3>
    dataset per sector, which diag_DOQSI_ham --sector reads."""
    import shutil

    from qsi_subspace_ed_gb300 import cli

    L = workloads.lattice("pyro_1x2x1")
    b = q.enumerate_basis(L)
    shutil.copy(L.path, tmp_path / "lat.json")
    q.write_basis_h5(tmp_path / "lat.0.basis.h5", b)
    out = cli.partition_main([str(tmp_path / "lat.0.basis.h5")])
    assert out == tmp_path / "lat.0.basis.partitioned.h5"
    assert out == cli.get_basis_file(tmp_path / "lat.json", 0, subspace=True)
    for counts, states in q.partition_basis(b, L).items():
        assert np.array_equal(q.read_basis_h5(out, q.sector_name(counts)), states)
    assert len(q.read_basis_h5(out, "basis_s4.4.4.4")) == 388
