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
