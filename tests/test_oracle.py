"""The oracle (CPU restatement) against the reference's golden data."""
import json

import numpy as np
import pytest

from helpers import GOLDEN, cases, golden_json, sha
from oracle import oracle as O


def test_oracle_term_compiler_matches_reference_masks():
    for kat in golden_json("term_kats.json"):
        toks = kat["spec"].split()
        t = O.terms_array([(1.0, "".join(x[-1] for x in toks), [int(x[:-1]) for x in toks])])
        words = t[0, 8:72].view(np.uint64)
        assert [str(int(w)) for w in words] == kat["masks"], kat["spec"]
        assert int(t[0, 72:76].view(np.int32)[0]) == kat["sign"], kat["spec"]


@pytest.mark.parametrize("name", ["golden48_JpmB", "ref32_g", "ref32_JpmB", "q0_32", "s4444"])
def test_oracle_triplets_match_reference_digest(name):
    basis, H = cases()[name]
    ref = golden_json("triplets.json")[name]
    assert len(basis) == ref["n_basis"] and sha(basis) == ref["basis_sha256"]
    r, c, v = O.triplets_port(basis, H.specs())
    assert len(r) == ref["n_triplets"]
    assert O.triplet_digest(r, c, v) == ref["sha256"]


def test_oracle_apply_matches_reference_apply():
    cs = cases()
    for fname, case in [("apply_ref32.npy", "ref32_g"), ("apply_q0_32.npy", "q0_32")]:
        x, y_ref = np.load(GOLDEN / fname)
        basis, H = cs[case]
        y = O.apply_port(basis, H.specs(), x, threads=1)
        np.testing.assert_allclose(y, y_ref, rtol=0, atol=1e-13 * np.abs(y_ref).max())


def test_oracle_wide_states_match_reference():
    """States up to 128 bits (spin i at bit 4i+3): connectivity digest and y = H x from the reference's own
    operator code."""
    from helpers import wide_case

    lohi, H, specs = wide_case()
    ref = golden_json("wide128.json")
    assert len(lohi) == ref["n_basis"] and sha(lohi) == ref["basis_sha256"]
    assert int(lohi[:, 1].max()) >> 62
    r, c, v = O.triplets_port(lohi, specs)
    assert len(r) == ref["n_triplets"] and O.triplet_digest(r, c, v) == ref["sha256"]
    x, y_ref = np.load(GOLDEN / "apply_wide128.npy")
    y = O.apply_port(lohi, specs, x, threads=1)
    np.testing.assert_allclose(y, y_ref, rtol=0, atol=1e-13 * np.abs(y_ref).max())


def test_oracle_golden_ground_state_energy():
    basis, H = cases()["golden48_JpmB"]
    g = golden_json("golden48.json")
    r, c, v = O.triplets_port(basis, H.specs())
    w, V = O.lowest_eigs(r, c, v, len(basis), k=1)
    assert abs(w[0] - g["E0"]) <= 1e-10
    ev = np.load(GOLDEN / "golden48_evec.npy").astype(np.float64)
    assert abs(abs(ev @ V[:, 0]) / np.linalg.norm(ev) - 1.0) < 1e-6


def test_two_block_recurrence_equals_three_term_recurrence():
    """The in-place two-block FTLM recurrence the GPU runs when three vector blocks do not fit
    (P <- H C - beta_prev P; alpha = <C, P>; P <- P - alpha C; beta = |P|; P /= beta; swap) gives the three-term
    recurrence's alphas and betas (W = H C; alpha = <C, W>; P <- W - alpha C - beta_prev P), FP64 numpy."""
    basis, H = cases()["s4444"]
    r, c, v = O.triplets_port(basis, H.specs())
    A = O.csr_from_triplets(r, c, v, len(basis))
    n, M = len(basis), 30
    q0 = np.random.default_rng(3).choice([-1.0, 1.0], size=n) / np.sqrt(n)
    a3, b3 = [], []
    C, P, bp = q0.copy(), np.zeros(n), 0.0
    for _ in range(M):
        W = A @ C
        al = C @ W
        P = W - al * C - bp * P
        bp = np.linalg.norm(P)
        a3.append(al), b3.append(bp)
        P, C = C, P / bp
    a2, b2 = [], []
    C, P, bp = q0.copy(), np.zeros(n), 0.0
    for _ in range(M):
        P = A @ C - bp * P
        al = C @ P
        P = P - al * C
        bp = np.linalg.norm(P)
        a2.append(al), b2.append(bp)
        P, C = C, P / bp
    np.testing.assert_allclose(a2[:20], a3[:20], rtol=0, atol=1e-12)
    np.testing.assert_allclose(b2[:20], b3[:20], rtol=0, atol=1e-12)


def test_oracle_q0_32spin_eigs():
    basis, H = cases()["q0_32"]
    ref = golden_json("eigs_q0_32.json")["evals"]
    r, c, v = O.triplets_port(basis, H.specs())
    w, _ = O.lowest_eigs(r, c, v, len(basis), k=5)
    np.testing.assert_allclose(w, ref[:5], atol=1e-12)


def test_oracle_ftlm_formula_approaches_exact():
    basis, H = cases()["s4444"]
    th = np.load(GOLDEN / "thermo_s4444.npz")
    r, c, v = O.triplets_port(basis, H.specs())
    f = O.ftlm_oracle(r, c, v, len(basis), R=32, M=60, seed=0, temps=th["T"])
    hi = th["T"] > 0.5  # FTLM with few vectors is accurate at high T
    np.testing.assert_allclose(f["C"][hi], th["C"][hi], rtol=0.15, atol=0.02)


# The reference's stored observables (.eigs.out.h5) were computed from an eigenvector that differs from the
# stored unit vector at the 1e-5 level (a different run), so the values agree to this absolute tolerance.
OBS_TOL = 2e-5


def test_oracle_observables_match_reference_output():
    """ring, ring_ring and partial_vol of the golden eigenvector (eval_observables) by the oracle's restated
    operators, products and expectation loops, against the reference's stored output."""
    import json

    obs = np.load(GOLDEN / "observables48.npz")
    lat = json.load(open(GOLDEN / "lattices" / "golden48.json"))
    basis = cases()["golden48_JpmB"][0]
    psi = np.load(GOLDEN / "golden48_evec.npy").astype(np.float64)
    rings = O.ring_terms_port(lat)
    e, c = O.expectations_port(basis, rings, psi, cross=True)
    np.testing.assert_allclose(e, obs["ring"], rtol=0, atol=OBS_TOL)
    np.testing.assert_allclose(c, obs["ring_ring"], rtol=0, atol=OBS_TOL)
    for sl in range(4):
        pv, _ = O.expectations_port(basis, O.partial_vol_terms_port(lat, rings, sl), psi)
        np.testing.assert_allclose(pv, obs[f"partial_vol_sl{sl}"], rtol=0, atol=OBS_TOL)


def test_oracle_term_product_matches_reference_kats():
    """operator*= restated in the oracle reproduces the reference's compiled products ("0Z 0X" etc.)."""
    for kat in golden_json("term_kats.json"):
        toks = kat["spec"].split()
        if len(toks) < 2 or len(set(int(t[:-1]) for t in toks)) != 1:
            continue
        # a product of single-site operators on one spin, built factor by factor
        factors = np.concatenate([O.terms_array([(1.0, t[-1], [int(t[:-1])])]) for t in toks])
        prod = O.term_product_port(factors)
        whole = O.terms_array([(1.0, "".join(t[-1] for t in toks), [int(t[:-1]) for t in toks])])
        sign_p, sign_w = prod.view(np.int32)[0, 18], whole.view(np.int32)[0, 18]
        assert sign_p == sign_w, kat["spec"]
        if sign_w != 0:  # a vanished operator's masks carry no meaning
            assert prod.tobytes() == whole.tobytes(), kat["spec"]


def test_term_compiler_and_apply_state_match_the_reference_on_random_strings():
    """2,000 seeded random operator strings (x X z Z + - p P q Q, repeated sites allowed, sites up to 127): the
    library's term compiler gives the reference SymbolicPMROperator's masks and sign, and applyState on random
    128-bit states gives its state and sign."""
    import qsi_subspace_ed_gb300 as q

    if O.ref() is None:
        pytest.skip("the reference checkout is absent")
    rng = np.random.default_rng(2024)
    alphabet = "xXzZ+-pPqQ"
    for _ in range(2000):
        k = int(rng.integers(1, 9))
        ops = "".join(rng.choice(list(alphabet), size=k))
        if rng.random() < 0.03:  # an operator letter neither accepts
            ops = ops[:-1] + "y"
        hi = 128 if rng.random() < 0.5 else 16  # small site ranges make repeated sites common
        ids = [int(v) for v in rng.integers(0, hi, size=k)]
        try:
            m_ref, sg_ref = O.term_masks_ref(ops, ids)
        except ValueError:
            with pytest.raises(q.QsiError):
                q.SymbolicPMROperator(ops, ids)
            continue
        op = q.SymbolicPMROperator(ops, ids)
        words = [op.t.x[0], op.t.x[1], op.t.z[0], op.t.z[1], op.t.up[0], op.t.up[1], op.t.down[0], op.t.down[1]]
        assert [int(w) for w in words] == [int(w) for w in m_ref], (ops, ids)
        assert op.sign == sg_ref, (ops, ids)
        for _ in range(4):
            s = int(rng.integers(0, 2**63)) | (int(rng.integers(0, 2**63)) << 64)
            if rng.random() < 0.5:  # states that satisfy the string's requirements as well
                s = (s | int(m_ref[4]) | (int(m_ref[5]) << 64)) & ~(int(m_ref[6]) | (int(m_ref[7]) << 64))
            assert op.applyState(s) == O.apply_state_ref(ops, ids, s), (ops, ids, s)


def test_oracle_connectivity_matches_the_reference_on_random_128_bit_bases():
    """Seeded random ring-like terms on sites up to 127 and bases grown from random states by those terms (hits
    inside, misses at the frontier): the oracle's triplets are the reference's bit for bit, and its applies agree."""
    if O.ref() is None:
        pytest.skip("the reference checkout is absent")
    rng = np.random.default_rng(77)
    for case in range(3):
        specs = []
        for _ in range(12):
            sites = [int(v) for v in rng.choice(128, size=6, replace=False)]
            c = float(rng.uniform(-1, 1))
            specs += [(c, "+-+-+-", sites), (c, "-+-+-+", sites)]
        specs += [(float(rng.uniform(-1, 1)), "z", [int(rng.integers(0, 128))]) for _ in range(4)]
        seen = set()
        frontier = []
        for _ in range(20):  # random states with as many rings as possible set to a flippable pattern
            s = int(rng.integers(0, 2**63)) | (int(rng.integers(0, 2**63)) << 64) | (1 << 127) * int(case == 2)
            fixed = {}
            for _, ops, ids in specs[0:24:2]:
                phase = int(rng.integers(0, 2))
                want = [(k % 2) ^ phase for k in range(6)]  # alternating, either phase
                if all(fixed.get(i, w) == w for i, w in zip(ids, want)):
                    for i, w in zip(ids, want):
                        fixed[i] = w
            for i, w in fixed.items():
                s = (s | (1 << i)) if w else (s & ~(1 << i))
            seen.add(s)
            frontier.append(s)
        while frontier and len(seen) < 3000:
            s = frontier.pop(0)
            for _, ops, ids in specs:
                t, sg = O.apply_state_ref(ops, ids, s)
                if sg and t not in seen and rng.random() < 0.7:  # leave some targets out: misses
                    seen.add(t)
                    frontier.append(t)
        states = sorted(seen)
        basis = np.array([[v & (2**64 - 1), v >> 64] for v in states], dtype=np.uint64)
        r1, c1, v1 = O.triplets_port(basis, specs)
        r2, c2, v2 = O.triplets_ref(basis, specs)
        assert len(basis) > 1000 and len(r1) > 4 * len(basis)  # off-diagonal hits present
        assert O.triplet_digest(r1, c1, v1) == O.triplet_digest(r2, c2, v2), case
        x = rng.standard_normal(len(basis))
        y1 = O.apply_port(basis, specs, x, threads=1)
        y2 = O.apply_ref(basis, specs, x, threads=1)
        np.testing.assert_allclose(y1, y2, rtol=0, atol=1e-13 * np.abs(y2).max())


def test_interp_search_restatement_matches_the_reference():
    """ZBasisInterp (high-word bounds + low-word bisection, the basis class of diag_DOQSI_ham and bench_apply):
    the restatement returns the reference's answer for members, absent states and unseen high words."""
    from helpers import wide_case

    if O.ref() is None:
        pytest.skip("the reference checkout is absent")
    rng = np.random.default_rng(5)
    bases = [cases()["q0_32"][0], wide_case()[0]]
    # a 128-bit basis with many high words and a few long runs of one high word
    pairs = sorted({(int(h) << 40, int(v)) for h, v in zip(rng.integers(0, 50, 6000), rng.integers(0, 2**63, 6000))})
    bases.append(np.array([[v, h] for h, v in pairs], dtype=np.uint64))
    for basis in bases:
        flipped = basis[rng.integers(0, len(basis), 400)].copy()
        flipped[:, 0] ^= np.uint64(1) << np.uint64(int(rng.integers(0, 64)))
        unseen = basis[rng.integers(0, len(basis), 100)].copy()
        unseen[:, 1] ^= np.uint64(1) << np.uint64(63)
        queries = np.concatenate([basis[rng.integers(0, len(basis), 500)], flipped, unseen])
        ix = O.InterpIndex(basis)
        got, want = ix.search(queries), O.search_interp_ref(basis, queries)
        assert np.array_equal(got, want)
        assert (got[:500] >= 0).all() and (got[-100:] == -2).all()


def test_interp_push_loop_equals_the_bisection_push_loop():
    """The push loop with ZBasisInterp lookups (the CPU baseline) gives the ZBasisBST push loop's y bitwise."""
    from helpers import wide_case

    for basis, specs in [(cases()["q0_32"][0], cases()["q0_32"][1].specs()), wide_case()[::2]]:
        terms = O.terms_array(specs)
        x = np.random.default_rng(1).standard_normal(len(basis))
        y1, y2 = np.zeros(len(basis)), np.zeros(len(basis))
        O.apply_rows_port(basis, terms, x, y1, 0, len(basis), threads=1)
        assert O.InterpIndex(basis).apply_rows(terms, x, y2, 0, len(basis), threads=1) == 0
        assert np.array_equal(y1, y2)


def test_oracle_enumerator_reproduces_reference_bases():
    """The oracle's restatement of the reference's enumerator gives the reference's stored bases (digests of
    test/data/*.reference.basis.h5 and the golden 48-spin basis)."""
    ref = golden_json("bases.json")
    for name in ["ref16", "ref32", "golden48"]:
        lat = json.load(open(GOLDEN / "lattices" / f"{name}.json"))
        b = O.enumerate_basis_oracle(lat)
        assert len(b) == ref[name]["n"] and sha(b) == ref[name]["sha256"], name


def test_oracle_enumerator_matches_the_engine_with_sectors_and_spinon_pairs():
    """Sectors and 1-2 spinon pairs (whose set depends on the reference's admission test and visiting order):
    the oracle's restatement and the engine's host enumerator give the same sorted bases."""
    import qsi_subspace_ed_gb300 as q
    from qsi_subspace_ed_gb300 import workloads

    l32, l64 = workloads.lattice("pyro_1x2x1"), workloads.lattice("pyro_1x2x2")
    for lat, sec, pairs, n in ((l32, None, 0, 3618), (l32, [4, 4, 4, 4], 0, 388), (l32, None, 1, 7236),
                               (l32, None, 2, 234044), (l64, [8, 8, 8, 8], 0, 221628), (l64, [6, 8, 9, 9], 0, None)):
        a = O.enumerate_basis_oracle(lat.data, sec, pairs)
        b = q.enumerate_basis(lat, n_spinon_pairs=pairs, sector=sec)
        assert np.array_equal(a, b), (lat.name(), sec, pairs)
        if n is not None:
            assert len(a) == n


def test_oracle_hamiltonian_specs_match_the_engine():
    """The oracle's ring/Zeeman/hopping term list equals the engine's, coefficients bitwise (the reference arm of
    the benchmark builds its operator from it without the engine's library)."""
    import qsi_subspace_ed_gb300 as q
    from qsi_subspace_ed_gb300 import workloads

    for name in ("pyro_1x2x1", "pyro_1x2x3"):
        lat = workloads.lattice(name)
        g, B = workloads.ring_zeeman_params(3, (0.2, 1.0), 0.5)
        for Jpm in (0.0, 0.05):
            a = O.ring_zeeman_specs(lat.data, g, B, Jpm)
            b = q.build_ring_zeeman(lat, g, B, Jpm).specs()
            assert [(c, ops, list(ids)) for c, ops, ids in a] == [(c, ops, list(ids)) for c, ops, ids in b]
