"""Pins the CPU oracle (oracle/bbs_oracle.c) to the reference.

* known-answer tests transcribed from test/MutationTree.cpp and
  test/TreeScorer.cpp (tests/golden/kat.json);
* golden vectors produced by the reference's own headers
  (tests/golden/ref_vectors.npz, tests/golden/make_golden.py);
* the fuzz property of test/MutationTree.cpp:663-744 with fixed seeds;
* the end-to-end test of test/Application.cpp:38-143 on the restated
  step loop;
* the FP64 sum-score gradient against central finite differences.
"""
import math

import numpy as np
import pytest

from bbscite_gb300 import data as D


def bits(s: str) -> int:
    return int(s, 2)


def rows_to_int(rows) -> list:
    return [int(r[0]) for r in rows]


# ----------------------------------------------------------------- KATs --

def test_kat_get_parent(orc, kat):
    k = kat["get_parent"]
    _, dm = orc.parent_to_matrix(k["parent_vector"])
    assert [orc.get_parent(dm, x) for x in range(5)] == k["expected"]


def test_kat_is_ancestor_and_descendant(orc, kat):
    am, dm = orc.parent_to_matrix(kat["is_ancestor"]["parent_vector"])
    for a, row in enumerate(kat["is_ancestor"]["expected_rows"]):
        for b, e in enumerate(row):
            assert ((int(am[a, 0]) >> b) & 1) == e
    for a, row in enumerate(kat["is_descendant"]["expected_rows"]):
        for b, e in enumerate(row):
            assert ((int(dm[a, 0]) >> b) & 1) == e


def test_kat_descendants_ancestors(orc, kat):
    pv = kat["get_descendants"]["parent_vector"]
    am, dm = orc.parent_to_matrix(pv)
    for x, exp in enumerate(kat["get_descendants"]["expected"]):
        assert [y for y in range(7) if (int(am[x, 0]) >> y) & 1] == exp
    for x, exp in enumerate(kat["get_ancestors"]["expected"]):
        assert [y for y in range(7) if (int(dm[x, 0]) >> y) & 1] == exp
    assert [orc.n_descendants(am, x) for x in range(7)] == \
        kat["get_n_descendants"]["expected"]
    assert [orc.n_ancestors(dm, x) for x in range(7)] == \
        kat["get_n_ancestors"]["expected"]


def test_kat_pruefer_and_matrix(orc, kat):
    k = kat["pruefer_code_to_parent_vector"]
    assert orc.pruefer_to_parent(k["code"]).tolist() == k["expected"]
    assert D.pruefer_to_parent(k["code"]).tolist() == k["expected"]
    k = kat["parent_vector_to_matrix"]
    am, dm = orc.parent_to_matrix(k["parent_vector"])
    assert rows_to_int(am) == [bits(s) for s in k["am"]]
    assert rows_to_int(dm) == [bits(s) for s in k["dm"]]


def test_kat_moves(orc, kat):
    beta = kat["moves"]["beta"]
    for case in kat["moves"]["cases"]:
        am, dm = orc.parent_to_matrix(case["start"])
        p = np.zeros(1, dtype=orc.MOD_PARAMS)
        for key, val in case["params"].items():
            p[key] = val
        nam, ndm, _ = orc.apply_move(am, dm, beta, p[0])
        eam, edm = orc.parent_to_matrix(case["expected"])
        assert (nam == eam).all() and (ndm == edm).all(), case["name"]
        assert orc.parent_vector(ndm).tolist() == case["expected"]


def test_kat_tree_scorer(orc, kat):
    k = kat["tree_scorer"]
    _, dm = orc.parent_to_matrix(k["parent_vector"])
    mut = np.array([[bits(s)] for s in k["is_mutated"]], dtype=np.uint64)
    known = np.array([[bits(s)] for s in k["is_known"]], dtype=np.uint64)
    a, b = k["alpha"], k["beta"]
    score, st, counts, attach = orc.logscore_tree(a, b, k["prior_sd"], dm,
                                                  mut, known)
    prior = orc.logscore_beta(a, b, k["prior_sd"], b)
    t = k["expected_terms"]
    true = (t["log(1-alpha)"] * math.log(1 - a) +
            t["log(1-beta)"] * math.log(1 - b) + t["log(beta)"] *
            math.log(b) + t["log(alpha)"] * math.log(a))
    assert (score - prior) == pytest.approx(true, rel=k["catch_approx_rel"])
    assert (st - prior) == pytest.approx(true, rel=k["catch_approx_rel"])
    # the same terms as integer class totals (n00, n01, n10, n11)
    assert counts.tolist() == [t["log(1-alpha)"], t["log(beta)"],
                               t["log(alpha)"], t["log(1-beta)"]]


# -------------------------------------------------------- golden vectors --

def test_golden_scores_bit_exact(orc, golden):
    for ci, (G, Cn) in enumerate(golden["score_cases"]):
        mut, known = D.matrix_to_bits(golden[f"score{ci}_matrix"])
        for t, pv in enumerate(golden[f"score{ci}_parents"]):
            _, dm = orc.parent_to_matrix(pv)
            for b, beta in enumerate(golden[f"score{ci}_betas"]):
                r, st, _, _ = orc.logscore_tree(1e-3, 0.2, 0.1, dm, mut,
                                                known, float(beta))
                want = golden[f"score{ci}_scores"][t, b]
                assert np.float32(r) == want, (G, Cn, t, b)
                f64 = orc.logscore_tree_f64(1e-3, float(beta), dm, mut,
                                            known, 0.2, 0.1, True)
                assert abs(st - f64) <= 1e-5 * abs(f64)


def test_golden_prior(orc, golden):
    for i, (a, bm, sd) in enumerate(golden["prior_params"]):
        for j, b in enumerate(golden["prior_betas"]):
            v = orc.logscore_beta(float(a), float(bm), float(sd), float(b))
            # NaN where float tgamma overflows (a+b > ~35), as in the
            # reference itself
            np.testing.assert_array_equal(np.float32(v),
                                          golden["prior_values"][i, j])


def _tree_hash(rows):
    h = np.uint64(1469598103934665603)
    with np.errstate(over="ignore"):
        for w in np.ascontiguousarray(rows, dtype=np.uint64).ravel():
            h = np.uint64((h ^ w) * np.uint64(1099511628211))
    return h


def test_golden_moves_bit_exact(orc, golden):
    for ci, (G, _) in enumerate(golden["move_cases"]):
        am, dm = orc.parent_to_matrix(golden[f"move{ci}_start"])
        beta = np.float32(0.3)
        raws = golden[f"move{ci}_raw"]
        for i in range(len(raws)):
            mp = orc.realize(am, dm, float(beta), raws[i])
            assert mp.tobytes() == golden[f"move{ci}_params"][i].tobytes()
            am, dm, beta = orc.apply_move(am, dm, float(beta), mp)
            assert np.float32(beta) == golden[f"move{ci}_betas"][i]
            assert _tree_hash(am) == golden[f"move{ci}_hashes"][i, 0]
            assert _tree_hash(dm) == golden[f"move{ci}_hashes"][i, 1]
            assert (orc.parent_vector(dm) ==
                    golden[f"move{ci}_parents"][i]).all()


def test_golden_chain_replay(orc, golden):
    """The restated step loop in reference score order reproduces the
    reference's proposals, decisions, final state and best score."""
    for ci, (G, Cn, steps, _) in enumerate(golden["chain_cases"]):
        G, Cn, steps = int(G), int(Cn), int(steps)
        mut, known = D.matrix_to_bits(golden[f"chain{ci}_matrix"])
        raw = golden[f"chain{ci}_raw"]
        res = orc.run_chain(1e-3, 0.2, 0.1, 1.0, golden[f"chain{ci}_start"],
                            mut, known, raw, score_mode=0)
        tr = res["trace"]
        assert (tr["proposed_score"] == golden[f"chain{ci}_prop_scores"]).all()
        assert (tr["accepted"] == golden[f"chain{ci}_accepted"]).all()
        assert (orc.parent_vector(res["dm"]) ==
                golden[f"chain{ci}_final_parent"]).all()
        assert np.float32(res["score"]) == golden[f"chain{ci}_final_score"]
        assert np.float32(res["beta"]) == golden[f"chain{ci}_final_beta"]
        assert np.float32(res["best_score"]) == \
            golden[f"chain{ci}_best_score"]
        assert _tree_hash(res["best_dm"]) == golden[f"chain{ci}_best_hash"]


def test_golden_chain_class_total_scores(orc, golden):
    """The class-total score (the CUDA path's form) keeps the reference's
    trajectory: decisions differ only inside a 1e-4 relative band around
    the acceptance level, and scores stay within 1e-5 relative."""
    for ci, (G, Cn, steps, _) in enumerate(golden["chain_cases"]):
        mut, known = D.matrix_to_bits(golden[f"chain{ci}_matrix"])
        res = orc.run_chain(1e-3, 0.2, 0.1, 1.0, golden[f"chain{ci}_start"],
                            mut, known, golden[f"chain{ci}_raw"],
                            score_mode=1,
                            forced=golden[f"chain{ci}_accepted"],
                            ambiguity=1e-4)
        tr = res["trace"]
        ref_prop = golden[f"chain{ci}_prop_scores"]
        np.testing.assert_allclose(tr["proposed_score"], ref_prop, rtol=1e-5)
        assert (tr["accepted"] == golden[f"chain{ci}_accepted"]).all()
        assert (orc.parent_vector(res["dm"]) ==
                golden[f"chain{ci}_final_parent"]).all()


def test_golden_chains_run_free_make_every_reference_decision(orc, golden):
    """Run free on the reference's recorded moves (no decision forced), the
    class-total chains make the reference's own decision -- taken on its
    cell-order score -- at every one of the 5,100 steps of the four golden
    chains, and end on its trees."""
    total = 0
    for ci, (G, Cn, steps, _) in enumerate(golden["chain_cases"]):
        mut, known = D.matrix_to_bits(golden[f"chain{ci}_matrix"])
        res = orc.run_chain(1e-3, 0.2, 0.1, 1.0, golden[f"chain{ci}_start"],
                            mut, known, golden[f"chain{ci}_raw"],
                            score_mode=1)
        acc = res["trace"]["accepted"]
        assert (acc == golden[f"chain{ci}_accepted"]).all()
        assert (orc.parent_vector(res["dm"]) ==
                golden[f"chain{ci}_final_parent"]).all()
        total += len(acc)
    assert total == 5100


# ------------------------------------------------------------- fuzzing --

def _parent_vector_move(pv, mp, am):
    """test/MutationTree.cpp:697-735: the move on the parent vector."""
    pv = list(int(x) for x in pv)
    v, w = int(mp["v"]), int(mp["w"])
    t = int(mp["move_type"])
    if t == 2:
        for i in range(len(pv)):
            if i != v and i != w:
                if pv[i] == v:
                    pv[i] = w
                elif pv[i] == w:
                    pv[i] = v
        if pv[v] == w:
            pv[v] = pv[w]
            pv[w] = v
        elif pv[w] == v:
            pv[w] = pv[v]
            pv[v] = w
        else:
            pv[v], pv[w] = pv[w], pv[v]
    elif t == 1:
        pv[v] = int(mp["nondescendant_of_v"])
    elif t == 3:
        pv[v] = int(mp["parent_of_w"])
        if (int(am[w, v // 64]) >> (v % 64)) & 1:
            pv[w] = int(mp["descendant_of_v"])
        else:
            pv[w] = int(mp["parent_of_v"])
    return pv


@pytest.mark.parametrize("seed,n_genes", [(1, 16), (2, 16), (3, 40),
                                          (4, 100), (5, 200)])
def test_fuzz_moves_match_parent_vector(orc, seed, n_genes):
    rng = np.random.default_rng(seed)
    mp_probs = orc.move_probs(0.0, 0.33, 0.33, 0.33)
    pv = D.random_parent_vector(rng, n_genes)
    am, dm = orc.parent_to_matrix(pv)
    moves = orc.sample_moves(mp_probs, n_genes + 1, seed, 0, 400)
    for raw in moves:
        mp = orc.realize(am, dm, 0.42, raw)
        if int(mp["move_type"]) == 0:
            continue
        exp = _parent_vector_move(pv, mp, am)
        nam, ndm, _ = orc.apply_move(am, dm, 0.42, mp)
        eam, edm = orc.parent_to_matrix(exp)
        assert (nam == eam).all() and (ndm == edm).all()
        # advance the tree (the reference's fuzz test keeps it fixed)
        pv, am, dm = exp, nam, ndm


# ------------------------------------------------------- Philox sampler --

def test_philox_known_answer(orc):
    # Random123's published known-answer vectors for philox4x32-10
    assert orc.philox([0, 0, 0, 0], [0, 0]).tolist() == \
        [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert orc.philox([0xffffffff] * 4, [0xffffffff] * 2).tolist() == \
        [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert orc.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                      [0xa4093822, 0x299f31d0]).tolist() == \
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_sampler_ranges(orc):
    mp = orc.move_probs(0.1, 0.55, 0.4, 0.05)
    mv = orc.sample_moves(mp, 20, 7, 3, 4000)
    assert set(np.unique(mv["move_type"])) == {0, 1, 2, 3}
    assert (mv["raw_v"] <= 18).all() and (mv["raw_w"] <= 18).all()
    assert (mv["raw_v"] != mv["raw_w"]).all()
    for f in ("raw_descendant_of_v", "raw_nondescendant_of_v",
              "acceptance_level"):
        assert (mv[f] >= 0).all() and (mv[f] < 1).all()
    frac = np.bincount(mv["move_type"], minlength=4) / len(mv)
    np.testing.assert_allclose(frac, [0.1 / 1.1, 0.55 / 1.1, 0.4 / 1.1,
                                      0.05 / 1.1], atol=0.03)


# --------------------------------------------------- FP64 sum-score grad --

def test_sumscore_gradient_fd(orc):
    m, _, _ = D.generate_dataset(11, 30, 40, 1e-3, 0.2, 0.1, 0.0)
    mut, known = D.matrix_to_bits(m)
    rng = np.random.default_rng(0)
    for _ in range(3):
        _, dm = orc.parent_to_matrix(D.random_parent_vector(rng, 30))
        a, b, h = 1e-2, 0.3, 1e-6
        f, da, db, post = orc.sumscore_grad_f64(a, b, dm, mut, known, True)
        fa = (orc.sumscore_grad_f64(a + h, b, dm, mut, known)[0] -
              orc.sumscore_grad_f64(a - h, b, dm, mut, known)[0]) / (2 * h)
        fb = (orc.sumscore_grad_f64(a, b + h, dm, mut, known)[0] -
              orc.sumscore_grad_f64(a, b - h, dm, mut, known)[0]) / (2 * h)
        assert da == pytest.approx(fa, rel=1e-6)
        assert db == pytest.approx(fb, rel=1e-6)
        np.testing.assert_allclose(post.sum(axis=1), 1.0, rtol=1e-12)


def test_golden_vectors_regenerate_bit_for_bit(orc, tmp_path):
    """tests/golden/ref_vectors.npz is exactly what its generator makes from
    the reference's own classes (oracle/_ref), array for array.  Needs the
    reference build, which exists only where the reference sources do."""
    import importlib.util
    import os
    if orc.ref_lib() is None:
        pytest.skip("oracle/_ref is not built here")
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(here, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    mg.OUT = str(tmp_path / "ref_vectors.npz")
    mg.main()
    old = np.load(os.path.join(here, "ref_vectors.npz"))
    new = np.load(mg.OUT)
    assert sorted(old.files) == sorted(new.files)
    for k in old.files:
        assert old[k].dtype == new[k].dtype and old[k].shape == new[k].shape, k
        assert old[k].tobytes() == new[k].tobytes(), k


def test_quality_fixture_scores(orc):
    """The committed reference results of the quality comparison are the
    reference's cell-order scores of their best trees."""
    import json
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                        "quality_ref.json")
    with open(path) as f:
        fx = json.load(f)
    w = fx["workload"]
    assert len(fx["results"]) == w["datasets"] == 64
    for row in fx["results"][:8]:
        m, _, _ = D.generate_dataset(row["dataset_seed"], w["n_genes"],
                                     w["n_cells"], w["alpha"], w["beta"],
                                     w["missing"], w["homozygous"])
        mut, known = D.matrix_to_bits(m)
        _, dm = orc.parent_to_matrix(np.array(row["best_parent"]))
        r, _, _, _ = orc.logscore_tree(w["alpha"], w["beta"], w["beta_sd"],
                                       dm, mut, known, w["beta"])
        assert np.float32(r) == np.float32(row["best_score"])


def _index_reached_count(am, mp, raw) -> bool:
    """Whether a realised move's k-th (non)descendant index reached its
    count: floor(u * count) in float (src/MutationTree.hpp:341-344), the
    case in which the reference's selection returns node 0."""
    n = am.shape[0]
    v = int(mp["v"])
    nd = sum(bin(int(am[v, k])).count("1") for k in range(am.shape[1]))
    nn = n - nd
    i_d = int(np.floor(np.float32(raw["raw_descendant_of_v"]) * np.float32(nd)))
    i_n = int(np.floor(np.float32(raw["raw_nondescendant_of_v"]) *
                       np.float32(nn)))
    return i_d >= nd or i_n >= nn


def test_parent_vector_moves_except_node0_fallbacks(orc):
    """The GPU's inherited counts follow each move on the parent vector, as
    the reference's test restates the moves (test/MutationTree.cpp:697-735).
    That form agrees with the reference's row update for every move except
    one whose k-th (non)descendant index reached its count: the reference
    then takes node 0, which need not be a (non)descendant of v.  The
    kernels flag exactly those moves and check their parent vectors against
    the rows.  Raw uniforms of 1.0 (edge values the golden move streams
    hold too) make the case certain."""
    rng = np.random.default_rng(97)
    top = np.float32(1.0)
    flagged = mismatched = 0
    for trial in range(12):
        G = int(rng.integers(4, 70))
        pv = D.random_parent_vector(rng, G)
        am, dm = orc.parent_to_matrix(pv)
        mp_probs = orc.move_probs(0.0, 0.4, 0.2, 0.4)
        raws = orc.sample_moves(mp_probs, G + 1, 500 + trial, 0, 300)
        edge = rng.random(len(raws)) < 0.3
        raws["raw_descendant_of_v"][edge] = top
        raws["raw_nondescendant_of_v"][edge] = top
        for raw in raws:
            mp = orc.realize(am, dm, 0.3, raw)
            if int(mp["move_type"]) == 0:
                continue
            nam, ndm, _ = orc.apply_move(am, dm, 0.3, mp)
            exp = _parent_vector_move(orc.parent_vector(dm), mp, am)
            agree = list(exp) == list(orc.parent_vector(ndm)) and (
                ndm == orc.parent_to_matrix(exp)[1]).all()
            if _index_reached_count(am, mp, raw):
                flagged += 1
                mismatched += not agree
            else:
                assert agree, (trial, mp)
                am, dm = nam, ndm  # advance along proper moves: trees only
    assert flagged > 0 and mismatched > 0


def test_golden_chains_parent_vector_mismatches_are_node0_fallbacks(orc,
                                                                    golden):
    """Along the reference's own recorded chains (its move streams and its
    accept decisions), the parent-vector form of a move disagrees with the
    row update only at moves whose k-th (non)descendant index reached its
    count -- the moves the kernels flag and check.  The first such
    disagreements of the four chains are steps 73, 153, none and 585.  A
    chain's cells held in registers (the launches whose warps hold all its
    cells) are the only ones scored from parent vectors, which is why a
    wrong vector shows at those steps only where the launch keeps the cells
    resident."""
    first = []
    for ci in range(len(golden["chain_cases"])):
        raws = golden[f"chain{ci}_raw"]
        acc = golden[f"chain{ci}_accepted"]
        am, dm = orc.parent_to_matrix(golden[f"chain{ci}_start"])
        beta = 0.2
        bad = []
        for i, raw in enumerate(raws):
            mp = orc.realize(am, dm, beta, raw)
            if int(mp["move_type"]) == 0:
                if acc[i]:
                    beta = float(mp["new_beta"])
                continue
            nam, ndm, _ = orc.apply_move(am, dm, beta, mp)
            pv = orc.parent_vector(dm)
            is_tree = (orc.parent_to_matrix(pv)[1] == dm).all()
            exp = _parent_vector_move(pv, mp, am)
            agree = list(exp) == list(orc.parent_vector(ndm)) and (
                ndm == orc.parent_to_matrix(exp)[1]).all()
            if is_tree and not agree:
                assert _index_reached_count(am, mp, raw), (ci, i)
                bad.append(i)
            if acc[i]:
                am, dm = nam, ndm
        first.append(bad[0] if bad else None)
    assert first == [73, 153, None, 585]


def test_application_kat_on_the_oracle(orc, kat):
    """The reference's end-to-end test (test/Application.cpp:38-143) on the
    oracle's restated step loop, in the reference's cell-order score: over
    the test's chain count and chain length, the best tree found scores
    like the true tree."""
    k = kat["application"]
    mut = np.array([[int(s, 2)] for s in k["is_mutated"]], dtype=np.uint64)
    known = np.array([[int(s, 2)] for s in k["is_known"]], dtype=np.uint64)
    rng = np.random.default_rng(38)
    parents = np.stack([D.random_parent_vector(rng, k["n_genes"])
                        for _ in range(k["n_chains"])])
    mp = orc.move_probs(beta_sd=k["beta_sd"])
    best, _ = orc.run_chains_mt(k["alpha"], k["beta"], k["beta_sd"], 1.0, mp,
                                143, parents, mut, known, k["chain_length"],
                                k["n_chains"], score_mode=0)
    _, dm = orc.parent_to_matrix(np.array(k["true_parent_vector"]))
    r, _, _, _ = orc.logscore_tree(k["alpha"], k["beta"], k["beta_sd"], dm,
                                   mut, known, k["beta"])
    assert best == pytest.approx(float(r), rel=1e-5)


def test_cpu_proxy_restatement_matches_reference_class(orc):
    """orc_cpu_proxy_scores -- the restated CPUTreeScorer that the CPU
    baseline times -- gives the reference class's scores bit for bit
    (tests/golden/proxy_vectors.npz, made from
    cpu_scoring_benchmark/CPUTreeScorer.hpp compiled unmodified)."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)),
                             "golden", "proxy_vectors.npz"))
    for i in range(3):
        a, b = (float(x) for x in g[f"rates{i}"])
        s = orc.cpu_proxy_scores(a, b, g["mutq"], g["knownq"], g["dmq"])
        assert s.view(np.uint32).tolist() == \
            g[f"scores{i}"].view(np.uint32).tolist()


def test_cpu_proxy_vectors_regenerate(orc, tmp_path):
    """tests/golden/proxy_vectors.npz is what its generator makes from the
    reference's own class (needs oracle/_ref, built only where the
    reference sources are)."""
    import importlib.util
    import os
    if orc.ref_lib() is None:
        pytest.skip("oracle/_ref is not built here")
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    spec = importlib.util.spec_from_file_location(
        "make_proxy_golden", os.path.join(here, "make_proxy_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    mg.OUT = str(tmp_path / "proxy_vectors.npz")
    mg.main()
    old = np.load(os.path.join(here, "proxy_vectors.npz"))
    new = np.load(mg.OUT)
    assert sorted(old.files) == sorted(new.files)
    for k in old.files:
        assert old[k].tobytes() == new[k].tobytes(), k
