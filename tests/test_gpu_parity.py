"""CUDA path vs the CPU oracle, through the C ABI.

Bit-exact: class counts, attachments, realised moves, proposed ancestor
rows, chain trajectories under recorded moves, and the FP32 class-total
score (host-computed log table; no contraction on either side).  Scores
are also held to 1e-5 relative of the FP64 restatement, and the adjoint
to 1e-4 relative of the FP64 gradient.
"""
import time

import numpy as np
import pytest

from bbscite_gb300 import data as D

pytestmark = pytest.mark.gpu

SCORE_RTOL = 1e-5   # FP32 score vs FP64 oracle
GRAD_RTOL = 1e-4    # FP32 adjoint vs FP64 gradient


def ctx_for(native, matrix, alpha, beta, sd=0.1, **kw):
    mut, known = D.matrix_to_bits(matrix)
    G, Cn = matrix.shape
    p = native.default_params(alpha_mean=alpha, beta_mean=beta, beta_sd=sd,
                              **kw)
    return native.Context(mut, known, Cn, G, p), mut, known


def tree_stack(orc, parents):
    return np.stack([orc.parent_to_matrix(pv)[1] for pv in parents])


# ------------------------------------------------------------- scoring --

def test_kat_tree_scorer(native, kat):
    k = kat["tree_scorer"]
    mut = np.array([[int(s, 2)] for s in k["is_mutated"]], dtype=np.uint64)
    known = np.array([[int(s, 2)] for s in k["is_known"]], dtype=np.uint64)
    p = native.default_params(alpha_mean=k["alpha"], beta_mean=k["beta"],
                              beta_sd=k["prior_sd"])
    with native.Context(mut, known, 6, 4, p) as c:
        _, dm = native.parent_to_matrix(k["parent_vector"])
        s, counts, att = c.score_trees(dm[None], k["beta"], attach=True)
    t = k["expected_terms"]
    assert counts[0].tolist() == [t["log(1-alpha)"], t["log(beta)"],
                                  t["log(alpha)"], t["log(1-beta)"]]
    # attachments of the KAT's comments: cells at nodes 4, 1, 1, 4, 0, 3
    assert att[0].tolist()[1] == 1 and att[0].tolist()[5] == 3


def test_score_trees_golden(native, orc, golden):
    for ci, (G, Cn) in enumerate(golden["score_cases"]):
        m = golden[f"score{ci}_matrix"]
        c, mut, known = ctx_for(native, m, 1e-3, 0.2)
        with c:
            dms = tree_stack(orc, golden[f"score{ci}_parents"])
            for b, beta in enumerate(golden[f"score{ci}_betas"]):
                s, counts, att = c.score_trees(dms, float(beta), attach=True)
                for t in range(len(dms)):
                    r, st, oc, oatt = orc.logscore_tree(
                        1e-3, 0.2, 0.1, dms[t], mut, known, float(beta))
                    assert np.float32(s[t]) == np.float32(st), (G, Cn, t, b)
                    assert (counts[t] == oc).all()
                    assert (att[t] == oatt).all()
                    f64 = orc.logscore_tree_f64(1e-3, float(beta), dms[t],
                                                mut, known, 0.2, 0.1, True)
                    assert abs(s[t] - f64) <= SCORE_RTOL * abs(f64)
                    ref = golden[f"score{ci}_scores"][t, b]
                    assert abs(s[t] - ref) <= SCORE_RTOL * abs(ref)


@pytest.mark.parametrize("G,Cn", [(2, 1), (31, 33), (32, 100), (63, 64),
                                  (64, 129), (95, 96), (127, 250),
                                  (128, 31), (200, 300), (255, 512)])
def test_score_random_shapes(native, orc, G, Cn):
    rng = np.random.default_rng(G * 1000 + Cn)
    m, _, _ = D.generate_dataset(G + Cn, G, Cn, 5e-3, 0.25, 0.1, 0.02)
    c, mut, known = ctx_for(native, m, 5e-3, 0.25)
    with c:
        parents = [D.random_parent_vector(rng, G) for _ in range(8)]
        dms = tree_stack(orc, parents)
        betas = rng.uniform(0.05, 0.6, size=8).astype(np.float32)
        s, counts, att = c.score_trees(dms, betas, attach=True)
        for t in range(8):
            _, st, oc, oatt = orc.logscore_tree(5e-3, 0.25, 0.1, dms[t], mut,
                                                known, float(betas[t]))
            assert np.float32(s[t]) == np.float32(st)
            assert (counts[t] == oc).all() and (att[t] == oatt).all()


def test_scratch_reuse_across_calls(native, orc):
    """The host-buffer entry points keep their device scratch in the
    context and grow it on demand: calls of mixed sizes and kinds on one
    context give bit-for-bit the results of the same calls on a fresh
    context, and scoring trees one at a time equals scoring them at once."""
    G, Cn = 95, 96
    m, _, _ = D.generate_dataset(5, G, Cn, 1e-3, 0.2, 0.1, 0.02)
    rng = np.random.default_rng(44)
    mp = orc.move_probs(0.1, 0.3, 0.3, 0.3)
    calls = []
    for n_trees in (1, 300, 7, 1000, 2):
        dms = tree_stack(orc, [D.random_parent_vector(rng, G)
                               for _ in range(n_trees)])
        betas = rng.uniform(0.05, 0.6, size=n_trees).astype(np.float32)
        raws = np.concatenate([orc.sample_moves(mp, G + 1, G, t, 1)
                               for t in range(n_trees)])
        calls.append((dms, betas, np.ascontiguousarray(raws).view(
            native.RAW_MOVE)))

    def run(c, dms, betas, raw):
        s, cnt, att = c.score_trees(dms, betas, attach=True)
        pout, out, bout = c.apply_moves(dms, betas, raw=raw)
        logl, da, db, post = c.sumscore_grad(dms, 1e-3, betas,
                                             posterior=len(dms) < 10)
        return [s, cnt, att, pout.tobytes(), out, bout, logl, da, db, post]

    c, _, _ = ctx_for(native, m, 1e-3, 0.2)
    with c:
        shared = [run(c, *call) for call in calls]
        dms, betas, _ = calls[3]
        one_by_one = [c.score_trees(dms[t:t + 1], betas[t:t + 1])[0][0]
                      for t in range(50)]
        np.testing.assert_array_equal(np.array(one_by_one, np.float32),
                                      shared[3][0][:50])
    for call, got in zip(calls, shared):
        c, _, _ = ctx_for(native, m, 1e-3, 0.2)
        with c:
            want = run(c, *call)
        for g, w in zip(got, want):
            if w is None:
                assert g is None
            elif isinstance(w, bytes):
                assert g == w
            else:
                np.testing.assert_array_equal(g, w)


# --------------------------------------------------------------- moves --

def test_apply_params_kat(native, kat):
    beta = kat["moves"]["beta"]
    for case in kat["moves"]["cases"]:
        n = len(case["start"])
        mut = np.zeros((1, 1), dtype=np.uint64)
        with native.Context(mut, mut, 1, n - 1) as c:
            _, dm = native.parent_to_matrix(case["start"])
            p = np.zeros(1, dtype=native.MOVE_PARAMS)
            for key, val in case["params"].items():
                p[key] = val
            _, out, _ = c.apply_moves(dm[None], beta, params=p)
            assert native.matrix_to_parent(out[0]).tolist() == \
                case["expected"], case["name"]
            _, edm = native.parent_to_matrix(case["expected"])
            assert (out[0] == edm).all()


def test_apply_moves_golden(native, orc, golden):
    for ci, (G, _) in enumerate(golden["move_cases"]):
        G = int(G)
        raws = golden[f"move{ci}_raw"]
        am, dm = orc.parent_to_matrix(golden[f"move{ci}_start"])
        beta = np.float32(0.3)
        trees, betas = [dm], [beta]
        for i in range(len(raws) - 1):
            mp = orc.realize(am, dm, float(beta), raws[i])
            am, dm, beta = orc.apply_move(am, dm, float(beta), mp)
            trees.append(dm)
            betas.append(np.float32(beta))
        mut = np.zeros((1, orc.words(G + 1)), dtype=np.uint64)
        with native.Context(mut, mut, 1, G) as c:
            raw = np.ascontiguousarray(raws).view(native.RAW_MOVE)
            pout, out, bout = c.apply_moves(np.stack(trees),
                                            np.array(betas, np.float32),
                                            raw=raw)
        want = golden[f"move{ci}_params"]
        assert pout.tobytes() == want.tobytes()
        for i in range(len(raws)):
            assert (native.matrix_to_parent(out[i]) ==
                    golden[f"move{ci}_parents"][i]).all(), (ci, i)
        np.testing.assert_array_equal(bout, golden[f"move{ci}_betas"])


@pytest.mark.parametrize("G", [2, 3, 30, 31, 32, 63, 64, 100, 127, 128, 129,
                               191, 255])
def test_apply_moves_fuzz(native, orc, G):
    rng = np.random.default_rng(G)
    n = G + 1
    k = 256
    parents = [D.random_parent_vector(rng, G) for _ in range(k)]
    mp = orc.move_probs(0.1, 0.3, 0.3, 0.3)
    raws = np.concatenate([orc.sample_moves(mp, n, G, t, 1) for t in
                           range(k)])
    edge = rng.random(k) < 0.1
    raws["raw_descendant_of_v"][edge] = 1.0
    betas = rng.uniform(0.05, 0.9, size=k).astype(np.float32)
    mut = np.zeros((1, orc.words(n)), dtype=np.uint64)
    with native.Context(mut, mut, 1, G) as c:
        dms = tree_stack(orc, parents)
        raw = np.ascontiguousarray(raws).view(native.RAW_MOVE)
        pout, out, bout = c.apply_moves(dms, betas, raw=raw)
    for t in range(k):
        am, dm = orc.parent_to_matrix(parents[t])
        p = orc.realize(am, dm, float(betas[t]), raws[t])
        nam, ndm, nb = orc.apply_move(am, dm, float(betas[t]), p)
        assert pout[t].tobytes() == p.tobytes(), t
        assert (out[t] == ndm).all(), t
        assert np.float32(bout[t]) == np.float32(nb)


# -------------------------------------------------------------- chains --

def _replay_check(native, orc, m, alpha, beta, start_parents, raws,
                  exact_scores=True, launch=None):
    c, mut, known = ctx_for(native, m, alpha, beta)
    n_chains, n_steps = raws.shape
    with c:
        c.init_chains(n_chains, np.stack(start_parents))
        if launch is not None:
            c.set_launch(*launch)
        tr = c.run(n_steps, moves=np.ascontiguousarray(raws).view(
            native.RAW_MOVE), trace=True)
        final = c.chains()
        best = c.best()
    best_score = -np.inf
    for ch in range(n_chains):
        res = orc.run_chain(alpha, beta, 0.1, 1.0, start_parents[ch], mut,
                            known, raws[ch], score_mode=1,
                            forced=tr["accepted"][ch], ambiguity=1e-5)
        t = res["trace"]
        assert (t["accepted"] == tr["accepted"][ch]).all()
        assert int(t["ambiguous"].sum()) <= 1
        assert (t["counts"] == tr["proposed_counts"][ch]).all()
        if exact_scores:
            assert (t["proposed_score"] == tr["proposed_score"][ch]).all()
        else:
            np.testing.assert_allclose(t["proposed_score"],
                                       tr["proposed_score"][ch], rtol=1e-6)
        assert (res["dm"] == final["dm"][ch]).all()
        if res["best_score"] > best_score:
            best_score = res["best_score"]
    assert best["score"] == pytest.approx(best_score, rel=1e-6)
    return tr


def test_mcmc_replay_golden(native, orc, golden):
    for ci, (G, Cn, steps, p_beta) in enumerate(golden["chain_cases"]):
        raw = golden[f"chain{ci}_raw"][None]
        tr = _replay_check(native, orc, golden[f"chain{ci}_matrix"], 1e-3,
                           0.2, [golden[f"chain{ci}_start"]], raw,
                           exact_scores=(p_beta == 0))
        # the reference's own recorded decisions (its cell-order score):
        # the class-total chains make every one of them (measured: all
        # 5,100 steps of the four chains); at most the replay's one
        # decision inside the rounding band may differ
        ref_acc = golden[f"chain{ci}_accepted"]
        assert int((tr["accepted"][0] != ref_acc).sum()) <= 1


@pytest.mark.parametrize("G,Cn,chains", [(16, 20, 7), (63, 64, 5),
                                         (95, 96, 4), (100, 200, 3),
                                         (255, 300, 2)])
def test_mcmc_replay_random(native, orc, G, Cn, chains):
    rng = np.random.default_rng(7 * G + Cn)
    m, _, _ = D.generate_dataset(G * Cn, G, Cn, 1e-3, 0.2, 0.1, 0.02)
    mp = orc.move_probs(0.0, 0.55, 0.4, 0.05)
    steps = 300
    raws = np.stack([orc.sample_moves(mp, G + 1, 99, ch, steps)
                     for ch in range(chains)])
    starts = [D.random_parent_vector(rng, G) for _ in range(chains)]
    _replay_check(native, orc, m, 1e-3, 0.2, starts, raws)


@pytest.mark.parametrize("G,Cn,launch", [(130, 100, (2, 1, 2)),
                                         (170, 120, (1, 2, 1)),
                                         (200, 150, (1, 1, 3)),
                                         (255, 300, (2, 1, 2)),
                                         (255, 300, (2, 3, 1))])
def test_wide_rows_replay_with_stars_and_node0_fallbacks(native, orc, G, Cn,
                                                         launch):
    """Rows of five to eight words take their counts through a ring of the
    last 64 nodes in the canonical order.  Chains started from star trees
    (every gene a child of the root: the order does not fit the ring, so
    masked popcounts score them until the moves deepen the tree), and moves
    whose k-th (non)descendant falls back to node 0 (u = 1.0: those
    proposals' parent vectors are checked against their rows), replay bit
    for bit against the oracle: decisions, class counts, scores and final
    rows, with one and with several warps per chain, at rows of five to
    eight words (131 to 256 nodes)."""
    rng = np.random.default_rng(G * 7 + Cn)
    m, _, _ = D.generate_dataset(G + Cn, G, Cn, 1e-3, 0.2, 0.1, 0.02)
    mp = orc.move_probs(0.0, 0.55, 0.4, 0.05)
    steps, chains = 300, 3
    raws = np.stack([orc.sample_moves(mp, G + 1, 41, ch, steps)
                     for ch in range(chains)])
    raws["raw_descendant_of_v"][rng.random(raws.shape) < 0.03] = 1.0
    raws["raw_nondescendant_of_v"][rng.random(raws.shape) < 0.03] = 1.0
    star = np.full(G + 1, G, dtype=np.uint32)
    starts = [star, star.copy(), D.random_parent_vector(rng, G)]
    _replay_check(native, orc, m, 1e-3, 0.2, starts, raws, launch=launch)


@pytest.fixture(scope="module")
def largest():
    """The largest problem the library takes: BBS_MAX_GENES genes and
    BBS_MAX_CELLS cells.  Class totals reach 1.5e7, just below 2^24, where
    FP32 still holds every integer; the fixed-point sums of the sum score
    reach 2^43 of their 2^48 range."""
    G, Cn = 255, 65535
    m, _, _ = D.generate_dataset(7 * G + Cn, G, Cn, 1e-3, 0.2, 0.05, 0.01)
    mut, known = D.matrix_to_bits(m)
    return G, Cn, m, mut, known


def test_largest_problem_scores(native, orc, largest):
    G, Cn, m, mut, known = largest
    rng = np.random.default_rng(65535)
    parents = [D.random_parent_vector(rng, G) for _ in range(3)]
    dms = tree_stack(orc, parents)
    betas = np.array([0.2, 0.05, 0.45], dtype=np.float32)
    c, _, _ = ctx_for(native, m, 1e-3, 0.2)
    with c:
        s, counts, att = c.score_trees(dms, betas, attach=True)
        logl, da, db, _ = c.sumscore_grad(dms, 1e-3, betas)
    for t in range(3):
        _, st, oc, oatt = orc.logscore_tree(1e-3, 0.2, 0.1, dms[t], mut,
                                            known, float(betas[t]))
        assert np.float32(s[t]) == np.float32(st)
        assert (counts[t] == oc).all() and (att[t] == oatt).all()
        # the four classes partition the known entries
        assert int(counts[t].sum()) == int(np.unpackbits(
            known.view(np.uint8)).sum())
        f64 = orc.logscore_tree_f64(1e-3, float(betas[t]), dms[t], mut, known,
                                    0.2, 0.1, True)
        assert abs(s[t] - f64) <= SCORE_RTOL * abs(f64)
        f, ga, gb, _ = orc.sumscore_grad_f64(1e-3, float(betas[t]), dms[t],
                                             mut, known)
        assert abs(logl[t] - f) <= SCORE_RTOL * abs(f)
        assert abs(da[t] - ga) <= GRAD_RTOL * abs(ga)
        assert abs(db[t] - gb) <= GRAD_RTOL * abs(gb)


def test_largest_problem_replays(native, orc, largest):
    G, Cn, m, _, _ = largest
    mp = orc.move_probs(0.0, 0.55, 0.4, 0.05)
    raws = orc.sample_moves(mp, G + 1, 77, 0, 20)[None]
    start = [D.random_parent_vector(np.random.default_rng(5), G)]
    _replay_check(native, orc, m, 1e-3, 0.2, start, raws)


def test_philox_stream_matches_oracle(native, orc):
    G, Cn = 40, 50
    m, _, _ = D.generate_dataset(1, G, Cn, 1e-3, 0.2, 0.1, 0.0)
    seed = 0x1234abcd
    c, mut, known = ctx_for(native, m, 1e-3, 0.2, seed=seed,
                            prob_beta_change=0.1)
    rng = np.random.default_rng(0)
    starts = np.stack([D.random_parent_vector(rng, G) for _ in range(3)])
    with c:
        c.init_chains(3, starts)
        tr = c.run(500, trace=True)
    mp = orc.move_probs(0.1, 0.55, 0.4, 0.05, 0.1, 10.0)
    for ch in range(3):
        want = orc.sample_moves(mp, G + 1, seed, ch, 500)
        got = tr["move"][ch]
        for f in ("move_type", "raw_v", "raw_w", "raw_descendant_of_v",
                  "raw_nondescendant_of_v", "acceptance_level"):
            assert (got[f] == want[f]).all(), f
        np.testing.assert_allclose(got["beta_jump"], want["beta_jump"],
                                   rtol=1e-5, atol=1e-8)


def test_resume_equals_single_run(native, orc):
    G, Cn = 50, 70
    m, _, _ = D.generate_dataset(2, G, Cn, 1e-3, 0.2, 0.1, 0.0)
    outs = []
    for split in ((400,), (150, 250)):
        c, _, _ = ctx_for(native, m, 1e-3, 0.2, seed=77)
        with c:
            c.init_chains(6)
            for s in split:
                c.run(s)
            outs.append((c.chains(), c.best()))
    (a, ba), (b, bb) = outs
    assert (a["dm"] == b["dm"]).all()
    np.testing.assert_array_equal(a["score"], b["score"])
    assert ba["score"] == bb["score"] and (ba["dm"] == bb["dm"]).all()


def test_best_is_consistent(native, orc):
    G, Cn = 63, 64
    m, _, _ = D.generate_dataset(9, G, Cn, 6.04e-5, 0.4309, 0.05, 0.0)
    c, mut, known = ctx_for(native, m, 6.04e-5, 0.4309)
    with c:
        c.init_chains(32)
        c.run(3000)
        best = c.best()
        s, counts, _ = c.score_trees(best["dm"][None], best["beta"])
    assert s[0] == best["score"]
    assert (counts[0] == best["counts"]).all()
    assert (native.dm_to_am(best["dm"]) == best["am"]).all()
    assert (native.matrix_to_parent(best["dm"]) == best["parent"]).all()
    f64 = orc.logscore_tree_f64(6.04e-5, best["beta"], best["dm"], mut, known,
                                0.4309, 0.1, True)
    assert abs(best["score"] - f64) <= SCORE_RTOL * abs(f64)


def test_application_kat(native, kat):
    """test/Application.cpp:38-143: the best tree found scores like the
    true tree (the reference's own stochastic sanity test)."""
    k = kat["application"]
    mut = np.array([[int(s, 2)] for s in k["is_mutated"]], dtype=np.uint64)
    known = np.array([[int(s, 2)] for s in k["is_known"]], dtype=np.uint64)
    p = native.default_params(alpha_mean=k["alpha"], beta_mean=k["beta"],
                              beta_sd=k["beta_sd"])
    with native.Context(mut, known, k["n_cells"], k["n_genes"], p) as c:
        c.init_chains(k["n_chains"])
        c.run(k["chain_length"])
        best = c.best()
        _, dm = native.parent_to_matrix(k["true_parent_vector"])
        s, _, _ = c.score_trees(dm[None], k["beta"])
    assert best["score"] == pytest.approx(float(s[0]), rel=1.2e-5)


def test_cancel_stops_a_run(native):
    m, _, _ = D.generate_dataset(4, 16, 20, 1e-3, 0.2)
    c, _, _ = ctx_for(native, m, 1e-3, 0.2)
    with c:
        c.init_chains(4)
        c.run_async(2_000_000)
        time.sleep(0.2)
        c.cancel()
        with pytest.raises(native.BbsError) as e:
            c.sync()
        assert e.value.code == native.BBS_ERR_TIMEOUT
        c.run(10)  # the context stays usable
        assert c.best()["score"] < 0


def test_run_rejects_bad_moves(native):
    m, _, _ = D.generate_dataset(4, 16, 20, 1e-3, 0.2)
    c, _, _ = ctx_for(native, m, 1e-3, 0.2)
    with c:
        c.init_chains(2)
        bad = np.zeros((2, 3), dtype=native.RAW_MOVE)
        bad["raw_v"][1, 2] = 17  # 17 nodes: 0..16
        with pytest.raises(native.BbsError) as e:
            c.run(3, moves=bad)
        assert e.value.code == native.BBS_ERR_INPUT
        with pytest.raises(native.BbsError):
            native.Context(np.zeros((2, 1), np.uint64),
                           np.zeros((2, 1), np.uint64), 2, 300)


# ------------------------------------------------------------- adjoint --

def test_sumscore_grad_vs_fp64(native, orc):
    G, Cn = 95, 96
    m, _, _ = D.generate_dataset(21, G, Cn, 1e-3, 0.2, 0.1, 0.02)
    c, mut, known = ctx_for(native, m, 1e-3, 0.2)
    rng = np.random.default_rng(3)
    parents = [D.random_parent_vector(rng, G) for _ in range(16)]
    dms = tree_stack(orc, parents)
    for (a, b) in ((1e-3, 0.2), (1e-2, 0.3)):
        with_post = a == 1e-3
        logl, da, db, post = c.sumscore_grad(dms, a, b, posterior=with_post)
        for t in range(len(dms)):
            f, ga, gb, opost = orc.sumscore_grad_f64(a, b, dms[t], mut, known,
                                                     posterior=with_post)
            assert abs(logl[t] - f) <= SCORE_RTOL * abs(f)
            assert abs(da[t] - ga) <= GRAD_RTOL * abs(ga)
            assert abs(db[t] - gb) <= GRAD_RTOL * abs(gb)
            if with_post:
                np.testing.assert_allclose(post[t], opost, atol=2e-5)
                np.testing.assert_allclose(post[t].sum(axis=1), 1.0,
                                           rtol=1e-4)
    c.close()


@pytest.mark.parametrize("G,Cn", [(95, 96), (40, 200), (127, 64), (200, 150)])
def test_launch_shapes_give_identical_chains(native, orc, G, Cn):
    """Every launch shape (cells per lane, warps per chain, chains per
    block) computes the same chains bit for bit."""
    m, _, _ = D.generate_dataset(G + 3 * Cn, G, Cn, 1e-3, 0.2, 0.1, 0.02)
    mut, known = D.matrix_to_bits(m)
    shapes = [(1, 1, 1), (2, 1, 2), (1, 2, 1), (1, 3, 1), (2, 2, 1),
              (1, 4, 1), (2, 1, 4)]
    qmax = 2 if G + 1 > 128 else 4
    outs = []
    for q, wpc, cpb in shapes:
        if q > qmax:
            continue
        p = native.default_params(alpha_mean=1e-3, beta_mean=0.2, seed=31,
                                  prob_beta_change=0.05)
        with native.Context(mut, known, Cn, G, p) as c:
            c.init_chains(9)
            c.set_launch(q, wpc, cpb)
            tr = c.run(150, trace=True)
            outs.append((c.chains(), c.best(), tr))
    ch0, b0, t0 = outs[0]
    for ch, b, t in outs[1:]:
        assert (ch["dm"] == ch0["dm"]).all()
        np.testing.assert_array_equal(ch["score"], ch0["score"])
        assert b["score"] == b0["score"] and (b["dm"] == b0["dm"]).all()
        assert (t["accepted"] == t0["accepted"]).all()
        assert (t["proposed_counts"] == t0["proposed_counts"]).all()


def test_autotune_keeps_chain_state(native):
    m, _, _ = D.generate_dataset(8, 60, 80, 1e-3, 0.2, 0.1, 0.0)
    mut, known = D.matrix_to_bits(m)
    p = native.default_params(alpha_mean=1e-3, beta_mean=0.2, seed=5)
    with native.Context(mut, known, 80, 60, p) as c:
        c.init_chains(16)
        c.run(100)
        before = c.chains()
        ms = c.autotune(32)
        assert ms > 0
        after = c.chains()
        assert (before["dm"] == after["dm"]).all()
        np.testing.assert_array_equal(before["score"], after["score"])
        q, wpc, cpb = c.launch()
        assert 1 <= q <= 4 and 1 <= wpc <= 4 and 1 <= cpb <= 4
        c.run(50)  # continues from the saved state


@pytest.mark.parametrize("G", [2, 3, 31, 32, 63, 64, 95, 127, 128, 200, 255])
def test_device_initial_trees_match_host(native, orc, G):
    """Random initial trees drawn on the device are the host helper's
    trees for the same seed (bbs_random_parent_vectors)."""
    m, _, _ = D.generate_dataset(G, G, 20, 1e-3, 0.2, 0.1, 0.0)
    mut, known = D.matrix_to_bits(m)
    seed = 0x5EED0000 + G
    p = native.default_params(alpha_mean=1e-3, beta_mean=0.2, seed=seed)
    with native.Context(mut, known, 20, G, p) as c:
        c.init_chains(37)
        dm = c.chains()["dm"]
    host = native.random_parents(seed, G, 37)
    for t in range(37):
        _, want = orc.parent_to_matrix(host[t])
        assert (dm[t] == want).all(), t
