"""Sum score, learned error rates and the batched form, through the C ABI.

Chains run on the GPU with a trace; the host replays every step in FP64
with the oracle: the proposed tree (bit-exact realisation + update), the
proposed score (1e-5 relative), the learned-move proposal (drift and
noise from the recorded uniforms) and the Metropolis-Hastings decision
(outside a band that covers FP32 score rounding).  The host follows the
GPU's decisions, and the final trees must match bit for bit.
"""
import math

import numpy as np
import pytest

from bbscite_gb300 import data as D

pytestmark = pytest.mark.gpu

SCORE_RTOL = 1e-5


def f32(x):
    return np.float32(x)


def prior_params(beta_mean, beta_sd):
    a = ((1 - beta_mean) * beta_mean ** 2 / beta_sd ** 2) - beta_mean
    return a, a * (1 / beta_mean - 1)


def geometry(alpha, beta, e, gamma, A, B):
    va, vb = alpha * (1 - alpha), beta * (1 - beta)
    dS_da = -e[0] / (1 - alpha) + e[2] / alpha
    dS_db = (e[1] / beta - e[3] / (1 - beta) + (A - 1) / beta -
             (B - 1) / (1 - beta))
    ga = gamma * va * dS_da + (1 - 2 * alpha)
    gb = gamma * vb * dS_db + (1 - 2 * beta)
    pa = 1 / (1 + gamma * (e[0] + e[2]) * va)
    pb = 1 / (1 + gamma * (e[1] + e[3] + max(A + B - 2, 0.0)) * vb)
    return ga, gb, pa, pb


def log_q(ta, tb, fa, fb, g, eps, drift):
    h = 0.5 * eps * eps if drift else 0.0
    ra = ta - fa - h * g[2] * g[0]
    rb = tb - fb - h * g[3] * g[1]
    return (-(ra * ra) / (2 * eps * eps * g[2]) -
            (rb * rb) / (2 * eps * eps * g[3]) -
            0.5 * (math.log(g[2]) + math.log(g[3])))


def logit(p):
    return math.log(p) - math.log1p(-p)


def replay(orc, native, m, p, start, trace, final_dm):
    """FP64 host replay of one traced chain; returns the number of
    decisions inside the rounding band."""
    mut, known = D.matrix_to_bits(m)
    sum_score = p.score_mode == native.SCORE_SUM
    gamma, eps = float(p.gamma), float(p.error_step)
    A, B = prior_params(float(p.beta_mean), float(p.beta_sd))
    am, dm = orc.parent_to_matrix(start)
    alpha, beta = f32(p.alpha_mean), f32(p.beta_mean)

    def evaluate(dmx, a, b):
        s, e = orc.score_counts_f64(float(a), float(b), dmx, mut, known,
                                    sum_score)
        return s + orc.logprior_beta_f64(float(p.beta_mean),
                                         float(p.beta_sd), float(b)), e

    S, e = evaluate(dm, alpha, beta)
    geo = geometry(float(alpha), float(beta), e, gamma, A, B)
    ambiguous = 0
    for t in trace:
        raw = t["move"]
        corr = 1.0
        nam, ndm, pa, pb = am, dm, alpha, beta
        if raw["move_type"] != 0:
            mp = orc.realize(am, dm, float(beta), _raw(orc, raw))
            nam, ndm, _ = orc.apply_move(am, dm, float(beta), mp)
            v, w = int(mp["v"]), int(mp["w"])
            if raw["move_type"] == 3 and (int(am[w, v // 64]) >> (v % 64)) & 1:
                corr = float(f32(orc.n_descendants(am, v)) /
                             f32(orc.n_descendants(am, w)))
        elif p.error_move == native.ERROR_BETA_WALK:
            nb = f32(beta + f32(raw["beta_jump"]))
            if nb < 0:
                nb = f32(abs(nb))
            if nb > 1:
                nb = f32(nb - f32(f32(2.0) * f32(nb - f32(1.0))))
            pb = nb
        else:
            pa, pb = f32(t["proposed_alpha"]), f32(t["proposed_beta"])
            # the proposal follows drift + preconditioned noise
            u1 = max(1.0 - float(raw["raw_descendant_of_v"]), 1e-30)
            r = math.sqrt(-2 * math.log(u1))
            z0 = r * math.cos(2 * math.pi * float(raw["raw_nondescendant_of_v"]))
            z1 = r * math.sin(2 * math.pi * float(raw["raw_nondescendant_of_v"]))
            h = 0.5 * eps * eps if p.error_move == native.ERROR_LANGEVIN else 0
            ea = logit(float(alpha)) + h * geo[2] * geo[0] + eps * math.sqrt(geo[2]) * z0
            eb = logit(float(beta)) + h * geo[3] * geo[1] + eps * math.sqrt(geo[3]) * z1
            if 1e-6 < pa < 1 - 1e-6 and 1e-6 < pb < 1 - 1e-6:
                assert abs(logit(float(pa)) - ea) < 2e-3 * max(1, abs(ea))
                assert abs(logit(float(pb)) - eb) < 2e-3 * max(1, abs(eb))
        S1, e1 = evaluate(ndm, pa, pb)
        assert abs(t["proposed_score"] - S1) <= SCORE_RTOL * abs(S1) + 1e-4
        smax, _ = orc.score_counts_f64(float(pa), float(pb), ndm, mut, known,
                                       False)
        smax += orc.logprior_beta_f64(float(p.beta_mean), float(p.beta_sd),
                                      float(pb))
        assert abs(t["proposed_max_score"] - smax) <= SCORE_RTOL * abs(smax) + 1e-4
        geo1 = geometry(float(pa), float(pb), e1, gamma, A, B)
        if raw["move_type"] == 0 and p.error_move != native.ERROR_BETA_WALK:
            fa, fb = logit(float(alpha)), logit(float(beta))
            ta, tb = logit(float(pa)), logit(float(pb))
            drift = p.error_move == native.ERROR_LANGEVIN
            logr = (gamma * (S1 - S) +
                    math.log(pa * (1 - pa)) + math.log(pb * (1 - pb)) -
                    math.log(alpha * (1 - alpha)) - math.log(beta * (1 - beta)) +
                    log_q(fa, fb, ta, tb, geo1, eps, drift) -
                    log_q(ta, tb, fa, fb, geo, eps, drift))
        else:
            logr = gamma * (S1 - S) + math.log(corr)
        lu = math.log(max(float(raw["acceptance_level"]), 1e-300))
        host = logr > lu
        if bool(t["accepted"]) != host:
            band = 3e-5 * abs(S) + 2e-3
            assert abs(logr - lu) < band, (logr, lu)
            ambiguous += 1
        if t["accepted"]:
            am, dm, alpha, beta, S, geo = nam, ndm, pa, pb, S1, geo1
    assert (dm == final_dm).all()
    return ambiguous


def _raw(orc, raw):
    out = np.zeros(1, dtype=orc.RAW_MOVE)
    out.view(np.uint8)[:] = np.frombuffer(raw.tobytes(), dtype=np.uint8)
    return out[0]


CASES = [
    # (score mode, error move, prob of an error move)
    ("sum", "beta_walk", 0.1),
    ("sum", "langevin", 0.25),
    ("sum", "random_walk", 0.25),
    ("max", "random_walk", 0.25),
    ("max", "langevin", 0.25),
]


@pytest.mark.parametrize("score,move,p_err", CASES)
def test_traced_chains_replay_in_fp64(native, orc, score, move, p_err):
    G, Cn, chains, steps = 30, 40, 3, 250
    m, _, _ = D.generate_dataset(101, G, Cn, 1e-3, 0.2, 0.1, 0.02)
    mut, known = D.matrix_to_bits(m)
    p = native.default_params(
        alpha_mean=1e-2, beta_mean=0.3, seed=17, prob_beta_change=p_err,
        score_mode=getattr(native, "SCORE_" + score.upper()),
        error_move=getattr(native, "ERROR_" + move.upper()))
    rng = np.random.default_rng(4)
    starts = np.stack([D.random_parent_vector(rng, G) for _ in range(chains)])
    with native.Context(mut, known, Cn, G, p) as c:
        c.init_chains(chains, starts)
        tr = c.run(steps, trace=True)
        final = c.chains()
    n_err = int((tr["move"]["move_type"] == 0).sum())
    assert n_err > 0
    amb = sum(replay(orc, native, m, p, starts[ch], tr[ch], final["dm"][ch])
              for ch in range(chains))
    assert amb <= 2


@pytest.mark.parametrize("score", ["max", "sum"])
def test_init_scores_match_fp64(native, orc, score):
    G, Cn = 95, 96
    m, _, _ = D.generate_dataset(55, G, Cn, 1e-3, 0.2, 0.1, 0.02)
    mut, known = D.matrix_to_bits(m)
    p = native.default_params(alpha_mean=1e-3, beta_mean=0.2,
                              score_mode=getattr(native, "SCORE_" + score.upper()))
    rng = np.random.default_rng(8)
    starts = np.stack([D.random_parent_vector(rng, G) for _ in range(16)])
    with native.Context(mut, known, Cn, G, p) as c:
        c.init_chains(16, starts)
        st = c.chains()
    for k in range(16):
        _, dm = orc.parent_to_matrix(starts[k])
        s, _ = orc.score_counts_f64(1e-3, 0.2, dm, mut, known, score == "sum")
        s += orc.logprior_beta_f64(0.2, 0.1, 0.2)
        assert abs(st["score"][k] - s) <= SCORE_RTOL * abs(s)


@pytest.mark.parametrize("score,move", [("max", "beta_walk"),
                                        ("sum", "langevin")])
def test_batch_equals_single_dataset_runs(native, score, move):
    """A dataset's chains in the batched launch are bit-identical to the
    same chains run alone (same Philox keys, same kernel code).  The two
    datasets of 200 and 220 genes share a launch group (rows of seven
    words), whose warps build their gene tables from either dataset's
    cells."""
    rng = np.random.default_rng(9)
    specs = [(int(rng.integers(16, 128)), int(rng.integers(16, 200)))
             for _ in range(7)] + [(200, 40), (33, 300), (220, 100)]
    datasets, params = [], []
    for i, (G, Cn) in enumerate(specs):
        m, _, _ = D.generate_dataset(300 + i, G, Cn, 1e-3, 0.2, 0.1, 0.0)
        mut, known = D.matrix_to_bits(m)
        datasets.append((mut, known, Cn, G))
        params.append(native.default_params(
            alpha_mean=float(10 ** rng.uniform(-5, -2)),
            beta_mean=float(rng.uniform(0.05, 0.45)), seed=1000 + i,
            prob_beta_change=0.1,
            score_mode=getattr(native, "SCORE_" + score.upper()),
            error_move=getattr(native, "ERROR_" + move.upper())))
    cpd, steps = 5, 120
    with native.Batch(datasets, params) as b:
        b.init_chains(cpd)
        b.run(steps)
        b.run(steps)  # graph replay
        bests = [b.best(d) for d in range(len(datasets))]
    for d, (mut, known, Cn, G) in enumerate(datasets):
        with native.Context(mut, known, Cn, G, params[d]) as c:
            c.init_chains(cpd)
            c.run(steps)
            c.run(steps)
            want = c.best()
        assert bests[d]["score"] == want["score"]
        assert (bests[d]["dm"] == want["dm"]).all()


@pytest.mark.parametrize("score", ["max", "sum"])
def test_batch_autotune_and_shapes_agree(native, score):
    """Every launch shape of the batched form -- cells per lane, warps per
    block, merged row widths, one-warp chains or chains of 2 and 4 warps --
    and the tuned one give the same chains, and every chain of every launch
    group runs all its steps."""
    # every row width of up to four words with 1-4 groups of 32 cells, and
    # two wider datasets
    specs = [(G, Cn) for G in (20, 50, 80, 110) for Cn in (20, 50, 80, 110)]
    specs += [(200, 40), (160, 300)]
    datasets = []
    for i, (G, Cn) in enumerate(specs):
        m, _, _ = D.generate_dataset(500 + i, G, Cn, 1e-3, 0.2, 0.1, 0.0)
        mut, known = D.matrix_to_bits(m)
        datasets.append((mut, known, Cn, G))
    nd = len(datasets)
    if score == "max":
        p = native.default_params(alpha_mean=1e-3, beta_mean=0.2, seed=3)
    else:
        p = _headline_params(native, seed=3)
    results = []
    # (cells per lane, warps per block, merged widths, warps per chain)
    for shape in ((1, 1, 0, 1), (2, 4, 0, 1), (4, 2, 1, 1), (3, 8, 0, 1),
                  (4, 7, 1, 1), (2, 0, 0, 2), (1, 0, 1, 4), (3, 0, 0, 4),
                  None):
        with native.Batch(datasets, p) as b:
            b.init_chains(4)
            if shape is None:
                assert b.autotune(40) > 0
            else:
                b.set_launch(*shape[:3])
                b.set_chain_warps(shape[3])
                assert b.chain_warps() == shape[3]
            b.run(150)
            img = b.save_chains()
            # every chain ran: its state (128 bytes, at the image's end)
            # counts 150 steps
            states = np.frombuffer(img[-128 * 4 * nd:], dtype=np.uint8)
            steps = states.reshape(4 * nd, 128)[:, 80:88].copy().view(
                np.uint64).ravel()
            assert (steps == 150).all(), (shape, steps)
            results.append(([b.best(d)["score"] for d in range(nd)],
                            img[-128 * 4 * nd:]))
    for r in results[1:]:
        assert r[0] == results[0][0]
        assert r[1] == results[0][1]  # the last chain states, byte for byte


def test_langevin_learns_alpha(native):
    """Data made with alpha=1e-3, beta=0.2; chains start at alpha=1e-2,
    beta=0.3 and learn both with the Langevin error move."""
    G, Cn = 40, 120
    m, _, _ = D.generate_dataset(77, G, Cn, 1e-3, 0.2, 0.05, 0.0)
    mut, known = D.matrix_to_bits(m)
    p = native.default_params(alpha_mean=1e-2, beta_mean=0.3, seed=5,
                              prob_beta_change=0.3,
                              score_mode=native.SCORE_SUM,
                              error_move=native.ERROR_LANGEVIN)
    with native.Context(mut, known, Cn, G, p) as c:
        c.init_chains(32)
        c.run(4000)
        st = c.chains()
    assert np.median(st["alpha"]) < 4e-3
    assert abs(np.median(st["beta"]) - 0.2) < 0.06
    acc = st["err_stats"][:, 1].sum() / max(1, st["err_stats"][:, 0].sum())
    assert 0.2 < acc < 0.98


@pytest.mark.parametrize("G,Cn,alpha,beta,score", [
    (255, 64, 1e-30, 0.5, "sum"),     # a cell's log-likelihood near -1.8e4
    (255, 40, 1e-3, 0.95, "sum"),     # (beta near 1 with sd 0.1 makes the
                                      # reference's Beta prior NaN)
    (2, 1, 1e-2, 0.3, "sum"),         # the smallest problem: moves need two
    (2, 1, 1e-2, 0.3, "max"),         # genes (two non-root nodes)
    (2, 3, 0.2, 0.45, "sum"),
    (255, 65535, 1e-3, 0.2, "sum"),   # the largest problem (fixed-point
                                      # sums near 2^43 of their 2^48 range)
])
def test_extreme_sizes_and_rates_replay_in_fp64(native, orc, G, Cn, alpha,
                                                beta, score):
    """Scores at the edges of the fixed-point range and of the sizes,
    replayed step by step in FP64."""
    m, _, _ = D.generate_dataset(7 * G + Cn, G, Cn, 1e-3, 0.2, 0.05, 0.0)
    p = native.default_params(
        alpha_mean=alpha, beta_mean=beta, seed=23,
        score_mode=getattr(native, "SCORE_" + score.upper()))
    mut, known = D.matrix_to_bits(m)
    rng = np.random.default_rng(12)
    # an FP64 evaluation of the largest problem takes about 0.4 s
    chains, steps = (1, 10) if G * Cn > 10 ** 6 else (2, 60)
    starts = np.stack([D.random_parent_vector(rng, G) for _ in range(chains)])
    with native.Context(mut, known, Cn, G, p) as c:
        c.init_chains(chains, starts)
        tr = c.run(steps, trace=True)
        final = c.chains()
    amb = sum(replay(orc, native, m, p, starts[ch], tr[ch], final["dm"][ch])
              for ch in range(chains))
    assert amb <= 2


# ---------------------------------------------------------------------
# The headline path: the sum score with counts inherited from the parent
# (rows of up to four words, cells held in registers, one warp per chain),
# replayed step by step in FP64, and the batched launch of one dataset
# shown to compute the same chains bit for bit.
# ---------------------------------------------------------------------

def _headline_params(native, move="langevin", p_err=0.1, seed=0xB5C17E):
    """The bench's batched+adjoint chains: sum score, learned error rates
    from the wrong start alpha=1e-2, beta=0.3."""
    return native.default_params(
        alpha_mean=1e-2, beta_mean=0.3, seed=seed, prob_beta_change=p_err,
        score_mode=native.SCORE_SUM,
        error_move=getattr(native, "ERROR_" + move.upper()))


@pytest.mark.parametrize("G,Cn,q", [(40, 50, 2), (95, 96, 3), (127, 64, 2)])
@pytest.mark.parametrize("move,p_err", [("langevin", 0.1),
                                        ("random_walk", 0.25)])
def test_inherited_count_chains_replay_in_fp64(native, orc, G, Cn, q, move,
                                               p_err):
    """Sum-score chains whose node loop inherits counts from the parent:
    41, 96 and 128 nodes (rows of 2, 3 and 4 32-bit words), every cell in
    registers (q cells per lane, one warp per chain, four chains per
    block -- at 95 x 96 the launch shape of the batched headline).  Each
    step is replayed in FP64: realised move, proposed rows, the sum score
    and the max score carried with it, the learned-rate proposal and the
    decision."""
    m, _, _ = D.generate_dataset(1000 + G, G, Cn, 1e-3, 0.2, 0.1, 0.02)
    mut, known = D.matrix_to_bits(m)
    p = _headline_params(native, move, p_err, seed=0xB5C17E + G)
    chains, steps = 4, 250
    rng = np.random.default_rng(G + Cn)
    starts = np.stack([D.random_parent_vector(rng, G) for _ in range(chains)])
    with native.Context(mut, known, Cn, G, p) as c:
        c.init_chains(chains, starts)
        c.set_launch(q, 1, 4)
        assert c.launch() == (q, 1, 4)
        tr = c.run(steps, trace=True)
        final = c.chains()
    assert int((tr["move"]["move_type"] == 0).sum()) > 0
    assert int(tr["accepted"].sum()) > 0
    for ch in range(chains):
        assert replay(orc, native, m, p, starts[ch], tr[ch],
                      final["dm"][ch]) <= 2


@pytest.mark.parametrize("G,Cn,launch", [(200, 150, (1, 1, 2)),
                                         (255, 300, (2, 1, 4)),
                                         (255, 300, (2, 2, 1))])
def test_wide_row_ring_chains_replay_in_fp64(native, orc, G, Cn, launch):
    """Sum-score chains with learned rates and rows of five to eight words:
    counts through the ring of the last 64 nodes in the canonical order,
    the cells streamed in chunks with a gene table per chunk.  Two chains
    start from star trees, whose order does not fit the ring (masked
    popcounts score them until the moves deepen the tree); every step of
    every chain is replayed in FP64."""
    m, _, _ = D.generate_dataset(3000 + G, G, Cn, 5e-4, 0.25, 0.08, 0.01)
    mut, known = D.matrix_to_bits(m)
    p = _headline_params(native, "langevin", 0.1, seed=0x51DE + G)
    chains, steps = 3, 200
    rng = np.random.default_rng(G + 3 * Cn)
    star = np.full(G + 1, G, dtype=np.uint32)
    starts = np.stack([star, star, D.random_parent_vector(rng, G)])
    with native.Context(mut, known, Cn, G, p) as c:
        c.init_chains(chains, starts)
        c.set_launch(*launch)
        tr = c.run(steps, trace=True)
        final = c.chains()
    assert int(tr["accepted"].sum()) > 0
    for ch in range(chains):
        assert replay(orc, native, m, p, starts[ch], tr[ch],
                      final["dm"][ch]) <= 2


@pytest.mark.parametrize("wpc", [1, 2])
def test_headline_batch_equals_replayed_chains(native, orc, wpc):
    """The batched launch of the bench's headline shape -- one 95 x 96
    dataset, 3 cells per lane, 4-warp blocks of one-warp chains (or chains
    of 2 warps, one per block), the dataset's increment tables built in the
    block -- leaves every chain (rows, best proposal and state)
    bit-identical to the same chains run alone with a trace, and those
    traced chains replay step by step in FP64."""
    G, Cn = 95, 96
    m, _, _ = D.generate_dataset(2026, G, Cn, 1e-3, 0.2, 0.1, 0.02)
    mut, known = D.matrix_to_bits(m)
    p = _headline_params(native)
    chains, steps = 8, 300
    with native.Batch([(mut, known, Cn, G)], p) as b:
        b.init_chains(chains)
        b.set_launch(3, 4, 0)
        b.set_chain_warps(wpc)
        assert b.launch()[:2] == (3, 4) and b.chain_warps() == wpc
        b.run(steps)
        img_b = b.save_chains()
    with native.Context(mut, known, Cn, G, p) as c:
        c.init_chains(chains)
        c.set_launch(3, 1, 4)
        starts = np.stack([native.matrix_to_parent(d)
                           for d in c.chains()["dm"]])
        tr = c.run(steps, trace=True)
        final = c.chains()
        img_c = c.save_chains()
    # both images end with the rows, the best proposals and the states of
    # the chains in the same layout
    n, W = G + 1, native.words(G + 1)
    tail = 2 * chains * n * W * 8 + 128 * chains
    assert img_b[-tail:] == img_c[-tail:]
    for ch in range(chains):
        assert replay(orc, native, m, p, starts[ch], tr[ch],
                      final["dm"][ch]) <= 2


@pytest.mark.parametrize("G,Cn", [(95, 96), (40, 200), (127, 64), (200, 150)])
def test_sum_launch_shapes_give_identical_chains(native, G, Cn):
    """Sum-score chains with learned rates are bit-identical under every
    launch shape: inherited counts (cells in registers, one or several
    warps per chain; for 200 genes the ring, over chunks of 32 to 256
    cells) and masked popcounts (streamed cells) add the same terms in the
    same order."""
    m, _, _ = D.generate_dataset(G + 5 * Cn, G, Cn, 1e-3, 0.2, 0.1, 0.02)
    mut, known = D.matrix_to_bits(m)
    shapes = [(3, 1, 4), (1, 1, 1), (2, 1, 2), (1, 2, 1), (1, 3, 1),
              (2, 2, 1), (1, 4, 1), (4, 1, 1), (4, 2, 1), (3, 1, 7),
              (3, 1, 8)]
    qmax = 2 if G + 1 > 128 else 4
    outs = []
    for q, wpc, cpb in shapes:
        if q > qmax:
            continue
        p = _headline_params(native, seed=77)
        with native.Context(mut, known, Cn, G, p) as c:
            c.init_chains(9)
            c.set_launch(q, wpc, cpb)
            try:
                tr = c.run(150, trace=True)
            except native.BbsError as e:
                # a block too large for this shape's shared memory is
                # refused before anything runs
                assert e.code == native.BBS_ERR_SIZE, e
                assert q >= 3 and cpb >= 7, e
                continue
            outs.append((c.chains(), c.best(), tr))
    ch0, b0, t0 = outs[0]
    for ch, b, t in outs[1:]:
        assert (ch["dm"] == ch0["dm"]).all()
        np.testing.assert_array_equal(ch["score"], ch0["score"])
        np.testing.assert_array_equal(ch["alpha"], ch0["alpha"])
        np.testing.assert_array_equal(ch["beta"], ch0["beta"])
        assert b["score"] == b0["score"] and (b["dm"] == b0["dm"]).all()
        assert (t["accepted"] == t0["accepted"]).all()
        np.testing.assert_array_equal(t["proposed_score"],
                                      t0["proposed_score"])
        np.testing.assert_array_equal(t["proposed_max_score"],
                                      t0["proposed_max_score"])


@pytest.mark.parametrize("G,Cn", [(95, 96), (255, 80)])
def test_autotune_skips_shapes_that_do_not_fit(native, G, Cn):
    """One dataset whose chains inherit counts: some launch shapes of the
    tuners' lists (8 warps of 4 cells per lane) need more shared memory
    than a block may have.  Both tuners skip them, pick a shape that runs,
    and leave the chains' states as they were."""
    m, _, _ = D.generate_dataset(G * Cn, G, Cn, 1e-3, 0.2, 0.1, 0.02)
    mut, known = D.matrix_to_bits(m)
    p = _headline_params(native)
    with native.Batch([(mut, known, Cn, G)], p) as b:
        b.init_chains(64)
        b.run(20)
        before = b.save_chains()
        assert b.autotune(16) > 0
        assert b.save_chains() == before
        b.run(20)
    with native.Context(mut, known, Cn, G, p) as c:
        c.init_chains(64)
        c.run(20)
        before = c.chains()
        assert c.autotune(16) > 0
        after = c.chains()
        assert (after["dm"] == before["dm"]).all()
        c.run(20)
