"""Generates tests/golden/ref_vectors.npz from the reference's own classes.

Run in a checkout where the reference sources exist (oracle/_ref is built
from them by `make -C oracle ref`):

    python tests/golden/make_golden.py

Every array in the output is produced by oracle/_ref/libbbs_ref.so, i.e. by
the reference's src/MutationTree.hpp, src/TreeScorer.hpp and
src/Parameters.hpp compiled unmodified, plus its step loop
(src/Application.hpp:408-487) restated around them in oracle/ref_driver.cpp.
Inputs come from seeded generators, so the file is reproducible.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(
    __file__))))
sys.path.insert(0, ROOT)

from bbscite_gb300 import data as D  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)),
                   "ref_vectors.npz")


def tree_hash(rows: np.ndarray) -> np.uint64:
    """Order-dependent 64-bit checksum of bit-matrix words."""
    h = np.uint64(1469598103934665603)
    with np.errstate(over="ignore"):
        for w in np.ascontiguousarray(rows, dtype=np.uint64).ravel():
            h = np.uint64((h ^ w) * np.uint64(1099511628211))
    return h


def random_raw_moves(rng, n_nodes, n, p_beta=0.1):
    raw = np.zeros(n, dtype=O.RAW_MOVE)
    t = rng.random(n)
    raw["move_type"] = np.where(t < p_beta, 0, np.where(
        t < p_beta + 0.45, 1, np.where(t < p_beta + 0.8, 2, 3)))
    v = rng.integers(0, n_nodes - 1, size=n)
    w = rng.integers(0, n_nodes - 2, size=n)
    w = w + (w >= v)
    raw["raw_v"], raw["raw_w"] = v, w
    edge = np.array([0.0, 1.0, np.float32(0.99999994)], dtype=np.float32)
    u1 = rng.random(n).astype(np.float32)
    u2 = rng.random(n).astype(np.float32)
    pick = rng.random(n)
    u1 = np.where(pick < 0.05, edge[rng.integers(0, 3, size=n)], u1)
    u2 = np.where(pick > 0.95, edge[rng.integers(0, 3, size=n)], u2)
    raw["raw_descendant_of_v"] = u1
    raw["raw_nondescendant_of_v"] = u2
    raw["beta_jump"] = rng.normal(0, 0.05, size=n).astype(np.float32)
    raw["acceptance_level"] = rng.random(n).astype(np.float32)
    return raw


def main() -> None:
    ref = O.ref_lib()
    if ref is None:
        raise SystemExit("oracle/_ref is not built (make -C oracle ref)")
    p = O._p
    out = {}

    # --- scores -----------------------------------------------------------
    score_cases = [(4, 6), (16, 20), (31, 32), (63, 64), (95, 96),
                   (127, 128), (127, 256), (255, 512)]
    for ci, (G, Cn) in enumerate(score_cases):
        rng = np.random.default_rng(1000 + ci)
        m, _, _ = D.generate_dataset(2000 + ci, G, Cn, 1e-3, 0.2, 0.1, 0.02)
        mut, known = D.matrix_to_bits(m)
        parents = np.stack([D.random_parent_vector(rng, G) for _ in range(3)])
        betas = np.array([0.2, 0.4309, 0.05], dtype=np.float32)
        scores = np.zeros((3, 3), dtype=np.float32)
        for t in range(3):
            _, dm = O.parent_to_matrix(parents[t])
            for b in range(3):
                scores[t, b] = ref.ref_score(1e-3, 0.2, 0.1, Cn, G, p(mut),
                                             p(known), p(dm), float(betas[b]))
        out[f"score{ci}_matrix"] = m
        out[f"score{ci}_parents"] = parents
        out[f"score{ci}_betas"] = betas
        out[f"score{ci}_scores"] = scores
    out["score_cases"] = np.array(score_cases, dtype=np.int32)

    # --- Beta prior -------------------------------------------------------
    prior_params = np.array([[1e-3, 0.2, 0.1], [6.04e-5, 0.4309, 0.1],
                             [1e-2, 0.25, 0.05], [1e-3, 0.45, 0.1]],
                            dtype=np.float32)
    prior_betas = np.array([0.05, 0.2, 0.3, 0.4309, 0.7], dtype=np.float32)
    prior_vals = np.zeros((len(prior_params), len(prior_betas)),
                          dtype=np.float32)
    for i, (a, bm, sd) in enumerate(prior_params):
        for j, b in enumerate(prior_betas):
            prior_vals[i, j] = ref.ref_logscore_beta(float(a), float(bm),
                                                     float(sd), float(b))
    out["prior_params"], out["prior_betas"] = prior_params, prior_betas
    out["prior_values"] = prior_vals

    # --- move realisation + update chains --------------------------------
    move_cases = [(3, 4), (16, 20), (63, 64), (95, 96), (127, 64), (255, 64)]
    for ci, (G, _) in enumerate(move_cases):
        rng = np.random.default_rng(3000 + ci)
        n = G + 1
        start = D.random_parent_vector(rng, G)
        am, dm = O.parent_to_matrix(start)
        beta = np.float32(0.3)
        n_moves = 64
        raw = random_raw_moves(rng, n, n_moves, p_beta=0.1)
        params = np.zeros(n_moves, dtype=O.MOD_PARAMS)
        pvs = np.zeros((n_moves, n), dtype=np.uint16)
        hashes = np.zeros((n_moves, 2), dtype=np.uint64)
        betas = np.zeros(n_moves, dtype=np.float32)
        for i in range(n_moves):
            ref.ref_realize(p(am), p(dm), n, float(beta), p(raw[i:i + 1]),
                            p(params[i:i + 1]))
            nam, ndm = np.zeros_like(am), np.zeros_like(dm)
            beta = np.float32(ref.ref_apply(p(am), p(dm), n, float(beta),
                                            p(params[i:i + 1]), p(nam),
                                            p(ndm)))
            am, dm = nam, ndm
            pvs[i] = [ref.ref_get_parent(p(am), p(dm), n, x) for x in range(n)]
            hashes[i] = (tree_hash(am), tree_hash(dm))
            betas[i] = beta
        out[f"move{ci}_start"] = start
        out[f"move{ci}_raw"] = raw
        out[f"move{ci}_params"] = params
        out[f"move{ci}_parents"] = pvs
        out[f"move{ci}_hashes"] = hashes
        out[f"move{ci}_betas"] = betas
    out["move_cases"] = np.array(move_cases, dtype=np.int32)

    # --- chain replays (the reference's own accept decisions) -------------
    chain_cases = [(16, 20, 2000, 0.0), (63, 64, 1000, 0.0),
                   (95, 96, 600, 0.0), (40, 50, 1500, 0.15)]
    for ci, (G, Cn, steps, p_beta) in enumerate(chain_cases):
        rng = np.random.default_rng(4000 + ci)
        n = G + 1
        alpha, beta_mean, sd, gamma = 1e-3, 0.2, 0.1, 1.0
        m, _, _ = D.generate_dataset(5000 + ci, G, Cn, alpha, beta_mean, 0.1,
                                     0.02)
        mut, known = D.matrix_to_bits(m)
        start = D.random_parent_vector(rng, G)
        am, dm = O.parent_to_matrix(start)
        raw = random_raw_moves(rng, n, steps, p_beta=p_beta)
        b = C.c_float(beta_mean)
        s0 = ref.ref_score(alpha, beta_mean, sd, Cn, G, p(mut), p(known),
                           p(dm), beta_mean)
        s = C.c_float(s0)
        best = C.c_float()
        best_dm = np.zeros_like(dm)
        prop = np.zeros(steps, dtype=np.float32)
        acc = np.zeros(steps, dtype=np.uint8)
        ref.ref_run_chain(alpha, beta_mean, sd, gamma, Cn, G, p(mut),
                          p(known), p(raw), steps, p(am), p(dm), C.byref(b),
                          C.byref(s), C.byref(best), p(best_dm), p(prop),
                          p(acc), None, 0.0, None)
        out[f"chain{ci}_matrix"] = m
        out[f"chain{ci}_start"] = start
        out[f"chain{ci}_raw"] = raw
        out[f"chain{ci}_initial_score"] = np.float32(s0)
        out[f"chain{ci}_prop_scores"] = prop
        out[f"chain{ci}_accepted"] = acc
        out[f"chain{ci}_final_parent"] = np.array(
            [ref.ref_get_parent(p(am), p(dm), n, x) for x in range(n)],
            dtype=np.uint16)
        out[f"chain{ci}_final_beta"] = np.float32(b.value)
        out[f"chain{ci}_final_score"] = np.float32(s.value)
        out[f"chain{ci}_best_score"] = np.float32(best.value)
        out[f"chain{ci}_best_hash"] = tree_hash(best_dm)
    out["chain_cases"] = np.array(chain_cases, dtype=np.float64)

    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({os.path.getsize(OUT)} bytes)")


if __name__ == "__main__":
    main()
