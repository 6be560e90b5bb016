"""Generates tests/golden/quality_ref.json: the reference's best-found
log-likelihoods on 64 seeded datasets of the 63-gene x 64-cell workload
(alpha=6.04e-5, beta=0.4309, 5% unknown, no homozygous entries), with
8 chains x 100,000 steps each.

Run where the reference sources exist (oracle/_ref is built from them by
`make -C oracle`):

    python tests/golden/make_quality_ref.py

Each chain's initial tree and moves come from the reference's own samplers
and URNG (MutationTree::sample_random_pruefer_code, RawMoveDistribution,
std::minstd_rand; oracle/ref_driver.cpp ref_sample_chain), and each chain
runs through the reference's MutationTree and TreeScorer classes with the
step loop of src/Application.hpp:408-487 (ref_run_chain).  The best over
the chains is the reference's own cell-order score.  Datasets come from
bbscite_gb300.data.generate_dataset with seed 3100 + i.
"""
from __future__ import annotations

import ctypes as C
import json
import multiprocessing as mp
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(
    __file__))))
sys.path.insert(0, ROOT)

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)),
                   "quality_ref.json")
WORKLOAD = dict(n_genes=63, n_cells=64, alpha=6.04e-5, beta=0.4309,
                beta_sd=0.1, missing=0.05, homozygous=0.0, chains=8,
                steps=100000, datasets=64, seed0=3100)


def run_dataset(i: int) -> dict:
    from bbscite_gb300 import data as D
    from oracle import oracle as O
    w = WORKLOAD
    ref = O.ref_lib()
    G, Cn = w["n_genes"], w["n_cells"]
    m, _, _ = D.generate_dataset(w["seed0"] + i, G, Cn, w["alpha"],
                                 w["beta"], w["missing"], w["homozygous"])
    mut, known = D.matrix_to_bits(m)
    n = G + 1

    def p(a):
        return a.ctypes.data_as(C.c_void_p)
    best_score, best_parent = None, None
    for ch in range(w["chains"]):
        parent = np.zeros(n, dtype=np.uint32)
        raw = np.zeros(w["steps"], dtype=O.RAW_MOVE)
        ref.ref_sample_chain(G, C.c_float(0.0), C.c_float(0.55),
                             C.c_float(0.4), C.c_float(0.05),
                             C.c_float(w["beta_sd"]), C.c_float(10.0),
                             C.c_uint32((w["seed0"] + i) * 16 + ch),
                             w["steps"], p(parent), p(raw))
        am, dm = O.parent_to_matrix(parent)
        s0 = ref.ref_score(w["alpha"], w["beta"], w["beta_sd"], Cn, G, p(mut),
                           p(known), p(dm), w["beta"])
        b, s = C.c_float(w["beta"]), C.c_float(s0)
        best = C.c_float()
        best_dm = np.zeros_like(dm)
        prop = np.zeros(w["steps"], dtype=np.float32)
        acc = np.zeros(w["steps"], dtype=np.uint8)
        ref.ref_run_chain(w["alpha"], w["beta"], w["beta_sd"], 1.0, Cn, G,
                          p(mut), p(known), p(raw), w["steps"], p(am), p(dm),
                          C.byref(b), C.byref(s), C.byref(best), p(best_dm),
                          p(prop), p(acc), None, 0.0, None)
        if best_score is None or best.value > best_score:
            best_score = best.value
            best_parent = O.parent_vector(best_dm).tolist()
    return {"dataset_seed": w["seed0"] + i, "best_score": best_score,
            "best_parent": best_parent}


def main() -> None:
    from oracle import oracle as O
    O.build()
    if O.ref_lib() is None:
        raise SystemExit("the reference's classes are not built here")
    with mp.get_context("spawn").Pool(os.cpu_count()) as pool:
        rows = pool.map(run_dataset, range(WORKLOAD["datasets"]))
    with open(OUT, "w") as f:
        json.dump({"workload": WORKLOAD, "results": rows}, f, indent=1)
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
