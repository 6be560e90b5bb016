#!/usr/bin/env python3
"""Chain-steps/s of the bbSCITE MCMC step path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Headline (`value`): the batched+adjoint form on 95 genes x 96 cells from
the seeded generator (alpha=1e-3, beta=0.2, 10% unknown, 2% homozygous):
1024 chains in the work-list launch, sum-over-attachments score with its
fused adjoint, Langevin error-rate moves (probability 0.1) learning alpha
and beta from 1e-2 / 0.3.  `plain` is the one-dataset kernel with the
reference's max score and fixed rates on the same chains.
`equal_best_logl` scores both forms' best trees with the reference's max
score at the generator's rates.  One bench step = one launch advancing
every chain by --chain-steps steps; chains continue across launches.
Inputs are resident in HBM before the timed region; a 256 MiB buffer is
written between launches to flush L2.

`value` is device-timed (CUDA events on the library's stream around each
launch); `e2e` is the same form through the C ABI with host buffers
(creation, host->device copies, the run and the device->host read of the
best tree inside the timed region).  `batched_mix` runs 512 uneven
datasets in one batched launch against one plain launch per dataset.

--impl reference runs the reference's CPU implementation of the path
(the C restatement in oracle/, threaded over chains) on the same data.
N > 1: one process per GPU, independent replicas (no data-path collective).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("chain-steps/s, 1 GB300, 95g x 96c: batched+adjoint vs plain at "
          "equal best logL")
UNIT = "chain-steps/s"
WORKLOAD = dict(n_genes=95, n_cells=96, alpha=1e-3, beta=0.2, missing=0.10,
                homozygous=0.02, data_seed=2026, chains=1024)


def popc_per_chain_step(n_genes: int, n_cells: int) -> int:
    """Algorithmic 32-bit POPC operations of one chain step: two masked
    popcounts per (cell, node) pair over ceil(G/32) words."""
    return n_cells * (n_genes + 1) * 2 * math.ceil(n_genes / 32)


def counted_bits_per_chain_step(n_genes: int, n_cells: int) -> int:
    """The paper's counted bits per step, 4 * cells * nodes^2."""
    return 4 * n_cells * (n_genes + 1) ** 2


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--chain-steps", type=int, default=20000,
                    help="chain steps per launch (one bench step)")
    ap.add_argument("--chains", type=int, default=WORKLOAD["chains"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="target length of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--quality-steps", type=int, default=200000,
                    help="untimed steps per chain of both forms before the "
                         "warm-up (the equal-best-logL comparison)")
    ap.add_argument("--autotune", type=int, default=1)
    ap.add_argument("--autotune-steps", type=int, default=200)
    ap.add_argument("--launch", default="",
                    help="plain form: cells_per_lane,warps_per_chain,"
                         "chains_per_block")
    ap.add_argument("--batch-launch", default="",
                    help="batched form: cells_per_lane,warps_per_block,"
                         "merge_rows[,warps_per_chain]")
    ap.add_argument("--mix-datasets", type=int, default=512)
    ap.add_argument("--mix-steps", type=int, default=20000,
                    help="512-dataset mix: steps per chain of the batched "
                         "and the sequential plain form")
    ap.add_argument("--mix-tuned-steps", type=int, default=2000,
                    help="512-dataset mix: steps per chain of the tuned "
                         "single-dataset form")
    ap.add_argument("--lvr-steps", type=int, default=400000,
                    help="Langevin vs random walk: steps per chain (0: off)")
    ap.add_argument("--lvr-seeds", type=int, default=8)
    ap.add_argument("--lvr-chains", type=int, default=256)
    ap.add_argument("--lvr-error-step", type=float, default=1.2)
    ap.add_argument("--caps-steps", type=int, default=500,
                    help="255x512 run: steps per launch (0: off)")
    ap.add_argument("--caps-chains", type=int, default=4096)
    ap.add_argument("--caps-profile", default="", choices=["", "batch", "plain"],
                    help="only the 255x512 kernel of one form at the shape "
                         "its tuner picks (batched: 2 cells per lane, chains "
                         "of 2 warps; plain: 2 cells per lane, chains of 4 "
                         "warps), one 20,000-step launch and one 100-step "
                         "launch, for an ncu capture of the second")
    return ap.parse_args(argv)


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def make_dataset(rank: int = 0):
    from bbscite_gb300 import data as D
    w = WORKLOAD
    m, _, _ = D.generate_dataset(w["data_seed"] + rank, w["n_genes"],
                                 w["n_cells"], w["alpha"], w["beta"],
                                 w["missing"], w["homozygous"])
    mut, known = D.matrix_to_bits(m)
    return m, mut, known


# ---------------------------------------------------------------- clocks --

class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"),
                stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None,
                    "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4)
                          if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------ baselines --

def cpu_baseline(seconds: float, rank: int = 0) -> dict:
    """The oracle port of the reference's step loop (reference cell-order
    score), threads over chains on all host cores, same 95x96 workload."""
    import numpy as np

    from bbscite_gb300 import data as D
    from oracle import oracle as O
    w = WORKLOAD
    _, mut, known = make_dataset(rank)
    threads = os.cpu_count() or 1
    mp = O.move_probs(0.0, 0.55, 0.4, 0.05, 0.1, 10.0)
    rng = np.random.default_rng(5)
    n_chains = max(threads, 32)
    parents = np.stack([D.random_parent_vector(rng, w["n_genes"])
                        for _ in range(n_chains)])
    # probe the rate, then size the sample to `seconds`
    probe_steps = 200
    t0 = time.perf_counter()
    O.run_chains_mt(w["alpha"], w["beta"], 0.1, 1.0, mp, 11, parents, mut,
                    known, probe_steps, threads, score_mode=0)
    rate = n_chains * probe_steps / (time.perf_counter() - t0)
    steps = max(probe_steps, int(rate * seconds / n_chains))
    t0 = time.perf_counter()
    best, _ = O.run_chains_mt(w["alpha"], w["beta"], 0.1, 1.0, mp, 12,
                              parents, mut, known, steps, threads,
                              score_mode=0)
    dt = time.perf_counter() - t0
    return {"value": n_chains * steps / dt, "unit": UNIT, "cores": threads,
            "kind": "port", "chains": n_chains,
            "sample": f"{n_chains} chains x {steps} steps of the 95x96 "
                      f"workload ({dt:.1f} s), oracle/bbs_oracle.c "
                      "orc_run_chains_mt, reference cell-order score",
            "best_logl": best}


def cpu_scoring_proxy_rate(seconds: float) -> dict:
    """The reference's CPU scoring benchmark restated
    (cpu_scoring_benchmark/CPUTreeScorer.hpp:97-213 at its fixed 128 cells
    x 127 genes): repeated scorings of fixed random trees on all host
    cores, as scorings/s and the paper's counted bits (4 * 128 * 128^2 per
    scoring; Table 4 quotes 233.05 k scorings/s and 1.95 Tbit/s on two Xeon
    Gold 6148)."""
    import numpy as np

    from bbscite_gb300 import data as D
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    m, _, _ = D.generate_dataset(128127, 127, 128, 1e-3, 0.2, 0.05, 0.0)
    # [quadword][gene] words with one bit per cell (128 cells, 128 slots)
    mutq = np.zeros((2, 128), dtype=np.uint64)
    knownq = np.zeros((2, 128), dtype=np.uint64)
    for g in range(127):
        for c in range(128):
            b = np.uint64(1) << np.uint64(c % 64)
            if m[g, c] != 3:
                knownq[c // 64, g] |= b
            if m[g, c] in (1, 2):
                mutq[c // 64, g] |= b
    # per tree [quadword][node] ancestor words
    rng = np.random.default_rng(128)
    trees = [np.ascontiguousarray(O.parent_to_matrix(
        D.random_parent_vector(rng, 127))[1].T) for _ in range(32)]
    n_trees = 64 * threads
    dmq = np.ascontiguousarray(np.stack([trees[t % 32]
                                         for t in range(n_trees)]))
    t0 = time.perf_counter()
    O.cpu_scoring_proxy(1e-3, 0.2, mutq, knownq, dmq, n_trees, 4, threads)
    rate = n_trees * 4 / (time.perf_counter() - t0)
    reps = max(4, int(rate * seconds / n_trees))
    t0 = time.perf_counter()
    O.cpu_scoring_proxy(1e-3, 0.2, mutq, knownq, dmq, n_trees, reps, threads)
    dt = time.perf_counter() - t0
    per_s = n_trees * reps / dt
    return {"scorings_per_s": per_s,
            "counted_tbit_per_s": per_s * 4 * 128 * 128 ** 2 / 1e12,
            "cores": threads, "kind": "port",
            "sample": f"{n_trees * reps} scorings at 128 cells x 127 genes "
                      f"({dt:.1f} s), oracle/bbs_oracle.c "
                      "orc_cpu_scoring_proxy"}


# What ties the CPU port to the reference's own code: the box has no
# reference sources, so the reference's classes cannot be compiled there.
PORT_PINNING = ("oracle/bbs_oracle.c restates the reference's step loop "
                "(src/Application.hpp:408-487) and scorer; it reproduces the "
                "reference classes compiled unmodified bit for bit (golden "
                "chains, scores and moves in tests/golden/ref_vectors.npz, "
                "CPUTreeScorer scores in tests/golden/proxy_vectors.npz)")


def run_reference(args) -> None:
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    w = WORKLOAD
    per_step = max(1.0, min(args.cpu_seconds, 8.0))
    vals = []
    info = None
    for i in range(args.warmup + args.steps):
        b = cpu_baseline(per_step)
        if i >= args.warmup:
            vals.append(b["value"])
            info = b
    value = statistics.mean(vals)
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64-popcount+f32", "data": "synthetic",
        "config": {"workload": f"{w['n_genes']} genes x {w['n_cells']} "
                   f"cells; a bounded sample of {info['chains']} chains of "
                   f"the {args.chains}-chain workload is timed; data "
                   "alpha=1e-3 beta=0.2 (10% unknown, 2% homozygous); the "
                   "reference's plain MCMC at fixed error rates (it has no "
                   "batched or adjoint form)",
                   "n_genes": w["n_genes"], "n_cells": w["n_cells"],
                   "chains": info["chains"],
                   "workload_chains": args.chains,
                   "parallelism": "host threads over chains"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": info["cores"],
                         "kind": info["kind"], "sample": info["sample"],
                         "pinned": PORT_PINNING},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "best_logl": info["best_logl"],
    }
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------------ ours --

PROFILE = "chain_kernels_95x96.json"


def _profile_figure(form: str, key: str, profile: str = PROFILE):
    """A figure of a chain kernel from a committed ncu summary (by default
    profiles/chain_kernels_95x96.json, the bench's shape; form "batch" or
    "plain"; warp instructions per chain-step, DRAM bytes per chain per
    launch), or None."""
    p = os.path.join(ROOT, "profiles", profile)
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return d.get(form, {}).get(key)


def max_over_ranks(dist, values, device):
    """Each timing maximised over the ranks: the job's clock is its slowest
    replica."""
    import torch
    if dist is None:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64,
                     device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


def global_best(dist, score, rank, world, device):
    """The best score over the replicas and the rank holding it (the lowest
    rank on ties): the one cross-replica step of the path, the final argmax
    of src/Application.hpp:470-487 over independent chain sets."""
    import torch
    if dist is None:
        return float(score), rank
    mine = torch.tensor([float(score), float(rank)], dtype=torch.float64,
                        device=device)
    parts = [torch.zeros_like(mine) for _ in range(world)]
    dist.all_gather(parts, mine)
    best, who = None, None
    for p in parts:
        s, r = float(p[0]), int(p[1])
        if best is None or s > best:
            best, who = s, r
    return best, who


def _timed(run, last_ms, steps, flush, barrier, torch):
    """Runs `steps` launches between barriers and device syncs; returns
    (sum of per-launch device ms, wall seconds, per-launch ms)."""
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ms = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        run()
        ms.append(last_ms())
    torch.cuda.synchronize()
    barrier()
    return sum(ms), time.perf_counter() - t0, ms


def mix_datasets(n_datasets: int, seed: int = 512):
    """The uneven mix: genes U[16,127], cells U[16,256], alpha log-uniform
    in [1e-5, 1e-2], beta U[0.05, 0.45], unknown U[0, 0.15]."""
    import numpy as np

    from bbscite_gb300 import data as D
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_datasets):
        G = int(rng.integers(16, 128))
        Cn = int(rng.integers(16, 257))
        a = float(10 ** rng.uniform(-5, -2))
        b = float(rng.uniform(0.05, 0.45))
        u = float(rng.uniform(0.0, 0.15))
        m, _, _ = D.generate_dataset(seed * 1000 + i, G, Cn, a, b, u, 0.0)
        mut, known = D.matrix_to_bits(m)
        out.append(((mut, known, Cn, G), a, b))
    return out


def run_mix(N, n_datasets, chains, steps, flush, torch, tuned_steps=None):
    """Batched launch (autotuned, CUDA graph) vs one plain launch per
    dataset, device time of the runs only, `steps` steps per chain in both.
    The plain form runs each chain on one warp (cells_per_lane =
    min(ceil(C/32), 4), one chain per block); the tuned single-dataset form
    (timed over tuned_steps steps per chain) lets each launch spread a
    chain's cells over up to 4 warps (the context's default launch
    heuristic)."""
    tuned_steps = tuned_steps or steps
    mix = mix_datasets(n_datasets)
    params = [N.default_params(alpha_mean=a, beta_mean=b, seed=900 + i)
              for i, (_, a, b) in enumerate(mix)]
    with N.Batch([d for d, _, _ in mix], params) as bt:
        bt.init_chains(chains)
        bt.autotune(max(16, steps // 10))
        bt.run(steps)
        flush.zero_()
        torch.cuda.synchronize()
        bt.run(steps)
        batched_ms = bt.last_run_ms()
        shape = bt.launch() + (bt.chain_warps(),)
    plain_ms = tuned_ms = 0.0
    for i, ((mut, known, Cn, G), _, _) in enumerate(mix):
        with N.Context(mut, known, Cn, G, params[i]) as c:
            c.init_chains(chains)
            c.run(tuned_steps)
            tuned_ms += c.last_run_ms()
            c.init_chains(chains)
            c.set_launch(min((Cn + 31) // 32, 4), 1, 1)
            c.run(steps)
            plain_ms += c.last_run_ms()
    total = n_datasets * chains * steps
    tuned_rate = n_datasets * chains * tuned_steps / (tuned_ms / 1e3)
    batched_rate = total / (batched_ms / 1e3)
    return {"datasets": n_datasets, "chains_per_dataset": chains,
            "steps": steps,
            "batched_chain_steps_per_s": batched_rate,
            "sequential_plain_chain_steps_per_s": total / (plain_ms / 1e3),
            "speedup": plain_ms / batched_ms,
            "tuned_steps": tuned_steps,
            "sequential_tuned_chain_steps_per_s": tuned_rate,
            "speedup_vs_tuned_single": batched_rate / tuned_rate,
            "pairs_per_chain_step": mix_pairs(mix),
            "batched_launch": {"cells_per_lane": shape[0],
                               "warps_per_block": shape[1],
                               "merged_row_widths": bool(shape[2]),
                               "warps_per_chain": shape[3]}}


def mix_pairs(mix) -> float:
    """Mean (cell, node) pairs scored per chain-step over the mix."""
    return sum(Cn * (G + 1) for (_, _, Cn, G), _, _ in mix) / len(mix)


def _logit(x):
    return math.log(x / (1.0 - x))


def run_langevin_vs_rw(N, mut, known, G, Cn, chains, total, seeds,
                       error_step, data_alpha, data_beta):
    """Steps-to-best of the adjoint-driven Langevin error-rate chain (sum
    score) against random-walk error-rate chains, all from alpha=1e-2,
    beta=0.3 with error-move probability 0.1, over `seeds` independent
    seeds (the same Philox seeds in every arm).  Arms: the preconditioned
    random walk on (logit alpha, logit beta) with the reference's max
    score; the reference's own beta random walk (alpha stays at its
    start); Langevin with the sum score; Langevin with the max score; and,
    as the bound no error-rate move can beat, the reference's chain
    started at the generator's rates (true_rates).  At
    every checkpoint (1,000-step chunks to 20,000 steps, then 10,000-step
    chunks) each arm's best tree is scored with the reference's max score
    at the generator's rates (a scale common to all arms: the chains rank
    proposals at their own rates), and the median over chains of
    logit(alpha) and logit(beta) is read.  Per seed: the first step count
    at which each arm is within 0.1 nats of a random-walk arm's final
    best, and the step count after which each arm's median rates stay
    within 0.25 (logit alpha) and 0.05 (logit beta) of their final
    values."""
    import numpy as np

    start = (1e-2, 0.3)
    arms = {"random_walk": (N.SCORE_MAX, N.ERROR_RANDOM_WALK, start),
            "langevin": (N.SCORE_SUM, N.ERROR_LANGEVIN, start),
            "langevin_max_score": (N.SCORE_MAX, N.ERROR_LANGEVIN, start),
            # the reference's own chain: its beta random walk (ChangeBeta,
            # src/MutationTree.hpp:345-351), alpha fixed at its start
            "reference_beta_walk": (N.SCORE_MAX, N.ERROR_BETA_WALK, start),
            # the bound: the reference's chain started at the generator's
            # rates, which no error-rate move can learn faster than
            "true_rates": (N.SCORE_MAX, N.ERROR_BETA_WALK,
                           (data_alpha, data_beta))}
    marks = list(range(1000, 20001, 1000)) + \
        list(range(30000, total + 1, 10000))
    res = {a: [] for a in arms}
    sp = N.default_params(alpha_mean=data_alpha, beta_mean=data_beta)
    with N.Context(mut, known, Cn, G, sp) as scorer:
        for sd in range(seeds):
            for name, (mode, move, (a0, b0)) in arms.items():
                p = N.default_params(alpha_mean=a0, beta_mean=b0,
                                     seed=0x1A6E + 7919 * sd,
                                     prob_beta_change=0.1, score_mode=mode,
                                     error_move=move, error_step=error_step)
                with N.Context(mut, known, Cn, G, p) as c:
                    c.init_chains(chains)
                    best, own, la, lb, done = [], [], [], [], 0
                    for mk in marks:
                        c.run(mk - done)
                        done = mk
                        b = c.best()
                        own.append(float(b["score"]))
                        best.append(float(scorer.score_trees(
                            b["dm"][None], data_beta)[0][0]))
                        st = c.chains()
                        la.append(float(np.median([_logit(x) for x in
                                                   st["alpha"]])))
                        lb.append(float(np.median([_logit(x) for x in
                                                   st["beta"]])))
                    e = c.chains()["err_stats"].sum(axis=0)
                settle = 0
                for k in range(len(marks)):
                    if abs(la[k] - la[-1]) > 0.25 or \
                            abs(lb[k] - lb[-1]) > 0.05:
                        settle = marks[k]
                res[name].append({"best": best, "own": own[-1],
                                  "settle": settle,
                                  "accept": float(e[1]) / max(1, int(e[0]))})
    def steps_to(arm, sd, base):
        """First checkpoint of `arm` within 0.1 nats of `base`'s final
        best, or None."""
        target = res[base][sd]["best"][-1] - 0.1
        return next((marks[k] for k, v in enumerate(res[arm][sd]["best"])
                     if v >= target), None)

    def median_ratio(arm, base):
        r = []
        for sd in range(seeds):
            a, b = steps_to(arm, sd, base), steps_to(base, sd, base)
            r.append(a / b if a is not None else math.inf)
        r.sort()
        med = r[len(r) // 2] if seeds % 2 else \
            0.5 * (r[seeds // 2 - 1] + r[seeds // 2])
        # never reached within the run: null in the JSON line
        return None if math.isinf(med) else med

    per_seed = [{"best": {a: round(res[a][sd]["best"][-1], 3) for a in arms},
                 "steps_to_rw_best": {a: steps_to(a, sd, "random_walk")
                                      for a in arms},
                 "steps_to_reference_best": {
                     a: steps_to(a, sd, "reference_beta_walk") for a in arms},
                 "best_at_own_rates": {a: round(res[a][sd]["own"], 3)
                                       for a in arms}}
                for sd in range(seeds)]
    ratios = {a: median_ratio(a, "random_walk") for a in arms
              if a not in ("random_walk", "reference_beta_walk")}
    ratios_ref = {a: median_ratio(a, "reference_beta_walk") for a in arms
                  if a not in ("random_walk", "reference_beta_walk",
                               "true_rates")}
    return {
        "chains": chains, "steps": total, "seeds": seeds,
        "error_step": error_step, "n_genes": G, "n_cells": Cn,
        "scored_with": f"reference max score at alpha={data_alpha:g} "
                       f"beta={data_beta:g}",
        "arms": {a: {"score": "sum" if m == N.SCORE_SUM else "max",
                     "error_move": {N.ERROR_LANGEVIN: "langevin",
                                    N.ERROR_RANDOM_WALK: "random_walk",
                                    N.ERROR_BETA_WALK: "beta_walk"}[e],
                     "start": [a0, b0]}
                 for a, (m, e, (a0, b0)) in arms.items()},
        # steps-to-best of a chain that knows the rates from step 0: no
        # error-rate move can do better than this, so a ratio above 0.5
        # here says the target is set by the shared tree moves
        "true_rates_step_ratio_over_rw": ratios["true_rates"],
        "per_seed": per_seed,
        "median_step_ratio_over_rw": ratios,
        "median_step_ratio_over_reference_beta_walk": ratios_ref,
        "target_half_met": ratios["langevin"] is not None
        and ratios["langevin"] <= 0.5,
        "target_half_met_vs_reference_beta_walk":
            ratios_ref["langevin"] is not None and ratios_ref["langevin"] <= 0.5,
        "rates_settle_steps": {a: [r["settle"] for r in res[a]] for a in arms},
        "error_move_acceptance": {a: [round(r["accept"], 3) for r in res[a]]
                                  for a in arms},
    }


CAPS_PROFILE = "chain_kernels_255x512.json"


def run_beyond_caps(N, chains, steps, flush, torch, warm=20000, early=1500):
    """255 genes x 512 cells (alpha=5e-4, beta=0.25, 8% unknown, 1%
    homozygous): the batched form with the sum score and Langevin error
    moves against the plain form (max score, fixed rates), device time of
    one launch of `steps` steps after `warm` steps from random trees: the
    regime of nearly all of a 1,000,000-step run.  The rate after `early`
    steps is reported too: there the sum score still sums many cells a
    second time, while their best attachment lies far below the bound it is
    taken against.  Launch shapes are tuned after `early` steps.  Both
    forms inherit counts through the ring (rows of eight words); the
    roofline is the issue slots, from the warp instructions per chain-step
    of the committed ncu summary (captured after `warm` steps)."""
    from bbscite_gb300 import data as D
    G, Cn = 255, 512
    m, _, _ = D.generate_dataset(5255, G, Cn, 5e-4, 0.25, 0.08, 0.01)
    mut, known = D.matrix_to_bits(m)
    adj = N.default_params(alpha_mean=5e-4, beta_mean=0.25, seed=5,
                           prob_beta_change=0.1, score_mode=N.SCORE_SUM,
                           error_move=N.ERROR_LANGEVIN)
    plain = N.default_params(alpha_mean=5e-4, beta_mean=0.25, seed=5)
    out = {"n_genes": G, "n_cells": Cn, "chains": chains, "steps": steps,
           "warm_up_steps": warm, "early_steps": early}

    def timed(run, last_ms):
        flush.zero_()
        torch.cuda.synchronize()
        run(steps)
        return chains * steps / (last_ms() / 1e3)

    with N.Batch([(mut, known, Cn, G)], adj) as bt:
        bt.init_chains(chains)
        bt.run(early)
        bt.autotune(max(8, steps // 4))
        out["batched_adjoint_after_early_steps"] = timed(bt.run,
                                                         bt.last_run_ms)
        bt.run(warm - early - steps)
        out["batched_adjoint_chain_steps_per_s"] = timed(bt.run,
                                                         bt.last_run_ms)
        out["batched_launch"] = list(bt.launch()) + [bt.chain_warps()]
    with N.Context(mut, known, Cn, G, plain) as c:
        c.init_chains(chains)
        c.run(early)
        c.autotune(max(8, steps // 4))
        out["plain_after_early_steps"] = timed(c.run, c.last_run_ms)
        c.run(warm - early - steps)
        out["plain_chain_steps_per_s"] = timed(c.run, c.last_run_ms)
        out["plain_launch"] = list(c.launch())
    out["batched_over_plain"] = (out["batched_adjoint_chain_steps_per_s"]
                                 / out["plain_chain_steps_per_s"])
    popc = popc_per_chain_step(G, Cn)
    peak, clk_hz = N.popc_peak()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    issue_peak = 4.0 * sms * clk_hz
    inst_b = _profile_figure("batch", "warp_instructions_per_chain_step",
                             CAPS_PROFILE)
    inst_p = _profile_figure("plain", "warp_instructions_per_chain_step",
                             CAPS_PROFILE)

    def issue_frac(r, inst):
        return None if inst is None else r * inst / issue_peak

    out["roofline"] = {
        "bound": "issue", "unit": "G warp-instructions/s",
        "peak": issue_peak / 1e9,
        "batched_adjoint_frac": issue_frac(
            out["batched_adjoint_chain_steps_per_s"], inst_b),
        "plain_frac": issue_frac(out["plain_chain_steps_per_s"], inst_p),
        "batched_adjoint_work_per_chain_step": inst_b,
        "plain_work_per_chain_step": inst_p,
        "work_source": f"smsp__inst_executed.sum per chain-step of the "
                       f"captured launch shapes, profiles/{CAPS_PROFILE}"}
    # POPC-equivalent work (the masked-popcount formulation's count; the
    # ring path issues none of these POPC)
    out["popc_per_chain_step"] = popc
    out["batched_adjoint_popc_equivalent_frac"] = \
        out["batched_adjoint_chain_steps_per_s"] * popc / peak
    out["plain_popc_equivalent_frac"] = \
        out["plain_chain_steps_per_s"] * popc / peak
    return out


def caps_profile(form: str, chains: int = 4096) -> None:
    """The 255x512 case of run_beyond_caps for an ncu capture: one form at
    a fixed launch shape, a 20,000-step launch (the timed regime), then the
    100-step launch to capture."""
    from bbscite_gb300 import data as D
    from bbscite_gb300 import native as N
    G, Cn = 255, 512
    m, _, _ = D.generate_dataset(5255, G, Cn, 5e-4, 0.25, 0.08, 0.01)
    mut, known = D.matrix_to_bits(m)
    steps = 100
    if form == "batch":
        p = N.default_params(alpha_mean=5e-4, beta_mean=0.25, seed=5,
                             prob_beta_change=0.1, score_mode=N.SCORE_SUM,
                             error_move=N.ERROR_LANGEVIN)
        with N.Batch([(mut, known, Cn, G)], p) as bt:
            bt.init_chains(chains)
            bt.set_launch(2, 2, 1)
            bt.set_chain_warps(2)
            bt.run(20000)
            bt.run(steps)
            rate = chains * steps / (bt.last_run_ms() / 1e3)
    else:
        p = N.default_params(alpha_mean=5e-4, beta_mean=0.25, seed=5)
        with N.Context(mut, known, Cn, G, p) as c:
            c.init_chains(chains)
            c.set_launch(2, 4, 1)
            c.run(20000)
            c.run(steps)
            rate = chains * steps / (c.last_run_ms() / 1e3)
    print(json.dumps({"caps_profile": form, "chain_steps_per_s": rate}))


def own_gpu(local: int) -> str:
    """Makes this rank's GPU the only visible one, before any CUDA call, so
    that torch and the library (which links its own CUDA runtime) both use
    it as device 0.  Returns the GPU's index for nvidia-smi."""
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    ids = [v for v in vis.split(",") if v.strip()] if vis else []
    gpu = ids[local] if local < len(ids) else str(local)
    os.environ["CUDA_VISIBLE_DEVICES"] = gpu
    return gpu


def run_ours(args) -> None:
    ws, rank, local = dist_info()
    gpu = own_gpu(local) if ws > 1 else str(local)

    import numpy as np
    import torch

    from bbscite_gb300 import native as N

    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(0 if ws > 1 else local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    w = WORKLOAD
    G, Cn, chains, L = w["n_genes"], w["n_cells"], args.chains, \
        args.chain_steps
    _, mut, known = make_dataset()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device="cuda")
    # batched+adjoint: sum score, Langevin error move learning (alpha,
    # beta) from the wrong start 1e-2 / 0.3, error-move probability 0.1
    adj = N.default_params(alpha_mean=1e-2, beta_mean=0.3,
                           seed=0xB5C17E + rank, prob_beta_change=0.1,
                           score_mode=N.SCORE_SUM,
                           error_move=N.ERROR_LANGEVIN)
    # plain: the reference's max score, fixed rates at the generator's
    plain = N.default_params(alpha_mean=w["alpha"], beta_mean=w["beta"],
                             seed=0xB5C17E + rank)

    bt = N.Batch([(mut, known, Cn, G)], adj)
    bt.init_chains(chains)
    if args.batch_launch:
        v = [int(x) for x in args.batch_launch.split(",")]
        bt.set_launch(*v[:3])
        if len(v) > 3:
            bt.set_chain_warps(v[3])
    ctx = N.Context(mut, known, Cn, G, plain)
    ctx.init_chains(chains)
    if args.launch:
        ctx.set_launch(*[int(x) for x in args.launch.split(",")])

    done = 0
    while done < args.quality_steps:
        k = min(L, args.quality_steps - done)
        bt.run(k)
        ctx.run(k)
        done += k
    # launch shapes tuned on the warmed-up chains, the regime timed (the
    # tuners restore the chains' states; every shape computes the same
    # chains)
    if args.autotune and not args.batch_launch:
        bt.autotune(args.autotune_steps)
    if args.autotune and not args.launch:
        ctx.autotune(args.autotune_steps)
    bshape = bt.launch() + (bt.chain_warps(),)
    pshape = ctx.launch()
    for _ in range(args.warmup):
        bt.run(L)
        ctx.run(L)
    clocks = ClockSampler(gpu)
    clocks.start()
    adj_ms, adj_wall, adj_list = _timed(lambda: bt.run(L), bt.last_run_ms,
                                        args.steps, flush, barrier, torch)
    pl_ms, pl_wall, pl_list = _timed(lambda: ctx.run(L), ctx.last_run_ms,
                                     args.steps, flush, barrier, torch)
    clk = clocks.stop()
    adj_ms, adj_wall, pl_ms, pl_wall = max_over_ranks(
        dist, [adj_ms, adj_wall, pl_ms, pl_wall], "cuda")
    steps_total = ws * chains * L * args.steps
    value = steps_total / (adj_ms / 1e3)
    plain_value = steps_total / (pl_ms / 1e3)

    # equal best logL: both best trees under the reference's max score at
    # the generator's rates (alpha=1e-3, beta=0.2)
    ab = bt.best(0)
    pb = ctx.best()
    s_adj, _, _ = ctx.score_trees(ab["dm"][None], w["beta"])
    s_pl, _, _ = ctx.score_trees(pb["dm"][None], w["beta"])
    bt.close()
    ctx.close()
    # replicas share the dataset and differ in their seeds: best over ranks
    s_adj = [global_best(dist, s_adj[0], rank, ws, "cuda")[0]]
    s_pl = [global_best(dist, s_pl[0], rank, ws, "cuda")[0]]

    # roofline of the headline kernel.  The binding resource is the issue
    # slot: four warp instructions per clock per SM, against the profiled
    # instructions per chain-step of the benched kernel (ncu).  The POPC
    # count of the masked-popcount formulation is kept as equivalent work.
    rate = chains * L / (statistics.mean(adj_list) / 1e3)
    plain_rate = chains * L / (statistics.mean(pl_list) / 1e3)
    popc_step = popc_per_chain_step(G, Cn)
    popc_peak, clk_hz = N.popc_peak()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    issue_peak = 4.0 * sms * clk_hz
    inst_step = _profile_figure("batch", "warp_instructions_per_chain_step")
    inst_plain = _profile_figure("plain", "warp_instructions_per_chain_step")
    dram = _profile_figure("batch", "dram_bytes_per_chain_per_launch")

    def issue_frac(r, inst):
        return None if inst is None else r * inst / issue_peak

    roofline = {
        "bound": "issue",
        "achieved": None if inst_step is None else rate * inst_step / 1e9,
        "peak": issue_peak / 1e9, "unit": "G warp-instructions/s",
        "frac": issue_frac(rate, inst_step),
        "traffic": (dram * chains) if dram is not None else None,
        "traffic_unit": "DRAM bytes per launch (ncu dram__bytes_read.sum + "
                        f"dram__bytes_write.sum, profiles/{PROFILE})",
        "peak_source": f"4 warp instructions per clock per SM x {sms} SMs "
                       f"at the SM clock measured live ({clk_hz / 1e6:.0f} "
                       "MHz, bbs_popc_peak)",
        "work_per_chain_step": f"{inst_step} warp instructions "
                               "(smsp__inst_executed.sum of the benched "
                               f"kernel per chain-step, profiles/{PROFILE})",
        "plain_frac": issue_frac(plain_rate, inst_plain),
        "plain_work_per_chain_step": inst_plain,
        "equivalent_work": {
            "unit": "G POPC/s", "achieved": rate * popc_step / 1e9,
            "peak": popc_peak / 1e9, "frac": rate * popc_step / popc_peak,
            "plain_frac": plain_rate * popc_step / popc_peak,
            "per_chain_step": popc_step,
            "note": "32-bit POPC of the masked-popcount formulation "
                    "(cells x nodes x 2 x ceil(genes/32)); the benched "
                    "kernels inherit counts and issue none of them in the "
                    "node loop, so this is work done, not a pipe's use"},
    }

    # end to end through the C ABI with host buffers (batched+adjoint)
    e2e_times = []
    for _ in range(args.e2e_steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        b2 = N.Batch([(mut, known, Cn, G)], adj)
        b2.init_chains(chains)
        b2.set_launch(*bshape[:3])
        b2.set_chain_warps(bshape[3])
        b2.run(L)
        b2.best(0)
        b2.close()
        e2e_times.append(time.perf_counter() - t)
    W64 = N.words(G + 1)
    # the cell rows go up; the initial trees are drawn on the device
    h2d = mut.nbytes + known.nbytes
    d2h = 128 * chains + (G + 1) * W64 * 8
    e2e_value = ws * chains * L / statistics.mean(e2e_times)

    mix = lvr = caps = None
    if rank == 0 and args.mix_datasets > 0:
        mix = run_mix(N, args.mix_datasets, 32, args.mix_steps, flush, torch,
                      args.mix_tuned_steps)
    if rank == 0 and args.lvr_steps > 0:
        lvr = run_langevin_vs_rw(N, mut, known, G, Cn, args.lvr_chains,
                                 args.lvr_steps, args.lvr_seeds,
                                 args.lvr_error_step, w["alpha"], w["beta"])
    if rank == 0 and args.caps_steps > 0:
        caps = run_beyond_caps(N, args.caps_chains, args.caps_steps, flush,
                               torch)

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": adj_wall * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "u32-popcount+f32",
        "data": "synthetic (seeded generator, verification/lib.py semantics)",
        "form": "batched+adjoint: work-list launch, sum-over-attachments "
                "score with its fused adjoint, Langevin error-rate move",
        "config": {
            "workload": f"{G} genes x {Cn} cells, {chains} chains; data "
                        "alpha=1e-3 beta=0.2 (10% unknown, 2% homozygous); "
                        "chains learn alpha, beta from 1e-2, 0.3 (error move "
                        "probability 0.1)",
            "n_genes": G, "n_cells": Cn, "chains": chains,
            "chain_steps_per_launch": L, "parallelism": f"replicas x{ws}",
            "launch": {"cells_per_lane": bshape[0],
                       "warps_per_block": bshape[1],
                       "warps_per_chain": bshape[3],
                       "autotuned": bool(args.autotune) and not args.batch_launch},
            "l2": "256 MiB buffer written between launches",
        },
        "plain": {
            "value": plain_value, "unit": UNIT,
            "form": "one-dataset persistent kernel, reference max score, "
                    "fixed alpha=1e-3 beta=0.2",
            "launch": {"cells_per_lane": pshape[0],
                       "warps_per_chain": pshape[1],
                       "chains_per_block": pshape[2]},
            "ms_per_step": pl_wall * 1e3 / args.steps,
        },
        "equal_best_logl": {
            "scored_with": "reference max score at alpha=1e-3 beta=0.2",
            "steps_per_chain": args.quality_steps
            + (args.warmup + args.steps) * L,
            "batched_adjoint": float(s_adj[0]), "plain": float(s_pl[0]),
            "difference": float(s_adj[0] - s_pl[0]),
            "within_0.1_nats": bool(s_adj[0] >= s_pl[0] - 0.1),
            "learned_alpha": ab["alpha"], "learned_beta": ab["beta"],
        },
        "roofline": roofline,
        "counted_tbit_per_s": value * counted_bits_per_chain_step(G, Cn)
        / 1e12,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": 2 * args.steps,
        "clocks": clk,
    }
    if lvr is not None:
        out["langevin_vs_random_walk"] = lvr
    if caps is not None:
        out["beyond_caps_255x512"] = caps
    if mix is not None:
        out["batched_mix"] = mix
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        b = cpu_baseline(args.cpu_seconds)
        cpu = b["value"]
        out["cpu_baseline"] = {k: b[k] for k in
                               ("value", "unit", "cores", "kind", "sample")}
        out["cpu_baseline"]["pinned"] = PORT_PINNING
        out["cpu_baseline"]["scoring_proxy"] = cpu_scoring_proxy_rate(
            min(5.0, args.cpu_seconds))
        # like for like: the plain form runs the reference's max score at
        # fixed rates, as the CPU port does; the headline form also learns
        # the rates with the sum score (a cross-form comparison)
        out["vs_cpu"] = {
            "plain_over_cpu": plain_value / cpu,
            "plain_e2e_basis": "device time",
            "batched_adjoint_over_cpu_cross_form": value / cpu,
            "batched_adjoint_e2e_over_cpu_cross_form": e2e_value / cpu,
        }
    # the key figures once more, last, where a tail of the line keeps them
    out["summary"] = {
        "batched_adjoint": value, "plain": plain_value,
        "e2e": e2e_value, "issue_frac": roofline["frac"],
        "plain_issue_frac": roofline["plain_frac"],
        "plain_over_cpu": plain_value / cpu if cpu else None,
        "mix_speedup": mix["speedup"] if mix else None,
        "mix_steps": mix["steps"] if mix else None,
        "langevin_half_met": lvr["target_half_met"] if lvr else None,
        "caps_batched_adjoint":
            caps["batched_adjoint_chain_steps_per_s"] if caps else None,
        "caps_plain": caps["plain_chain_steps_per_s"] if caps else None,
        "caps_batched_over_plain": caps["batched_over_plain"] if caps else None,
        "caps_batched_issue_frac":
            caps["roofline"]["batched_adjoint_frac"] if caps else None,
        "caps_plain_issue_frac":
            caps["roofline"]["plain_frac"] if caps else None,
    }
    if rank == 0:
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main(argv=None) -> None:
    args = parse_args(argv)
    if args.impl == "reference":
        run_reference(args)
    elif args.caps_profile:
        caps_profile(args.caps_profile, args.caps_chains)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
