#!/usr/bin/env python3
"""Chain-steps/s of the bbSCITE MCMC step path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Workload (the headline configuration): 95 genes x 96 cells from the seeded
generator (alpha=1e-3, beta=0.2, 10% unknown, 2% of true mutations
recorded as homozygous), 1024 chains, fixed error rates, Philox moves,
max-over-attachments score.  One bench step = one persistent launch that
advances every chain by --chain-steps steps; chains continue across
launches.  Inputs are resident in HBM before the timed region; a 256 MiB
buffer is written between launches to flush L2.

Prints one JSON line (rank 0).  `value` is device-timed (CUDA events on the
library's stream around each launch), `e2e` the same metric through the C
ABI with host buffers (context creation, host->device copies, the run and
the device->host read of the best tree inside the timed region).

--impl reference runs the reference's CPU implementation of the path
(the C restatement in oracle/, threaded over chains) on the same workload.
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
    ap.add_argument("--autotune", type=int, default=1)
    ap.add_argument("--autotune-steps", type=int, default=200)
    ap.add_argument("--launch", default="",
                    help="cells_per_lane,warps_per_chain,chains_per_block")
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
            "kind": "port",
            "sample": f"{n_chains} chains x {steps} steps of the 95x96 "
                      f"workload ({dt:.1f} s), oracle/bbs_oracle.c "
                      "orc_run_chains_mt, reference cell-order score",
            "best_logl": best}


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
                   "cells, plain MCMC, fixed error rates",
                   "parallelism": "host threads over chains"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": info["cores"],
                         "kind": info["kind"], "sample": info["sample"]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "best_logl": info["best_logl"],
    }
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------------ ours --

def _traffic_from_profile():
    """DRAM bytes per launch of the chain kernel from the committed ncu
    summary (profiles/mcmc_95x96_dram.json), or None."""
    p = os.path.join(ROOT, "profiles", "mcmc_95x96_dram.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return d.get("dram_bytes_per_chain_per_launch")


def run_ours(args) -> None:
    import numpy as np
    import torch

    from bbscite_gb300 import native as N

    ws, rank, local = dist_info()
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(local)
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
    _, mut, known = make_dataset(rank)
    params = N.default_params(alpha_mean=w["alpha"], beta_mean=w["beta"],
                              seed=0xB5C17E + rank)
    ctx = N.Context(mut, known, Cn, G, params)
    ctx.init_chains(chains)
    # launch shape from the autotuner (chain state is restored afterwards)
    if args.launch:
        ctx.set_launch(*[int(x) for x in args.launch.split(",")])
    elif args.autotune:
        ctx.autotune(args.autotune_steps)
    shape = ctx.launch()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device="cuda")

    for _ in range(args.warmup):
        ctx.run(L)
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    kernel_ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        ctx.run(L)
        kernel_ms.append(ctx.last_run_ms())
    torch.cuda.synchronize()
    barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    dev_s = sum(kernel_ms) / 1e3
    if dist is not None:
        t = torch.tensor([dev_s, wall], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_s, wall = float(t[0]), float(t[1])
    total_steps = ws * chains * L * args.steps
    value = total_steps / dev_s
    best = ctx.best()
    ctx.close()

    # roofline of the chain kernel (integer pipe: POPC)
    popc_step = popc_per_chain_step(G, Cn)
    launch_s = statistics.mean(kernel_ms) / 1e3
    achieved = popc_step * chains * L / launch_s
    peak, clk_hz = N.popc_peak()
    traffic = _traffic_from_profile()

    # end to end through the C ABI with host buffers
    e2e_times = []
    h2d = d2h = 0
    for _ in range(args.e2e_steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        c2 = N.Context(mut, known, Cn, G, params)
        parents = N.random_parents(params.seed, G, chains)
        c2.init_chains(chains, parents)
        c2.set_launch(*shape)
        c2.run(L)
        b2 = c2.best()
        c2.close()
        e2e_times.append(time.perf_counter() - t)
        h2d = mut.nbytes + known.nbytes + chains * (G + 1) * N.words(G + 1) * 8
        d2h = chains * 64 + (G + 1) * N.words(G + 1) * 8
        del b2
    e2e_value = ws * chains * L / statistics.mean(e2e_times)

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": wall * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32-popcount+f32",
        "data": "synthetic (seeded generator, verification/lib.py semantics)",
        "form": "plain persistent chain kernel (one warp per chain)",
        "config": {
            "workload": f"{G} genes x {Cn} cells, {chains} chains, plain MCMC,"
                        " fixed error rates alpha=1e-3 beta=0.2, Philox moves",
            "n_genes": G, "n_cells": Cn, "chains": chains,
            "chain_steps_per_launch": L, "parallelism": f"replicas x{ws}",
            "launch": {"cells_per_lane": shape[0],
                       "warps_per_chain": shape[1],
                       "chains_per_block": shape[2],
                       "autotuned": bool(args.autotune)},
            "l2": "256 MiB buffer written between launches",
        },
        "roofline": {
            "bound": "int (POPC pipe)", "achieved": achieved / 1e9,
            "peak": peak / 1e9, "unit": "Gop/s",
            "frac": achieved / peak,
            "traffic": (traffic * chains) if traffic is not None else None,
            "traffic_unit": "bytes per launch (ncu dram read+write, "
                            "profiles/mcmc_95x96_dram.json)",
            "peak_source": "bbs_popc_peak microbenchmark on this GPU "
                           f"(SM clock {clk_hz / 1e6:.0f} MHz)",
            "work_per_chain_step": f"{popc_step} POPC (32-bit)",
        },
        "counted_tbit_per_s": value * counted_bits_per_chain_step(G, Cn)
        / 1e12,
        "best_logl": best["score"],
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": args.steps,
        "clocks": clk,
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        b = cpu_baseline(args.cpu_seconds)
        out["cpu_baseline"] = {k: b[k] for k in
                               ("value", "unit", "cores", "kind", "sample")}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main(argv=None) -> None:
    args = parse_args(argv)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
