"""bench.py's reference arm on the host (no GPU): one JSON line with the
keys the benchmark contract names, on the same metric and workload as the
GPU arm, and the helpers that turn a rate into roofline figures."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_reference_arm_prints_one_contract_line():
    import bench
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"),
                        "--impl", "reference", "--steps", "1", "--warmup",
                        "0", "--cpu-seconds", "1"], cwd=ROOT,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["higher_is_better"] is True
    assert (d["n_gpus"], d["steps"], d["warmup"]) == (1, 1, 0)
    assert d["value"] > 0
    w = bench.WORKLOAD
    # the workload of the GPU arm; the chains named are those timed
    assert (d["config"]["n_genes"], d["config"]["n_cells"],
            d["config"]["workload_chains"]) == (w["n_genes"], w["n_cells"],
                                                w["chains"])
    assert 1 <= d["config"]["chains"] <= w["chains"]
    assert f"{d['config']['chains']} chains" in d["cpu_baseline"]["sample"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"],
                        "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_work_per_chain_step():
    import bench
    # two masked popcounts per (cell, node) pair over ceil(G/32) words
    assert bench.popc_per_chain_step(95, 96) == 96 * 96 * 2 * 3 == 55296
    assert bench.popc_per_chain_step(63, 64) == 16384
    assert bench.popc_per_chain_step(255, 512) == 2097152
    # the paper's counted bits, 4 * cells * nodes^2
    assert bench.counted_bits_per_chain_step(95, 96) == 4 * 96 * 96 ** 2


def test_profile_figures_the_bench_reads():
    """The committed ncu summaries give the warp instructions per chain-step
    that turn each timed rate into an issue-slot fraction: the 95 x 96
    kernels of the headline and the 255 x 512 kernels (the shapes and the
    regime the bench times)."""
    import bench
    for form in ("batch", "plain"):
        for prof in (bench.PROFILE, bench.CAPS_PROFILE):
            w = bench._profile_figure(form, "warp_instructions", prof)
            cs = bench._profile_figure(form, "chain_steps", prof)
            per = bench._profile_figure(form,
                                        "warp_instructions_per_chain_step",
                                        prof)
            assert isinstance(per, int) and per > 0, (form, prof)
            assert abs(w / cs - per) <= 1, (form, prof)
    # 95 x 96: 1024 chains x 2000 steps; 255 x 512: 4096 chains x 100 steps
    assert bench._profile_figure("batch", "chain_steps") == 1024 * 2000
    assert bench._profile_figure("batch", "chain_steps",
                                 bench.CAPS_PROFILE) == 4096 * 100
