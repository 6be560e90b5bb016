"""The CLI and the C++ wrappers on the GPU: the five output files of
src/main.cpp:171-214 in the reference's formats, identical to the best
tree of the same run through the Python binding; the MutationTree update
constructor on the reference's move known answers (test/MutationTree.cpp:
410-611); realize_raw_move_sample against the oracle; TreeScorer on the
reference's scoring known answer (test/TreeScorer.cpp:33-93)."""
import os
import subprocess

import numpy as np
import pytest

from bbscite_gb300 import data as D

pytestmark = pytest.mark.gpu


def test_cli_outputs_match_api(native, tmp_path):
    from bbscite_gb300 import build as B
    G, Cn = 24, 40
    m, _, _ = D.generate_dataset(77, G, Cn, 1e-3, 0.25, 0.05, 0.0)
    D.write_csv(m, str(tmp_path / "data.csv"))
    r = subprocess.run([B.CLI, "-i", "data.csv", "-r", "16", "-l", "3000",
                        "-fd", "0.001", "-ad", "0.25", "-seed", "9"],
                       cwd=tmp_path, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    assert lines[0].startswith("Move generation makespan: ")
    assert lines[1].startswith("Time elapsed: ") and lines[1].endswith(" ms")
    base = tmp_path / "data"
    am_txt = (tmp_path / "data_ml0_am.txt").read_text().splitlines()
    dm_txt = (tmp_path / "data_ml0_dm.txt").read_text().splitlines()
    n = G + 1
    assert len(am_txt) == n and all(len(x) == n for x in am_txt)
    am = np.array([[c == "1" for c in row] for row in am_txt])
    dm = np.array([[c == "1" for c in row] for row in dm_txt])
    assert (am == dm.T).all()

    mut, known = D.matrix_to_bits(m)
    p = native.default_params(alpha_mean=1e-3, beta_mean=0.25, seed=9)
    with native.Context(mut, known, Cn, G, p) as c:
        c.init_chains(16)
        c.run(3000)
        best = c.best()
    for x in range(n):
        for y in range(n):
            assert am[x, y] == bool((int(best["am"][x, y // 64]) >> (y % 64)) & 1)
    gv = (tmp_path / "data_ml0.gv").read_text()
    nw = (tmp_path / "data_ml0.newick").read_text()
    assert gv == native.to_graphviz(best["parent"])
    assert nw == native.to_newick(best["parent"])
    beta_txt = (tmp_path / "data_ml0_beta.txt").read_text()
    assert beta_txt.endswith("\n")
    assert np.float32(float(beta_txt)) == pytest.approx(best["beta"], rel=1e-5)
    assert str(base)  # output base is the input path without its suffix


def test_cpp_update_constructor_kats(probe, kat):
    mv = kat["moves"]
    lines = []
    for case in mv["cases"]:
        p = case["params"]
        lines.append(f"tree {mv['beta']} " + " ".join(map(str, case["start"])))
        lines.append("update {move_type} {v} {w} {parent_of_v} {parent_of_w} "
                     "{descendant_of_v} {nondescendant_of_v} {new_beta}"
                     .format(**p))
    out, _ = probe(lines)
    for i, case in enumerate(mv["cases"]):
        parts = dict(p.strip().split(" ", 1) for p in out[2 * i + 1].split(" | "))
        assert [int(x) for x in parts["parent"].split()] == case["expected"], \
            case["name"]


def test_cpp_realize_vs_oracle(probe, orc):
    rng = np.random.default_rng(8)
    lines, cases = [], []
    for G in (5, 40, 130):
        pv = D.random_parent_vector(rng, G)
        lines.append("tree 0.3 " + " ".join(map(str, pv)))
        for _ in range(20):
            t = int(rng.integers(0, 4))
            v, w = rng.integers(0, G), rng.integers(0, G - 1)
            ud, un, j = rng.random(), rng.random(), rng.normal() * 0.01
            lines.append(f"realize {t} {v} {w} {ud:.9g} {un:.9g} {j:.9g}")
            cases.append((pv, t, v, w, ud, un, j))
    out, _ = probe(lines)
    got = [l for l in out if not l.startswith("parent")]
    for (pv, t, v, w, ud, un, j), line in zip(cases, got):
        am, dm = orc.parent_to_matrix(pv)
        raw = np.zeros(1, dtype=orc.RAW_MOVE)
        raw["move_type"], raw["raw_v"], raw["raw_w"] = t, v, w
        raw["raw_descendant_of_v"] = np.float32(float(f"{ud:.9g}"))
        raw["raw_nondescendant_of_v"] = np.float32(float(f"{un:.9g}"))
        raw["beta_jump"] = np.float32(float(f"{j:.9g}"))
        ref = orc.realize(am, dm, np.float32(0.3), raw[0])
        vals = line.split()
        assert [int(x) for x in vals[:7]] == [int(ref[k]) for k in (
            "move_type", "v", "w", "parent_of_v", "parent_of_w",
            "descendant_of_v", "nondescendant_of_v")]
        assert np.float32(vals[7]) == ref["new_beta"]


def test_cpp_tree_scorer_kat(probe, kat, orc):
    k = kat["tree_scorer"]
    mut = [int(s, 2) for s in k["is_mutated"]]
    known = [int(s, 2) for s in k["is_known"]]
    lines = [f"scorer {k['alpha']} {k['beta']} {k['prior_sd']} {k['n_cells']} "
             f"{k['n_genes']} " + " ".join(map(str, mut + known)),
             f"tree {k['beta']} " + " ".join(map(str, k["parent_vector"])),
             "score", f"prior {k['beta']}"]
    out, _ = probe(lines)
    score, prior = float(out[2]), float(out[3])
    want_prior = orc.logscore_beta(k["alpha"], k["beta"], k["prior_sd"],
                                   k["beta"])
    assert np.float32(prior) == np.float32(want_prior)
    import math
    t, a, b = k["expected_terms"], k["alpha"], k["beta"]
    want = (t["log(1-alpha)"] * math.log(1 - a) + t["log(1-beta)"]
            * math.log(1 - b) + t["log(beta)"] * math.log(b)
            + t["log(alpha)"] * math.log(a) + want_prior)
    assert score == pytest.approx(want, rel=k["catch_approx_rel"])


def test_cpp_application_checkpoint(probe):
    """Application::save_chains / load_chains: a run of 300 + 200 steps
    split by a checkpoint into a second Application ends where one run of
    500 steps does."""
    G, Cn = 20, 30
    m, _, _ = D.generate_dataset(11, G, Cn, 1e-3, 0.2, 0.1, 0.02)
    mut, known = D.matrix_to_bits(m)
    words = " ".join(str(int(w)) for w in list(mut.ravel()) +
                     list(known.ravel()))
    out, _ = probe([f"resume {Cn} {G} 300 200 {words} -i in.csv -r 4 "
                    "-fd 0.001 -ad 0.2 -e 0.1 -seed 9"])
    f = out[0].split()
    assert f[0] == "whole" and f[2] == "resumed"
    assert float(f[1]) == float(f[3])
    assert f[5] == "1"


def test_cli_application_kat(native, orc, kat, tmp_path):
    """The reference's end-to-end test (test/Application.cpp:38-143)
    through the command line: the tree in _ml0 scores like the true tree
    under the reference's scorer."""
    from bbscite_gb300 import build as B
    k = kat["application"]
    G, Cn = k["n_genes"], k["n_cells"]
    m = np.array([[(int(k["is_mutated"][c], 2) >> g) & 1 for c in range(Cn)]
                  for g in range(G)], dtype=np.int8)
    D.write_csv(m, str(tmp_path / "app.csv"))
    r = subprocess.run([B.CLI, "-i", "app.csv", "-r", str(k["n_chains"]),
                        "-l", str(k["chain_length"]), "-fd", str(k["alpha"]),
                        "-ad", str(k["beta"]), "-sd", str(k["beta_sd"]),
                        "-seed", "1"], cwd=tmp_path, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    from bbscite_gb300.verification import lib as L
    found = L.parse_newick((tmp_path / "app_ml0.newick").read_text())
    mut, known = D.matrix_to_bits(m)
    _, dm_found = orc.parent_to_matrix(found)
    _, dm_true = orc.parent_to_matrix(np.array(k["true_parent_vector"]))
    s_found = orc.logscore_tree(k["alpha"], k["beta"], k["beta_sd"], dm_found,
                                mut, known, k["beta"])[0]
    s_true = orc.logscore_tree(k["alpha"], k["beta"], k["beta_sd"], dm_true,
                               mut, known, k["beta"])[0]
    assert s_found == pytest.approx(s_true, rel=1.2e-5)
