"""Search quality against the reference: on 64 seeded 63-gene x 64-cell
datasets (8 chains x 100,000 steps each), the best trees this path finds,
scored with the reference's own cell-order score, are no worse than the
best the reference's classes found with their own samplers and URNG
(tests/golden/quality_ref.json, made by tests/golden/make_quality_ref.py):
the one-sided test of the reference's verification tool (mean difference
above minus one bit flip, 95 %) rejects inferiority, and without that
margin the data show no shortfall either -- the upper 95 % confidence
bound of the mean difference is at least zero and a sign test over the
seeds finds no side better at the 5 % level.  Also the `score` command of
the verification harness."""
import json
import os

import numpy as np
import pytest

from bbscite_gb300 import data as D
from bbscite_gb300.verification import lib as L

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_best_found_no_worse_than_reference(native, orc):
    with open(os.path.join(HERE, "golden", "quality_ref.json")) as f:
        fx = json.load(f)
    w = fx["workload"]
    diffs = []
    for row in fx["results"]:
        m, _, _ = D.generate_dataset(row["dataset_seed"], w["n_genes"],
                                     w["n_cells"], w["alpha"], w["beta"],
                                     w["missing"], w["homozygous"])
        mut, known = D.matrix_to_bits(m)
        p = native.default_params(alpha_mean=w["alpha"], beta_mean=w["beta"],
                                  beta_sd=w["beta_sd"],
                                  seed=row["dataset_seed"])
        with native.Context(mut, known, w["n_cells"], w["n_genes"], p) as c:
            c.init_chains(w["chains"])
            c.run(w["steps"])
            best = c.best()
        ref_order, _, _, _ = orc.logscore_tree(
            w["alpha"], w["beta"], w["beta_sd"], best["dm"], mut, known,
            best["beta"])
        diffs.append(float(ref_order) - row["best_score"])
    from scipy.stats import binomtest, t as student_t
    r = L.tost(diffs, w["alpha"], w["beta"], n_bits=1)
    d = np.asarray(diffs)
    upper = d.mean() + student_t.ppf(0.95, len(d) - 1) * d.std(ddof=1) / \
        np.sqrt(len(d))
    n_side = r["better"] + r["worse"]
    sign_p = binomtest(r["better"], n_side, 0.5).pvalue if n_side else 1.0
    print(f"\nbest-found differences (ours - reference) over "
          f"{len(diffs)} seeds: {r}; upper 95% bound of the mean "
          f"{upper:.3f}; sign test p {sign_p:.3f}")
    assert r["non_inferior"], r
    assert upper >= 0.0, (upper, r)
    assert sign_p > 0.05 or r["better"] > r["worse"], (sign_p, r)


def test_score_command(native, orc, tmp_path, capsys):
    from bbscite_gb300.verification.__main__ import main as vmain
    G, Cn, a, b = 40, 60, 1e-3, 0.25
    m, parent, _ = D.generate_dataset(8, G, Cn, a, b, 0.05, 0.0)
    D.write_csv(m, str(tmp_path / "m.csv"))
    (tmp_path / "t.newick").write_text(native.to_newick(parent))
    assert vmain(["score", "-a", str(a), "-b", str(b), "-t",
                  str(tmp_path / "t.newick"), "-m", str(tmp_path / "m.csv"),
                  "-x", "-o", str(tmp_path / "truth.csv")]) == 0
    ll = float(capsys.readouterr().out.strip())
    mut, known = D.matrix_to_bits(m)
    _, dm = orc.parent_to_matrix(parent)
    want = orc.logscore_tree_f64(np.float32(a), np.float32(b), dm, mut, known,
                                 b, 0.1, False)
    assert ll == pytest.approx(want, rel=1e-6)
    assert D.read_csv(str(tmp_path / "truth.csv")).shape == m.shape
