"""The co-optimal tree list (SCITE's -max_treelist_size, parsed but unused
by the reference at src/Parameters.hpp:223-231): on data where genes
without known entries make many trees score alike, the list holds
distinct trees that all score exactly the best score, the best first;
keeping it does not change the chains; the CLI writes one _ml<i> set per
tree."""
import subprocess

import numpy as np
import pytest

from bbscite_gb300 import data as D

pytestmark = pytest.mark.gpu


def tied_dataset():
    m, _, _ = D.generate_dataset(91, 12, 30, 1e-3, 0.2, 0.0, 0.0)
    m[3, :] = 3   # genes with no known entry: their placement never
    m[7, :] = 3   # changes a score
    return m


def run(native, m, k, steps=20000):
    mut, known = D.matrix_to_bits(m)
    G, Cn = m.shape
    p = native.default_params(alpha_mean=1e-3, beta_mean=0.2, seed=12,
                              treelist_size=k)
    c = native.Context(mut, known, Cn, G, p)
    c.init_chains(32)
    c.run(steps)
    return c


def test_treelist_collects_distinct_ties(native, orc):
    m = tied_dataset()
    with run(native, m, 16) as c:
        tl = c.treelist(64)
        best = c.best()
        scores, _, _ = c.score_trees(tl["dm"], tl["betas"])
    k = len(tl["dm"])
    assert k >= 2
    assert (tl["dm"][0] == best["dm"]).all()
    assert tl["score"] == best["score"]
    for i in range(k):
        for j in range(i):
            assert not (tl["dm"][i] == tl["dm"][j]).all()
    assert (scores == np.float32(best["score"])).all()


def test_treelist_does_not_change_the_chains(native):
    m = tied_dataset()
    with run(native, m, 1, 5000) as a, run(native, m, 16, 5000) as b:
        sa, sb = a.chains(), b.chains()
        for key in ("dm", "beta", "score", "counts"):
            assert (sa[key] == sb[key]).all(), key
        ba, bb = a.best(), b.best()
        assert ba["score"] == bb["score"] and (ba["dm"] == bb["dm"]).all()
        # with one tree per chain the list holds the chains' own bests
        # that reach the top score, at most one per chain
        ta, tb = a.treelist(64), b.treelist(64)
        assert 1 <= len(ta["dm"]) <= 32 and (ta["dm"][0] == ba["dm"]).all()
        assert len(tb["dm"]) >= len(ta["dm"])


def test_cli_writes_the_tree_list(native, tmp_path):
    from bbscite_gb300 import build as B
    D.write_csv(tied_dataset(), str(tmp_path / "t.csv"))
    r = subprocess.run([B.CLI, "-i", "t.csv", "-r", "32", "-l", "20000",
                        "-fd", "0.001", "-ad", "0.2", "-seed", "12",
                        "-max_treelist_size", "5"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    files = sorted(p.name for p in tmp_path.glob("t_ml*.newick"))
    assert files[0] == "t_ml0.newick" and 2 <= len(files) <= 5
    texts = [(tmp_path / f).read_text() for f in files]
    assert len(set(texts)) == len(texts)
