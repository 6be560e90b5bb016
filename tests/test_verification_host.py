"""The verification harness on the host: Newick parsing, the likelihood at
given attachments, the equivalence test, and the generate / tost commands
of the reference's verification tool."""
import math
import os

import numpy as np
import pytest

from bbscite_gb300 import data as D
from bbscite_gb300.verification import lib as L
from bbscite_gb300.verification.__main__ import main as vmain


def test_newick_round_trip(native):
    rng = np.random.default_rng(5)
    for G in (1, 2, 7, 40, 200):
        pv = D.random_parent_vector(rng, G)
        assert (L.parse_newick(native.to_newick(pv)) == pv).all()
    with pytest.raises(ValueError):
        L.parse_newick("((0,1)2,3")


def test_likelihood_at_best_attachments_is_the_max_score(orc):
    G, Cn, a, b = 30, 40, 1e-3, 0.2
    m, parent, attach = D.generate_dataset(11, G, Cn, a, b, 0.1, 0.05)
    mut, known = D.matrix_to_bits(m)
    am, dm = orc.parent_to_matrix(parent)
    _, _, _, best = orc.logscore_tree(a, b, 0.1, dm, mut, known, b)
    f64 = orc.logscore_tree_f64(a, b, dm, mut, known, b, 0.1, False)
    assert L.log_likelihood(m, parent, best, a, b) == pytest.approx(
        f64, rel=1e-12)
    # at the true attachments the likelihood is at most the maximum
    assert L.log_likelihood(m, parent, attach, a, b) <= f64 + 1e-9


def test_tost_decisions():
    a, b = 1e-6, 0.25
    eps = L.max_bit_flip_difference(a, b)
    assert eps == pytest.approx(abs(math.log(1e-6) - math.log(0.75)))
    r = L.tost(np.zeros(32), a, b)
    assert r["non_inferior"] and r["equivalent"] and r["equal"] == 32
    rng = np.random.default_rng(0)
    r = L.tost(rng.normal(0.0, 0.5, 32), a, b)
    assert r["non_inferior"] and r["equivalent"]
    r = L.tost(rng.normal(-3 * eps, 0.5, 32), a, b)
    assert not r["non_inferior"]


def test_generate_and_tost_commands(native, tmp_path, capsys):
    assert vmain(["generate", "-o", str(tmp_path / "g"), "-n", "12", "-m",
                  "20", "-a", "0.01", "-b", "0.2", "-e", "0.05", "-s", "4",
                  "-x"]) == 0
    ll = float(capsys.readouterr().out.strip())
    m, parent, attach = D.generate_dataset(4, 12, 20, 0.01, 0.2, 0.05, 0.0)
    assert (D.read_csv(str(tmp_path / "g" / "input.csv")) == m).all()
    assert (L.parse_newick((tmp_path / "g" / "true_tree.newick").read_text())
            == parent).all()
    assert ll == pytest.approx(L.log_likelihood(m, parent, attach, 0.01, 0.2))
    base = tmp_path / "q"
    for i, (x, y) in enumerate([(-10.0, -10.0), (-12.5, -12.0),
                                (-9.0, -9.5), (-20.0, -20.0)]):
        for name, v in (("bbSCITE", x), ("SCITE", y)):
            d = base / f"in{i}" / name
            d.mkdir(parents=True)
            (d / "likelihood.txt").write_text(f"{v}\n")
    rc = vmain(["tost", "-d", str(base), "-a", "1e-6", "-b", "0.25"])
    out = capsys.readouterr().out
    assert rc == 0 and "non-inferior to SCITE!" in out
    assert "no. inputs both equal: 2" in out
