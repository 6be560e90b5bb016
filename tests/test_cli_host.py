"""The SCITE-compatible surface on the host (no GPU): the C++ Parameters
wrapper against the reference's own Parameters class (argument values and
the exact stderr text, when the reference builds here) and against fixed
expectations; the C++ MutationTree wrapper against the reference's
known answers (test/MutationTree.cpp); the CLI's argument and input-file
errors (src/main.cpp:42-101) with their messages and exit codes."""
import ctypes as C
import os
import shlex
import subprocess

import numpy as np
import pytest

from bbscite_gb300 import data as D

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

ARGV_CASES = [
    "-i in.csv -r 4 -l 100",
    "-i in.csv -r 4 -l 100 -fd 0.01 -ad 0.2 -sd 0.05 -g 2.5 -x 5",
    "-i in.csv -r 4 -l 100 -ad 0.2 0.1",
    "-i in.csv -r 4 -l 100 -e 0.1 -move_probs 0.5 0.3 0.2",
    "-i in.csv -r 4 -l 100 -max_treelist_size 7 -t -n 5 -m 6 -a -p -s "
    "-transpose -no_tree_list -names x -cc 1",
    "-i in.dat.csv -o out/base -r 1000 -l 5000000",
    "",
    "-i in.csv -r 4",
    "-i in.csv -r 4 -l 100 -zz",
    "-i in.csv -r 4 -l 100 -e -1",
    "-i in.csv -r 4 -l 100 -e 0 -move_probs 0 0 0",
    "-i",
    "-i in.csv -r 4 -l 100 -move_probs 0.5",
    "-i in.csv -r 4 -l 100 -ad",
]


def parse_probe_line(line):
    tok = line.split()
    out = {}
    for k, v in zip(tok[0::2], tok[1::2]):
        out[k] = v
    return out


def test_parameters_fixed_expectations(probe):
    out, err = probe(["params " + a for a in ARGV_CASES[:6]])
    r = [parse_probe_line(x) for x in out]
    assert all(x["ok"] == "1" for x in r)
    # defaults, src/Parameters.hpp:39-45
    assert float(r[0]["alpha"]) == np.float32(6.04e-5)
    assert float(r[0]["beta"]) == np.float32(0.4309)
    assert (r[0]["chains"], r[0]["length"], r[0]["out"]) == ("4", "100", "in")
    assert float(r[1]["gamma"]) == 2.5 and float(r[1]["chi"]) == 5.0
    # -ad a b sums in double, then rounds to float
    assert float(r[2]["beta"]) == np.float32(np.float64(np.float32(0.2)) + 0.1)
    assert "Summing false negative probabilites." in err
    # probabilities normalised by their sum
    assert float(r[3]["e"]) == pytest.approx(0.1 / 1.1, rel=1e-6)
    assert r[4]["max_trees"] == "7"
    assert r[5]["out"] == "out/base" and r[5]["length"] == "5000000"


def test_parameters_errors(probe):
    out, err = probe(["params " + a for a in ARGV_CASES[6:]])
    assert all(parse_probe_line(x)["ok"] == "0" for x in out)
    for msg in ("Error: Missing input file path. Did you forget to set the "
                "-i paramater?",
                "Error: Missing markov chain length. Did you forget to set "
                "the -l parameter?",
                "Error: Unknown parameter -zz.",
                "Error: Move probabilities may not be negative.",
                "Error: The sum of the move type probabilities is zero.",
                "Error: Missing argument to parameter -i.",
                "Error: Missing argument to parameter -move_probs.",
                "Error: Missing argument to parameter -ad."):
        assert msg in err, msg


def test_parameters_match_reference_class(probe, orc, capfd):
    """Values and stderr text against the reference's Parameters class
    (compiled from its sources by oracle/Makefile; skipped where absent)."""
    ref = orc.ref_lib()
    if ref is None:
        pytest.skip("reference sources not built here")
    for case in ARGV_CASES:
        argv = ["bbscite"] + shlex.split(case)
        arr = (C.c_char_p * len(argv))(*[a.encode() for a in argv])
        vals = np.zeros(12, dtype=np.float32)
        capfd.readouterr()
        ok = ref.ref_parse_args(len(argv), arr, vals.ctypes.data)
        ref_err = capfd.readouterr().err
        out, err = probe(["params " + case])
        got = parse_probe_line(out[0])
        assert int(got["ok"]) == ok, case
        assert err == ref_err, case
        assert np.float32(got["alpha"]) == vals[0], case
        assert np.float32(got["beta"]) == vals[1], case
        assert np.float32(got["sd"]) == vals[2], case
        assert np.float32(got["chi"]) == vals[7], case
        assert np.float32(got["gamma"]) == vals[8], case
        assert int(got["max_trees"]) == int(vals[11]), case
        if ok:
            for k, i in (("e", 3), ("prune", 4), ("swap", 5),
                         ("subtrees", 6)):
                assert np.float32(got[k]) == vals[i], (case, k)
            assert int(got["chains"]) == int(vals[9])
            assert int(got["length"]) == int(vals[10])


def test_mutation_tree_wrapper_kats(probe, kat):
    code = kat["pruefer_code_to_parent_vector"]
    out, _ = probe(["pruefer " + " ".join(map(str, code["code"]))])
    assert [int(x) for x in out[0].split()] == code["expected"]

    def queries(entry):
        pv = kat[entry]["parent_vector"]
        out, _ = probe(["tree 0.42 " + " ".join(map(str, pv))])
        return dict(p.strip().split(" ", 1) for p in out[0].split(" | "))

    ints = lambda s: [int(x) for x in s.split()]  # noqa: E731
    assert ints(queries("get_parent")["parent"]) == \
        kat["get_parent"]["expected"]
    assert ints(queries("get_n_descendants")["n_desc"]) == \
        kat["get_n_descendants"]["expected"]
    assert ints(queries("get_n_ancestors")["n_anc"]) == \
        kat["get_n_ancestors"]["expected"]
    anc = queries("is_ancestor")["anc"].split()
    for x, row in enumerate(kat["is_ancestor"]["expected_rows"]):
        assert [c == "1" for c in anc[x]] == [bool(v) for v in row]
    desc = queries("is_descendant")["desc"].split()
    for x, row in enumerate(kat["is_descendant"]["expected_rows"]):
        assert [c == "1" for c in desc[x]] == [bool(v) for v in row]

    g = kat["to_graphviz"]
    out, _ = probe(["tree 0.42 " + " ".join(map(str, g["parent_vector"]))])
    parts = dict(p.strip().split(" ", 1) for p in out[0].split(" | "))
    assert parts["gv"].replace("\\n", "\n") == g["expected"]
    nw = kat["to_newick"]
    out, _ = probe(["tree 0.42 " + " ".join(map(str, nw["parent_vector"]))])
    parts = dict(p.strip().split(" ", 1) for p in out[0].split(" | "))
    assert parts["newick"].replace("\\n", "\n") == nw["expected"]


def test_mutation_tree_wrapper_vs_oracle(probe, orc):
    """Queries of the wrapper against the oracle on random trees."""
    rng = np.random.default_rng(17)
    lines, trees = [], []
    for G in (3, 17, 64, 100):
        pv = D.random_parent_vector(rng, G)
        trees.append(pv)
        lines.append("tree 0.3 " + " ".join(map(str, pv)))
    out, _ = probe(lines)
    for pv, line in zip(trees, out):
        parts = dict(p.strip().split(" ", 1) for p in line.split(" | "))
        n = len(pv)
        am, dm = orc.parent_to_matrix(pv)
        assert [int(x) for x in parts["parent"].split()] == \
            [orc.get_parent(dm, x) for x in range(n)]
        kd = [int(x) for x in parts["kth_desc"].split()]
        kn = [int(x) for x in parts["kth_nondesc"].split()]
        i = j = 0
        for x in range(n):
            nd = orc.n_descendants(am, x)
            for k in range(nd + 1):
                assert kd[i] == orc.descendant_or_nondescendant(am, x, k, True)
                i += 1
            for k in range(n - nd + 1):
                assert kn[j] == orc.descendant_or_nondescendant(am, x, k,
                                                                False)
                j += 1


# ------------------------------------------------------------------ CLI --

def cli():
    from bbscite_gb300 import build as B
    return B.CLI


def run_cli(args, cwd):
    return subprocess.run([cli()] + args, capture_output=True, text=True,
                          cwd=cwd, timeout=300)


def test_cli_argument_errors(native, tmp_path):
    r = run_cli([], tmp_path)
    assert r.returncode == 1
    assert r.stderr.splitlines() == [
        "Error: Missing input file path. Did you forget to set the -i "
        "paramater?",
        "Error: Missing number of markov chains to simulate. Did you forget "
        "to set the -r parameter?",
        "Error: Missing markov chain length. Did you forget to set the -l "
        "parameter?",
        "Quitting due to CLI argument errors."]


@pytest.mark.parametrize("content,message", [
    ("0 1 0\n1 x 0\n", "Error: Illegal character x in the input file!"),
    ("0 1 0\n1 0\n", "Error: Inconsistent rows in the input file!"),
    ("", "Error: Empty input file!"),
    ("\n".join(["0 1"] * 256) + "\n",
     "Error: This build of bbSCITE only supports up 255 genes. The input "
     "data contains 256 genes."),
])
def test_cli_input_errors(native, tmp_path, content, message):
    (tmp_path / "in.csv").write_text(content)
    r = run_cli(["-i", "in.csv", "-r", "2", "-l", "10"], tmp_path)
    assert r.returncode == 1
    assert message in r.stderr.splitlines()


def test_cli_without_gpu_fails_loudly(native, tmp_path):
    from conftest import has_gpu
    if has_gpu():
        pytest.skip("a GPU is present")
    m, _, _ = D.generate_dataset(3, 6, 8, 0.01, 0.2, 0.0, 0.0)
    D.write_csv(m, str(tmp_path / "in.csv"))
    r = run_cli(["-i", "in.csv", "-r", "2", "-l", "10"], tmp_path)
    assert r.returncode == 1
    assert r.stderr.startswith("Error: ")
    assert not (tmp_path / "in_ml0.gv").exists()
