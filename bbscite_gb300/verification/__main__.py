"""python -m bbscite_gb300.verification {generate,score,tost}

The data-generation, tree-scoring and quality-test commands of the
reference's verification tool (verification/__main__.py:13-163), over this
project's generator and GPU scorer.  Differences: the generator is
bbscite_gb300.data.generate_dataset (numpy PCG64 instead of Python's
random and networkx), the likelihood uses the corrected error classes of
bbscite_gb300/verification/lib.py, and `tost` prints no histogram."""
from __future__ import annotations

import argparse
import math
import os
import sys
from pathlib import Path

import numpy as np

from bbscite_gb300 import data as D
from bbscite_gb300.verification import lib as L


def generate(args) -> int:
    out = Path(args.out_dir or ".")
    out.mkdir(parents=True, exist_ok=True)
    seed = args.seed if args.seed is not None else int.from_bytes(
        os.urandom(4), "little")
    m, parent, attach = D.generate_dataset(seed, args.genes, args.cells,
                                           args.alpha, args.beta,
                                           args.missing, 0.0)
    from bbscite_gb300 import native as N
    (out / "true_tree.gv").write_text(N.to_graphviz(parent))
    (out / "true_tree.newick").write_text(N.to_newick(parent))
    D.write_csv(m, str(out / "input.csv"))
    (out / "true_attachments.csv").write_text(
        " ".join(str(int(a)) for a in attach) + "\n")
    ll = L.log_likelihood(m, parent, attach, args.alpha, args.beta)
    if args.compact:
        print(ll)
    else:
        print(f"True mutation tree likelihood: {math.exp(ll)} = exp({ll})")
    return 0


def score(args) -> int:
    from bbscite_gb300 import native as N
    m = D.read_csv(str(args.matrix))
    n_genes, n_cells = m.shape
    parent = L.parse_newick(Path(args.tree).read_text())
    if len(parent) != n_genes + 1:
        print("Error: the tree and the matrix disagree in the number of "
              "genes", file=sys.stderr)
        return 1
    mut, known = D.matrix_to_bits(m)
    p = N.default_params(alpha_mean=args.alpha, beta_mean=args.beta)
    with N.Context(mut, known, n_cells, n_genes, p) as ctx:
        _, dm = N.parent_to_matrix(parent)
        _, _, attach = ctx.score_trees(dm[None], args.beta, attach=True)
    ll = L.log_likelihood(m, parent, attach[0], args.alpha, args.beta)
    if args.compact:
        print(ll)
    else:
        print(f"Mutation tree likelihood: {math.exp(ll)} = log({ll})")
    if args.out_matrix is not None:
        truth = np.zeros_like(m)
        for c in range(n_cells):
            for g in L.root_path(parent, int(attach[0][c])):
                if g < n_genes:
                    truth[g, c] = 1
        D.write_csv(truth, str(args.out_matrix))
    return 0


def quality(args) -> int:
    def get(d: Path) -> float:
        return float((d / "likelihood.txt").read_text().split()[0])
    diffs = [get(d / "bbSCITE") - get(d / "SCITE")
             for d in sorted(Path(args.basedir).iterdir()) if d.is_dir()]
    r = L.tost(diffs, args.alpha, args.beta, args.n_bits,
               args.confidence_level)
    flip = L.max_bit_flip_difference(args.alpha, args.beta)
    print(f"Mean differences: {r['mean']:.2f} ≌ "
          f"{abs(r['mean']) / flip:.2f} bit flips")
    print(f"H0: µ <= -{r['epsilon']:.2f} or µ >= {r['epsilon']:.2f}")
    print(f"H1: -{r['epsilon']:.2f} < µ < {r['epsilon']:.2f}")
    print(f"p-value for lower part of H0: {r['lower_p']}")
    print(f"p-value for upper part of H0: {r['upper_p']}")
    print(f"maximal p-value to reject H0 parts: {r['p_bound']:.4f}")
    ok = r["equivalent"]
    print("bbSCITE is non-inferior to SCITE!" if ok else
          "bbSCITE may not be non-inferior to SCITE!")
    print()
    print("# Additional statistics:")
    print(f"max difference (bbSCITE better): {max(diffs):.2f} ≌ "
          f"{max(diffs) / flip:.2f} bit flips")
    print(f"min difference (SCITE better): {min(diffs):.2f} ≌ "
          f"{min(diffs) / flip:.2f} bit flips")
    print(f"no. inputs bbSCITE better: {r['better']}")
    print(f"no. inputs both equal: {r['equal']}")
    print(f"no. inputs SCITE better: {r['worse']}")
    return 0 if ok else 1


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m bbscite_gb300.verification")
    sub = ap.add_subparsers(dest="subcommand", required=True)
    g = sub.add_parser("generate", help="Generate a random input")
    g.add_argument("-o", "--out-dir", type=Path)
    g.add_argument("-n", "--genes", required=True, type=int)
    g.add_argument("-m", "--cells", required=True, type=int)
    g.add_argument("-a", "--alpha", required=True, type=float)
    g.add_argument("-b", "--beta", required=True, type=float)
    g.add_argument("-e", "--missing", required=True, type=float)
    g.add_argument("-s", "--seed", type=int)
    g.add_argument("-x", "--compact", action="store_true")
    s = sub.add_parser("score", help="Score a tree on a matrix")
    s.add_argument("-a", "--alpha", required=True, type=float)
    s.add_argument("-b", "--beta", required=True, type=float)
    s.add_argument("-t", "--tree", required=True, type=Path)
    s.add_argument("-m", "--matrix", required=True, type=Path)
    s.add_argument("-o", "--out-matrix", type=Path)
    s.add_argument("-x", "--compact", action="store_true")
    t = sub.add_parser("tost", help="Equivalence test of best likelihoods")
    t.add_argument("-d", "--basedir", default=Path("./quality_benchmark.out"),
                   type=Path)
    t.add_argument("-n", "--n-bits", default=1, type=int)
    t.add_argument("-a", "--alpha", default=1e-6, type=float)
    t.add_argument("-b", "--beta", default=0.25, type=float)
    t.add_argument("-c", "--confidence-level", default=0.95, type=float)
    args = ap.parse_args(argv)
    return {"generate": generate, "score": score, "tost": quality}[
        args.subcommand](args)


if __name__ == "__main__":
    sys.exit(main())
