"""Host-side helpers of the verification harness: Newick parsing, the
log-likelihood of a tree with given attachments, and the equivalence
(TOST) test of best-found likelihoods.

Follows verification/lib.py and verification/__main__.py of the reference
with two documented corrections:
  - the off-diagonal error classes use log(alpha) for observed 1 / true 0
    and log(beta) for observed 0 / true 1 (the reference's
    MutationTree.get_log_likelihood, verification/lib.py:85-88, swaps them;
    its get_most_likely_attachment, :188-191, and src/TreeScorer.hpp:99-106
    do not);
  - an entry 2 counts as an observed mutation, as src/main.cpp:129-133 reads
    it (verification/lib.py:81 and :185 skip it as unknown).
"""
from __future__ import annotations

import math

import numpy as np


def parse_newick(text: str) -> np.ndarray:
    """Parent vector of a Newick tree "(children)label" with integer node
    labels (the format of src/MutationTree.hpp:818-837); the root is its own
    parent."""
    s = text.strip().rstrip(";").strip()
    parent: dict[int, int] = {}
    pos = 0

    def node() -> int:
        nonlocal pos
        children = []
        if pos < len(s) and s[pos] == "(":
            pos += 1
            while True:
                children.append(node())
                if pos >= len(s):
                    raise ValueError("unbalanced parentheses")
                if s[pos] == ",":
                    pos += 1
                    continue
                if s[pos] == ")":
                    pos += 1
                    break
                raise ValueError(f"bad Newick at {pos}: {s[pos]!r}")
        start = pos
        while pos < len(s) and s[pos].isdigit():
            pos += 1
        if start == pos:
            raise ValueError(f"missing node label at {pos}")
        label = int(s[start:pos])
        for c in children:
            parent[c] = label
        return label

    root = node()
    if pos != len(s):
        raise ValueError(f"trailing text at {pos}")
    parent[root] = root
    n = len(parent)
    if sorted(parent) != list(range(n)) or root != n - 1:
        raise ValueError("nodes must be 0..n-1 with the root n-1")
    return np.array([parent[x] for x in range(n)], dtype=np.uint32)


def root_path(parent, node: int) -> set:
    out = {int(node)}
    while int(parent[node]) != int(node):
        node = int(parent[node])
        out.add(node)
    return out


def log_likelihood(matrix: np.ndarray, parent, attachments, alpha: float,
                   beta: float) -> float:
    """Sum over known entries of log P(observed | true) with the true state
    from each cell's attachment node (its root path carries the mutated
    genes)."""
    matrix = np.asarray(matrix)
    n_genes, n_cells = matrix.shape
    occ = np.zeros((2, 2), dtype=np.int64)  # [observed][true]
    for c in range(n_cells):
        genes = root_path(parent, int(attachments[c]))
        for g in range(n_genes):
            o = int(matrix[g, c])
            if o == 3:
                continue
            occ[1 if o in (1, 2) else 0, 1 if g in genes else 0] += 1
    return (occ[0, 0] * math.log(1.0 - alpha) + occ[1, 0] * math.log(alpha)
            + occ[0, 1] * math.log(beta) + occ[1, 1] * math.log(1.0 - beta))


def max_bit_flip_difference(alpha: float, beta: float) -> float:
    """verification/__main__.py:109-110"""
    return max(abs(math.log(alpha) - math.log(1 - beta)),
               abs(math.log(beta) - math.log(1 - alpha)))


def tost(differences, alpha: float, beta: float, n_bits: int = 1,
         confidence: float = 0.95) -> dict:
    """Two one-sided t-tests of the mean likelihood difference against
    +-n_bits bit flips (verification/__main__.py:96-160): `non_inferior`
    rejects mu <= -epsilon, `equivalent` rejects both mu <= -epsilon and
    mu >= epsilon, each at (1 - confidence) / 2."""
    from scipy.stats import ttest_1samp
    d = np.asarray(differences, dtype=np.float64)
    eps = n_bits * max_bit_flip_difference(alpha, beta)
    bound = (1.0 - confidence) / 2.0
    if np.all(d == d[0]):
        # no spread: the t statistic is undefined; decide by the value
        lower_p = 0.0 if d[0] > -eps else 1.0
        upper_p = 0.0 if d[0] < eps else 1.0
    else:
        lower_p = float(ttest_1samp(d, -eps, alternative="greater").pvalue)
        upper_p = float(ttest_1samp(d, eps, alternative="less").pvalue)
    return {"epsilon": eps, "mean": float(d.mean()),
            "lower_p": lower_p, "upper_p": upper_p, "p_bound": bound,
            "non_inferior": lower_p < bound,
            "equivalent": lower_p < bound and upper_p < bound,
            "better": int((d > 0).sum()), "equal": int((d == 0).sum()),
            "worse": int((d < 0).sum())}
