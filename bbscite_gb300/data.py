"""Mutation data formats and the seeded synthetic generator.

* SCITE CSV: one row per gene, one space-separated entry per cell, entries
  0 (not mutated), 1 (mutated), 2 (homozygous mutated, read as 1) and
  3 (unknown) -- src/main.cpp:50-144.
* Bit rows: per cell, ceil(n_nodes/64) little-endian uint64 words with bit g
  set for gene g (`is_mutated`, `is_known`), src/main.cpp:103-144.  Bits at
  and beyond the root index n_genes are zero.
* Generator: a uniform random rooted tree over n_genes gene nodes plus the
  root n_genes (uniform Pruefer code, decoded as src/MutationTree.hpp:
  427-476), each cell attached to a uniform node, true profile = genes on the
  root path, then sequencing noise (verification/lib.py:92-98, 199-223):
  true 0 -> 1 with probability alpha, true 1 -> 0 with beta, then unknown
  (3) with `missing`, then a `homozygous` fraction of observed true
  mutations recorded as 2.  numpy's PCG64 makes the output identical on
  every platform for a given seed.
"""
from __future__ import annotations

import heapq
import os

import numpy as np


def n_words(n_nodes: int) -> int:
    return (n_nodes + 63) // 64


def pruefer_to_parent(code) -> np.ndarray:
    """Pruefer code (length n-2, entries in [0, n-1]) -> parent vector with
    root n-1 whose own entry is n-1.  Same tree as the reference's scan for
    the smallest degree-1 node (a min-heap of leaves)."""
    code = [int(c) for c in code]
    n = len(code) + 2
    degree = [1] * n
    for c in code:
        degree[c] += 1
    parent = np.full(n, n - 1, dtype=np.uint32)
    leaves = [j for j in range(n) if degree[j] == 1]
    heapq.heapify(leaves)
    for c in code:
        j = heapq.heappop(leaves)
        parent[j] = c
        degree[c] -= 1
        degree[j] -= 1
        if degree[c] == 1:
            heapq.heappush(leaves, c)
    for j in range(n):
        if degree[j] == 1:
            parent[j] = n - 1
            break
    return parent


def random_parent_vector(rng: np.random.Generator, n_genes: int) -> np.ndarray:
    n = n_genes + 1
    return pruefer_to_parent(rng.integers(0, n, size=n - 2))


def ancestors_of(parent: np.ndarray, x: int) -> list:
    root = len(parent) - 1
    out = []
    while x != root:
        out.append(x)
        x = int(parent[x])
    return out


def generate_dataset(seed: int, n_genes: int, n_cells: int, alpha: float,
                     beta: float, missing: float = 0.0,
                     homozygous: float = 0.0):
    """Returns (matrix[int8, n_genes x n_cells], true parent vector,
    attachments)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    parent = random_parent_vector(rng, n_genes)
    attach = rng.integers(0, n_genes + 1, size=n_cells)
    truth = np.zeros((n_genes, n_cells), dtype=np.int8)
    for c in range(n_cells):
        for g in ancestors_of(parent, int(attach[c])):
            truth[g, c] = 1
    u_flip = rng.random((n_genes, n_cells))
    u_miss = rng.random((n_genes, n_cells))
    u_homo = rng.random((n_genes, n_cells))
    obs = np.where(truth == 0, (u_flip < alpha).astype(np.int8),
                   (u_flip >= beta).astype(np.int8)).astype(np.int8)
    obs = np.where(u_miss < missing, np.int8(3), obs)
    homo = (truth == 1) & (obs == 1) & (u_homo < homozygous)
    obs = np.where(homo, np.int8(2), obs).astype(np.int8)
    return obs, parent, attach


def matrix_to_bits(matrix: np.ndarray, n_nodes: int | None = None):
    """SCITE matrix (genes x cells) -> (is_mutated, is_known) bit rows of
    shape (n_cells, n_words(n_nodes))."""
    matrix = np.asarray(matrix)
    n_genes, n_cells = matrix.shape
    n_nodes = n_genes + 1 if n_nodes is None else n_nodes
    W = n_words(n_nodes)
    mut = np.zeros((n_cells, W), dtype=np.uint64)
    known = np.zeros((n_cells, W), dtype=np.uint64)
    for g in range(n_genes):
        word, bit = divmod(g, 64)
        b = np.uint64(1) << np.uint64(bit)
        row = matrix[g]
        known[:, word] |= np.where(row != 3, b, np.uint64(0))
        mut[:, word] |= np.where((row == 1) | (row == 2), b, np.uint64(0))
    return mut, known


def write_csv(matrix: np.ndarray, path: str) -> None:
    with open(path, "w") as f:
        for row in np.asarray(matrix):
            f.write(" ".join(str(int(x)) for x in row) + "\n")


def read_csv(path: str) -> np.ndarray:
    with open(path) as f:
        rows = [[int(x) for x in line.split()] for line in f
                if line.strip()]
    return np.array(rows, dtype=np.int8)


def dataset_files(out_dir: str, seed: int, n_genes: int, n_cells: int,
                  alpha: float, beta: float, missing: float = 0.0,
                  homozygous: float = 0.0) -> str:
    """Writes input.csv (+ true_tree.newick, true_attachments.csv) like
    `tool.py generate` and returns the CSV path."""
    os.makedirs(out_dir, exist_ok=True)
    m, parent, attach = generate_dataset(seed, n_genes, n_cells, alpha, beta,
                                         missing, homozygous)
    path = os.path.join(out_dir, "input.csv")
    write_csv(m, path)
    with open(os.path.join(out_dir, "true_attachments.csv"), "w") as f:
        f.write(" ".join(str(int(a)) for a in attach) + "\n")
    with open(os.path.join(out_dir, "true_parent.txt"), "w") as f:
        f.write(" ".join(str(int(p)) for p in parent) + "\n")
    return path
