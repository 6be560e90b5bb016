"""Generates tests/golden/proxy_vectors.npz: scores of the reference's own
CPU scoring benchmark class (cpu_scoring_benchmark/CPUTreeScorer.hpp,
compiled unmodified into oracle/_ref by `make -C oracle ref`) on seeded
inputs at its fixed 128 cells x 127 genes, to pin the restatement
orc_cpu_proxy_scores that the CPU baseline times.

    python tests/golden/make_proxy_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
OUT = os.path.join(HERE, "proxy_vectors.npz")

from bbscite_gb300 import data as D  # noqa: E402
from oracle import oracle as O  # noqa: E402


def inputs():
    """The benchmark's layout: [quadword][cell] data words with one bit per
    gene, [quadword][node] ancestor words per tree."""
    m, _, _ = D.generate_dataset(128127, 127, 128, 1e-3, 0.2, 0.05, 0.02)
    mutq = np.zeros((2, 128), dtype=np.uint64)
    knownq = np.zeros((2, 128), dtype=np.uint64)
    mut, known = D.matrix_to_bits(m)  # [cell][word] rows over the genes
    mutq[:, :] = mut.T
    knownq[:, :] = known.T
    rng = np.random.default_rng(128)
    trees = [np.ascontiguousarray(O.parent_to_matrix(
        D.random_parent_vector(rng, 127))[1].T) for _ in range(12)]
    return mutq, knownq, np.ascontiguousarray(np.stack(trees))


def main():
    O.build()
    if O.ref_lib() is None:
        raise SystemExit("oracle/_ref is not built (make -C oracle ref)")
    mutq, knownq, dmq = inputs()
    out = {"mutq": mutq, "knownq": knownq, "dmq": dmq}
    for i, (a, b) in enumerate(((1e-3, 0.2), (6.04e-5, 0.4309), (0.05, 0.05))):
        out[f"rates{i}"] = np.array([a, b], dtype=np.float32)
        out[f"scores{i}"] = O.cpu_proxy_scores(a, b, mutq, knownq, dmq,
                                               reference=True)
    np.savez_compressed(OUT, **out)


if __name__ == "__main__":
    main()
