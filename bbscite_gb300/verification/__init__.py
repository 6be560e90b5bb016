"""Verification harness over the GB300 path: data generation, tree scoring
and the non-inferiority test of the reference's verification/ tool, plus
the autograd wrapper of the sum-score adjoint."""
