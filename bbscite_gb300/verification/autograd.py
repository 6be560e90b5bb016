"""torch.autograd.Function over the sum-score adjoint (bbs_sumscore_grad).

The forward pass returns, per tree, logL = sum_c logsumexp_j s_cj at the
tree's (alpha, beta); the backward pass multiplies the incoming gradient by
the kernel's dlogL/dalpha and dlogL/dbeta.  The sum score has no
counterpart in the reference's code (SCITE's sum score is described in
docs/thesis/chapters/conclusion/open_directions.tex:13 only), so the
definition is the one stated here: s_cj is the reference's cell score
(src/TreeScorer.hpp:131-210) of cell c attached below node j.

This wrapper is harness code: the library's own chains use the adjoint in
the kernel and never go through torch.
"""
from __future__ import annotations

import numpy as np
import torch


class SumScore(torch.autograd.Function):
    """logL(alpha, beta) of a fixed batch of trees on one dataset."""

    @staticmethod
    def forward(ctx, alpha: torch.Tensor, beta: torch.Tensor, context,
                dm: np.ndarray):
        a = alpha.detach().to("cpu", torch.float64).numpy()
        b = beta.detach().to("cpu", torch.float64).numpy()
        logl, da, db, _ = context.sumscore_grad(dm, a, b)
        ctx.save_for_backward(torch.from_numpy(da.astype(np.float64)),
                              torch.from_numpy(db.astype(np.float64)))
        return torch.from_numpy(logl.astype(np.float64)).to(alpha.dtype)

    @staticmethod
    def backward(ctx, grad):
        da, db = ctx.saved_tensors
        g = grad.to(torch.float64)
        return (g * da).to(grad.dtype), (g * db).to(grad.dtype), None, None


def sum_score(context, dm: np.ndarray, alpha: torch.Tensor,
              beta: torch.Tensor) -> torch.Tensor:
    """Per-tree sum score; differentiable in alpha and beta (tensors of
    one entry per tree, or scalars broadcast over the trees)."""
    n = dm.shape[0]
    alpha = alpha.expand(n) if alpha.dim() == 0 else alpha
    beta = beta.expand(n) if beta.dim() == 0 else beta
    return SumScore.apply(alpha, beta, context, dm)
