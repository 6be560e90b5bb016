"""Sum-score adjoint on 4096 random trees at 95 genes x 96 cells, through
the autograd wrapper of the verification harness: forward logL within
1e-5 relative of FP64, dlogL/dalpha and dlogL/dbeta within 1e-4 relative
of the FP64 gradient and of central finite differences (h = 1e-6) of the
FP64 sum score, per-cell attachment posteriors against FP64."""
import numpy as np
import pytest

from bbscite_gb300 import data as D

pytestmark = pytest.mark.gpu

SCORE_RTOL = 1e-5
GRAD_RTOL = 1e-4
FD_H = 1e-6
N_TREES = 4096


@pytest.fixture(scope="module")
def setup(native, orc):
    torch = pytest.importorskip("torch")
    from bbscite_gb300.verification.autograd import sum_score
    G, Cn = 95, 96
    m, _, _ = D.generate_dataset(404, G, Cn, 1e-3, 0.2, 0.1, 0.02)
    mut, known = D.matrix_to_bits(m)
    p = native.default_params(alpha_mean=1e-3, beta_mean=0.2)
    ctx = native.Context(mut, known, Cn, G, p)
    rng = np.random.default_rng(4096)
    dms = np.stack([orc.parent_to_matrix(D.random_parent_vector(rng, G))[1]
                    for _ in range(N_TREES)])
    yield torch, sum_score, ctx, dms, mut, known
    ctx.close()


@pytest.mark.parametrize("alpha,beta", [(1e-3, 0.2), (1e-2, 0.3)])
def test_gradcheck_4096_trees(setup, orc, alpha, beta):
    torch, sum_score, ctx, dms, mut, known = setup
    # evaluation point exactly representable in FP32 (the kernel's input)
    a0, b0 = float(np.float32(alpha)), float(np.float32(beta))
    a = torch.full((N_TREES,), a0, dtype=torch.float64, requires_grad=True)
    b = torch.full((N_TREES,), b0, dtype=torch.float64, requires_grad=True)
    logl = sum_score(ctx, dms, a, b)
    logl.sum().backward()
    ga, gb = a.grad.numpy(), b.grad.numpy()
    worst = {"f": 0.0, "ga": 0.0, "gb": 0.0, "fd_a": 0.0, "fd_b": 0.0}
    for t in range(N_TREES):
        f, ra, rb, _ = orc.sumscore_grad_f64(a0, b0, dms[t], mut, known)
        fa = [orc.score_counts_f64(a0 + s * FD_H, b0, dms[t], mut, known,
                                   True)[0] for s in (1, -1)]
        fb = [orc.score_counts_f64(a0, b0 + s * FD_H, dms[t], mut, known,
                                   True)[0] for s in (1, -1)]
        fd_a = (fa[0] - fa[1]) / (2 * FD_H)
        fd_b = (fb[0] - fb[1]) / (2 * FD_H)
        worst["f"] = max(worst["f"], abs(logl[t].item() - f) / abs(f))
        worst["ga"] = max(worst["ga"], abs(ga[t] - ra) / abs(ra))
        worst["gb"] = max(worst["gb"], abs(gb[t] - rb) / abs(rb))
        worst["fd_a"] = max(worst["fd_a"], abs(ga[t] - fd_a) / abs(fd_a))
        worst["fd_b"] = max(worst["fd_b"], abs(gb[t] - fd_b) / abs(fd_b))
    print(f"\nworst relative errors over {N_TREES} trees at "
          f"alpha={a0:g} beta={b0:g}: {worst}")
    assert worst["f"] <= SCORE_RTOL
    assert worst["ga"] <= GRAD_RTOL and worst["gb"] <= GRAD_RTOL
    assert worst["fd_a"] <= GRAD_RTOL and worst["fd_b"] <= GRAD_RTOL


def test_posteriors_sample(setup, orc):
    _, _, ctx, dms, mut, known = setup
    sel = dms[:64]
    _, _, _, post = ctx.sumscore_grad(sel, 1e-3, 0.2, posterior=True)
    for t in range(len(sel)):
        _, _, _, ref = orc.sumscore_grad_f64(float(np.float32(1e-3)),
                                             float(np.float32(0.2)), sel[t],
                                             mut, known, posterior=True)
        np.testing.assert_allclose(post[t], ref, atol=2e-5)


def test_autograd_chain_rule(setup):
    """Gradients flow through the wrapper into a torch graph: the
    derivative of logL(sigmoid(u)) in u is dlogL/dalpha * a (1 - a)."""
    torch, sum_score, ctx, dms, _, _ = setup
    u = torch.tensor(np.log(1e-3 / (1 - 1e-3)), dtype=torch.float64,
                     requires_grad=True)
    b = torch.tensor(0.2, dtype=torch.float64)
    out = sum_score(ctx, dms[:8], torch.sigmoid(u), b).sum()
    out.backward()
    a = torch.sigmoid(u.detach())
    _, da, _, _ = ctx.sumscore_grad(dms[:8], a.item(), 0.2)
    want = float(np.sum(da.astype(np.float64))) * a.item() * (1 - a.item())
    assert abs(u.grad.item() - want) <= 1e-9 * abs(want)
