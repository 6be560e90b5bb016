"""bbs_score_trees_noalloc: scoring for callers that cannot allocate GPU
memory at scoring time (for example a framework that has given all device
memory to its own pool, or a latency-critical loop where an allocation
would synchronise the device).  The entry point takes device buffers from
the caller and keeps its scratch in a fixed device array.

Checked through the C ABI against bbs_score_trees on the same trees, on two
calls in a row (the second call reuses the scratch the first one left).
The test allocates its device buffers with torch; the entry point itself
allocates nothing.
"""
import ctypes as C

import numpy as np
import pytest

from bbscite_gb300 import data as D

pytestmark = pytest.mark.gpu


def _bind(native):
    L = native.lib()
    fn = L.bbs_score_trees_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                   C.c_void_p, C.c_void_p]
    return fn


def _random_trees(native, rng, n_genes, n_trees):
    parents = np.stack([D.random_parent_vector(rng, n_genes)
                        for _ in range(n_trees)])
    return np.stack([native.parent_to_matrix(p)[1] for p in parents])


def test_noalloc_matches_score_trees_twice(native):
    torch = pytest.importorskip("torch")
    fn = _bind(native)
    G, Cn = 95, 96
    m, _, _ = D.generate_dataset(77, G, Cn, 1e-3, 0.2, 0.1, 0.02)
    mut, known = D.matrix_to_bits(m)
    p = native.default_params(alpha_mean=1e-3, beta_mean=0.2)
    rng = np.random.default_rng(12)
    with native.Context(mut, known, Cn, G, p) as ctx:
        for n_trees in (600, 37):  # two calls in a row, different sizes
            dm = _random_trees(native, rng, G, n_trees)
            betas = rng.uniform(0.05, 0.6, size=n_trees).astype(np.float32)
            want_s, want_c, _ = ctx.score_trees(dm, betas)

            d_dm = torch.from_numpy(dm.view(np.int64).copy()).cuda()
            d_scores = torch.full((n_trees,), float("nan"),
                                  dtype=torch.float32, device="cuda")
            d_counts = torch.zeros((n_trees, 4), dtype=torch.int64,
                                   device="cuda")
            torch.cuda.synchronize()
            rc = fn(ctx._h, C.c_void_p(d_dm.data_ptr()),
                    betas.ctypes.data_as(C.c_void_p), n_trees,
                    C.c_void_p(d_scores.data_ptr()),
                    C.c_void_p(d_counts.data_ptr()))
            native.check(rc)
            got_s = d_scores.cpu().numpy()
            got_c = d_counts.cpu().numpy().view(np.uint64)
            # same kernel, same host log table: bit-exact
            np.testing.assert_array_equal(got_s, want_s)
            np.testing.assert_array_equal(got_c, want_c)


@pytest.mark.parametrize("G,Cn,with_counts", [(255, 40, True),
                                               (95, 96, False)])
def test_noalloc_wide_rows_and_no_counts(native, G, Cn, with_counts):
    """Rows of four 64-bit words (255 genes), and a call without the
    optional counts buffer: the same scores as bbs_score_trees."""
    torch = pytest.importorskip("torch")
    fn = _bind(native)
    m, _, _ = D.generate_dataset(G + Cn, G, Cn, 1e-3, 0.2, 0.1, 0.02)
    mut, known = D.matrix_to_bits(m)
    p = native.default_params(alpha_mean=1e-3, beta_mean=0.2)
    rng = np.random.default_rng(G)
    with native.Context(mut, known, Cn, G, p) as ctx:
        for n_trees in (70, 5):
            dm = _random_trees(native, rng, G, n_trees)
            betas = rng.uniform(0.05, 0.6, size=n_trees).astype(np.float32)
            want_s, want_c, _ = ctx.score_trees(dm, betas)
            d_dm = torch.from_numpy(dm.view(np.int64).copy()).cuda()
            d_scores = torch.full((n_trees,), float("nan"),
                                  dtype=torch.float32, device="cuda")
            d_counts = (torch.zeros((n_trees, 4), dtype=torch.int64,
                                    device="cuda") if with_counts else None)
            torch.cuda.synchronize()
            rc = fn(ctx._h, C.c_void_p(d_dm.data_ptr()),
                    betas.ctypes.data_as(C.c_void_p), n_trees,
                    C.c_void_p(d_scores.data_ptr()),
                    C.c_void_p(d_counts.data_ptr()) if with_counts else None)
            native.check(rc)
            np.testing.assert_array_equal(d_scores.cpu().numpy(), want_s)
            if with_counts:
                np.testing.assert_array_equal(
                    d_counts.cpu().numpy().view(np.uint64), want_c)


def test_noalloc_rejects_too_many_trees(native):
    torch = pytest.importorskip("torch")
    fn = _bind(native)
    m, _, _ = D.generate_dataset(3, 20, 30, 1e-3, 0.2)
    mut, known = D.matrix_to_bits(m)
    with native.Context(mut, known, 30, 20) as ctx:
        n = 16385  # one more than BBS_NOALLOC_MAX_TREES
        betas = np.full(n, 0.2, dtype=np.float32)
        d_buf = torch.zeros(8, dtype=torch.int64, device="cuda")
        rc = fn(ctx._h, C.c_void_p(d_buf.data_ptr()),
                betas.ctypes.data_as(C.c_void_p), n,
                C.c_void_p(d_buf.data_ptr()), None)
        assert rc == native.BBS_ERR_SIZE
        assert b"at most 16384 trees" in native.lib().bbs_last_error()
