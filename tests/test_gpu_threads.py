"""Contexts on several host threads at once.

Each context owns its device memory and one CUDA stream, and the last
error is kept per thread, so two contexts and a batch driven from three
threads at the same time (ctypes releases the GIL during each call) give
exactly the results of the same runs one after another.
"""
import threading

import numpy as np
import pytest

from bbscite_gb300 import data as D

pytestmark = pytest.mark.gpu


def ctx_run(native, seed, G, Cn, out, key):
    m, _, _ = D.generate_dataset(seed, G, Cn, 1e-3, 0.2, 0.1, 0.02)
    mut, known = D.matrix_to_bits(m)
    p = native.default_params(alpha_mean=1e-3, beta_mean=0.2, seed=seed,
                              prob_beta_change=0.1)
    with native.Context(mut, known, Cn, G, p) as c:
        c.init_chains(64)
        for _ in range(4):  # about a second: the threads overlap
            c.run(5000)
        out[key] = (c.chains()["dm"].copy(), c.best()["score"])


def batch_run(native, out, key):
    data = []
    for i, (g, cn) in enumerate([(30, 40), (90, 96)]):
        m, _, _ = D.generate_dataset(90 + i, g, cn, 1e-3, 0.2, 0.1, 0.02)
        mut, known = D.matrix_to_bits(m)
        data.append((mut, known, cn, g))
    p = native.default_params(alpha_mean=1e-2, beta_mean=0.3, seed=5,
                              prob_beta_change=0.1,
                              score_mode=native.SCORE_SUM,
                              error_move=native.ERROR_LANGEVIN)
    with native.Batch(data, p) as bt:
        bt.init_chains(32)
        for _ in range(4):
            bt.run(5000)
        out[key] = [(bt.best(d)["dm"].copy(), bt.best(d)["score"])
                    for d in range(2)]


def errors_stay_per_thread(native, out, key):
    """A failing call on this thread leaves its own message, whatever the
    other threads do meanwhile."""
    msgs = []
    for _ in range(200):
        with pytest.raises(native.BbsError) as e:
            native.Context(np.zeros((2, 1), np.uint64),
                           np.zeros((2, 1), np.uint64), 2, 300)
        msgs.append(str(e.value))
    out[key] = msgs


def test_contexts_on_three_threads_match_sequential_runs(native):
    jobs = [(ctx_run, (native, 71, 63, 64)), (ctx_run, (native, 72, 95, 96)),
            (batch_run, (native,)), (errors_stay_per_thread, (native,))]
    seq = {}
    for i, (fn, args) in enumerate(jobs[:3]):
        fn(*args, seq, i)
    par = {}
    errs = []

    def wrap(fn, args, i):
        try:
            fn(*args, par, i)
        except BaseException as exc:  # reported on the main thread
            errs.append(exc)
    threads = [threading.Thread(target=wrap, args=(fn, args, i))
               for i, (fn, args) in enumerate(jobs)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=600)
    assert not errs, errs
    assert all(not t.is_alive() for t in threads)
    for i in (0, 1):
        np.testing.assert_array_equal(par[i][0], seq[i][0])
        assert par[i][1] == seq[i][1]
    for (dm_p, s_p), (dm_s, s_s) in zip(par[2], seq[2]):
        np.testing.assert_array_equal(dm_p, dm_s)
        assert s_p == s_s
    assert all("gene count 300" in m for m in par[3]), set(par[3])
