"""Chain checkpoints through the C ABI (bbs_save_chains / bbs_load_chains).

A run that is stopped, saved, destroyed and restored into a new context
continues bit for bit like the same run done in one go: the image holds
each chain's trees, best proposals, co-optimal lists, rates, scores and
Philox position.  Images of another dataset or other parameters, and
damaged images, are refused on the host before anything reaches the GPU,
and the refusing context keeps its own chains.
"""
import ctypes as C

import numpy as np
import pytest

from bbscite_gb300 import data as D

pytestmark = pytest.mark.gpu

G, CN = 40, 70


def make(native, m, **kw):
    mut, known = D.matrix_to_bits(m)
    p = native.default_params(alpha_mean=1e-3, beta_mean=0.2, seed=77, **kw)
    return native.Context(mut, known, CN, G, p)


def snapshot(c):
    ch = c.chains()
    return ch, c.best()


def assert_same(a, b):
    (ca, ba), (cb, bb) = a, b
    for k in ("dm", "alpha", "beta", "score", "counts", "err_stats"):
        np.testing.assert_array_equal(ca[k], cb[k], err_msg=k)
    assert ba["score"] == bb["score"] and ba["beta"] == bb["beta"]
    assert (ba["dm"] == bb["dm"]).all()


MODES = {
    "max-beta-walk": dict(prob_beta_change=0.1),
    "sum-langevin-treelist": dict(prob_beta_change=0.1, treelist_size=4,
                                  error_step=0.3),
}


@pytest.mark.parametrize("mode", list(MODES))
def test_resume_from_checkpoint_equals_one_run(native, mode):
    kw = dict(MODES[mode])
    if mode.startswith("sum"):
        kw.update(score_mode=native.SCORE_SUM,
                  error_move=native.ERROR_LANGEVIN)
    m, _, _ = D.generate_dataset(3, G, CN, 1e-3, 0.2, 0.1, 0.02)
    with make(native, m, **kw) as c:
        c.init_chains(6)
        c.run(700)
        whole = snapshot(c)
        whole_list = c.treelist(64) if "treelist" in mode else None
    with make(native, m, **kw) as c:
        c.init_chains(6)
        c.run(250)
        image = c.save_chains()
    with make(native, m, **kw) as c:
        c.init_chains(2)  # replaced by the image
        c.load_chains(image)
        assert c.n_chains == 6
        c.run(450)
        assert_same(snapshot(c), whole)
        if whole_list is not None:
            got = c.treelist(64)
            assert got["score"] == whole_list["score"]
            np.testing.assert_array_equal(got["dm"], whole_list["dm"])
            np.testing.assert_array_equal(got["betas"], whole_list["betas"])
        # a second save of the restored chains is the same image format
        again = c.save_chains()
        assert len(again) == len(image) and again[:8] == b"BBSCHKPT"


def test_checkpoint_refusals_keep_the_chains(native):
    m, _, _ = D.generate_dataset(4, G, CN, 1e-3, 0.2, 0.1, 0.02)
    other, _, _ = D.generate_dataset(5, G, CN, 1e-3, 0.2, 0.1, 0.02)
    with make(native, m) as c:
        c.init_chains(3)
        c.run(50)
        image = bytearray(c.save_chains())
    n = G + 1
    W = (n + 63) // 64
    header = 80
    bad = {
        "truncated": bytes(image[:-8]),
        "magic": b"XXXXXXXX" + bytes(image[8:]),
    }
    # node 5 of chain 1 without its own bit: no tree has such a row
    flipped = bytearray(image)
    off = header + 8 * ((1 * n + 5) * W)
    assert flipped[off] & 0x20
    flipped[off] ^= 0x20
    bad["not a tree"] = bytes(flipped)
    # chain 0 claiming more listed trees than the list holds
    listed = bytearray(image)
    states = header + 8 * (3 * n * W) * 2
    listed[states + 96:states + 100] = (5).to_bytes(4, "little")  # list_count
    bad["list count"] = bytes(listed)

    with make(native, other) as c:
        c.init_chains(2)
        c.run(20)
        before = snapshot(c)
        with pytest.raises(native.BbsError) as e:
            c.load_chains(bytes(image))
        assert e.value.code == native.BBS_ERR_INPUT
        assert_same(snapshot(c), before)
    with make(native, m, gamma=0.5) as c:
        c.init_chains(2)
        with pytest.raises(native.BbsError) as e:
            c.load_chains(bytes(image))
        assert e.value.code == native.BBS_ERR_INPUT
    with make(native, m) as c:
        c.init_chains(2)
        c.run(20)
        before = snapshot(c)
        for name in ("truncated", "magic", "not a tree", "list count"):
            with pytest.raises(native.BbsError) as e:
                c.load_chains(bad[name])
            assert e.value.code == native.BBS_ERR_INPUT, name
        assert_same(snapshot(c), before)
        c.load_chains(bytes(image))  # the intact image still loads
        assert c.n_chains == 3


def test_save_reports_the_size_it_needs(native):
    m, _, _ = D.generate_dataset(6, G, CN, 1e-3, 0.2)
    with make(native, m) as c:
        c.init_chains(4)
        L = native.lib()
        size = C.c_size_t()
        native.check(L.bbs_save_chains(c._h, None, C.byref(size)))
        n = G + 1
        W = (n + 63) // 64
        assert size.value == 80 + 2 * 8 * 4 * n * W + 128 * 4
        small = C.c_size_t(size.value - 1)
        buf = C.create_string_buffer(size.value)
        assert L.bbs_save_chains(c._h, buf, C.byref(small)) == \
            native.BBS_ERR_SIZE
        assert small.value == size.value


def test_batch_resume_from_checkpoint_equals_one_run(native):
    """A batch of three datasets (three row widths), sum score with
    Langevin error moves: 200 steps, checkpoint, a new batch, 300 steps
    end where 500 steps in one batch do."""
    shapes = [(20, 30), (70, 100), (150, 64)]
    data = []
    for i, (g, cn) in enumerate(shapes):
        m, _, _ = D.generate_dataset(40 + i, g, cn, 1e-3, 0.2, 0.1, 0.02)
        mut, known = D.matrix_to_bits(m)
        data.append((mut, known, cn, g))
    p = native.default_params(alpha_mean=1e-2, beta_mean=0.3, seed=13,
                              prob_beta_change=0.1,
                              score_mode=native.SCORE_SUM,
                              error_move=native.ERROR_LANGEVIN)

    def bests(bt):
        return [bt.best(d) for d in range(len(shapes))]

    with native.Batch(data, p) as bt:
        bt.init_chains(5)
        bt.run(500)
        whole = bests(bt)
    with native.Batch(data, p) as bt:
        bt.init_chains(5)
        bt.run(200)
        image = bt.save_chains()
    with native.Batch(data, p) as bt:
        bt.init_chains(1)
        bt.load_chains(image)
        bt.run(300)
        got = bests(bt)
    for w, g in zip(whole, got):
        assert (w["dm"] == g["dm"]).all()
        assert (w["alpha"], w["beta"], w["score"]) == \
            (g["alpha"], g["beta"], g["score"])
    # other datasets refuse the image and keep their chains
    with native.Batch(data[:2] + [data[0]], p) as bt:
        bt.init_chains(2)
        bt.run(10)
        before = bests(bt)
        with pytest.raises(native.BbsError) as e:
            bt.load_chains(image)
        assert e.value.code == native.BBS_ERR_INPUT
        after = bests(bt)
        for w, g in zip(before, after):
            assert (w["dm"] == g["dm"]).all() and w["score"] == g["score"]
