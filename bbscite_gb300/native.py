"""ctypes binding of the C ABI in include/bbscite_gb300.h.

The shared library is built in-tree (bbscite_gb300/libbbscite_gb300.so by
bbscite_gb300/build.py).  The environment variable BBSCITE_GB300_LIB names
another build of it to load instead, such as the one with device checks
(libbbscite_gb300_checked.so).  There is no fallback: if the library is
missing or a call fails, a BbsError is raised.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("BBSCITE_GB300_LIB") or os.path.join(
    PKG, "libbbscite_gb300.so")

BBS_OK, BBS_ERR_INPUT, BBS_ERR_SIZE, BBS_ERR_CUDA, BBS_ERR_TIMEOUT, \
    BBS_ERR_STATE, BBS_ERR_IO, BBS_ERR_ALLOC, BBS_ERR_DEVICE_CHECK = range(9)
MAX_GENES = 255
MAX_CELLS = 65535

RAW_MOVE = np.dtype([("move_type", "<i4"), ("raw_v", "<u4"), ("raw_w", "<u4"),
                     ("raw_descendant_of_v", "<f4"),
                     ("raw_nondescendant_of_v", "<f4"),
                     ("beta_jump", "<f4"), ("acceptance_level", "<f4"),
                     ("reserved", "<u4")])
MOVE_PARAMS = np.dtype([("move_type", "<i4"), ("v", "<u4"), ("w", "<u4"),
                        ("parent_of_v", "<u4"), ("parent_of_w", "<u4"),
                        ("descendant_of_v", "<u4"),
                        ("nondescendant_of_v", "<u4"), ("new_beta", "<f4")])
STEP_TRACE = np.dtype([("move", RAW_MOVE), ("proposed_score", "<f4"),
                       ("current_score", "<f4"), ("proposed_beta", "<f4"),
                       ("accepted", "<u4"), ("proposed_alpha", "<f4"),
                       ("proposed_max_score", "<f4"),
                       ("reserved", "<u4", (2,)),
                       ("proposed_counts", "<u8", (4,))])
assert RAW_MOVE.itemsize == 32 and STEP_TRACE.itemsize == 96

SCORE_MAX, SCORE_SUM = 0, 1
ERROR_BETA_WALK, ERROR_RANDOM_WALK, ERROR_LANGEVIN = 0, 1, 2


class BbsError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


class Params(C.Structure):
    _fields_ = [("alpha_mean", C.c_float), ("beta_mean", C.c_float),
                ("beta_sd", C.c_float), ("prob_beta_change", C.c_float),
                ("prob_prune_n_reattach", C.c_float),
                ("prob_swap_nodes", C.c_float),
                ("prob_swap_subtrees", C.c_float),
                ("beta_jump_scaling_chi", C.c_float), ("gamma", C.c_float),
                ("treelist_size", C.c_uint32), ("seed", C.c_uint64),
                ("score_mode", C.c_uint32), ("error_move", C.c_uint32),
                ("error_step", C.c_float), ("reserved1", C.c_uint32)]


_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise BbsError(BBS_ERR_STATE,
                       f"native library not built: {LIB_PATH} "
                       "(run python -m bbscite_gb300.build)")
    L = C.CDLL(LIB_PATH)
    v, u32, u64, f32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float
    sig = {
        "bbs_last_error": (C.c_char_p, []),
        "bbs_version": (C.c_char_p, []),
        "bbs_words": (u32, [u32]),
        "bbs_params_default": (None, [v]),
        "bbs_pruefer_to_parent_vector": (C.c_int, [v, u32, v]),
        "bbs_parent_vector_to_matrix": (C.c_int, [v, u32, v, v]),
        "bbs_matrix_to_parent_vector": (C.c_int, [v, u32, v]),
        "bbs_dm_to_am": (C.c_int, [v, u32, v]),
        "bbs_tree_to_graphviz": (C.c_int, [v, u32, v, C.c_size_t, v]),
        "bbs_tree_to_newick": (C.c_int, [v, u32, v, C.c_size_t, v]),
        "bbs_random_parent_vectors": (C.c_int, [u64, u32, u32, v]),
        "bbs_read_csv": (C.c_int, [C.c_char_p, v, v, v, v]),
        "bbs_create": (C.c_int, [v, v, v, u32, u32, v]),
        "bbs_destroy": (None, [v]),
        "bbs_get_sizes": (C.c_int, [v, v, v, v]),
        "bbs_init_chains": (C.c_int, [v, u32, v]),
        "bbs_run": (C.c_int, [v, u32, v, v]),
        "bbs_run_async": (C.c_int, [v, u32]),
        "bbs_sync": (C.c_int, [v]),
        "bbs_cancel": (C.c_int, [v]),
        "bbs_last_run_ms": (C.c_int, [v, v]),
        "bbs_set_launch": (C.c_int, [v, C.c_int, C.c_int, C.c_int]),
        "bbs_get_launch": (C.c_int, [v, v, v, v]),
        "bbs_autotune": (C.c_int, [v, u32, v]),
        "bbs_get_best": (C.c_int, [v, v, v, v, v, v, v, v]),
        "bbs_get_chains": (C.c_int, [v, v, v, v, v, v, v]),
        "bbs_get_best_alpha": (C.c_int, [v, v]),
        "bbs_get_treelist": (C.c_int, [v, u32, v, v, v, v]),
        "bbs_save_chains": (C.c_int, [v, v, v]),
        "bbs_load_chains": (C.c_int, [v, v, C.c_size_t]),
        "bbs_batch_create": (C.c_int, [v, u32, v, v, v, v, v]),
        "bbs_batch_destroy": (None, [v]),
        "bbs_batch_init_chains": (C.c_int, [v, u32]),
        "bbs_batch_run": (C.c_int, [v, u32]),
        "bbs_batch_last_run_ms": (C.c_int, [v, v]),
        "bbs_batch_set_launch": (C.c_int, [v, C.c_int, C.c_int, C.c_int]),
        "bbs_batch_get_launch": (C.c_int, [v, v, v, v]),
        "bbs_batch_set_chain_warps": (C.c_int, [v, C.c_int]),
        "bbs_batch_get_chain_warps": (C.c_int, [v, v]),
        "bbs_batch_autotune": (C.c_int, [v, u32, v]),
        "bbs_batch_get_best": (C.c_int, [v, u32, v, v, v, v, v]),
        "bbs_batch_save_chains": (C.c_int, [v, v, v]),
        "bbs_batch_load_chains": (C.c_int, [v, v, C.c_size_t]),
        "bbs_score_trees": (C.c_int, [v, v, v, u32, v, v, v]),
        "bbs_apply_moves": (C.c_int, [v, v, v, u32, v, v, v, v, v]),
        "bbs_sumscore_grad": (C.c_int, [v, v, v, v, u32, v, v, v, v]),
        "bbs_popc_peak": (C.c_int, [v, v]),
        "bbs_device_check_selftest": (C.c_int, [v, v, v, v]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def check(code: int) -> None:
    if code != BBS_OK:
        raise BbsError(code, lib().bbs_last_error().decode())


def words(n_nodes: int) -> int:
    return (n_nodes + 63) // 64


def default_params(**kw) -> Params:
    p = Params()
    lib().bbs_params_default(C.byref(p))
    for k, val in kw.items():
        setattr(p, k, val)
    return p


# ---- host tree helpers --------------------------------------------------

def pruefer_to_parent(code) -> np.ndarray:
    code = np.ascontiguousarray(code, dtype=np.uint32)
    out = np.zeros(len(code) + 2, dtype=np.uint32)
    check(lib().bbs_pruefer_to_parent_vector(_p(code), len(code), _p(out)))
    return out


def parent_to_matrix(parent):
    parent = np.ascontiguousarray(parent, dtype=np.uint32)
    n = len(parent)
    am = np.zeros((n, words(n)), dtype=np.uint64)
    dm = np.zeros((n, words(n)), dtype=np.uint64)
    check(lib().bbs_parent_vector_to_matrix(_p(parent), n, _p(am), _p(dm)))
    return am, dm


def matrix_to_parent(dm) -> np.ndarray:
    dm = np.ascontiguousarray(dm, dtype=np.uint64)
    out = np.zeros(dm.shape[0], dtype=np.uint32)
    check(lib().bbs_matrix_to_parent_vector(_p(dm), dm.shape[0], _p(out)))
    return out


def dm_to_am(dm) -> np.ndarray:
    dm = np.ascontiguousarray(dm, dtype=np.uint64)
    am = np.zeros_like(dm)
    check(lib().bbs_dm_to_am(_p(dm), dm.shape[0], _p(am)))
    return am


def _text(fn, parent) -> str:
    parent = np.ascontiguousarray(parent, dtype=np.uint32)
    n = C.c_size_t()
    check(fn(_p(parent), len(parent), None, 0, C.byref(n)))
    buf = C.create_string_buffer(n.value + 1)
    check(fn(_p(parent), len(parent), buf, n.value + 1, C.byref(n)))
    return buf.value.decode()


def to_graphviz(parent) -> str:
    return _text(lib().bbs_tree_to_graphviz, parent)


def to_newick(parent) -> str:
    return _text(lib().bbs_tree_to_newick, parent)


def random_parents(seed: int, n_genes: int, n_trees: int) -> np.ndarray:
    out = np.zeros((n_trees, n_genes + 1), dtype=np.uint32)
    check(lib().bbs_random_parent_vectors(seed, n_genes, n_trees, _p(out)))
    return out


def read_csv(path: str):
    nc, ng = C.c_uint32(), C.c_uint32()
    check(lib().bbs_read_csv(path.encode(), C.byref(nc), C.byref(ng), None,
                             None))
    W = words(ng.value + 1)
    mut = np.zeros((nc.value, W), dtype=np.uint64)
    known = np.zeros((nc.value, W), dtype=np.uint64)
    check(lib().bbs_read_csv(path.encode(), C.byref(nc), C.byref(ng),
                             _p(mut), _p(known)))
    return mut, known, nc.value, ng.value


def popc_peak():
    ops, clk = C.c_double(), C.c_double()
    check(lib().bbs_popc_peak(C.byref(ops), C.byref(clk)))
    return ops.value, clk.value


class Context:
    """One dataset on the GPU (Application + TreeScorer data side)."""

    def __init__(self, mut, known, n_cells: int, n_genes: int,
                 params: Params | None = None):
        self.params = params if params is not None else default_params()
        self.mut = np.ascontiguousarray(mut, dtype=np.uint64)
        self.known = np.ascontiguousarray(known, dtype=np.uint64)
        self.n_cells, self.n_genes = n_cells, n_genes
        self.n_nodes = n_genes + 1
        self.W = words(self.n_nodes)
        h = C.c_void_p()
        check(lib().bbs_create(C.byref(h), _p(self.mut), _p(self.known),
                               n_cells, n_genes, C.byref(self.params)))
        self._h = h
        self.n_chains = 0

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().bbs_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- chains --
    def init_chains(self, n_chains: int, parents=None) -> None:
        p = None
        if parents is not None:
            p = np.ascontiguousarray(parents, dtype=np.uint32)
            assert p.shape == (n_chains, self.n_nodes)
        check(lib().bbs_init_chains(self._h, n_chains, _p(p)))
        self.n_chains = n_chains

    def run(self, n_steps: int, moves=None, trace: bool = False):
        mv = None
        if moves is not None:
            mv = np.ascontiguousarray(moves, dtype=RAW_MOVE)
            assert mv.shape == (self.n_chains, n_steps)
        tr = (np.zeros((self.n_chains, n_steps), dtype=STEP_TRACE)
              if trace else None)
        check(lib().bbs_run(self._h, n_steps, _p(mv), _p(tr)))
        return tr

    def run_async(self, n_steps: int) -> None:
        check(lib().bbs_run_async(self._h, n_steps))

    def sync(self) -> None:
        check(lib().bbs_sync(self._h))

    def cancel(self) -> None:
        check(lib().bbs_cancel(self._h))

    def set_launch(self, cells_per_lane=0, warps_per_chain=0,
                   chains_per_block=0) -> None:
        check(lib().bbs_set_launch(self._h, cells_per_lane, warps_per_chain,
                                   chains_per_block))

    def launch(self) -> tuple:
        q, w, b = C.c_int(), C.c_int(), C.c_int()
        check(lib().bbs_get_launch(self._h, C.byref(q), C.byref(w),
                                   C.byref(b)))
        return q.value, w.value, b.value

    def autotune(self, probe_steps: int = 64) -> float:
        ms = C.c_float()
        check(lib().bbs_autotune(self._h, probe_steps, C.byref(ms)))
        return ms.value

    def last_run_ms(self) -> float:
        """Device time of the last run (CUDA events on the context's
        stream around the chain kernel)."""
        ms = C.c_float()
        check(lib().bbs_last_run_ms(self._h, C.byref(ms)))
        return ms.value

    def best(self) -> dict:
        n, W = self.n_nodes, self.W
        am = np.zeros((n, W), dtype=np.uint64)
        dm = np.zeros((n, W), dtype=np.uint64)
        parent = np.zeros(n, dtype=np.uint32)
        beta, score = C.c_float(), C.c_float()
        counts = np.zeros(4, dtype=np.uint64)
        chain = C.c_uint32()
        check(lib().bbs_get_best(self._h, _p(am), _p(dm), _p(parent),
                                 C.byref(beta), C.byref(score), _p(counts),
                                 C.byref(chain)))
        return dict(am=am, dm=dm, parent=parent, beta=beta.value,
                    score=score.value, counts=counts, chain=chain.value)

    def chains(self) -> dict:
        dm = np.zeros((self.n_chains, self.n_nodes, self.W), dtype=np.uint64)
        alpha = np.zeros(self.n_chains, dtype=np.float32)
        beta = np.zeros(self.n_chains, dtype=np.float32)
        score = np.zeros(self.n_chains, dtype=np.float32)
        counts = np.zeros((self.n_chains, 4), dtype=np.uint64)
        err = np.zeros((self.n_chains, 2), dtype=np.uint32)
        check(lib().bbs_get_chains(self._h, _p(dm), _p(alpha), _p(beta),
                                   _p(score), _p(counts), _p(err)))
        return dict(dm=dm, alpha=alpha, beta=beta, score=score,
                    counts=counts, err_stats=err)

    def treelist(self, max_trees: int = 128) -> dict:
        """Distinct trees tied with the best proposal (up to
        params.treelist_size per chain): dm (k x n x W), betas, score."""
        dm = np.zeros((max_trees, self.n_nodes, self.W), dtype=np.uint64)
        betas = np.zeros(max_trees, dtype=np.float32)
        score, k = C.c_float(), C.c_uint32()
        check(lib().bbs_get_treelist(self._h, max_trees, _p(dm), _p(betas),
                                     C.byref(score), C.byref(k)))
        return dict(dm=dm[:k.value], betas=betas[:k.value], score=score.value)

    def best_alpha(self) -> float:
        a = C.c_float()
        check(lib().bbs_get_best_alpha(self._h, C.byref(a)))
        return a.value

    def save_chains(self) -> bytes:
        """Every chain's state as one checkpoint image (bbs_save_chains)."""
        size = C.c_size_t()
        check(lib().bbs_save_chains(self._h, None, C.byref(size)))
        buf = C.create_string_buffer(size.value)
        check(lib().bbs_save_chains(self._h, buf, C.byref(size)))
        return buf.raw[:size.value]

    def load_chains(self, image: bytes) -> None:
        """Replaces the chains with those of a checkpoint image made with
        the same dataset and parameters (bbs_load_chains)."""
        check(lib().bbs_load_chains(self._h, image, len(image)))
        n = C.c_uint32()
        check(lib().bbs_get_sizes(self._h, None, None, C.byref(n)))
        self.n_chains = n.value

    # -- batch primitives --
    def score_trees(self, dm, betas, attach: bool = False):
        dm = np.ascontiguousarray(dm, dtype=np.uint64)
        n_trees = dm.shape[0]
        betas = np.ascontiguousarray(
            np.broadcast_to(np.asarray(betas, dtype=np.float32), (n_trees,)))
        scores = np.zeros(n_trees, dtype=np.float32)
        counts = np.zeros((n_trees, 4), dtype=np.uint64)
        att = (np.zeros((n_trees, self.n_cells), dtype=np.uint32)
               if attach else None)
        check(lib().bbs_score_trees(self._h, _p(dm), _p(betas), n_trees,
                                    _p(scores), _p(counts), _p(att)))
        return scores, counts, att

    def apply_moves(self, dm, betas, raw=None, params=None):
        dm = np.ascontiguousarray(dm, dtype=np.uint64)
        n_trees = dm.shape[0]
        betas = np.ascontiguousarray(
            np.broadcast_to(np.asarray(betas, dtype=np.float32), (n_trees,)))
        rw = (np.ascontiguousarray(raw, dtype=RAW_MOVE)
              if raw is not None else None)
        pr = (np.ascontiguousarray(params, dtype=MOVE_PARAMS)
              if params is not None else None)
        pout = np.zeros(n_trees, dtype=MOVE_PARAMS)
        out = np.zeros_like(dm)
        bout = np.zeros(n_trees, dtype=np.float32)
        check(lib().bbs_apply_moves(self._h, _p(dm), _p(betas), n_trees,
                                    _p(rw), _p(pr), _p(pout), _p(out),
                                    _p(bout)))
        return pout, out, bout

    def sumscore_grad(self, dm, alphas, betas, posterior: bool = False):
        dm = np.ascontiguousarray(dm, dtype=np.uint64)
        n_trees = dm.shape[0]
        al = np.ascontiguousarray(
            np.broadcast_to(np.asarray(alphas, dtype=np.float32), (n_trees,)))
        be = np.ascontiguousarray(
            np.broadcast_to(np.asarray(betas, dtype=np.float32), (n_trees,)))
        logl = np.zeros(n_trees, dtype=np.float32)
        da = np.zeros(n_trees, dtype=np.float32)
        db = np.zeros(n_trees, dtype=np.float32)
        post = (np.zeros((n_trees, self.n_cells, self.n_nodes),
                         dtype=np.float32) if posterior else None)
        check(lib().bbs_sumscore_grad(self._h, _p(dm), _p(al), _p(be),
                                      n_trees, _p(logl), _p(da), _p(db),
                                      _p(post)))
        return logl, da, db, post


class Batch:
    """Many datasets whose chains run in one launch per row width."""

    def __init__(self, datasets, params):
        """datasets: list of (mut, known, n_cells, n_genes); params: one
        Params or a list of one per dataset."""
        n = len(datasets)
        if isinstance(params, Params):
            params = [params] * n
        self._keep = []
        self.n_datasets = n
        self.n_cells = np.array([d[2] for d in datasets], dtype=np.uint32)
        self.n_genes = np.array([d[3] for d in datasets], dtype=np.uint32)
        muts = (C.c_void_p * n)()
        knowns = (C.c_void_p * n)()
        for i, (mut, known, _, _) in enumerate(datasets):
            mu = np.ascontiguousarray(mut, dtype=np.uint64)
            kn = np.ascontiguousarray(known, dtype=np.uint64)
            self._keep += [mu, kn]
            muts[i] = mu.ctypes.data
            knowns[i] = kn.ctypes.data
        parr = (Params * n)(*params)
        h = C.c_void_p()
        check(lib().bbs_batch_create(C.byref(h), n, _p(self.n_cells),
                                     _p(self.n_genes), muts, knowns, parr))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().bbs_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def init_chains(self, chains_per_dataset: int) -> None:
        check(lib().bbs_batch_init_chains(self._h, chains_per_dataset))

    def run(self, n_steps: int) -> None:
        check(lib().bbs_batch_run(self._h, n_steps))

    def last_run_ms(self) -> float:
        ms = C.c_float()
        check(lib().bbs_batch_last_run_ms(self._h, C.byref(ms)))
        return ms.value

    def set_launch(self, cells_per_lane=0, warps_per_block=0,
                   merge_rows=-1) -> None:
        check(lib().bbs_batch_set_launch(self._h, cells_per_lane,
                                         warps_per_block, merge_rows))

    def launch(self) -> tuple:
        q, w, m = C.c_int(), C.c_int(), C.c_int()
        check(lib().bbs_batch_get_launch(self._h, C.byref(q), C.byref(w),
                                         C.byref(m)))
        return q.value, w.value, m.value

    def set_chain_warps(self, warps_per_chain: int) -> None:
        check(lib().bbs_batch_set_chain_warps(self._h, warps_per_chain))

    def chain_warps(self) -> int:
        w = C.c_int()
        check(lib().bbs_batch_get_chain_warps(self._h, C.byref(w)))
        return w.value

    def autotune(self, probe_steps: int = 64) -> float:
        ms = C.c_float()
        check(lib().bbs_batch_autotune(self._h, probe_steps, C.byref(ms)))
        return ms.value

    def save_chains(self) -> bytes:
        """Every chain of every dataset as one checkpoint image."""
        size = C.c_size_t()
        check(lib().bbs_batch_save_chains(self._h, None, C.byref(size)))
        buf = C.create_string_buffer(size.value)
        check(lib().bbs_batch_save_chains(self._h, buf, C.byref(size)))
        return buf.raw[:size.value]

    def load_chains(self, image: bytes) -> None:
        """Replaces the chains with those of a checkpoint image made with
        the same datasets and parameters."""
        check(lib().bbs_batch_load_chains(self._h, image, len(image)))

    def best(self, dataset: int) -> dict:
        n = int(self.n_genes[dataset]) + 1
        dm = np.zeros((n, words(n)), dtype=np.uint64)
        parent = np.zeros(n, dtype=np.uint32)
        a, b, s = C.c_float(), C.c_float(), C.c_float()
        check(lib().bbs_batch_get_best(self._h, dataset, _p(dm), _p(parent),
                                       C.byref(a), C.byref(b), C.byref(s)))
        return dict(dm=dm, parent=parent, alpha=a.value, beta=b.value,
                    score=s.value)

