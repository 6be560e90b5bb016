"""ctypes access to the CPU oracle (test infrastructure only).

Loads oracle/liboracle.so (the C restatement in bbs_oracle.c) and, when it
was built, oracle/_ref/libbbs_ref.so (the reference's own headers compiled
against oracle/shim).  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline / reference arm import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libbbs_ref.so")

RAW_MOVE = np.dtype([("move_type", "<i4"), ("raw_v", "<u4"), ("raw_w", "<u4"),
                     ("raw_descendant_of_v", "<f4"),
                     ("raw_nondescendant_of_v", "<f4"),
                     ("beta_jump", "<f4"), ("acceptance_level", "<f4"),
                     ("pad_", "<u4")])
MOD_PARAMS = np.dtype([("move_type", "<i4"), ("v", "<u4"), ("w", "<u4"),
                       ("parent_of_v", "<u4"), ("parent_of_w", "<u4"),
                       ("descendant_of_v", "<u4"),
                       ("nondescendant_of_v", "<u4"), ("new_beta", "<f4")])
STEP_TRACE = np.dtype([("proposed_score", "<f4"), ("current_score", "<f4"),
                       ("current_beta", "<f4"), ("accepted", "<u4"),
                       ("ambiguous", "<u4"), ("pad_", "<u4"),
                       ("counts", "<u8", (4,))])

CHANGE_BETA, PRUNE_REATTACH, SWAP_NODES, SWAP_SUBTREES = range(4)


class _Scorer(C.Structure):
    _fields_ = [("l00", C.c_float), ("l01", C.c_float), ("l10", C.c_float),
                ("l11", C.c_float), ("bpriora", C.c_float),
                ("bpriorb", C.c_float)]


class _ChainParams(C.Structure):
    _fields_ = [("alpha_mean", C.c_float), ("beta_mean", C.c_float),
                ("beta_sd", C.c_float), ("gamma", C.c_float),
                ("score_mode", C.c_int32)]


class _MoveProbs(C.Structure):
    _fields_ = [("cum_beta", C.c_float), ("cum_prune", C.c_float),
                ("cum_swap", C.c_float), ("beta_jump_sd", C.c_float)]


def _foreign(path: str) -> bool:
    """True when `path` exists but was built for another machine."""
    import platform
    want = {"x86_64": 0x3E, "aarch64": 0xB7}.get(platform.machine())
    try:
        with open(path, "rb") as f:
            head = f.read(20)
    except OSError:
        return False
    return (want is not None and len(head) == 20
            and int.from_bytes(head[18:20], "little") != want)


def build(ref: bool = True) -> None:
    """Builds liboracle.so (and _ref when the reference sources exist)."""
    import shutil
    for path in (LIB_PATH, REF_PATH):
        if _foreign(path):
            os.unlink(path)
    if shutil.which("make"):
        target = "all" if ref else "oracle"
        subprocess.run(["make", "-s", "-C", HERE, target], check=True)
        return
    import platform
    arch = ["-mpopcnt"] if platform.machine() == "x86_64" else []
    subprocess.run(["gcc", "-O3", "-fPIC", "-ffp-contract=off", "-std=c11",
                    *arch, "-shared", "-o", LIB_PATH,
                    os.path.join(HERE, "bbs_oracle.c"), "-lm", "-lpthread"],
                   check=True)


_lib = None
_ref = None


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or _foreign(LIB_PATH):
            build(ref=False)
        _lib = C.CDLL(LIB_PATH)
        v = C.c_void_p
        u32, f32 = C.c_uint32, C.c_float
        _lib.orc_words.restype = u32
        _lib.orc_get_parent.restype = u32
        _lib.orc_get_n_descendants.restype = u32
        _lib.orc_get_n_ancestors.restype = u32
        _lib.orc_get_descendant_or_nondescendant.restype = u32
        _lib.orc_is_parent.restype = C.c_int
        _lib.orc_apply_move.restype = f32
        _lib.orc_apply_move.argtypes = [v, v, u32, f32, v, v, v]
        _lib.orc_realize_raw_move.argtypes = [v, v, u32, f32, v, v]
        _lib.orc_logscore_tree.restype = f32
        _lib.orc_logscore_tree.argtypes = [v, v, u32, v, v, u32, f32, v, v, v]
        _lib.orc_logscore_beta.restype = f32
        _lib.orc_logscore_beta.argtypes = [v, f32]
        _lib.orc_scorer_init.argtypes = [v, f32, f32, f32]
        _lib.orc_score_from_totals.restype = f32
        _lib.orc_score_from_totals.argtypes = [v, v, f32]
        _lib.orc_logscore_tree_f64.restype = C.c_double
        _lib.orc_logscore_tree_f64.argtypes = [
            C.c_double, C.c_double, C.c_double, C.c_double, v, u32, v, v,
            u32, C.c_int]
        _lib.orc_sumscore_grad_f64.restype = C.c_double
        _lib.orc_sumscore_grad_f64.argtypes = [
            C.c_double, C.c_double, v, u32, v, v, u32, v, v, v]
        for fn in ("orc_sumscore_counts_f64", "orc_maxscore_counts_f64"):
            getattr(_lib, fn).restype = C.c_double
            getattr(_lib, fn).argtypes = [C.c_double, C.c_double, v, u32, v,
                                          v, u32, v]
        _lib.orc_logprior_beta_f64.restype = C.c_double
        _lib.orc_logprior_beta_f64.argtypes = [C.c_double] * 3
        _lib.orc_run_chain.argtypes = [v, u32, v, v, u32, v, u32, v, v, v, v,
                                       v, v, v, v, v, v, v, f32]
        _lib.orc_philox4x32_10.argtypes = [v, v, v]
        _lib.orc_move_probs_from_params.argtypes = [v, f32, f32, f32, f32,
                                                    f32, f32]
        _lib.orc_sample_move.argtypes = [v, u32, C.c_uint64, u32, C.c_uint64,
                                         v]
        _lib.orc_run_chains_mt.restype = f32
        _lib.orc_run_chains_mt.argtypes = [v, v, C.c_uint64, u32, v, v, u32,
                                           v, u32, u32, u32, v]
        _lib.orc_cpu_scoring_proxy.restype = C.c_double
        _lib.orc_cpu_scoring_proxy.argtypes = [f32, f32, v, v, v, u32, u32,
                                               u32]
    return _lib


def ref_lib():
    """The reference's own classes, or None when they were not built."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        _ref = C.CDLL(REF_PATH)
        v = C.c_void_p
        u32, f32 = C.c_uint32, C.c_float
        _ref.ref_get_parent.restype = u32
        _ref.ref_realize.argtypes = [v, v, u32, f32, v, v]
        _ref.ref_apply.restype = f32
        _ref.ref_apply.argtypes = [v, v, u32, f32, v, v, v]
        _ref.ref_score.restype = f32
        _ref.ref_score.argtypes = [f32, f32, f32, u32, u32, v, v, v, f32]
        _ref.ref_logscore_beta.restype = f32
        _ref.ref_logscore_beta.argtypes = [f32, f32, f32, f32]
        _ref.ref_run_chain.argtypes = [f32, f32, f32, f32, u32, u32, v, v, v,
                                       u32, v, v, v, v, v, v, v, v, v, f32, v]
        _ref.ref_to_graphviz.argtypes = [v, v, u32, C.c_char_p, C.c_int]
        _ref.ref_to_newick.argtypes = [v, v, u32, C.c_char_p, C.c_int]
        _ref.ref_parse_args.argtypes = [C.c_int, v, v]
    return _ref


# ---------------------------------------------------------------------------
# numpy-level helpers
# ---------------------------------------------------------------------------

def words(n_nodes: int) -> int:
    return (n_nodes + 63) // 64


def pruefer_to_parent(code) -> np.ndarray:
    code = np.ascontiguousarray(code, dtype=np.uint32)
    parent = np.zeros(len(code) + 2, dtype=np.uint32)
    lib().orc_pruefer_to_parent_vector(_p(code), C.c_uint32(len(code)),
                                       _p(parent))
    return parent


def parent_to_matrix(parent):
    parent = np.ascontiguousarray(parent, dtype=np.uint32)
    n = len(parent)
    am = np.zeros((n, words(n)), dtype=np.uint64)
    dm = np.zeros((n, words(n)), dtype=np.uint64)
    lib().orc_parent_vector_to_matrix(_p(parent), C.c_uint32(n), _p(am),
                                      _p(dm))
    return am, dm


def get_parent(dm, x: int) -> int:
    n = dm.shape[0]
    return int(lib().orc_get_parent(_p(dm), C.c_uint32(n), C.c_uint32(x)))


def parent_vector(dm) -> np.ndarray:
    n = dm.shape[0]
    return np.array([get_parent(dm, x) for x in range(n)], dtype=np.uint32)


def n_descendants(am, x: int) -> int:
    return int(lib().orc_get_n_descendants(_p(am), C.c_uint32(am.shape[0]),
                                           C.c_uint32(x)))


def n_ancestors(dm, x: int) -> int:
    return int(lib().orc_get_n_ancestors(_p(dm), C.c_uint32(dm.shape[0]),
                                         C.c_uint32(x)))


def descendant_or_nondescendant(am, x: int, k: int, descendant: bool) -> int:
    """src/MutationTree.hpp:840-878: the k-th descendant (or non-descendant)
    of x, 0 when k is out of range."""
    return int(lib().orc_get_descendant_or_nondescendant(
        _p(am), C.c_uint32(am.shape[0]), C.c_uint32(x), C.c_uint32(k),
        C.c_int(1 if descendant else 0)))


def realize(am, dm, beta: float, raw) -> np.ndarray:
    out = np.zeros(1, dtype=MOD_PARAMS)
    raw = np.ascontiguousarray(np.asarray(raw, dtype=RAW_MOVE).reshape(1))
    lib().orc_realize_raw_move(_p(am), _p(dm), am.shape[0], beta, _p(raw),
                               _p(out))
    return out[0]


def apply_move(am, dm, beta: float, params):
    n = am.shape[0]
    params = np.ascontiguousarray(
        np.asarray(params, dtype=MOD_PARAMS).reshape(1))
    nam = np.zeros_like(am)
    ndm = np.zeros_like(dm)
    nb = lib().orc_apply_move(_p(am), _p(dm), n, beta, _p(params), _p(nam),
                              _p(ndm))
    return nam, ndm, float(nb)


def scorer(alpha: float, beta_mean: float, beta_sd: float) -> _Scorer:
    s = _Scorer()
    lib().orc_scorer_init(C.byref(s), alpha, beta_mean, beta_sd)
    return s


def logscore_tree(alpha, beta_mean, beta_sd, dm, mut, known, beta=None):
    """Returns (reference-order score, class-total score, counts[4],
    attachments)."""
    s = scorer(alpha, beta_mean, beta_sd)
    beta = beta_mean if beta is None else beta
    n_cells = mut.shape[0]
    counts = np.zeros(4, dtype=np.uint64)
    st = C.c_float()
    attach = np.zeros(n_cells, dtype=np.uint32)
    r = lib().orc_logscore_tree(C.byref(s), _p(dm), dm.shape[0], _p(mut),
                                _p(known), n_cells, beta, _p(counts),
                                C.byref(st), _p(attach))
    return float(r), float(st.value), counts, attach


def logscore_beta(alpha, beta_mean, beta_sd, beta) -> float:
    s = scorer(alpha, beta_mean, beta_sd)
    return float(lib().orc_logscore_beta(C.byref(s), beta))


def logscore_tree_f64(alpha, beta, dm, mut, known, beta_mean=None,
                      beta_sd=0.1, with_prior=False) -> float:
    bm = beta if beta_mean is None else beta_mean
    return float(lib().orc_logscore_tree_f64(
        alpha, beta, bm, beta_sd, _p(dm), dm.shape[0], _p(mut), _p(known),
        mut.shape[0], int(with_prior)))


def sumscore_grad_f64(alpha, beta, dm, mut, known, posterior=False):
    da, db = C.c_double(), C.c_double()
    post = (np.zeros((mut.shape[0], dm.shape[0]), dtype=np.float64)
            if posterior else None)
    r = lib().orc_sumscore_grad_f64(alpha, beta, _p(dm), dm.shape[0],
                                    _p(mut), _p(known), mut.shape[0],
                                    C.byref(da), C.byref(db), _p(post))
    return float(r), float(da.value), float(db.value), post


def score_counts_f64(alpha, beta, dm, mut, known, sum_score: bool):
    """FP64 (sum or max) score without prior and its (expected) class
    counts (n00, n01, n10, n11)."""
    e = np.zeros(4, dtype=np.float64)
    fn = (lib().orc_sumscore_counts_f64 if sum_score
          else lib().orc_maxscore_counts_f64)
    r = fn(alpha, beta, _p(dm), dm.shape[0], _p(mut), _p(known),
           mut.shape[0], _p(e))
    return float(r), e


def logprior_beta_f64(beta_mean, beta_sd, beta) -> float:
    return float(lib().orc_logprior_beta_f64(beta_mean, beta_sd, beta))


def move_probs(prob_beta_change=0.0, prob_prune=0.55, prob_swap=0.4,
               prob_subtrees=0.05, beta_sd=0.1, chi=10.0) -> _MoveProbs:
    mp = _MoveProbs()
    lib().orc_move_probs_from_params(C.byref(mp), prob_beta_change,
                                     prob_prune, prob_swap, prob_subtrees,
                                     beta_sd, chi)
    return mp


def sample_moves(mp, n_nodes: int, seed: int, chain: int, n_steps: int,
                 start: int = 0) -> np.ndarray:
    out = np.zeros(n_steps, dtype=RAW_MOVE)
    for i in range(n_steps):
        lib().orc_sample_move(C.byref(mp), n_nodes, C.c_uint64(seed), chain,
                              C.c_uint64(start + i),
                              out[i:i + 1].ctypes.data_as(C.c_void_p))
    return out


def philox(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    lib().orc_philox4x32_10(_p(c), _p(k), _p(o))
    return o


def run_chain(alpha, beta_mean, beta_sd, gamma, dm_parent, mut, known, moves,
              score_mode=1, beta=None, score=None, forced=None,
              ambiguity=0.0):
    """Replays recorded moves on one chain.  Returns a dict with the final
    state, the best proposal and the per-step trace."""
    am, dm = parent_to_matrix(dm_parent)
    n = am.shape[0]
    cp = _ChainParams(alpha, beta_mean, beta_sd, gamma, score_mode)
    beta = beta_mean if beta is None else beta
    if score is None:
        r, st, _, _ = logscore_tree(alpha, beta_mean, beta_sd, dm, mut, known,
                                    beta)
        score = st if score_mode else r
    b = C.c_float(beta)
    s = C.c_float(score)
    bv = C.c_int(0)
    best_am = np.zeros_like(am)
    best_dm = np.zeros_like(dm)
    bb, bs = C.c_float(), C.c_float()
    moves = np.ascontiguousarray(moves, dtype=RAW_MOVE)
    trace = np.zeros(len(moves), dtype=STEP_TRACE)
    forced_arr = (np.ascontiguousarray(forced, dtype=np.uint8)
                  if forced is not None else None)
    lib().orc_run_chain(C.byref(cp), n, _p(mut), _p(known), mut.shape[0],
                        _p(moves), len(moves), _p(am), _p(dm), C.byref(b),
                        C.byref(s), C.byref(bv), _p(best_am), _p(best_dm),
                        C.byref(bb), C.byref(bs), _p(trace), _p(forced_arr),
                        ambiguity)
    return dict(am=am, dm=dm, beta=b.value, score=s.value, best_am=best_am,
                best_dm=best_dm, best_beta=bb.value, best_score=bs.value,
                trace=trace)


def run_chains_mt(alpha, beta_mean, beta_sd, gamma, mp, seed, parents, mut,
                  known, n_steps, n_threads, score_mode=1):
    parents = np.ascontiguousarray(parents, dtype=np.uint32)
    n_chains, n = parents.shape
    cp = _ChainParams(alpha, beta_mean, beta_sd, gamma, score_mode)
    finals = np.zeros(n_chains, dtype=np.float32)
    best = lib().orc_run_chains_mt(C.byref(cp), C.byref(mp),
                                   C.c_uint64(seed), n, _p(mut), _p(known),
                                   mut.shape[0], _p(parents), n_chains,
                                   n_steps, n_threads, _p(finals))
    return float(best), finals


def cpu_proxy_scores(alpha, beta, mutq, knownq, dmq, reference=False):
    """Per-tree scores of the CPUTreeScorer proxy at 128 cells x 127 genes
    (mutq / knownq: [quadword][cell] words, dmq: trees x [quadword][node]),
    by the restatement or, with reference=True, by the reference's own
    class (None when oracle/_ref was not built)."""
    n = dmq.shape[0]
    out = np.zeros(n, dtype=np.float32)
    args = (C.c_float(alpha), C.c_float(beta), _p(mutq), _p(knownq), _p(dmq),
            C.c_uint32(n), _p(out))
    if reference:
        r = ref_lib()
        if r is None:
            return None
        r.ref_proxy_scores(*args)
    else:
        lib().orc_cpu_proxy_scores(*args)
    return out


def cpu_scoring_proxy(alpha, beta, mutq, knownq, dmq, n_trees, reps,
                      n_threads) -> float:
    return float(lib().orc_cpu_scoring_proxy(alpha, beta, _p(mutq),
                                             _p(knownq), _p(dmq), n_trees,
                                             reps, n_threads))
