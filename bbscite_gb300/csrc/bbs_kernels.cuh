// bbs_kernels.cuh -- kernel templates of the GB300 path.
//
//   mcmc_kernel   persistent chain runner, src/Application.hpp:398-496.
//                 A chain is one warp, or `wpc` warps that split its cells
//                 (the block is then that one chain).  The chain's current
//                 and proposed ancestor rows are double-buffered in shared
//                 memory; cell rows stay in registers (or are re-read per
//                 chunk for wide datasets).
//   score_kernel  TreeScorer::logscore_tree over a batch (warp per tree).
//   apply_kernel  realize_raw_move_sample + update ctor over a batch.
//   grad_kernel   sum-over-attachments score with its fused adjoint.
#pragma once
#include <cuda_runtime.h>

#include <cmath>

#include "bbs_device.cuh"

namespace bbs {

// Rows x = 32 r + lane for the node groups r owned by warp `wic` of `wpc`.
template <int W32>
__device__ __forceinline__ void copy_rows_part(const uint32_t *src,
                                               uint32_t *dst, int n, int wpc,
                                               int wic, int lane) {
  constexpr int RS = rs_of_w32(W32);
  for (int r = wic; r < W32; r += wpc) {
    const int x = 32 * r + lane;
    if (x < n) {
      uint32_t v[W32];
      ld_row<W32>(src + x * RS, v);
      st_row<W32>(dst + x * RS, v);
    }
  }
}

template <int W32>
__device__ __forceinline__ void copy_rows(const uint32_t *src, uint32_t *dst,
                                          int n, int lane) {
  copy_rows_part<W32>(src, dst, n, 1, 0, lane);
}

// The scratch pieces of a slot: parent vectors and warp wic's scratch.
// (Host-callable too: the layout test walks it over every shape.)
struct SlotSum {
  uint8_t *par0, *par1;
  SumCtx sx;
};

__host__ __device__ __forceinline__ SlotSum slot_sum(uint8_t *slot, int n,
                                                     int rs, int wpc, int wic,
                                                     int w32, int q,
                                                     bool counts) {
  SlotSum o{};
  uint8_t *p = slot + slot_head_bytes(n, rs, wpc);
  o.par0 = p;
  o.par1 = p + n;
  p += align16(2 * n) + wic * sum_warp_bytes(n, w32, q, counts);
  o.sx.ord = reinterpret_cast<uint16_t *>(p);
  p += align16(2 * n);
  o.sx.hist = reinterpret_cast<int *>(p);
  p += align16(4 * 32 * ((n + 31) / 32));
  if (counts && w32 <= 4) o.sx.cnt = reinterpret_cast<uint32_t *>(p);
  if (counts && w32 > 4) {
    o.sx.ring = reinterpret_cast<uint32_t *>(p);
    o.sx.gt = reinterpret_cast<uint32_t *>(p + align16(ring_bytes(q)));
  }
  return o;
}

// The block's increment tables: for warp part wic of wpc and lane l, the
// cells c = 32 wic + 32 wpc q + l (q < Q; zero past the dataset's cells),
// as load_cells takes them; gene j's entry packs D bit | M bit << 8 of each
// such cell as the count table packs counts.  Cell rows are read with the
// stride rs that load_cells uses.
template <int Q>
__device__ __forceinline__ void build_increments(uint8_t *table, int wpc,
                                                 const DatasetDev &ds, int rs) {
  constexpr int NW = kPackWords<Q>;
  const int n = ds.n_nodes;
  for (int idx = threadIdx.x; idx < wpc * n * 32; idx += blockDim.x) {
    const int wic = idx / (n * 32);
    const int rem = idx - wic * n * 32;
    const int j = rem >> 5, l = rem & 31;
    uint32_t k[NW];
#pragma unroll
    for (int w = 0; w < NW; w++) k[w] = 0u;
#pragma unroll
    for (int q = 0; q < Q; q++) {
      const int c = 32 * wic + 32 * wpc * q + l;
      uint32_t v = 0;
      if (c < ds.n_cells) {
        const uint32_t kw = __ldg(ds.K + (size_t)c * rs + (j >> 5));
        const uint32_t mw = __ldg(ds.M + (size_t)c * rs + (j >> 5));
        const uint32_t bit = 1u << (j & 31);
        v = ((kw & ~mw & bit) ? 1u : 0u) | ((mw & bit) ? 256u : 0u);
      }
      k[q >> 1] |= v << (16 * (q & 1));
    }
    st_pack<Q>(reinterpret_cast<uint32_t *>(table + (size_t)wic * inc_table_bytes(n, Q)),
               j * 32 + l, k);
  }
}

// Evaluates a tree for the whole chain (all wpc warps): returns the score
// S = data term + prior and the (exact or expected) class counts e[4];
// sk, sm are the class sums of the max score and smax the max score itself
// (S for the max score; for the sum score, sum_c max_j s_cj + prior).
template <int W32, int Q, bool SUM>
__device__ __forceinline__ float evaluate(const uint32_t *rows, int n,
                                          const DatasetDev &ds,
                                          Cells<W32, Q> &cb, bool resident,
                                          const LogTable &L, float prior,
                                          int wpc, int wic, int lane,
                                          int *part, int parity,
                                          const SumCtx &sx,
                                          float (&e)[4], int &sk, int &sm,
                                          float &smax) {
  if constexpr (!SUM) {
    int a, b;
    score_part<W32, Q>(rows, n, ds, cb, resident, L, wpc, wic, lane, a, b, sx);
    if (wpc > 1) {
      int *pp = part + parity * 12 * wpc;
      if (lane == 0) {
        pp[12 * wic] = a;
        pp[12 * wic + 1] = b;
      }
      __syncthreads();
      a = b = 0;
      for (int w = 0; w < wpc; w++) {
        a += pp[12 * w];
        b += pp[12 * w + 1];
      }
    }
    sk = a;
    sm = b;
    int N[4];
    class_totals(ds, sk, sm, N);
#pragma unroll
    for (int i = 0; i < 4; i++) e[i] = (float)N[i];
    smax = tree_score(ds, sk, sm, L, prior);
    return smax;
  } else {
    long long acc[6];
    sum_part<W32, Q>(rows, n, ds, cb, resident, L, wpc, wic, lane, acc, sx);
    if (wpc > 1) {
      long long *pp = reinterpret_cast<long long *>(part) + parity * 6 * wpc;
      if (lane == 0)
        for (int i = 0; i < 6; i++) pp[6 * wic + i] = acc[i];
      __syncthreads();
      for (int i = 0; i < 6; i++) acc[i] = 0;
      for (int w = 0; w < wpc; w++)
        for (int i = 0; i < 6; i++) acc[i] += pp[6 * w + i];
    }
    complete_expected_counts(ds, acc);
    sk = sm = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) e[i] = ll_to_float(acc[i + 1]) * (1.0f / kFixScale);
    smax = __fadd_rn(ll_to_float(acc[5]) * (1.0f / kScoreScale), prior);
    return __fadd_rn(ll_to_float(acc[0]) * (1.0f / kScoreScale), prior);
  }
}

// One chain for n_steps steps: src/Application.hpp:408-487 with the
// error-rate move chosen by md.error_move.  `chain_id` keys the Philox
// stream.  All wpc warps of the chain run this with the same arguments.
template <int W32, int Q, bool SUM>
__device__ __forceinline__ void run_chain(
    const DatasetDev &ds, const ModelDev &md, uint32_t chain_id,
    uint32_t *g, uint32_t *gbest, uint64_t *lhash, float *lbeta, int K,
    ChainState *gstate,
    const bbs_raw_move *moves, bbs_step_trace *trace, int n_steps,
    const volatile int *cancel, int *status, uint32_t *buf0, uint32_t *buf1,
    int *part, volatile int *sflag, uint4 *pbuf, const SlotSum &ss,
    Cells<W32, Q> &cb, bool resident, int wpc, int wic, int lane) {
  const int n = ds.n_nodes;
  const bool multi = wpc > 1;
  const ChainState st = *gstate;
  copy_rows_part<W32>(g, buf0, n, wpc, wic, lane);
  if (multi) __syncthreads(); else __syncwarp();
  uint32_t *cur = buf0, *prop = buf1;
  // Inherited counts (rows of up to four words): the parent vectors of the
  // current tree and of the proposal follow the rows.  A parent vector is
  // used only after it has been checked against its rows: a realised move
  // whose k-th (non)descendant fell back to node 0 (the reference's rule
  // when floor(u * count) reaches the count) changes the rows in a way the
  // parent-vector form does not follow, and may leave rows that are no tree.
  // Such trees are scored with masked popcounts, which take any rows.
  // Rows of five to eight words inherit through the ring, which needs the
  // parent vectors too (any cells, resident or streamed).
  uint8_t *cpar = nullptr, *ppar = nullptr;
  bool cur_par_ok = false;  // cpar describes cur
  const bool track = W32 <= 4 ? ss.sx.inc != nullptr && resident
                              : ss.sx.ring != nullptr;
  if (track) {
    cpar = ss.par0;
    ppar = ss.par1;
    if (wic == 0) derive_parents<W32>(cur, n, cpar, ss.sx.hist, lane);
    if (multi) __syncthreads(); else __syncwarp();
    cur_par_ok = parents_match_rows<W32>(cur, n, cpar, lane);
  }
  SumCtx sx = ss.sx;
  float alpha = st.alpha, beta = st.beta, score = st.score, prior = st.prior;
  LogTable L{st.l00, st.l10, st.l01, st.l11};
  float ec[4] = {st.ec[0], st.ec[1], st.ec[2], st.ec[3]};
  int csk = st.sk, csm = st.sm;
  bool has_best = st.has_best != 0;
  float best_score = st.best_score, best_alpha = st.best_alpha,
        best_beta = st.best_beta;
  int bsk = st.best_sk, bsm = st.best_sm;
  uint32_t err_prop = st.err_proposed, err_acc = st.err_accepted;
  uint32_t lcount = st.list_count;  // co-optimal trees listed (K > 1)
  const bool learn = md.error_move != 0;
  int i = 0;
  bool cancelled = false;
  for (; i < n_steps; i++) {
    if (cancel != nullptr && (i & 255) == 0) {
      // one reader, then a chain-uniform decision
      if (wic == 0 && lane == 0) *sflag = *cancel;
      if (multi) __syncthreads(); else __syncwarp();
      const int c = *sflag;
      if (multi) __syncthreads(); else __syncwarp();
      if (c) {
        cancelled = true;
        break;
      }
    }
    // Philox blocks of the next 16 steps (a warp-uniform condition; the
    // previous step's reads ended at its closing __syncwarp)
    if (moves == nullptr && (i & 15) == 0) {
      philox_fill(pbuf, md.seed, chain_id, st.steps_done + (uint64_t)i, lane);
      __syncwarp();
    }
    const bbs_raw_move raw =
        moves != nullptr
            ? moves[i]
            : move_from_words(md.mp, (uint32_t)n, pbuf[2 * (i & 15)],
                              pbuf[2 * (i & 15) + 1], trace != nullptr);
    const bool err_move = raw.move_type == BBS_MOVE_CHANGE_BETA;
    float palpha = alpha, pbeta = beta, pprior = prior;
    LogTable PL = L;
    const uint32_t *scored = cur;
    float corr = 1.0f;
    float fa = 0.0f, fb = 0.0f, ta = 0.0f, tb = 0.0f;
    ErrorGeom geo{};  // of the current state, on learned error moves
    bool fallback_move = false;  // the realised move took node 0 by fallback
    uint32_t Dv[W32], Dw[W32];
    if (!err_move) {
      const Realized R = realize_move<W32>(cur, n, beta, raw, lane, Dv, Dw);
      const uint32_t top = max(max(max(R.p.v, R.p.w), max(R.p.parent_of_v, R.p.parent_of_w)),
                               max(R.p.descendant_of_v, R.p.nondescendant_of_v));
      if (!device_check(top < (uint32_t)n, status, kCheckMoveNode, top, (uint32_t)n)) {
        cancelled = true;  // the chain stops where it is
        break;
      }
      build_proposal<W32>(cur, prop, n, R.p, Dv, Dw, R.related, wpc, wic,
                          lane);
      fallback_move = R.fallback;
      if (cur_par_ok && wic == 0)
        propose_parents(cpar, ppar, n, R.p, R.related, lane);
      scored = prop;
      // src/Application.hpp:443-450
      if (raw.move_type == BBS_MOVE_SWAP_SUBTREES && R.related)
        corr = __fdiv_rn((float)R.ndv, (float)R.ndw);
    } else if (!learn) {
      // reference ChangeBeta: beta + jump reflected into [0, 1]
      // (src/MutationTree.hpp:345-351)
      float nb = __fadd_rn(beta, raw.beta_jump);
      if (nb < 0.0f) nb = fabsf(nb);
      if (nb > 1.0f) nb = __fsub_rn(nb, __fmul_rn(2.0f, __fsub_rn(nb, 1.0f)));
      pbeta = nb;
      beta_terms(ds, pbeta, PL.l01, PL.l11, pprior);
    } else {
      // (preconditioned) random walk or Langevin step in logit space, with
      // the geometry of the current state from its class counts
      geo = error_geometry(ds, alpha, beta, md.gamma, ec);
      float z0, z1;
      error_normals(raw, z0, z1);
      const float eps = md.error_step;
      const float h = md.error_move == 2 ? 0.5f * eps * eps : 0.0f;
      fa = logit(alpha);
      fb = logit(beta);
      ta = fa + h * geo.prec_a * geo.grad_a + eps * sqrtf(geo.prec_a) * z0;
      tb = fb + h * geo.prec_b * geo.grad_b + eps * sqrtf(geo.prec_b) * z1;
      palpha = fminf(fmaxf(sigmoid(ta), 1.0e-7f), 1.0f - 1.0e-7f);
      pbeta = fminf(fmaxf(sigmoid(tb), 1.0e-7f), 1.0f - 1.0e-7f);
      ta = logit(palpha);
      tb = logit(pbeta);
      alpha_terms_f(palpha, PL.l00, PL.l10);
      beta_terms_f(ds, pbeta, PL.l01, PL.l11, pprior);
    }
    if (multi) __syncthreads(); else __syncwarp();
    // The evaluated tree's parent vector.  It is checked against the rows
    // where it can be wrong -- a proposal whose move took node 0 by
    // fallback -- and used only where it checks out; checked builds check
    // every one and record a mismatch outside that case as a failed device
    // check.
    bool par_ok = false;
    if (cpar != nullptr && cur_par_ok) {
      const bool suspect = scored != cur && fallback_move;
      bool check = suspect;
#ifdef BBS_CHECKED
      check = true;
#endif
      par_ok = true;
      if (check) {
        par_ok = parents_match_rows<W32>(scored, n,
                                         scored == cur ? cpar : ppar, lane);
#ifdef BBS_CHECKED
        if (!suspect)
          device_check(par_ok, status, kCheckParent,
                       (uint32_t)raw.move_type, 4u);
#endif
      }
    }
    sx.par = par_ok ? (scored == cur ? cpar : ppar) : nullptr;
    const bool prop_par_ok = par_ok && scored != cur;
    float e[4], psmax;
    int sk, sm;
    const float pscore = evaluate<W32, Q, SUM>(scored, n, ds, cb, resident, PL,
                                               pprior, wpc, wic, lane, part,
                                               i & 1, sx, e, sk, sm, psmax);
    bool accept;
    if (err_move && learn) {
      const ErrorGeom pgeo = error_geometry(ds, palpha, pbeta, md.gamma, e);
      const float logj = logf(alpha * (1.0f - alpha)) + logf(beta * (1.0f - beta));
      const float plogj =
          logf(palpha * (1.0f - palpha)) + logf(pbeta * (1.0f - pbeta));
      const bool drift = md.error_move == 2;
      const float logr = md.gamma * (pscore - score) + plogj - logj +
                         log_q(fa, fb, ta, tb, pgeo, md.error_step, drift) -
                         log_q(ta, tb, fa, fb, geo, md.error_step, drift);
      accept = logr > logf(raw.acceptance_level);
      err_prop++;
      if (accept) err_acc++;
    } else {
      // src/Application.hpp:452-455
      const float ratio = __fmul_rn(
          corr, expf(__fmul_rn(__fsub_rn(pscore, score), md.gamma)));
      accept = ratio > raw.acceptance_level;
      if (err_move) {
        err_prop++;
        if (accept) err_acc++;
      }
    }
    // src/Application.hpp:456, best over proposals by the reference's max
    // score (the chain's own score unless it samples the sum score)
    if (!has_best || psmax > best_score) {
      has_best = true;
      best_score = psmax;
      best_alpha = palpha;
      best_beta = pbeta;
      bsk = sk;
      bsm = sm;
      copy_rows_part<W32>(scored, gbest, n, wpc, wic, lane);
      if (K > 1) {
        // a new best: the co-optimal list restarts with it
        const uint64_t h = tree_hash<W32>(scored, n, lane);
        if (wic == 0 && lane == 0) {
          lhash[0] = h;
          lbeta[0] = pbeta;
        }
        lcount = 1;
      }
    } else if (K > 1 && psmax == best_score && lcount < (uint32_t)K) {
      // a tie with the best: listed when it is a tree not listed yet
      const uint64_t h = tree_hash<W32>(scored, n, lane);
      const bool seen =
          __any_sync(BBS_FULL_MASK, lane < (int)lcount && lhash[lane] == h);
      if (!seen) {
        copy_rows_part<W32>(scored, gbest + (size_t)lcount * n * rs_of_w32(W32),
                            n, wpc, wic, lane);
        if (wic == 0 && lane == 0) {
          lhash[lcount] = h;
          lbeta[lcount] = pbeta;
        }
        lcount++;
      }
    }
    if (trace != nullptr && wic == 0 && lane == 0) {
      bbs_step_trace *t = trace + i;
      t->move = raw;
      t->proposed_score = pscore;
      t->current_score = accept ? pscore : score;
      t->proposed_beta = pbeta;
      t->accepted = accept ? 1u : 0u;
      t->proposed_alpha = palpha;
      t->proposed_max_score = psmax;
#pragma unroll
      for (int k = 0; k < 2; k++) t->reserved[k] = 0;
#pragma unroll
      for (int k = 0; k < 4; k++)
        t->proposed_counts[k] = SUM ? 0ull : (uint64_t)e[k];
    }
    if (accept) {
      if (!err_move) {
        uint32_t *t = cur;
        cur = prop;
        prop = t;
        uint8_t *tp = cpar;
        cpar = ppar;
        ppar = tp;
        cur_par_ok = prop_par_ok;
        if (cpar != nullptr && !cur_par_ok) {
          // the new tree's own parent vector, where its rows are a tree
          if (multi) __syncthreads(); else __syncwarp();
          if (wic == 0) derive_parents<W32>(cur, n, cpar, ss.sx.hist, lane);
          if (multi) __syncthreads(); else __syncwarp();
          cur_par_ok = parents_match_rows<W32>(cur, n, cpar, lane);
        }
      }
      alpha = palpha;
      beta = pbeta;
      score = pscore;
      prior = pprior;
      L = PL;
#pragma unroll
      for (int k = 0; k < 4; k++) ec[k] = e[k];
      csk = sk;
      csm = sm;
    }
    __syncwarp();
  }
  copy_rows_part<W32>(cur, g, n, wpc, wic, lane);
  if (wic == 0 && lane == 0) {
    ChainState o = st;
    o.alpha = alpha;
    o.beta = beta;
    o.score = score;
    o.prior = prior;
    o.l00 = L.l00;
    o.l10 = L.l10;
    o.l01 = L.l01;
    o.l11 = L.l11;
#pragma unroll
    for (int k = 0; k < 4; k++) o.ec[k] = ec[k];
    o.sk = csk;
    o.sm = csm;
    o.has_best = has_best ? 1u : 0u;
    o.best_alpha = best_alpha;
    o.best_beta = best_beta;
    o.best_score = best_score;
    o.best_sk = bsk;
    o.best_sm = bsm;
    o.steps_done = st.steps_done + (uint64_t)i;
    o.err_proposed = err_prop;
    o.err_accepted = err_acc;
    o.list_count = lcount;
    *gstate = o;
    if (cancelled && status != nullptr) atomicOr(status, 1);
  }
  if (multi) __syncthreads(); else __syncwarp();
}

// Launch bounds of each cells-per-lane variant (bbs_layout.h).
template <int Q>
struct ChainBounds {
  static constexpr int threads = chain_max_threads(Q);
  static constexpr int min_blocks = chain_min_blocks(Q);
};

// One dataset: chains 0..n_chains-1, one warp per chain (blocks of `cpb`
// chains) or wpc warps per chain (the block is one chain).  REC: recorded
// moves and/or a step trace (replays and tests); without them the move and
// trace paths compile away.
template <int W32, int Q, bool SUM, bool REC>
__global__ void __launch_bounds__(ChainBounds<Q>::threads,
                                  ChainBounds<Q>::min_blocks)
    mcmc_kernel(const RunArgs a) {
  extern __shared__ __align__(16) uint32_t smem[];
  constexpr int RS = rs_of_w32(W32);
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const int wpc = a.wpc;
  const int cpb = wpb / wpc;
  const int slot = wib / wpc, wic = wib - slot * wpc;
  const int n = a.ds.n_nodes;
  // rows of five to eight words stream their cells per evaluation (their
  // counts come through the ring and a gene table built per chunk)
  const bool resident = W32 <= 4 && a.ds.n_cells <= 32 * wpc * Q;
  // the same decisions as the launcher's, for the whole block
  const bool counts = inherits_counts(W32, a.ds.n_cells, 32 * wpc * Q);
  const bool scratch = SUM || counts;
  const int sb = slot_bytes(n, RS, wpc, scratch, W32, Q, counts);
  uint8_t *slot_base = reinterpret_cast<uint8_t *>(smem) + (size_t)slot * sb;
  uint32_t *buf0 = reinterpret_cast<uint32_t *>(slot_base);
  uint32_t *buf1 = buf0 + n * RS;
  int *part = reinterpret_cast<int *>(buf0 + 2 * n * RS);
  volatile int *sflag = part + 24 * wpc;
  uint4 *pbuf = reinterpret_cast<uint4 *>(
      slot_base + 4 * (2 * n * RS + 24 * wpc + 4) + kPhiloxBytes * wic);
  Cells<W32, Q> cb;
  if (resident) load_cells<W32, Q>(cb, a.ds, 32 * wic, 32 * wpc, lane);
  SlotSum ss{};
  if (scratch) {
    ss = slot_sum(slot_base, n, RS, wpc, wic, W32, Q, counts);
    if constexpr (W32 <= 4) {
      if (counts) {
        uint8_t *table = reinterpret_cast<uint8_t *>(smem) + (size_t)cpb * sb;
        build_increments<Q>(table, wpc, a.ds, RS);
        __syncthreads();
        ss.sx.inc = reinterpret_cast<const uint32_t *>(
            table + (size_t)wic * inc_table_bytes(n, Q));
      }
    }
  }
  for (int chain = blockIdx.x * cpb + slot; chain < a.n_chains;
       chain += gridDim.x * cpb) {
    const bbs_raw_move *moves = nullptr;
    bbs_step_trace *trace = nullptr;
    if constexpr (REC) {
      if (a.moves != nullptr) moves = a.moves + (size_t)chain * a.n_steps;
      if (a.trace != nullptr) trace = a.trace + (size_t)chain * a.n_steps;
    }
    const int K = a.list_hash != nullptr ? a.md.treelist : 1;
    run_chain<W32, Q, SUM>(
        a.ds, a.md, (uint32_t)chain, a.rows + (size_t)chain * n * RS,
        a.best_rows + (size_t)chain * K * n * RS,
        K > 1 ? a.list_hash + (size_t)chain * K : nullptr,
        K > 1 ? a.list_beta + (size_t)chain * K : nullptr, K, a.states + chain,
        moves, trace,
        a.n_steps, a.cancel, a.status, buf0, buf1, part, sflag, pbuf, ss, cb,
        resident, wpc, wic, lane);
  }
}

// One work unit of the batched launch: chain `chain` of dataset `d`, run
// by the wpc warps of its slot (warp wic of them).
template <int W32, int Q, bool SUM>
__device__ __forceinline__ void batch_unit(const BatchArgs &b,
                                           const DatasetDev &ds,
                                           const ModelDev &md, uint32_t chain,
                                           uint32_t d, uint32_t *buf0,
                                           int *part, volatile int *sflag,
                                           uint4 *pbuf, const SlotSum &ss_in,
                                           Cells<W32, Q> &cb, int wpc,
                                           int wic, int lane) {
  constexpr int RS = rs_of_w32(W32);
  // the dataset's node count is within this launch's row width
  uint32_t *buf1 = buf0 + ds.n_nodes * RS;
  // rows of five to eight words stream their cells per evaluation (their
  // counts come through the ring and a gene table built per chunk)
  const bool resident = W32 <= 4 && ds.n_cells <= 32 * wpc * Q;
  if (resident) load_cells<W32, Q>(cb, ds, 32 * wic, 32 * wpc, lane);
  const uint64_t off = b.chain_off[chain];
  // Philox key: the chain's number within its dataset, so a dataset's
  // chains draw the same moves here as in a one-dataset run.
  const uint32_t local = chain - d * (uint32_t)b.chains_per_dataset;
  // the increment table holds the cells of dataset b.table_ds only
  SlotSum ss = ss_in;
  if ((int)d != b.table_ds) ss.sx.inc = nullptr;
  run_chain<W32, Q, SUM>(ds, md, local, b.rows + off, b.best_rows + off,
                         nullptr, nullptr, 1, b.states + chain, nullptr,
                         nullptr, b.n_steps, b.cancel, b.status, buf0, buf1,
                         part, sflag, pbuf, ss, cb, resident, wpc, wic, lane);
}

// Many datasets: warps take chains from a shared work list (costliest
// first); each chain brings its own dataset and rules.  One warp per chain
// (blocks of one-warp slots), or wpc warps per chain (the block is one
// slot and takes its chains together).
// Rows of five to eight words leave the register count free (up to 255):
// a one-warp slot there takes about 31 KB of shared memory, so at most 7
// such blocks fit an SM whatever their registers, and with the tighter
// bound of two cells per lane (168) the sum score's kernel spilled
// (measured at 255 x 512: 7.5 M against 6.7 M chain-steps/s).
// MULTI: chains of b.wpc > 1 warps; without it every chain is one warp,
// known at compile time.
template <int W32, int Q, bool SUM, bool MULTI>
__global__ void __launch_bounds__(ChainBounds<Q>::threads,
                                  W32 > 4 ? 1 : ChainBounds<Q>::min_blocks)
    batch_kernel(const BatchArgs b) {
  extern __shared__ __align__(16) uint32_t smem[];
  constexpr int RS = rs_of_w32(W32);
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpc = MULTI ? b.wpc : 1;
  const int slot = wib / wpc, wic = wib - slot * wpc;
  // inherited counts (the host's decision, the same in every thread)
  const bool counts = b.with_counts != 0;
  const bool scratch = SUM || counts;
  const int sb = slot_bytes(b.max_nodes, RS, wpc, scratch, W32, Q, counts);
  uint8_t *slot_base = reinterpret_cast<uint8_t *>(smem) + (size_t)slot * sb;
  uint32_t *buf0 = reinterpret_cast<uint32_t *>(slot_base);
  int *part = reinterpret_cast<int *>(buf0 + 2 * b.max_nodes * RS);
  volatile int *sflag = part + 24 * wpc;
  // the slot's next unit, shared by its warps (the flag words' second)
  volatile unsigned int *sunit =
      reinterpret_cast<volatile unsigned int *>(sflag + 1);
  uint4 *pbuf = reinterpret_cast<uint4 *>(
      slot_base + 4 * (2 * b.max_nodes * RS + 24 * wpc + 4) +
      kPhiloxBytes * wic);
  SlotSum ss{};
  if (scratch) {
    ss = slot_sum(slot_base, b.max_nodes, RS, wpc, wic, W32, Q, counts);
    if constexpr (W32 <= 4) {
      if (counts) {
        // one increment table per warp part of a chain (the launch's one
        // dataset)
        uint8_t *table = reinterpret_cast<uint8_t *>(smem) +
                         (size_t)((blockDim.x >> 5) / wpc) * sb;
        const DatasetDev &tds = b.ds[b.table_ds];
        build_increments<Q>(table, wpc, tds, RS);
        __syncthreads();
        ss.sx.inc = reinterpret_cast<const uint32_t *>(
            table + (size_t)wic * inc_table_bytes(tds.n_nodes, Q));
      }
    }
  }
  Cells<W32, Q> cb;
  for (;;) {
    unsigned int unit = 0;
    if constexpr (!MULTI) {
      if (lane == 0) unit = atomicAdd(b.next_unit, 1u);
      unit = __shfl_sync(BBS_FULL_MASK, unit, 0);
    } else {
      // the block's warps take each unit together (the previous unit's
      // reads of *sunit ended before the first barrier)
      __syncthreads();
      if (threadIdx.x == 0) *sunit = atomicAdd(b.next_unit, 1u);
      __syncthreads();
      unit = *sunit;
    }
    if (unit >= (unsigned int)b.n_units) break;
    const uint32_t chain = b.units[unit];
    if (!device_check(chain < (uint32_t)b.n_chains, b.status, kCheckUnit, chain,
                      (uint32_t)b.n_chains))
      continue;
    const uint32_t d = b.chain_ds[chain];
    if (!device_check(d < (uint32_t)b.n_datasets, b.status, kCheckDataset, d,
                      (uint32_t)b.n_datasets))
      continue;
    // The sum score reads the dataset and model tables in place (fewer
    // registers, measured faster); the max score keeps register copies
    // (measured faster there).
    if constexpr (SUM) {
      batch_unit<W32, Q, SUM>(b, b.ds[d], b.md[d], chain, d, buf0, part,
                              sflag, pbuf, ss, cb, wpc, wic, lane);
    } else {
      const DatasetDev ds = b.ds[d];
      const ModelDev md = b.md[d];
      batch_unit<W32, Q, SUM>(b, ds, md, chain, d, buf0, part, sflag, pbuf,
                              ss, cb, wpc, wic, lane);
    }
  }
}

// Initial chain states: each chain's tree evaluated at (alpha_mean,
// beta_mean); one warp per chain.
template <int W32, int Q, bool SUM>
__global__ void __launch_bounds__(128) init_kernel(const InitArgs a) {
  extern __shared__ __align__(16) uint32_t smem[];
  constexpr int RS = rs_of_w32(W32);
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const int idx = blockIdx.x * wpb + wib;
  if (idx >= a.n_chains) return;  // whole warp
  const int chain = a.chain_list != nullptr ? (int)a.chain_list[idx] : idx;
  const uint32_t d = a.chain_ds != nullptr ? a.chain_ds[chain] : 0u;
  const DatasetDev ds = a.ds[d];
  const ModelDev md = a.md[d];
  const int n = ds.n_nodes;
  const uint64_t off = a.chain_off != nullptr ? a.chain_off[chain]
                                              : (uint64_t)chain * n * RS;
  // per warp: the tree's rows, then (sum score) the canonical order and
  // its histogram
  const int wb = 4 * a.max_nodes * RS +
                 (SUM ? align16(2 * a.max_nodes) + align16(4 * 32 * ((a.max_nodes + 31) / 32)) : 0);
  uint8_t *mine = reinterpret_cast<uint8_t *>(smem) + (size_t)wib * wb;
  uint32_t *rows = reinterpret_cast<uint32_t *>(mine);
  SumCtx sx{};
  if constexpr (SUM) {
    sx.ord = reinterpret_cast<uint16_t *>(mine + 4 * a.max_nodes * RS);
    sx.hist = reinterpret_cast<int *>(mine + 4 * a.max_nodes * RS + align16(2 * a.max_nodes));
  }
  copy_rows<W32>(a.rows + off, rows, n, lane);
  __syncwarp();
  const float *tm = a.terms + 8 * (size_t)d;
  const LogTable L{tm[2], tm[3], tm[4], tm[5]};
  const float alpha = tm[0], beta = tm[1], prior = tm[6];
  Cells<W32, Q> cb;
  float e[4], smax;
  int sk, sm;
  const float S = evaluate<W32, Q, SUM>(rows, n, ds, cb, false, L, prior, 1, 0,
                                        lane, nullptr, 0, sx, e, sk, sm, smax);
  if (lane == 0) {
    ChainState o;
    o.alpha = alpha;
    o.beta = beta;
    o.score = S;
    o.prior = prior;
    o.l00 = L.l00;
    o.l10 = L.l10;
    o.l01 = L.l01;
    o.l11 = L.l11;
#pragma unroll
    for (int k = 0; k < 4; k++) o.ec[k] = e[k];
    o.sk = sk;
    o.sm = sm;
    o.has_best = 0;
    o.best_alpha = alpha;
    o.best_beta = beta;
    o.best_score = -INFINITY;
    o.best_sk = 0;
    o.best_sm = 0;
    o.steps_done = 0;
    o.err_proposed = 0;
    o.err_accepted = 0;
    o.list_count = 0;
    for (int k = 0; k < 7; k++) o.pad[k] = 0;
    a.states[chain] = o;
  }
}

template <int W32, int Q, bool ATTACH>
__global__ void __launch_bounds__(128) score_kernel(const ScoreArgs a) {
  extern __shared__ __align__(16) uint32_t smem[];
  constexpr int RS = rs_of_w32(W32);
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const int tree = blockIdx.x * wpb + wib;
  if (tree >= a.n_trees) return;  // whole warp
  const int n = a.ds.n_nodes;
  uint32_t *rows = smem + (size_t)wib * n * RS;
  copy_rows<W32>(a.rows + (size_t)tree * n * RS, rows, n, lane);
  __syncwarp();
  const float *bt = a.beta_terms + 4 * (size_t)tree;
  const LogTable L{a.ds.l00, a.ds.l10, bt[1], bt[2]};
  const float prior = bt[3];
  Cells<W32, Q> cb;
  int k = 0, m = 0;
  for (int c0 = 0; c0 < a.ds.n_cells; c0 += 32 * Q) {
    load_cells<W32, Q>(cb, a.ds, c0, 32, lane);
    int bj[Q];
    best_nodes<W32, Q>(rows, n, cb, L.l00, L.l01, L.l10, L.l11, a.ds.neg_zero,
                          bj);
    counts_at<W32, Q>(rows, cb, bj, k, m);
    if constexpr (ATTACH) {
#pragma unroll
      for (int q = 0; q < Q; q++) {
        const int c = c0 + 32 * q + lane;
        if (c < a.ds.n_cells)
          a.attach[(size_t)tree * a.ds.n_cells + c] = (uint32_t)bj[q];
      }
    }
  }
  const int sk = (int)__reduce_add_sync(BBS_FULL_MASK, (uint32_t)k);
  const int sm = (int)__reduce_add_sync(BBS_FULL_MASK, (uint32_t)m);
  if (lane == 0) {
    const float s = tree_score(a.ds, sk, sm, L, prior);
    if (a.scores) a.scores[tree] = s;
    if (a.counts) {
      int N[4];
      class_totals(a.ds, sk, sm, N);
      for (int q = 0; q < 4; q++) a.counts[4 * (size_t)tree + q] = (uint64_t)N[q];
    }
  }
}

template <int W32>
__global__ void __launch_bounds__(128) apply_kernel(const ApplyArgs a) {
  extern __shared__ __align__(16) uint32_t smem[];
  constexpr int RS = rs_of_w32(W32);
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const int tree = blockIdx.x * wpb + wib;
  if (tree >= a.n_trees) return;
  const int n = a.n_nodes;
  uint32_t *rows = smem + (size_t)wib * n * RS;
  copy_rows<W32>(a.rows + (size_t)tree * n * RS, rows, n, lane);
  __syncwarp();
  const float beta = a.betas[tree];
  uint32_t Dv[W32], Dw[W32];
  bbs_move_params p;
  bool related;
  if (a.raw != nullptr) {
    const Realized R = realize_move<W32>(rows, n, beta, a.raw[tree], lane, Dv, Dw);
    p = R.p;
    related = R.related;
  } else {
    p = a.params[tree];
    p.v = min(p.v, (uint32_t)(n - 1));
    p.w = min(p.w, (uint32_t)(n - 1));
    descendant_sets<W32>(rows, n, p.v, p.w, lane, Dv, Dw);
    related = has_bit<W32>(Dw, p.v);
  }
  uint32_t *out = a.rows_out + (size_t)tree * n * RS;
  build_proposal<W32>(rows, out, n, p, Dv, Dw, related, 1, 0, lane);
  if (lane == 0) {
    if (a.params_out) a.params_out[tree] = p;
    if (a.beta_out)
      a.beta_out[tree] = p.move_type == BBS_MOVE_CHANGE_BETA ? p.new_beta : beta;
  }
}

// Sum-over-attachments score and adjoint.  Per cell an online logsumexp
// over nodes carries the softmax-weighted sums of k = popc(K & A_j) and
// m = popc(M & A_j); the expected class counts follow from the identity
// above, and dlogL/dtheta = sum_c sum_k E_pi[n_k] dl_k/dtheta.
template <int W32, int Q>
__global__ void __launch_bounds__(128) grad_kernel(const GradArgs a) {
  extern __shared__ __align__(16) uint32_t smem[];
  constexpr int RS = rs_of_w32(W32);
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const int tree = blockIdx.x * wpb + wib;
  if (tree >= a.n_trees) return;
  const int n = a.ds.n_nodes;
  uint32_t *rows = smem + (size_t)wib * n * RS;
  copy_rows<W32>(a.rows + (size_t)tree * n * RS, rows, n, lane);
  __syncwarp();
  const float *tb = a.tables + 6 * (size_t)tree;
  const float l00 = tb[2], l01 = tb[3], l10 = tb[4], l11 = tb[5];
  float acc_lse = 0.0f, acc_n00 = 0.0f, acc_n01 = 0.0f, acc_n10 = 0.0f,
        acc_n11 = 0.0f;
  Cells<W32, Q> cb;
  for (int c0 = 0; c0 < a.ds.n_cells; c0 += 32 * Q) {
    load_cells<W32, Q>(cb, a.ds, c0, 32, lane);
    float mx[Q], z[Q], ek[Q], em[Q];
#pragma unroll
    for (int q = 0; q < Q; q++) {
      mx[q] = -INFINITY;
      z[q] = ek[q] = em[q] = 0.0f;
    }
    for (int j = 0; j < n; j++) {
      uint32_t r[W32];
      ld_row<W32>(rows + j * RS, r);
#pragma unroll
      for (int q = 0; q < Q; q++) {
        const int d = masked_popc<W32>(cb.D[q], r);
        const int m = masked_popc<W32>(cb.M[q], r);
        const int k = d + m;
        const float s = pair_score(d, m, cb.pdb[q], cb.pmb[q], l00, l01, l10, l11);
        if (s > mx[q]) {
          const float sc = expf(mx[q] - s);
          z[q] = z[q] * sc + 1.0f;
          ek[q] = ek[q] * sc + (float)k;
          em[q] = em[q] * sc + (float)m;
          mx[q] = s;
        } else {
          const float e = expf(s - mx[q]);
          z[q] += e;
          ek[q] += e * (float)k;
          em[q] += e * (float)m;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < Q; q++) {
      const int c = c0 + 32 * q + lane;
      if (c >= a.ds.n_cells) continue;
      const float lse = mx[q] + logf(z[q]);
      const float Ek = ek[q] / z[q], Em = em[q] / z[q];
      const float pm = cb.pmb[q] - 8388608.0f;
      const float pkm = cb.pdb[q] - 8388608.0f;
      acc_lse += lse;
      acc_n11 += Em;
      acc_n01 += Ek - Em;
      acc_n10 += pm - Em;
      acc_n00 += pkm - Ek + Em;
      if (a.posterior != nullptr) {
        float *post = a.posterior + ((size_t)tree * a.ds.n_cells + c) * n;
        for (int j = 0; j < n; j++) {
          uint32_t r[W32];
          ld_row<W32>(rows + j * RS, r);
          const float s = pair_score(masked_popc<W32>(cb.D[q], r),
                                     masked_popc<W32>(cb.M[q], r), cb.pdb[q],
                                     cb.pmb[q], l00, l01, l10, l11);
          post[j] = expf(s - lse);
        }
      }
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    acc_lse += __shfl_xor_sync(BBS_FULL_MASK, acc_lse, off);
    acc_n00 += __shfl_xor_sync(BBS_FULL_MASK, acc_n00, off);
    acc_n01 += __shfl_xor_sync(BBS_FULL_MASK, acc_n01, off);
    acc_n10 += __shfl_xor_sync(BBS_FULL_MASK, acc_n10, off);
    acc_n11 += __shfl_xor_sync(BBS_FULL_MASK, acc_n11, off);
  }
  if (lane == 0) {
    const double al = tb[0], be = tb[1];
    a.logl[tree] = acc_lse;
    if (a.dalpha)
      a.dalpha[tree] = (float)(-(double)acc_n00 / (1.0 - al) + (double)acc_n10 / al);
    if (a.dbeta)
      a.dbeta[tree] = (float)((double)acc_n01 / be - (double)acc_n11 / (1.0 - be));
  }
}

}  // namespace bbs
