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

// Shared-memory words per chain slot: two row buffers, the partial class
// sums of both step parities (2 x wpc x 2 ints) and a flag word, padded to
// 16 bytes.
__host__ __device__ inline int slot_words(int n, int rs, int wpc) {
  return 2 * n * rs + 4 * wpc + 4;
}

// Resident 128-thread blocks per SM the register budget aims for: fewer
// cells per lane leave room for more warps.
template <int W32, int Q>
struct McmcOccupancy {
  static constexpr int min_blocks = Q == 1 ? 4 : (Q == 2 ? 3 : 2);
};

template <int W32, int Q>
__global__ void __launch_bounds__(128, McmcOccupancy<W32, Q>::min_blocks)
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
  uint32_t *buf0 = smem + (size_t)slot * slot_words(n, RS, wpc);
  uint32_t *buf1 = buf0 + n * RS;
  int *part = reinterpret_cast<int *>(buf0 + 2 * n * RS);
  volatile int *sflag = part + 4 * wpc;
  const bool multi = wpc > 1;  // block-uniform
  const bool resident = a.ds.n_cells <= 32 * wpc * Q;
  Cells<W32, Q> cb;
  if (resident) load_cells<W32, Q>(cb, a.ds, 32 * wic, 32 * wpc, lane);

  for (int chain = blockIdx.x * cpb + slot; chain < a.n_chains;
       chain += gridDim.x * cpb) {
    const ChainState st = a.states[chain];
    uint32_t *g = a.rows + (size_t)chain * n * RS;
    uint32_t *gbest = a.best_rows + (size_t)chain * n * RS;
    copy_rows_part<W32>(g, buf0, n, wpc, wic, lane);
    if (multi) __syncthreads(); else __syncwarp();
    uint32_t *cur = buf0, *prop = buf1;
    float beta = st.beta, score = st.score;
    float l01 = st.l01, l11 = st.l11, prior = st.prior;
    int csk = st.sk, csm = st.sm;
    bool has_best = st.has_best != 0;
    float best_score = st.best_score, best_beta = st.best_beta;
    int bsk = st.best_sk, bsm = st.best_sm;
    int i = 0;
    bool cancelled = false;
    for (; i < a.n_steps; i++) {
      if (a.cancel != nullptr && (i & 255) == 0) {
        // one reader, then a chain-uniform decision
        if (wic == 0 && lane == 0) *sflag = *a.cancel;
        if (multi) __syncthreads(); else __syncwarp();
        const int c = *sflag;
        if (multi) __syncthreads(); else __syncwarp();
        if (c) {
          cancelled = true;
          break;
        }
      }
      const uint64_t step = st.steps_done + (uint64_t)i;
      const bbs_raw_move raw =
          a.moves != nullptr
              ? a.moves[(size_t)chain * a.n_steps + i]
              : sample_move(a.mp, (uint32_t)n, a.seed, (uint32_t)chain, step,
                            a.trace != nullptr);
      uint32_t Dv[W32], Dw[W32];
      const Realized R = realize_move<W32>(cur, n, beta, raw, lane, Dv, Dw);
      const bool beta_move = raw.move_type == BBS_MOVE_CHANGE_BETA;
      const uint32_t *scored = cur;
      float pbeta = beta, pl01 = l01, pl11 = l11, pprior = prior;
      if (beta_move) {
        pbeta = R.p.new_beta;
        beta_terms(a.ds, pbeta, pl01, pl11, pprior);
      } else {
        build_proposal<W32>(cur, prop, n, R.p, Dv, Dw, R.related, wpc, wic,
                            lane);
        scored = prop;
      }
      if (multi) __syncthreads(); else __syncwarp();
      int sk, sm;
      score_part<W32, Q>(scored, n, a.ds, cb, resident, pl01, pl11, wpc, wic,
                         lane, sk, sm);
      if (multi) {
        int *pp = part + (i & 1) * 2 * wpc;
        if (lane == 0) {
          pp[2 * wic] = sk;
          pp[2 * wic + 1] = sm;
        }
        __syncthreads();
        sk = sm = 0;
        for (int w = 0; w < wpc; w++) {
          sk += pp[2 * w];
          sm += pp[2 * w + 1];
        }
      }
      const float pscore = tree_score(a.ds, sk, sm, pl01, pl11, pprior);
      // src/Application.hpp:443-456
      float corr = 1.0f;
      if (raw.move_type == BBS_MOVE_SWAP_SUBTREES && R.related)
        corr = __fdiv_rn((float)R.ndv, (float)R.ndw);
      const float ratio = __fmul_rn(
          corr, expf(__fmul_rn(__fsub_rn(pscore, score), a.gamma)));
      const bool accept = ratio > raw.acceptance_level;
      if (!has_best || pscore > best_score) {
        has_best = true;
        best_score = pscore;
        best_beta = pbeta;
        bsk = sk;
        bsm = sm;
        copy_rows_part<W32>(scored, gbest, n, wpc, wic, lane);
      }
      if (a.trace != nullptr && wic == 0 && lane == 0) {
        bbs_step_trace *t = a.trace + (size_t)chain * a.n_steps + i;
        t->move = raw;
        t->proposed_score = pscore;
        t->current_score = accept ? pscore : score;
        t->proposed_beta = pbeta;
        t->accepted = accept ? 1u : 0u;
        int N[4];
        class_totals(a.ds, sk, sm, N);
#pragma unroll
        for (int k = 0; k < 4; k++) t->proposed_counts[k] = (uint64_t)N[k];
      }
      if (accept) {
        if (!beta_move) {
          uint32_t *t = cur;
          cur = prop;
          prop = t;
        }
        beta = pbeta;
        score = pscore;
        l01 = pl01;
        l11 = pl11;
        prior = pprior;
        csk = sk;
        csm = sm;
      }
      __syncwarp();
    }
    copy_rows_part<W32>(cur, g, n, wpc, wic, lane);
    if (wic == 0 && lane == 0) {
      ChainState o = st;
      o.beta = beta;
      o.score = score;
      o.l01 = l01;
      o.l11 = l11;
      o.prior = prior;
      o.sk = csk;
      o.sm = csm;
      o.has_best = has_best ? 1u : 0u;
      o.best_beta = best_beta;
      o.best_score = best_score;
      o.best_sk = bsk;
      o.best_sm = bsm;
      o.steps_done = st.steps_done + (uint64_t)i;
      a.states[chain] = o;
      if (cancelled && a.status != nullptr) atomicOr(a.status, 1);
    }
    if (multi) __syncthreads(); else __syncwarp();
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
  const float l01 = bt[1], l11 = bt[2], prior = bt[3];
  Cells<W32, Q> cb;
  int k = 0, m = 0;
  for (int c0 = 0; c0 < a.ds.n_cells; c0 += 32 * Q) {
    load_cells<W32, Q>(cb, a.ds, c0, 32, lane);
    int bj[Q];
    best_nodes<W32, Q>(rows, n, cb, a.ds.l00, l01, a.ds.l10, l11, bj);
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
    const float s = tree_score(a.ds, sk, sm, l01, l11, prior);
    if (a.scores) a.scores[tree] = s;
    if (a.counts) {
      int N[4];
      class_totals(a.ds, sk, sm, N);
      for (int q = 0; q < 4; q++) a.counts[4 * (size_t)tree + q] = (uint64_t)N[q];
    }
    if (a.states) {
      ChainState o;
      o.beta = bt[0];
      o.score = s;
      o.l01 = l01;
      o.l11 = l11;
      o.prior = prior;
      o.sk = sk;
      o.sm = sm;
      o.has_best = 0;
      o.best_beta = bt[0];
      o.best_score = -INFINITY;
      o.best_sk = 0;
      o.best_sm = 0;
      o.steps_done = 0;
      o.pad[0] = o.pad[1] = 0;
      a.states[tree] = o;
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
