// bbs_internal.h -- host/device shared structs of the GB300 path.
#pragma once
#include <cstdint>

#include "bbscite_gb300.h"

namespace bbs {

// Row storage: a bit row over n nodes (or genes) is stored as
// RS = 2 * ceil(n/64) 32-bit words -- the little-endian image of the ABI's
// uint64 row -- of which W32 = ceil(n/32) are significant.
inline constexpr int kMaxW32 = 8;  // 256 nodes
inline constexpr int kMaxQ = 4;    // cells per lane per chunk

__host__ __device__ constexpr int rs_of_w32(int w32) {
  return 2 * ((w32 + 1) / 2);
}
__host__ __device__ constexpr int w32_of_nodes(int n) { return (n + 31) / 32; }

// Cumulative move thresholds and jump sd (src/RawMoveDistribution.hpp:
// 119-131, src/Parameters.hpp:451-584).
struct MoveProbs {
  float cum_beta, cum_prune, cum_swap, beta_jump_sd;
};

// One dataset as the kernels see it.
struct DatasetDev {
  const uint32_t *K;  // known rows  [n_cells][RS]
  const uint32_t *M;  // mutated rows [n_cells][RS], pre-masked with K
  int n_cells, n_nodes;
  int sum_k, sum_m;   // sum over cells of popc(K), popc(M)
  float l00, l10;     // log(1-alpha), log(alpha) (src/TreeScorer.hpp:99-106)
  float bpa, bpb;     // Beta prior parameters (src/TreeScorer.hpp:108-111)
  float lg_ab, lg_a, lg_b;  // log(tgamma(a+b)), log(tgamma(a)), log(tgamma(b))
};

// Persistent per-chain state (64 bytes).
struct ChainState {
  float beta, score;
  float l01, l11, prior;  // log(beta), log(1-beta), logscore_beta(beta)
  int32_t sk, sm;         // class sums of the current tree
  uint32_t has_best;
  float best_beta, best_score;
  int32_t best_sk, best_sm;
  uint64_t steps_done;    // Philox step counter
  uint32_t pad[2];
};
static_assert(sizeof(ChainState) == 64, "ChainState layout");

struct RunArgs {
  DatasetDev ds;
  MoveProbs mp;
  float gamma;
  int n_chains, n_steps;
  uint64_t seed;
  uint32_t *rows;       // [n_chains][n_nodes][RS] current trees
  uint32_t *best_rows;  // [n_chains][n_nodes][RS] best proposals
  ChainState *states;
  const bbs_raw_move *moves;  // [n_chains][n_steps] or null
  bbs_step_trace *trace;      // [n_chains][n_steps] or null
  const volatile int *cancel; // host-writable flag (mapped) or null
  int *status;                // device status word (0 = ok, 1 = cancelled)
  int wpc;                    // warps per chain (cells split over them)
};

struct ScoreArgs {
  DatasetDev ds;
  const uint32_t *rows;  // [n_trees][n_nodes][RS]
  const float *beta_terms;  // [n_trees][4]: beta, l01, l11, prior (host libm)
  int n_trees;
  float *scores;
  uint64_t *counts;      // [n_trees][4] or null
  uint32_t *attach;      // [n_trees][n_cells] or null
  ChainState *states;    // when set: write score/sk/sm/l01/l11/prior
};

struct ApplyArgs {
  int n_nodes, n_trees;
  const uint32_t *rows;
  const float *betas;
  const bbs_raw_move *raw;         // realise first when set
  const bbs_move_params *params;   // else apply these
  bbs_move_params *params_out;
  uint32_t *rows_out;
  float *beta_out;
};

struct GradArgs {
  DatasetDev ds;
  const uint32_t *rows;
  const float *tables;  // [n_trees][6]: alpha, beta, l00, l01, l10, l11
  int n_trees;
  float *logl, *dalpha, *dbeta;
  float *posterior;  // [n_trees][n_cells][n_nodes] or null
};

// Host launchers (bbs_kernels.cu).  Return a cudaError_t as int.
// chains_per_block must be 1 when a.wpc > 1 (the block is one chain).
int launch_mcmc(const RunArgs &a, int q, int chains_per_block, int n_sms,
                void *stream);
int launch_score(const ScoreArgs &a, int q, void *stream);
int launch_apply(const ApplyArgs &a, void *stream);
int launch_grad(const GradArgs &a, int q, void *stream);
int run_popc_bench(double *popc_per_s, double *clock_hz);
size_t mcmc_smem_bytes(int n_nodes, int wpc, int chains_per_block);
int pick_q(int n_cells);

}  // namespace bbs
