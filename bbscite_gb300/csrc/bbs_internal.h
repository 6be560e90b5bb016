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
// Status words of a run: bit 0 of [0] a cancelled run, bit 1 a failed
// device check (BBS_CHECKED builds) whose code, value and limit are [1..3].
inline constexpr int kStatusWords = 4;
inline constexpr int kCheckMoveNode = 1, kCheckUnit = 2, kCheckDataset = 3,
                     kCheckSelfTest = 4, kCheckParent = 5;

__host__ __device__ constexpr int rs_of_w32(int w32) {
  return 2 * ((w32 + 1) / 2);
}
__host__ __device__ constexpr int w32_of_nodes(int n) { return (n + 31) / 32; }
// Chains inherit counts from the parent (max or sum score):
//   - rows of up to four words, when all their cells stay in registers (at
//     most cells_per_pass = 32 x cells per lane x warps per chain): the
//     block's increment tables and each warp's count table of every node
//     exist then;
//   - rows of five to eight words, always: each warp keeps a ring of the
//     counts of the last kRing nodes in the canonical order and a gene
//     table of the cells it is scoring, rebuilt per chunk of streamed
//     cells.
inline constexpr int kRing = 64;
__host__ __device__ constexpr bool inherits_counts(int w32, int n_cells,
                                                   int cells_per_pass) {
  return w32 > 4 || n_cells <= cells_per_pass;
}

// Cumulative move thresholds and jump sd (src/RawMoveDistribution.hpp:
// 119-131, src/Parameters.hpp:451-584).  The first threshold is the
// error-rate move (the reference's ChangeBeta).
struct MoveProbs {
  float cum_beta, cum_prune, cum_swap, beta_jump_sd;
};

// One dataset as the kernels see it.
struct DatasetDev {
  const uint32_t *K;  // known rows  [n_cells][RS]
  const uint32_t *M;  // mutated rows [n_cells][RS], pre-masked with K
  int n_cells, n_nodes;
  int sum_k, sum_m;   // sum over cells of popc(K), popc(M)
  float l00, l10;     // log(1-alpha), log(alpha) of alpha_mean
                      // (src/TreeScorer.hpp:99-106)
  float bpa, bpb;     // Beta prior parameters (src/TreeScorer.hpp:108-111)
  float lg_ab, lg_a, lg_b;  // log(tgamma(a+b)), log(tgamma(a)), log(tgamma(b))
  float neg_zero;     // -0.0f.  Paired products are taken as fused
                      // multiply-adds of this addend: read from memory, it
                      // cannot be folded, so the compiler cannot contract a
                      // product with the sum that follows it (it does so for
                      // a paired multiply, whatever its rounding modifier)
};

// The sampling rules of one dataset's chains.
struct ModelDev {
  MoveProbs mp;
  float gamma;
  int32_t score_mode;  // 0: max over attachments, 1: sum (logsumexp)
  int32_t error_move;  // 0: reference beta walk, 1: preconditioned random
                       // walk on (logit alpha, logit beta), 2: Langevin
  float error_step;    // step size of error moves 1 and 2
  int32_t treelist;    // co-optimal trees kept per chain (1: the best only)
  uint64_t seed;       // Philox key
};

// Persistent per-chain state (128 bytes).
struct ChainState {
  float alpha, beta, score, prior;  // score = data term + log prior(beta)
  float l00, l10, l01, l11;         // log table of (alpha, beta)
  float ec[4];                      // class counts n00, n01, n10, n11 of
                                    // the current tree at the current rates
                                    // (expected counts for the sum score):
                                    // the error moves' gradient source
  int32_t sk, sm;                   // class sums (max score)
  uint32_t has_best;
  float best_alpha, best_beta, best_score;
  int32_t best_sk, best_sm;
  uint64_t steps_done;              // Philox step counter
  uint32_t err_proposed, err_accepted;
  uint32_t list_count;              // trees in the chain's co-optimal list
  uint32_t pad[7];
};
static_assert(sizeof(ChainState) == 128, "ChainState layout");

struct RunArgs {
  DatasetDev ds;
  ModelDev md;
  int n_chains, n_steps;
  uint32_t *rows;       // [n_chains][n_nodes][RS] current trees
  uint32_t *best_rows;  // [n_chains][treelist][n_nodes][RS] best proposal
                        // and the trees tied with it
  uint64_t *list_hash;  // [n_chains][treelist] tree hashes (treelist > 1)
  float *list_beta;     // [n_chains][treelist]
  ChainState *states;
  const bbs_raw_move *moves;  // [n_chains][n_steps] or null
  bbs_step_trace *trace;      // [n_chains][n_steps] or null
  const volatile int *cancel; // host-writable flag (mapped) or null
  int *status;                // device status word (0 = ok, 1 = cancelled)
  int wpc;                    // warps per chain (cells split over them)
};

// Many datasets in one launch: chains are listed by unit (chain index in
// an order of decreasing cost); each chain names its dataset and row offset.
struct BatchArgs {
  const DatasetDev *ds;      // [n_datasets]
  const ModelDev *md;        // [n_datasets]
  const uint32_t *chain_ds;  // [n_chains] dataset of each chain
  const uint64_t *chain_off; // [n_chains] word offset of its rows
  const uint32_t *units;     // chains of this launch, costliest first
  int n_units, n_steps;
  int n_chains, n_datasets;  // bounds of units[] and chain_ds[] entries
  int chains_per_dataset;    // chain c is number c - d * this of dataset d
  uint32_t *rows, *best_rows;
  ChainState *states;
  unsigned int *next_unit;   // work counter (zeroed before the launch)
  const volatile int *cancel;
  int *status;
  int max_nodes;             // shared memory is sized for this
  int table_ds;              // the launch's only dataset, or -1
  int with_counts;           // 1: the chains inherit counts (rows of up to
                             // four words, one dataset whose cells stay in
                             // registers; wider rows always); shared memory
                             // holds the count and increment tables, or
                             // the rings and gene tables, only then
  int wpc;                   // warps per chain: 1 (blocks of one-warp
                             // chains), or 2-4 (a block is one chain)
};

// Initial state of each chain: evaluate its tree at (alpha_mean,
// beta_mean) with host-computed log-table terms.
struct InitArgs {
  const DatasetDev *ds;      // [n_datasets]
  const ModelDev *md;
  const uint32_t *chain_ds;  // null: every chain uses dataset 0
  const uint64_t *chain_off; // null: chain * n_nodes * RS
  const float *terms;        // [n_datasets][8]: alpha, beta, l00, l10,
                             //   l01, l11, prior, unused
  const uint32_t *chain_list; // null: chains 0..n_chains-1
  int n_chains;
  const uint32_t *rows;
  ChainState *states;
  int max_nodes;             // shared memory is sized for this
};

// Random initial trees on the device: per chain a uniform Pruefer code
// from Philox (seed of the chain's dataset, stream 0x7265, counter (entry
// group, chain number in its dataset)), decoded smallest leaf first, as
// ancestor rows.  Same trees as the host's bbs_random_parent_vectors.
struct TreeArgs {
  const DatasetDev *ds;      // [n_datasets]
  const ModelDev *md;
  const uint32_t *chain_ds;  // null: every chain uses dataset 0
  const uint64_t *chain_off; // null: chain * n_nodes * RS
  int chains_per_dataset;    // chain number in its dataset: c - d * this
  int n_chains;
  uint32_t *rows;
  int max_nodes;             // shared memory is sized for this
};

struct ScoreArgs {
  DatasetDev ds;
  const uint32_t *rows;  // [n_trees][n_nodes][RS]
  const float *beta_terms;  // [n_trees][4]: beta, l01, l11, prior (host libm)
  int n_trees;
  float *scores;
  uint64_t *counts;      // [n_trees][4] or null
  uint32_t *attach;      // [n_trees][n_cells] or null
  ChainState *states;    // unused (kept zero)
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

// Host launchers (bbs_aux.cu, bbs_mcmc_*.cu).  Return a cudaError_t as int.
// chains_per_block must be 1 when a.wpc > 1 (the block is one chain).
int launch_mcmc(const RunArgs &a, int q, int chains_per_block, int n_sms,
                void *stream);
int launch_batch(const BatchArgs &b, int w32, int q, bool sum,
                 int warps_per_block, int n_sms, void *stream);
// Launch groups: every chain of a launch must store its rows with the
// stride rs_of_w32(w32) of the launch (w32 at least the chains' own).
int launch_init(const InitArgs &a, int w32, bool sum, void *stream);
int launch_trees(const TreeArgs &a, void *stream);
int launch_score(const ScoreArgs &a, int q, void *stream);
int launch_apply(const ApplyArgs &a, void *stream);
int launch_grad(const GradArgs &a, int q, void *stream);
int run_popc_bench(double *popc_per_s, double *clock_hz);
// Records one failing device check (code kCheckSelfTest, value 7, limit 5)
// in status[0..3] without any out-of-range access; 1 when the library was
// built with device checks (BBS_CHECKED), else 0 and status untouched.
int run_check_selftest(int *status_device, int *enabled);
int pick_q(int n_cells);

}  // namespace bbs
