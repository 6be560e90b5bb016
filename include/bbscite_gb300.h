/*
 * bbscite_gb300.h -- C ABI of the GB300 (sm_103a) implementation of
 * bbSCITE's MCMC mutation-tree search.
 *
 * Plain C types only: caller-owned host buffers, sizes, an opaque context.
 * No function throws or aborts; every entry point returns a BBS_* status and
 * leaves a message for bbs_last_error().  One context is used by one host
 * thread at a time; each context owns its device memory and one CUDA stream.
 *
 * Bit-row layout (identical to the reference's ac_int rows, little-endian):
 *   n_nodes = n_genes + 1, root = n_nodes - 1, W = bbs_words(n_nodes)
 *   uint64 words per row.  A tree is given by its ancestor rows
 *   dm[x] (bit y <=> y is an ancestor of x, x itself and the root included)
 *   and/or its descendant rows am[x] (bit y <=> x is an ancestor of y):
 *   `descendant` / `ancestor` in src/MutationTree.hpp:40-71.
 *   Cell data: per cell one row of W words, bit g = gene g:
 *   `is_mutated` / `is_known` in src/main.cpp:103-144.
 *
 * References below are file:line in Janonard/bbSCITE.
 */
#ifndef BBSCITE_GB300_H
#define BBSCITE_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define BBS_API __attribute__((visibility("default")))
#else
#define BBS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference returns 1 from main / throws
 * std::out_of_range: src/main.cpp:45-48, src/Parameters.hpp:465-467) ---- */
#define BBS_OK 0
#define BBS_ERR_INPUT 1   /* invalid argument or data */
#define BBS_ERR_SIZE 2    /* size outside the supported range */
#define BBS_ERR_CUDA 3    /* CUDA runtime error (no device, launch, ...) */
#define BBS_ERR_TIMEOUT 4 /* a bounded run was cancelled / gave up */
#define BBS_ERR_STATE 5   /* call order (e.g. run before init_chains) */
#define BBS_ERR_IO 6      /* file could not be read or written */
#define BBS_ERR_ALLOC 7   /* host or device allocation failed */
#define BBS_ERR_DEVICE_CHECK 8 /* a device-side index check failed (builds
                                  with BBS_CHECKED defined) */

#define BBS_MAX_GENES 255   /* replaces the compile-time 63/95 caps */
#define BBS_MAX_CELLS 65535 /* integer class totals stay exact in FP32 */
#define BBS_MAX_TREELIST_PER_CHAIN 16

/* src/MoveType.hpp:23-42 */
#define BBS_MOVE_CHANGE_BETA 0
#define BBS_MOVE_PRUNE_REATTACH 1
#define BBS_MOVE_SWAP_NODES 2
#define BBS_MOVE_SWAP_SUBTREES 3

/* Run parameters: the CLI surface of src/Parameters.hpp:39-45, 61-281.
 * Move probabilities are normalised by their sum (Parameters.hpp:451-612). */
typedef struct bbs_params {
  float alpha_mean;            /* -fd  */
  float beta_mean;             /* -ad  */
  float beta_sd;               /* -sd  */
  float prob_beta_change;      /* -e   */
  float prob_prune_n_reattach; /* -move_probs a b c */
  float prob_swap_nodes;
  float prob_swap_subtrees;
  float beta_jump_scaling_chi; /* -x   */
  float gamma;                 /* -g   */
  uint32_t treelist_size;      /* co-optimal trees kept per chain (1: the best
                                  only), at most BBS_MAX_TREELIST_PER_CHAIN;
                                  single-dataset contexts (a batch keeps the
                                  best only) */
  uint64_t seed; /* Philox key for moves and random initial trees */
  /* Extensions without a counterpart in the reference (defaults reproduce
   * it): the score and the error-rate move taken with probability
   * prob_beta_change. */
  uint32_t score_mode; /* BBS_SCORE_MAX (reference) or BBS_SCORE_SUM */
  uint32_t error_move; /* BBS_ERROR_BETA_WALK (reference), _RANDOM_WALK,
                          _LANGEVIN */
  float error_step;    /* step of the learned error moves (preconditioned) */
  uint32_t reserved1;
} bbs_params;

/* Score: the reference's max over attachments (src/TreeScorer.hpp:131-210)
 * or the sum over attachments, log sum_j exp s_cj per cell. */
#define BBS_SCORE_MAX 0
#define BBS_SCORE_SUM 1
/* Error-rate move: the reference's beta random walk reflected into [0,1]
 * (src/MutationTree.hpp:345-351, sd = beta_sd / chi); a preconditioned
 * random walk on (logit alpha, logit beta); or a Langevin (MALA) step
 * driven by the adjoint gradient of the score.  The last two learn alpha
 * as well and accept with the exact Metropolis-Hastings ratio. */
#define BBS_ERROR_BETA_WALK 0
#define BBS_ERROR_RANDOM_WALK 1
#define BBS_ERROR_LANGEVIN 2

/* One recorded move, src/RawMoveDistribution.hpp:44-50 (32 bytes). */
typedef struct bbs_raw_move {
  int32_t move_type;
  uint32_t raw_v, raw_w;
  float raw_descendant_of_v, raw_nondescendant_of_v;
  float beta_jump;
  float acceptance_level;
  uint32_t reserved;
} bbs_raw_move;

/* A realised move, src/MutationTree.hpp:84-89 (32 bytes). */
typedef struct bbs_move_params {
  int32_t move_type;
  uint32_t v, w, parent_of_v, parent_of_w, descendant_of_v,
      nondescendant_of_v;
  float new_beta;
} bbs_move_params;

/* Per-step record written by bbs_run when a trace buffer is given. */
typedef struct bbs_step_trace {
  bbs_raw_move move;      /* the move as drawn (Philox) or read */
  float proposed_score;   /* score of the proposal */
  float current_score;    /* chain score after the step */
  float proposed_beta;
  uint32_t accepted;
  float proposed_alpha;
  float proposed_max_score; /* the reference's max score of the proposal
                               (equal to proposed_score with that score) */
  uint32_t reserved[2];
  uint64_t proposed_counts[4]; /* class totals n00,n01,n10,n11 (max score) */
} bbs_step_trace;

typedef struct bbs_ctx bbs_ctx;

/* ---- library ---- */
BBS_API const char *bbs_last_error(void);
BBS_API const char *bbs_version(void);
BBS_API uint32_t bbs_words(uint32_t n_nodes);
/* Parameters() defaults, src/Parameters.hpp:39-45 */
BBS_API void bbs_params_default(bbs_params *p);

/* ---- host tree helpers (MutationTree host methods) ---- */
/* src/MutationTree.hpp:427-476 */
BBS_API int bbs_pruefer_to_parent_vector(const uint32_t *code, uint32_t code_len,
                                 uint32_t *parent);
/* src/MutationTree.hpp:379-409 */
BBS_API int bbs_parent_vector_to_matrix(const uint32_t *parent, uint32_t n_nodes,
                                uint64_t *am, uint64_t *dm);
/* get_parent for every node, src/MutationTree.hpp:549-596 */
BBS_API int bbs_matrix_to_parent_vector(const uint64_t *dm, uint32_t n_nodes,
                                uint32_t *parent);
/* descendant rows from ancestor rows (transpose) */
BBS_API int bbs_dm_to_am(const uint64_t *dm, uint32_t n_nodes, uint64_t *am);
/* to_graphviz / to_newick, src/MutationTree.hpp:799-837, 880-894.
 * Writes at most cap bytes (NUL-terminated) and the full length. */
BBS_API int bbs_tree_to_graphviz(const uint32_t *parent, uint32_t n_nodes, char *buf,
                         size_t cap, size_t *len);
BBS_API int bbs_tree_to_newick(const uint32_t *parent, uint32_t n_nodes, char *buf,
                       size_t cap, size_t *len);
/* Uniform random trees as in src/Application.hpp:149-157 (uniform Pruefer
 * code, decoded), drawn from Philox(seed) instead of minstd_rand. */
BBS_API int bbs_random_parent_vectors(uint64_t seed, uint32_t n_genes,
                              uint32_t n_trees, uint32_t *parents);

/* ---- input file (src/main.cpp:50-144) ----
 * Parses a SCITE matrix (gene rows, cell columns, entries 0/1/2/3).  Call
 * with mut == NULL to get the sizes; then with buffers of
 * n_cells * bbs_words(n_genes + 1) words each. */
BBS_API int bbs_read_csv(const char *path, uint32_t *n_cells, uint32_t *n_genes,
                 uint64_t *is_mutated, uint64_t *is_known);

/* ---- single-dataset context: Application + TreeScorer ---- */
/* Application ctor data side + TreeScorer ctor (src/Application.hpp:88-117,
 * src/TreeScorer.hpp:92-117): copies the cell bit rows to the device and
 * builds the log table and the Beta prior. */
BBS_API int bbs_create(bbs_ctx **ctx, const uint64_t *is_mutated,
               const uint64_t *is_known, uint32_t n_cells, uint32_t n_genes,
               const bbs_params *params);
BBS_API void bbs_destroy(bbs_ctx *ctx);
BBS_API int bbs_get_sizes(const bbs_ctx *ctx, uint32_t *n_cells, uint32_t *n_genes,
                  uint32_t *n_chains);

/* Initial chain states, src/Application.hpp:119-164: n_chains trees from
 * `parents` (n_chains x n_nodes) or, when NULL, uniform random trees from
 * the seed; beta = beta_mean; scores computed on the device.  Any chain
 * count is accepted (the reference rounds up to the pipeline capacity,
 * src/Application.hpp:105-117). */
BBS_API int bbs_init_chains(bbs_ctx *ctx, uint32_t n_chains, const uint32_t *parents);

/* The work kernel, src/Application.hpp:366-498: advances every chain by
 * n_steps steps.  moves == NULL draws moves on the device from Philox
 * (seed, chain, step); otherwise `moves` holds n_chains x n_steps recorded
 * moves (chain-major, the emulator's order src/Application.hpp:313-354 with
 * pipeline capacity 1).  `trace` (n_chains x n_steps, optional) receives
 * every step.  Blocks until done.  The best proposal over all chains and
 * all runs is kept (src/Application.hpp:456). */
BBS_API int bbs_run(bbs_ctx *ctx, uint32_t n_steps, const bbs_raw_move *moves,
            bbs_step_trace *trace);
/* Same, returning immediately; bbs_sync waits and reports the status. */
BBS_API int bbs_run_async(bbs_ctx *ctx, uint32_t n_steps);
BBS_API int bbs_sync(bbs_ctx *ctx);
/* Asks a running kernel to stop after its current step block; the run then
 * returns BBS_ERR_TIMEOUT.  Safe from another host thread. */
BBS_API int bbs_cancel(bbs_ctx *ctx);

/* Launch shape of the chain kernel (no counterpart in the reference, whose
 * FPGA pipeline has a fixed chain-group size, src/main.cpp:28-32):
 * cells per lane per chunk (1-4; 1-2 above 128 nodes), warps per chain
 * (1-4; the cells are split over them) and chains per block (one-warp
 * chains only: 1-4, or 1-8 with 3-4 cells per lane; a run with a larger
 * block fails).  0 keeps a value.  bbs_init_chains picks a default. */
BBS_API int bbs_set_launch(bbs_ctx *ctx, int cells_per_lane,
                           int warps_per_chain, int chains_per_block);
BBS_API int bbs_get_launch(const bbs_ctx *ctx, int *cells_per_lane,
                           int *warps_per_chain, int *chains_per_block);
/* Times probe_steps steps of every launch shape on the current chains
 * (their state is restored afterwards) and keeps the fastest; best_ms
 * (optional) receives its time. */
BBS_API int bbs_autotune(bbs_ctx *ctx, uint32_t probe_steps, float *best_ms);

/* Device time in milliseconds of the last completed bbs_run / bbs_sync,
 * measured with CUDA events recorded on the context's stream around the
 * chain kernel (src/Application.hpp:197-219 reports the kernel makespan). */
BBS_API int bbs_last_run_ms(const bbs_ctx *ctx, float *ms);

/* get_best_am/dm/beta/score, src/Application.hpp:224-256; also the parent
 * vector, the class totals (n00,n01,n10,n11) and the chain index.  Any
 * output pointer may be NULL.  The best proposal is chosen by the
 * reference's max score also when chains sample the sum score (whose
 * class totals are then not recorded: counts are zero). */
BBS_API int bbs_get_best(bbs_ctx *ctx, uint64_t *am, uint64_t *dm, uint32_t *parent,
                 float *beta, float *score, uint64_t *counts,
                 uint32_t *chain);
/* The co-optimal tree list: SCITE's -max_treelist_size, parsed but
 * unused by the reference (src/Parameters.hpp:223-231).  Each chain keeps
 * up to params.treelist_size distinct trees whose score equals its best
 * proposal's; this gathers the distinct trees of every chain whose best
 * equals the overall best, in chain order, the bbs_get_best tree first.
 * dm: max_trees x n_nodes x W ancestor rows; betas: max_trees (may be
 * NULL); *score the common score; *n_trees the number written. */
BBS_API int bbs_get_treelist(bbs_ctx *ctx, uint32_t max_trees, uint64_t *dm,
                             float *betas, float *score, uint32_t *n_trees);

/* The alpha of the best proposal (equal to alpha_mean unless alpha is
 * learned by the error move). */
BBS_API int bbs_get_best_alpha(bbs_ctx *ctx, float *alpha);
/* Current chain states (dm rows n_chains x n_nodes x W, alphas, betas,
 * scores, class totals); error-move statistics (proposed, accepted) per
 * chain in err_stats (n_chains x 2).  Any output may be NULL. */
BBS_API int bbs_get_chains(bbs_ctx *ctx, uint64_t *dm, float *alpha, float *beta,
                   float *score, uint64_t *counts, uint32_t *err_stats);

/* Chain checkpoints (no counterpart in the reference, whose chain state
 * lives only inside the FPGA pipeline, src/Application.hpp:490-495).
 * bbs_save_chains writes every chain's state -- current and best trees,
 * the co-optimal lists, rates, scores, error-move statistics and the
 * position in its Philox stream -- into buf as one byte image of *size
 * bytes; with buf == NULL it only sets *size.  A buffer that is too small
 * gives BBS_ERR_SIZE with the size needed in *size.  bbs_load_chains
 * restores such an image into a context created with the same dataset and
 * parameters (in this process or another), replacing its chains; the
 * chains then continue exactly as if they had never stopped.  An image of
 * another dataset or other parameters, a damaged image or one holding
 * something other than trees gives BBS_ERR_INPUT and leaves the context's
 * chains as they were.  The launch shape returns to its default. */
BBS_API int bbs_save_chains(bbs_ctx *ctx, void *buf, size_t *size);
BBS_API int bbs_load_chains(bbs_ctx *ctx, const void *buf, size_t size);

/* TreeScorer::logscore_tree for a batch, src/TreeScorer.hpp:131-210:
 * dm = n_trees x n_nodes x W ancestor rows, betas (n_trees).  Outputs:
 * scores (class-total form: ((l00*N00 + l01*N01) + l10*N10) + l11*N11 plus
 * logscore_beta), counts (n_trees x 4, may be NULL), attach (n_trees x
 * n_cells first-max attachment nodes, may be NULL).  This call, and
 * bbs_apply_moves and bbs_sumscore_grad, keep their device scratch in the
 * context: it grows to the largest call made so far and is freed by
 * bbs_destroy, so a caller scoring one tree at a time allocates device
 * memory on its first call only. */
BBS_API int bbs_score_trees(bbs_ctx *ctx, const uint64_t *dm, const float *betas,
                    uint32_t n_trees, float *scores, uint64_t *counts,
                    uint32_t *attach);

/* TreeScorer::logscore_beta, src/TreeScorer.hpp:122-126: the log Beta
 * prior of `beta` with the context's (beta_mean, beta_sd), in FP32 through
 * log(tgamma(.)) as the reference computes it (NaN where tgammaf
 * overflows, a + b above about 35). */
BBS_API int bbs_logscore_beta(const bbs_ctx *ctx, float beta, float *out);

/* realize_raw_move_sample + update constructor for a batch,
 * src/MutationTree.hpp:123-363.  When `raw` is non-NULL each move is
 * realised first (params_out, optional, receives the result); otherwise
 * `params` are applied as given.  dm_out receives the proposed ancestor
 * rows, beta_out the proposed beta. */
BBS_API int bbs_apply_moves(bbs_ctx *ctx, const uint64_t *dm, const float *betas,
                    uint32_t n_trees, const bbs_raw_move *raw,
                    const bbs_move_params *params,
                    bbs_move_params *params_out, uint64_t *dm_out,
                    float *beta_out);

/* ---- many datasets in one launch (no counterpart in the reference,
 * whose FPGA build takes one dataset per run) ----
 * Datasets of up to BBS_MAX_GENES genes, each with its own cells and
 * parameters; chains of all datasets run in one persistent launch per
 * row-width group, taken costliest first from a shared work list. */
typedef struct bbs_batch bbs_batch;
/* is_mutated[d] / is_known[d]: n_cells[d] x bbs_words(n_genes[d] + 1). */
BBS_API int bbs_batch_create(bbs_batch **batch, uint32_t n_datasets,
                             const uint32_t *n_cells, const uint32_t *n_genes,
                             const uint64_t *const *is_mutated,
                             const uint64_t *const *is_known,
                             const bbs_params *params);
BBS_API void bbs_batch_destroy(bbs_batch *batch);
/* chains_per_dataset random initial trees per dataset (from each
 * dataset's seed). */
BBS_API int bbs_batch_init_chains(bbs_batch *batch, uint32_t chains_per_dataset);
/* Advances every chain by n_steps; the launches are replayed from a CUDA
 * graph captured on the first run with this n_steps. */
BBS_API int bbs_batch_run(bbs_batch *batch, uint32_t n_steps);
BBS_API int bbs_batch_last_run_ms(const bbs_batch *batch, float *ms);
/* Launch shape: cells per lane (1-4; 1-2 above 128 nodes) and warps per
 * block (1-8; a launch group with 1-2 cells per lane takes at most 4, and
 * a block too large for its shared memory fails the run with
 * BBS_ERR_SIZE);
 * merge_rows != 0 runs trees of an odd number of 32-bit row words (1, 3,
 * 5, 7) with the next even width, which has the same row stride (one
 * launch per pair of widths instead of two). */
BBS_API int bbs_batch_set_launch(bbs_batch *batch, int cells_per_lane,
                                 int warps_per_block, int merge_rows);
BBS_API int bbs_batch_get_launch(const bbs_batch *batch, int *cells_per_lane,
                                 int *warps_per_block, int *merge_rows);
/* Chain-to-warp mapping: 1 (default) runs each chain on one warp, in
 * blocks of warps_per_block chains; 2-4 splits each chain's cells over that
 * many warps, one chain per block (warps_per_block is then ignored).
 * Chains are bit-identical under every mapping. */
BBS_API int bbs_batch_set_chain_warps(bbs_batch *batch, int warps_per_chain);
BBS_API int bbs_batch_get_chain_warps(const bbs_batch *batch,
                                      int *warps_per_chain);
/* Times probe_steps steps per launch shape -- cells per lane, one-warp
 * chains in blocks of 1, 2, 4, 7 or 8, or chains of 2 or 4 warps, with and
 * without merged row widths (chain states restored) -- and keeps the
 * fastest. */
BBS_API int bbs_batch_autotune(bbs_batch *batch, uint32_t probe_steps,
                               float *best_ms);
/* Best proposal of one dataset (over its chains). */
BBS_API int bbs_batch_get_best(bbs_batch *batch, uint32_t dataset, uint64_t *dm,
                               uint32_t *parent, float *alpha, float *beta,
                               float *score);
/* Checkpoints of a batch, as bbs_save_chains / bbs_load_chains: every
 * chain of every dataset, restored into a batch created with the same
 * datasets and parameters. */
BBS_API int bbs_batch_save_chains(bbs_batch *batch, void *buf, size_t *size);
BBS_API int bbs_batch_load_chains(bbs_batch *batch, const void *buf, size_t size);

/* Sum-over-attachments score and its adjoint (no counterpart in the
 * reference; SCITE's "-s" score, see docs/thesis/chapters/conclusion/
 * open_directions.tex:13): logL = sum_c logsumexp_j s_cj(alpha, beta) and
 * dlogL/dalpha, dlogL/dbeta for a batch of trees with per-tree (alpha,
 * beta); posterior (n_trees x n_cells x n_nodes, optional) receives the
 * attachment posteriors softmax_j s_cj.  No Beta prior term. */
BBS_API int bbs_sumscore_grad(bbs_ctx *ctx, const uint64_t *dm, const float *alphas,
                      const float *betas, uint32_t n_trees, float *logl,
                      float *dalpha, float *dbeta, float *posterior);

/* bbs_score_trees for callers that cannot allocate GPU memory (no
 * counterpart in the reference).  Some callers cannot call cudaMalloc at
 * scoring time: a framework that has handed all device memory to its own
 * pool, a latency-critical loop where an allocation would synchronise the
 * device, or code that must leave the allocator untouched between set-up
 * and teardown.  This entry point allocates nothing.  The caller passes
 * device buffers: dm_device (n_trees x n_nodes x W ancestor rows),
 * scores_device (n_trees floats) and counts_device (n_trees x 4, may be
 * NULL), plus the betas in host memory.  The per-tree log-table scratch
 * lives in a fixed device array of BBS_NOALLOC_MAX_TREES entries (256 KB),
 * which every GPU that loads this library holds until the process exits;
 * more trees per call are rejected with BBS_ERR_SIZE.  The first call on a
 * device looks that array's address up (cudaGetSymbolAddress) and keeps it
 * for the life of the process; make that first call before any stream
 * capture.  The kept address does not survive cudaDeviceReset: do not call
 * this entry point again after resetting the device.  All calls share the
 * array, so calls that overlap on the GPU (several host threads or
 * contexts at once) race; serialise them.  The context's device must be
 * the current device.  The call runs on the context's own stream, not the
 * caller's, and returns when the scores are written (it waits for that
 * stream): finish writing dm_device (synchronise the stream that produced
 * it) before the call. */
#define BBS_NOALLOC_MAX_TREES 16384
BBS_API int bbs_score_trees_noalloc(bbs_ctx *ctx, const uint64_t *dm_device,
                                    const float *betas, uint32_t n_trees,
                                    float *scores_device,
                                    uint64_t *counts_device);

/* Integer-pipe calibration: 32-bit POPC throughput of this device in
 * operations per second (a timed microbenchmark). */
/* Device checks (no counterpart in the reference).  A build with
 * BBS_CHECKED defined (python -m bbscite_gb300.build --checked, giving
 * libbbscite_gb300_checked.so) tests the device indices that come from
 * data -- the nodes of every realised move, work-list entries and dataset
 * numbers -- and skips what a bad index would reach; a run in which a
 * check failed returns BBS_ERR_DEVICE_CHECK naming the check, the value
 * and its limit.  bbs_device_check_selftest makes one check fail on
 * purpose (index 7 against limit 5, no access) and reports what was
 * recorded: *enabled is 1 in a checked build (then *code = 4, *value = 7,
 * *limit = 5) and 0 otherwise (nothing recorded, *code = 0). */
BBS_API int bbs_device_check_selftest(int *enabled, uint32_t *code,
                                      uint32_t *value, uint32_t *limit);

BBS_API int bbs_popc_peak(double *popc_per_s, double *sm_clock_hz);

#ifdef __cplusplus
}
#endif
#endif
