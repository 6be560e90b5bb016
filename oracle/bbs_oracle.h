/*
 * bbs_oracle.h -- CPU restatement of bbSCITE's MCMC hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle is the checker for the CUDA path in
 * bbscite_gb300/: only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline / reference arm may load it.  The product never links it.
 *
 * Bit-row convention (shared with the C ABI in include/bbscite_gb300.h):
 *   a tree over n_nodes nodes (root = n_nodes-1) is two row-major bit
 *   matrices of n_nodes rows x W = ceil(n_nodes/64) uint64 words:
 *     am[x] bit y  <=>  x is an ancestor of y   (descendant set of x)
 *     dm[x] bit y  <=>  y is an ancestor of x   (ancestor set of x)
 *   exactly as `ancestor` / `descendant` in src/MutationTree.hpp:40-71.
 *   Cell data: per cell one row of ceil(n_genes/64)... words; here the
 *   same W as the tree (bit g = gene g), src/main.cpp:103-144.
 */
#ifndef BBS_ORACLE_H
#define BBS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* src/MoveType.hpp:23-42 */
enum { ORC_CHANGE_BETA = 0, ORC_PRUNE_REATTACH = 1, ORC_SWAP_NODES = 2,
       ORC_SWAP_SUBTREES = 3 };

/* src/RawMoveDistribution.hpp:44-50 (32-byte record) */
typedef struct {
  int32_t move_type;
  uint32_t raw_v, raw_w;
  float raw_descendant_of_v, raw_nondescendant_of_v;
  float beta_jump;
  float acceptance_level;
  uint32_t pad_;
} orc_raw_move;

/* src/MutationTree.hpp:84-89 */
typedef struct {
  int32_t move_type;
  uint32_t v, w, parent_of_v, parent_of_w, descendant_of_v,
      nondescendant_of_v;
  float new_beta;
} orc_mod_params;

/* src/TreeScorer.hpp:92-117 scorer constants */
typedef struct {
  float l00, l01, l10, l11; /* log table [observed][true] */
  float bpriora, bpriorb;   /* Beta prior parameters */
} orc_scorer;

uint32_t orc_words(uint32_t n_nodes);

/* ---- tree construction (host helpers) ---- */
void orc_pruefer_to_parent_vector(const uint32_t *code, uint32_t code_len,
                                  uint32_t *parent);
void orc_parent_vector_to_matrix(const uint32_t *parent, uint32_t n_nodes,
                                 uint64_t *am, uint64_t *dm);
/* parent vector from a descendant matrix (get_parent for every node) */
void orc_matrix_to_parent_vector(const uint64_t *am, const uint64_t *dm,
                                 uint32_t n_nodes, uint32_t *parent);

/* ---- tree queries ---- */
int orc_is_parent(const uint64_t *dm, uint32_t n_nodes, uint32_t parent,
                  uint32_t child);
uint32_t orc_get_parent(const uint64_t *dm, uint32_t n_nodes, uint32_t x);
uint32_t orc_get_n_descendants(const uint64_t *am, uint32_t n_nodes,
                               uint32_t x);
uint32_t orc_get_n_ancestors(const uint64_t *dm, uint32_t n_nodes,
                             uint32_t x);
uint32_t orc_get_descendant_or_nondescendant(const uint64_t *am,
                                             uint32_t n_nodes, uint32_t x,
                                             uint32_t k, int descendant);

/* ---- moves ---- */
void orc_realize_raw_move(const uint64_t *am, const uint64_t *dm,
                          uint32_t n_nodes, float beta,
                          const orc_raw_move *raw, orc_mod_params *out);
/* update constructor: writes the proposed tree and returns its beta */
float orc_apply_move(const uint64_t *am, const uint64_t *dm, uint32_t n_nodes,
                     float beta, const orc_mod_params *p, uint64_t *new_am,
                     uint64_t *new_dm);

/* ---- scoring ---- */
void orc_scorer_init(orc_scorer *s, float alpha_mean, float beta_mean,
                     float beta_sd);
void orc_scorer_set_beta(orc_scorer *s, float beta);
float orc_logscore_beta(const orc_scorer *s, float beta);
/*
 * Max-over-attachments score of one tree.  Returns the score exactly as
 * src/TreeScorer.hpp:131-210 sums it (per-cell maxima added in cell order);
 * also returns, when non-NULL:
 *   counts[4]  = integer error-class totals at the first-max attachment
 *                (n00, n01, n10, n11) = [observed][true]
 *   score_totals = the class-total form used by the CUDA path:
 *                ((l00*N00 + l01*N01) + l10*N10) + l11*N11 + prior(beta)
 *   attach[c]  = first-max attachment node of cell c
 * `mut` and `known` hold n_cells rows of W words (W from n_nodes).
 */
float orc_logscore_tree(const orc_scorer *s, const uint64_t *dm,
                        uint32_t n_nodes, const uint64_t *mut,
                        const uint64_t *known, uint32_t n_cells, float beta,
                        uint64_t *counts, float *score_totals,
                        uint32_t *attach);
float orc_score_from_totals(const orc_scorer *s, const uint64_t *counts,
                            float beta);

/* FP64 restatement of the same max score (log table in double) */
double orc_logscore_tree_f64(double alpha, double beta, double beta_mean,
                             double beta_sd, const uint64_t *dm,
                             uint32_t n_nodes, const uint64_t *mut,
                             const uint64_t *known, uint32_t n_cells,
                             int with_prior);

/*
 * FP64 sum-over-attachments score logL = sum_c logsumexp_j s_cj (no prior)
 * and its exact gradient; posteriors (n_cells x n_nodes) optional.
 */
double orc_sumscore_grad_f64(double alpha, double beta, const uint64_t *dm,
                             uint32_t n_nodes, const uint64_t *mut,
                             const uint64_t *known, uint32_t n_cells,
                             double *dalpha, double *dbeta,
                             double *posterior);

/* FP64 sum score logL = sum_c logsumexp_j s_cj (no prior) and the expected
 * class counts e[4] = sum_c sum_j pi_cj (n00, n01, n10, n11). */
double orc_sumscore_counts_f64(double alpha, double beta, const uint64_t *dm,
                               uint32_t n_nodes, const uint64_t *mut,
                               const uint64_t *known, uint32_t n_cells,
                               double *e);
/* FP64 class totals at the first-max attachment of the max score. */
double orc_maxscore_counts_f64(double alpha, double beta, const uint64_t *dm,
                               uint32_t n_nodes, const uint64_t *mut,
                               const uint64_t *known, uint32_t n_cells,
                               double *e);
/* FP64 log Beta prior of beta with the reference's parameters from
 * (beta_mean, beta_sd), src/TreeScorer.hpp:108-126. */
double orc_logprior_beta_f64(double beta_mean, double beta_sd, double beta);

/* ---- chain driver (src/Application.hpp:408-487) ---- */
typedef struct {
  float alpha_mean, beta_mean, beta_sd, gamma;
  int32_t score_mode; /* 0: reference cell-order sum, 1: class totals */
} orc_chain_params;

typedef struct {
  float proposed_score;
  float current_score; /* after the step */
  float current_beta;
  uint32_t accepted;
  uint32_t ambiguous;  /* decision taken from `forced_accept` */
  uint64_t counts[4];  /* class totals of the proposed tree */
} orc_step_trace;

/*
 * Runs one chain over `n_steps` recorded moves starting from (am, dm,
 * beta, score); updates the state in place.  The best proposal seen
 * (strict '>' after the first proposal, src/Application.hpp:456) is
 * tracked in best_* when `*best_valid` is 0 or its score is exceeded.
 * If `forced_accept` is non-NULL, a decision whose acceptance ratio lies
 * within `ambiguity` (relative) of the acceptance level takes
 * forced_accept[i] instead and is flagged.
 */
void orc_run_chain(const orc_chain_params *cp, uint32_t n_nodes,
                   const uint64_t *mut, const uint64_t *known,
                   uint32_t n_cells, const orc_raw_move *moves,
                   uint32_t n_steps, uint64_t *am, uint64_t *dm, float *beta,
                   float *score, int *best_valid, uint64_t *best_am,
                   uint64_t *best_dm, float *best_beta, float *best_score,
                   orc_step_trace *trace, const uint8_t *forced_accept,
                   float ambiguity);

/* ---- Philox4x32-10 move sampler shared with the CUDA path ---- */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]);
typedef struct {
  float cum_beta, cum_prune, cum_swap; /* cumulative move thresholds */
  float beta_jump_sd;
} orc_move_probs;
void orc_move_probs_from_params(orc_move_probs *mp, float prob_beta_change,
                                float prob_prune_n_reattach,
                                float prob_swap_nodes,
                                float prob_swap_subtrees, float beta_sd,
                                float beta_jump_scaling_chi);
void orc_sample_move(const orc_move_probs *mp, uint32_t n_nodes,
                     uint64_t seed, uint32_t chain, uint64_t step,
                     orc_raw_move *out);

/* ---- multi-threaded plain run (CPU baseline) ---- */
/*
 * Runs n_chains independent chains for n_steps Philox moves each using
 * n_threads POSIX threads; initial trees from `parents` (n_chains rows of
 * n_nodes).  Returns the best score; writes per-chain final scores.
 */
float orc_run_chains_mt(const orc_chain_params *cp,
                        const orc_move_probs *mp, uint64_t seed,
                        uint32_t n_nodes, const uint64_t *mut,
                        const uint64_t *known, uint32_t n_cells,
                        const uint32_t *parents, uint32_t n_chains,
                        uint32_t n_steps, uint32_t n_threads,
                        float *final_scores);

/* ---- CPUTreeScorer restatement (cpu_scoring_benchmark) ---- */
/*
 * The transposed scoring loop of cpu_scoring_benchmark/CPUTreeScorer.hpp:
 * 165-213 at its fixed 128 cells x 127 genes, 2 quadwords: for each node,
 * max over cells, summed over nodes.  `dmq` is [2][128] words (quadword,
 * node); `mutq`, `knownq` are [2][128] words (quadword, gene) with cell
 * bits.  Runs `n_trees` x `reps` scorings over n_threads threads and
 * returns the checksum of scores.
 */
void orc_cpu_proxy_scores(float alpha, float beta, const uint64_t *mutq,
                          const uint64_t *knownq, const uint64_t *dmq,
                          uint32_t n_trees, float *out);
double orc_cpu_scoring_proxy(float alpha, float beta, const uint64_t *mutq,
                             const uint64_t *knownq, const uint64_t *dmq,
                             uint32_t n_trees, uint32_t reps,
                             uint32_t n_threads);

#ifdef __cplusplus
}
#endif
#endif
