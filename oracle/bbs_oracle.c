/*
 * bbs_oracle.c -- CPU restatement of bbSCITE's MCMC hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path, and the CPU
 * baseline that bench.py times.  Nothing in bbscite_gb300/ links or loads
 * this file.  Every function names the reference lines it restates
 * (paths relative to the Janonard/bbSCITE project root).
 *
 * Parity pinning: tests/test_oracle.py checks these functions against the
 * reference's own known-answer tests (test/MutationTree.cpp,
 * test/TreeScorer.cpp, transcribed into tests/golden/kat.json) and against
 * golden vectors produced by the reference's own headers compiled on the
 * host (oracle/ref_driver.cpp, tests/golden/make_golden.py).
 *
 * Build: gcc -O3 -ffp-contract=off -fPIC -shared (see oracle/Makefile).
 * Floating-point contraction is off so that every float operation rounds
 * exactly as the reference's source order says.
 */
#include "bbs_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ORC_MAX_WORDS 8 /* 512 nodes */

uint32_t orc_words(uint32_t n_nodes) { return (n_nodes + 63u) / 64u; }

static inline int getb(const uint64_t *row, uint32_t i) {
  return (int)((row[i >> 6] >> (i & 63u)) & 1u);
}
static inline void setb(uint64_t *row, uint32_t i, int b) {
  uint64_t m = 1ull << (i & 63u);
  if (b)
    row[i >> 6] |= m;
  else
    row[i >> 6] &= ~m;
}
static inline int popc64(uint64_t x) { return __builtin_popcountll(x); }

/* ------------------------------------------------------------------ */
/* Tree construction                                                   */
/* ------------------------------------------------------------------ */

/* src/MutationTree.hpp:427-476 (Pruefer decoding, root = n_nodes-1) */
void orc_pruefer_to_parent_vector(const uint32_t *code, uint32_t code_len,
                                  uint32_t *parent) {
  uint32_t n_nodes = code_len + 2;
  uint32_t *degree = (uint32_t *)malloc(sizeof(uint32_t) * n_nodes);
  for (uint32_t i = 0; i < n_nodes; i++) {
    degree[i] = 1;
    parent[i] = n_nodes - 1;
  }
  for (uint32_t i = 0; i < code_len; i++)
    degree[code[i]]++;
  for (uint32_t i = 0; i < code_len; i++) {
    for (uint32_t j = 0; j < n_nodes; j++) {
      if (degree[j] == 1) {
        parent[j] = code[i];
        degree[code[i]]--;
        degree[j]--;
        break;
      }
    }
  }
  for (uint32_t i = 0; i < n_nodes; i++) {
    if (degree[i] == 1) {
      parent[i] = n_nodes - 1;
      break;
    }
  }
  free(degree);
}

/* src/MutationTree.hpp:379-409 */
void orc_parent_vector_to_matrix(const uint32_t *parent, uint32_t n_nodes,
                                 uint64_t *am, uint64_t *dm) {
  uint32_t W = orc_words(n_nodes), root = n_nodes - 1;
  memset(am, 0, sizeof(uint64_t) * W * n_nodes);
  memset(dm, 0, sizeof(uint64_t) * W * n_nodes);
  for (uint32_t i = 0; i < n_nodes; i++) {
    uint32_t anc = i;
    uint32_t guard = 0;
    while (anc != root && guard++ <= n_nodes) {
      setb(am + (size_t)anc * W, i, 1);
      setb(dm + (size_t)i * W, anc, 1);
      anc = parent[anc];
    }
    setb(am + (size_t)i * W, i, 1);
    setb(dm + (size_t)i * W, i, 1);
    setb(am + (size_t)root * W, i, 1);
    setb(dm + (size_t)i * W, root, 1);
  }
}

void orc_matrix_to_parent_vector(const uint64_t *am, const uint64_t *dm,
                                 uint32_t n_nodes, uint32_t *parent) {
  (void)am;
  for (uint32_t x = 0; x < n_nodes; x++)
    parent[x] = orc_get_parent(dm, n_nodes, x);
}

/* ------------------------------------------------------------------ */
/* Queries                                                             */
/* ------------------------------------------------------------------ */

/* src/MutationTree.hpp:549-575: `parent` is the parent of `child` iff it
 * is an ancestor of child and their ancestor sets agree everywhere except
 * at child; the root is its own parent. */
int orc_is_parent(const uint64_t *dm, uint32_t n_nodes, uint32_t parent,
                  uint32_t child) {
  uint32_t W = orc_words(n_nodes);
  const uint64_t *pa = dm + (size_t)parent * W;
  const uint64_t *ca = dm + (size_t)child * W;
  if (!getb(ca, parent))
    return 0;
  if (parent == child)
    return child == n_nodes - 1;
  for (uint32_t i = 0; i < n_nodes; i++) {
    if (i == child)
      continue;
    if (getb(pa, i) != getb(ca, i))
      return 0;
  }
  return 1;
}

/* src/MutationTree.hpp:585-596 (last matching node wins) */
uint32_t orc_get_parent(const uint64_t *dm, uint32_t n_nodes, uint32_t x) {
  uint32_t parent = 0;
  for (uint32_t j = 0; j < n_nodes; j++)
    if (orc_is_parent(dm, n_nodes, j, x))
      parent = j;
  return parent;
}

/* src/MutationTree.hpp:661-674 */
uint32_t orc_get_n_descendants(const uint64_t *am, uint32_t n_nodes,
                               uint32_t x) {
  uint32_t W = orc_words(n_nodes), n = 0;
  for (uint32_t i = 0; i < n_nodes; i++)
    n += (uint32_t)getb(am + (size_t)x * W, i);
  return n;
}

/* src/MutationTree.hpp:733-746 */
uint32_t orc_get_n_ancestors(const uint64_t *dm, uint32_t n_nodes,
                             uint32_t x) {
  uint32_t W = orc_words(n_nodes), n = 0;
  for (uint32_t i = 0; i < n_nodes; i++)
    n += (uint32_t)getb(dm + (size_t)x * W, i);
  return n;
}

/* src/MutationTree.hpp:840-878: the k-th (0-based) set bit of the
 * (complemented) descendant row among the first n_nodes bits; 0 if there
 * is none. */
uint32_t orc_get_descendant_or_nondescendant(const uint64_t *am,
                                             uint32_t n_nodes, uint32_t x,
                                             uint32_t k, int descendant) {
  uint32_t W = orc_words(n_nodes);
  const uint64_t *row = am + (size_t)x * W;
  for (uint32_t i = 0; i < n_nodes; i++) {
    int b = getb(row, i);
    if (!descendant)
      b = !b;
    if (b) {
      if (k == 0)
        return i;
      k--;
    }
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* Moves                                                               */
/* ------------------------------------------------------------------ */

/* src/MutationTree.hpp:323-363 */
void orc_realize_raw_move(const uint64_t *am, const uint64_t *dm,
                          uint32_t n_nodes, float beta,
                          const orc_raw_move *raw, orc_mod_params *out) {
  uint32_t W = orc_words(n_nodes);
  uint32_t v = raw->raw_v, w = raw->raw_w;
  if (getb(am + (size_t)v * W, w)) { /* is_ancestor(v, w) */
    uint32_t t = v;
    v = w;
    w = t;
  }
  uint32_t parent_of_v = orc_get_parent(dm, n_nodes, v);
  uint32_t parent_of_w = orc_get_parent(dm, n_nodes, w);
  uint32_t n_desc = orc_get_n_descendants(am, n_nodes, v);
  uint32_t n_nondesc = n_nodes - n_desc;
  /* float product, floor, then conversion to uint32 */
  float fd = floorf(raw->raw_descendant_of_v * (float)n_desc);
  float fn = floorf(raw->raw_nondescendant_of_v * (float)n_nondesc);
  uint32_t i_desc = (uint32_t)fd;
  uint32_t i_nondesc = (uint32_t)fn;
  out->move_type = raw->move_type;
  out->v = v;
  out->w = w;
  out->parent_of_v = parent_of_v;
  out->parent_of_w = parent_of_w;
  out->descendant_of_v =
      orc_get_descendant_or_nondescendant(am, n_nodes, v, i_desc, 1);
  out->nondescendant_of_v =
      orc_get_descendant_or_nondescendant(am, n_nodes, v, i_nondesc, 0);
  float nb = beta + raw->beta_jump;
  if (nb < 0)
    nb = fabsf(nb);
  if (nb > 1)
    nb = nb - 2.0f * (nb - 1.0f);
  out->new_beta = nb;
}

/* src/MutationTree.hpp:123-307, the bitwise update constructor, restated
 * bit by bit (x over nodes, y over all row bits). */
float orc_apply_move(const uint64_t *am, const uint64_t *dm, uint32_t n_nodes,
                     float beta, const orc_mod_params *p, uint64_t *new_am,
                     uint64_t *new_dm) {
  uint32_t W = orc_words(n_nodes), max_y = W * 64u;
  float new_beta = beta;
  if (p->move_type == ORC_CHANGE_BETA)
    new_beta = p->new_beta;
  uint32_t v = p->v, w = p->w;
  const uint64_t *v_desc = am + (size_t)v * W, *w_desc = am + (size_t)w * W;
  const uint64_t *v_anc = dm + (size_t)v * W, *w_anc = dm + (size_t)w * W;
  uint32_t v_target = 0, w_target = 0;
  switch (p->move_type) {
  case ORC_SWAP_SUBTREES:
    v_target = p->parent_of_w;
    w_target = getb(w_desc, v) ? p->descendant_of_v : p->parent_of_v;
    break;
  case ORC_PRUNE_REATTACH:
    v_target = p->nondescendant_of_v;
    w_target = 0;
    break;
  default:
    v_target = w_target = 0;
  }
  const uint64_t *vt_anc = dm + (size_t)v_target * W;
  const uint64_t *wt_anc = dm + (size_t)w_target * W;

  for (uint32_t x = 0; x < n_nodes; x++) {
    const uint64_t *x_desc = am + (size_t)x * W, *x_anc = dm + (size_t)x * W;
    uint64_t *na = new_am + (size_t)x * W, *nd = new_dm + (size_t)x * W;
    for (uint32_t k = 0; k < W; k++) {
      na[k] = x_desc[k];
      nd[k] = x_anc[k];
    }
    for (uint32_t y = 0; y < max_y; y++) {
      int x_to_y, y_to_x;
      switch (p->move_type) {
      case ORC_SWAP_NODES:
        if (x == v) {
          if (y == v) {
            x_to_y = y_to_x = 1;
          } else if (y == w) {
            x_to_y = getb(w_desc, v);
            y_to_x = getb(v_desc, w);
          } else {
            x_to_y = getb(w_desc, y);
            y_to_x = getb(w_anc, y);
          }
        } else if (x == w) {
          if (y == v) {
            x_to_y = getb(v_desc, w);
            y_to_x = getb(w_desc, v);
          } else if (y == w) {
            x_to_y = y_to_x = 1;
          } else {
            x_to_y = getb(v_desc, y);
            y_to_x = getb(v_anc, y);
          }
        } else {
          if (y == v) {
            x_to_y = getb(x_desc, w);
            y_to_x = getb(x_anc, w);
          } else if (y == w) {
            x_to_y = getb(x_desc, v);
            y_to_x = getb(x_anc, v);
          } else {
            x_to_y = getb(x_desc, y);
            y_to_x = getb(x_anc, y);
          }
        }
        break;
      case ORC_PRUNE_REATTACH:
        if (getb(v_desc, y))
          x_to_y = getb(x_desc, v_target) ||
                   (getb(v_desc, x) && getb(x_desc, y));
        else
          x_to_y = getb(x_desc, y);
        if (getb(v_desc, x))
          y_to_x = getb(vt_anc, y) || (getb(x_anc, y) && getb(v_desc, y));
        else
          y_to_x = getb(x_anc, y);
        break;
      case ORC_SWAP_SUBTREES:
        if (getb(w_desc, v)) {
          int cx = getb(v_desc, x) ? 2 : (getb(w_desc, x) ? 1 : 0);
          int cy = getb(v_desc, y) ? 2 : (getb(w_desc, y) ? 1 : 0);
          if (cx == cy || (cx == 0 && (cy == 1 || cy == 2)))
            x_to_y = getb(x_desc, y);
          else if (cx == 2 && cy == 1)
            x_to_y = getb(x_desc, w_target);
          else
            x_to_y = 0;
          if (cx == cy || (cy == 0 && (cx == 1 || cx == 2)))
            y_to_x = getb(x_anc, y);
          else if (cy == 2 && cx == 1)
            y_to_x = getb(wt_anc, y);
          else
            y_to_x = 0;
        } else {
          if (getb(v_desc, y) && !getb(w_desc, y))
            x_to_y = getb(x_desc, v_target) ||
                     (getb(v_desc, x) && getb(x_desc, y));
          else if (!getb(v_desc, y) && getb(w_desc, y))
            x_to_y = getb(x_desc, w_target) ||
                     (getb(w_desc, x) && getb(x_desc, y));
          else
            x_to_y = getb(x_desc, y);
          if (getb(v_desc, x) && !getb(w_desc, x))
            y_to_x = getb(vt_anc, y) || (getb(v_desc, y) && getb(x_anc, y));
          else if (!getb(v_desc, x) && getb(w_desc, x))
            y_to_x = getb(wt_anc, y) || (getb(w_desc, y) && getb(x_anc, y));
          else
            y_to_x = getb(x_anc, y);
        }
        break;
      case ORC_CHANGE_BETA:
      default:
        x_to_y = getb(x_desc, y);
        y_to_x = getb(x_anc, y);
        break;
      }
      setb(na, y, x_to_y);
      setb(nd, y, y_to_x);
    }
  }
  return new_beta;
}

/* ------------------------------------------------------------------ */
/* Scoring                                                             */
/* ------------------------------------------------------------------ */

/* src/TreeScorer.hpp:99-111: the log table (double math rounded to
 * float for the 1-x entries, float logf for the x entries) and the Beta
 * prior parameters (std::pow(float,int) promotes to double). */
void orc_scorer_init(orc_scorer *s, float alpha_mean, float beta_mean,
                     float beta_sd) {
  s->l00 = (float)log(1.0 - (double)alpha_mean);
  s->l10 = logf(alpha_mean);
  s->l01 = logf(beta_mean);
  s->l11 = (float)log(1.0 - (double)beta_mean);
  s->bpriora = (float)(((double)(1.0f - beta_mean) *
                        pow((double)beta_mean, 2.0) /
                        pow((double)beta_sd, 2.0)) -
                       (double)beta_mean);
  s->bpriorb = s->bpriora * ((1.0f / beta_mean) - 1.0f);
}

/* src/TreeScorer.hpp:136-137 */
void orc_scorer_set_beta(orc_scorer *s, float beta) {
  s->l01 = logf(beta);
  s->l11 = (float)log(1.0 - (double)beta);
}

/* src/TreeScorer.hpp:122-126 (float tgamma/log) */
float orc_logscore_beta(const orc_scorer *s, float beta) {
  float a = s->bpriora, b = s->bpriorb;
  float r = logf(tgammaf(a + b));
  r = r + (a - 1.0f) * logf(beta);
  r = r + (b - 1.0f) * logf(1.0f - beta);
  r = r - logf(tgammaf(a));
  r = r - logf(tgammaf(b));
  return r;
}

float orc_score_from_totals(const orc_scorer *s, const uint64_t *counts,
                            float beta) {
  float t = (float)counts[0] * s->l00;
  t = t + (float)counts[1] * s->l01;
  t = t + (float)counts[2] * s->l10;
  t = t + (float)counts[3] * s->l11;
  return t + orc_logscore_beta(s, beta);
}

/* src/TreeScorer.hpp:131-210.  The scorer reads the ancestor rows
 * (get_ancestors = dm row); for every node j and cell c the four class
 * counts popcount(known & (o ? mut : ~mut) & (t ? anc_j : ~anc_j)) are
 * weighted by the log table in the order (0,0),(0,1),(1,0),(1,1); the
 * per-cell maximum keeps the first node on ties (std::max(old, new));
 * the cell maxima are summed in cell order and the Beta prior is added.
 * The table's beta entries are refreshed from `beta` first. */
float orc_logscore_tree(const orc_scorer *s0, const uint64_t *dm,
                        uint32_t n_nodes, const uint64_t *mut,
                        const uint64_t *known, uint32_t n_cells, float beta,
                        uint64_t *counts, float *score_totals,
                        uint32_t *attach) {
  orc_scorer s = *s0;
  orc_scorer_set_beta(&s, beta);
  const float l00 = s.l00, l01 = s.l01, l10 = s.l10, l11 = s.l11;
  uint32_t W = orc_words(n_nodes);
  uint64_t tot[4] = {0, 0, 0, 0};
  float tree_score = 0.0f;
  for (uint32_t c = 0; c < n_cells; c++) {
    const uint64_t *M = mut + (size_t)c * W, *K = known + (size_t)c * W;
    float best = 0.0f;
    uint32_t best_j = 0, best_n[4] = {0, 0, 0, 0};
    for (uint32_t j = 0; j < n_nodes; j++) {
      const uint64_t *A = dm + (size_t)j * W;
      /* popcount(known & (o ? mut : ~mut) & (t ? anc : ~anc)) */
      uint32_t n00 = 0, n01 = 0, n10 = 0, n11 = 0;
      for (uint32_t k = 0; k < W; k++) {
        const uint64_t kn = K[k], mu = M[k], a = A[k];
        n00 += (uint32_t)popc64(kn & ~mu & ~a);
        n01 += (uint32_t)popc64(kn & ~mu & a);
        n10 += (uint32_t)popc64(kn & mu & ~a);
        n11 += (uint32_t)popc64(kn & mu & a);
      }
      /* weighted in the order (0,0), (0,1), (1,0), (1,1) */
      float sc = 0.0f;
      sc += (float)n00 * l00;
      sc += (float)n01 * l01;
      sc += (float)n10 * l10;
      sc += (float)n11 * l11;
      if (j == 0 || best < sc) {
        best = sc;
        best_j = j;
        best_n[0] = n00;
        best_n[1] = n01;
        best_n[2] = n10;
        best_n[3] = n11;
      }
    }
    tree_score += best;
    for (int q = 0; q < 4; q++)
      tot[q] += best_n[q];
    if (attach)
      attach[c] = best_j;
  }
  float prior = orc_logscore_beta(&s, beta);
  if (counts)
    memcpy(counts, tot, sizeof(tot));
  if (score_totals)
    *score_totals = orc_score_from_totals(&s, tot, beta);
  return tree_score + prior;
}

/* FP64 restatement of the max score (same formula, double arithmetic). */
double orc_logscore_tree_f64(double alpha, double beta, double beta_mean,
                             double beta_sd, const uint64_t *dm,
                             uint32_t n_nodes, const uint64_t *mut,
                             const uint64_t *known, uint32_t n_cells,
                             int with_prior) {
  double L[2][2] = {{log(1.0 - alpha), log(beta)},
                    {log(alpha), log(1.0 - beta)}};
  uint32_t W = orc_words(n_nodes);
  double total = 0.0;
  for (uint32_t c = 0; c < n_cells; c++) {
    const uint64_t *M = mut + (size_t)c * W, *K = known + (size_t)c * W;
    double best = -INFINITY;
    for (uint32_t j = 0; j < n_nodes; j++) {
      const uint64_t *A = dm + (size_t)j * W;
      double sc = 0.0;
      for (int o = 0; o < 2; o++)
        for (int t = 0; t < 2; t++) {
          uint32_t cnt = 0;
          for (uint32_t k = 0; k < W; k++)
            cnt += (uint32_t)popc64(K[k] & (o ? M[k] : ~M[k]) &
                                    (t ? A[k] : ~A[k]));
          sc += (double)cnt * L[o][t];
        }
      if (j == 0 || sc > best)
        best = sc;
    }
    total += best;
  }
  if (with_prior) {
    double a = ((1.0 - beta_mean) * beta_mean * beta_mean /
                (beta_sd * beta_sd)) -
               beta_mean;
    double b = a * (1.0 / beta_mean - 1.0);
    total += lgamma(a + b) + (a - 1.0) * log(beta) +
             (b - 1.0) * log(1.0 - beta) - lgamma(a) - lgamma(b);
  }
  return total;
}

/* Sum-over-attachments score in FP64 and its gradient.  s_cj is the same
 * per-(cell,node) log-likelihood as above; logL = sum_c logsumexp_j s_cj;
 * d s_cj / d alpha = -n00/(1-alpha) + n10/alpha,
 * d s_cj / d beta  =  n01/beta - n11/(1-beta),
 * d logL / d theta = sum_c sum_j pi_cj d s_cj / d theta, pi = softmax_j. */
double orc_sumscore_grad_f64(double alpha, double beta, const uint64_t *dm,
                             uint32_t n_nodes, const uint64_t *mut,
                             const uint64_t *known, uint32_t n_cells,
                             double *dalpha, double *dbeta,
                             double *posterior) {
  double L[2][2] = {{log(1.0 - alpha), log(beta)},
                    {log(alpha), log(1.0 - beta)}};
  uint32_t W = orc_words(n_nodes);
  double *sc = (double *)malloc(sizeof(double) * n_nodes);
  double *dn = (double *)malloc(sizeof(double) * n_nodes * 4);
  double total = 0.0, ga = 0.0, gb = 0.0;
  for (uint32_t c = 0; c < n_cells; c++) {
    const uint64_t *M = mut + (size_t)c * W, *K = known + (size_t)c * W;
    double mx = -INFINITY;
    for (uint32_t j = 0; j < n_nodes; j++) {
      const uint64_t *A = dm + (size_t)j * W;
      double s = 0.0;
      for (int o = 0; o < 2; o++)
        for (int t = 0; t < 2; t++) {
          uint32_t cnt = 0;
          for (uint32_t k = 0; k < W; k++)
            cnt += (uint32_t)popc64(K[k] & (o ? M[k] : ~M[k]) &
                                    (t ? A[k] : ~A[k]));
          dn[j * 4 + o * 2 + t] = (double)cnt;
          s += (double)cnt * L[o][t];
        }
      sc[j] = s;
      if (s > mx)
        mx = s;
    }
    double z = 0.0;
    for (uint32_t j = 0; j < n_nodes; j++)
      z += exp(sc[j] - mx);
    total += mx + log(z);
    for (uint32_t j = 0; j < n_nodes; j++) {
      double pi = exp(sc[j] - mx) / z;
      if (posterior)
        posterior[(size_t)c * n_nodes + j] = pi;
      ga += pi * (-dn[j * 4 + 0] / (1.0 - alpha) + dn[j * 4 + 2] / alpha);
      gb += pi * (dn[j * 4 + 1] / beta - dn[j * 4 + 3] / (1.0 - beta));
    }
  }
  free(sc);
  free(dn);
  if (dalpha)
    *dalpha = ga;
  if (dbeta)
    *dbeta = gb;
  return total;
}

/* Per-(cell,node) class counts. */
static void pair_counts(const uint64_t *K, const uint64_t *M,
                        const uint64_t *A, uint32_t W, double n[4]) {
  uint32_t c[4] = {0, 0, 0, 0};
  for (uint32_t k = 0; k < W; k++) {
    c[0] += (uint32_t)popc64(K[k] & ~M[k] & ~A[k]);
    c[1] += (uint32_t)popc64(K[k] & ~M[k] & A[k]);
    c[2] += (uint32_t)popc64(K[k] & M[k] & ~A[k]);
    c[3] += (uint32_t)popc64(K[k] & M[k] & A[k]);
  }
  for (int q = 0; q < 4; q++)
    n[q] = (double)c[q];
}

double orc_sumscore_counts_f64(double alpha, double beta, const uint64_t *dm,
                               uint32_t n_nodes, const uint64_t *mut,
                               const uint64_t *known, uint32_t n_cells,
                               double *e) {
  const double L[4] = {log(1.0 - alpha), log(beta), log(alpha),
                       log(1.0 - beta)};
  uint32_t W = orc_words(n_nodes);
  double *sc = (double *)malloc(sizeof(double) * n_nodes);
  double *cn = (double *)malloc(sizeof(double) * n_nodes * 4);
  double total = 0.0, acc[4] = {0, 0, 0, 0};
  for (uint32_t c = 0; c < n_cells; c++) {
    const uint64_t *M = mut + (size_t)c * W, *K = known + (size_t)c * W;
    double mx = -INFINITY;
    for (uint32_t j = 0; j < n_nodes; j++) {
      pair_counts(K, M, dm + (size_t)j * W, W, cn + 4 * j);
      double s = 0.0;
      for (int q = 0; q < 4; q++)
        s += cn[4 * j + q] * L[q];
      sc[j] = s;
      if (s > mx)
        mx = s;
    }
    double z = 0.0;
    for (uint32_t j = 0; j < n_nodes; j++)
      z += exp(sc[j] - mx);
    total += mx + log(z);
    for (uint32_t j = 0; j < n_nodes; j++) {
      const double pi = exp(sc[j] - mx) / z;
      for (int q = 0; q < 4; q++)
        acc[q] += pi * cn[4 * j + q];
    }
  }
  free(sc);
  free(cn);
  if (e)
    for (int q = 0; q < 4; q++)
      e[q] = acc[q];
  return total;
}

double orc_maxscore_counts_f64(double alpha, double beta, const uint64_t *dm,
                               uint32_t n_nodes, const uint64_t *mut,
                               const uint64_t *known, uint32_t n_cells,
                               double *e) {
  const double L[4] = {log(1.0 - alpha), log(beta), log(alpha),
                       log(1.0 - beta)};
  uint32_t W = orc_words(n_nodes);
  double total = 0.0, acc[4] = {0, 0, 0, 0};
  for (uint32_t c = 0; c < n_cells; c++) {
    const uint64_t *M = mut + (size_t)c * W, *K = known + (size_t)c * W;
    double best = -INFINITY, bn[4] = {0, 0, 0, 0};
    for (uint32_t j = 0; j < n_nodes; j++) {
      double n[4];
      pair_counts(K, M, dm + (size_t)j * W, W, n);
      double s = 0.0;
      for (int q = 0; q < 4; q++)
        s += n[q] * L[q];
      if (j == 0 || s > best) {
        best = s;
        memcpy(bn, n, sizeof(bn));
      }
    }
    total += best;
    for (int q = 0; q < 4; q++)
      acc[q] += bn[q];
  }
  if (e)
    for (int q = 0; q < 4; q++)
      e[q] = acc[q];
  return total;
}

double orc_logprior_beta_f64(double beta_mean, double beta_sd, double beta) {
  const double a = ((1.0 - beta_mean) * beta_mean * beta_mean /
                    (beta_sd * beta_sd)) -
                   beta_mean;
  const double b = a * (1.0 / beta_mean - 1.0);
  return lgamma(a + b) + (a - 1.0) * log(beta) + (b - 1.0) * log(1.0 - beta) -
         lgamma(a) - lgamma(b);
}

/* ------------------------------------------------------------------ */
/* Chain driver                                                        */
/* ------------------------------------------------------------------ */

/* src/Application.hpp:408-487, one chain, recorded moves. */
void orc_run_chain(const orc_chain_params *cp, uint32_t n_nodes,
                   const uint64_t *mut, const uint64_t *known,
                   uint32_t n_cells, const orc_raw_move *moves,
                   uint32_t n_steps, uint64_t *am, uint64_t *dm, float *beta,
                   float *score, int *best_valid, uint64_t *best_am,
                   uint64_t *best_dm, float *best_beta, float *best_score,
                   orc_step_trace *trace, const uint8_t *forced_accept,
                   float ambiguity) {
  uint32_t W = orc_words(n_nodes);
  size_t nw = (size_t)W * n_nodes;
  orc_scorer sc;
  orc_scorer_init(&sc, cp->alpha_mean, cp->beta_mean, cp->beta_sd);
  uint64_t *pam = (uint64_t *)malloc(sizeof(uint64_t) * nw);
  uint64_t *pdm = (uint64_t *)malloc(sizeof(uint64_t) * nw);
  float cur_beta = *beta, cur_score = *score;
  for (uint32_t i = 0; i < n_steps; i++) {
    orc_mod_params mp;
    orc_realize_raw_move(am, dm, n_nodes, cur_beta, &moves[i], &mp);
    float prop_beta = orc_apply_move(am, dm, n_nodes, cur_beta, &mp, pam, pdm);
    uint64_t counts[4];
    float st;
    float sref = orc_logscore_tree(&sc, pdm, n_nodes, mut, known, n_cells,
                                   prop_beta, counts, &st, NULL);
    float prop_score = cp->score_mode ? st : sref;
    float corr;
    if (moves[i].move_type == ORC_SWAP_SUBTREES &&
        getb(am + (size_t)mp.w * W, mp.v))
      corr = (float)orc_get_n_descendants(am, n_nodes, mp.v) /
             (float)orc_get_n_descendants(am, n_nodes, mp.w);
    else
      corr = 1.0f;
    float ratio = corr * expf((prop_score - cur_score) * cp->gamma);
    int accept = ratio > moves[i].acceptance_level;
    int ambiguous = 0;
    if (forced_accept) {
      float u = moves[i].acceptance_level;
      float d = fabsf(ratio - u);
      if (d <= ambiguity * fabsf(u) || d <= ambiguity * fabsf(ratio)) {
        ambiguous = (accept != (int)forced_accept[i]);
        accept = forced_accept[i];
      }
    }
    if (!*best_valid || prop_score > *best_score) {
      *best_valid = 1;
      *best_score = prop_score;
      *best_beta = prop_beta;
      if (best_am)
        memcpy(best_am, pam, sizeof(uint64_t) * nw);
      if (best_dm)
        memcpy(best_dm, pdm, sizeof(uint64_t) * nw);
    }
    if (accept) {
      memcpy(am, pam, sizeof(uint64_t) * nw);
      memcpy(dm, pdm, sizeof(uint64_t) * nw);
      cur_beta = prop_beta;
      cur_score = prop_score;
    }
    if (trace) {
      trace[i].proposed_score = prop_score;
      trace[i].current_score = cur_score;
      trace[i].current_beta = cur_beta;
      trace[i].accepted = (uint32_t)accept;
      trace[i].ambiguous = (uint32_t)ambiguous;
      memcpy(trace[i].counts, counts, sizeof(counts));
    }
  }
  *beta = cur_beta;
  *score = cur_score;
  free(pam);
  free(pdm);
}

/* ------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers:  */
/* as easy as 1, 2, 3", SC'11) and the move sampler of the CUDA path.  */
/* ------------------------------------------------------------------ */

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

/* src/Parameters.hpp:451-541 (probabilities normalised by their float
 * sum) and src/RawMoveDistribution.hpp:119-131 (cumulative thresholds
 * accumulated in float in this order); jump sd = beta_sd / chi
 * (src/Parameters.hpp:582-584). */
void orc_move_probs_from_params(orc_move_probs *mp, float prob_beta_change,
                                float prob_prune_n_reattach,
                                float prob_swap_nodes,
                                float prob_swap_subtrees, float beta_sd,
                                float beta_jump_scaling_chi) {
  float sum = prob_beta_change + prob_prune_n_reattach + prob_swap_nodes +
              prob_swap_subtrees;
  float pb = prob_beta_change / sum, pp = prob_prune_n_reattach / sum,
        ps = prob_swap_nodes / sum;
  mp->cum_beta = pb;
  mp->cum_prune = pb + pp;
  mp->cum_swap = pb + pp + ps;
  mp->beta_jump_sd = beta_sd / beta_jump_scaling_chi;
}

static inline float u01_24(uint32_t x) {
  return (float)(x >> 8) * (1.0f / 16777216.0f);
}
static inline uint32_t uniform_below(uint32_t x, uint32_t n) {
  return (uint32_t)(((uint64_t)x * (uint64_t)n) >> 32);
}

/*
 * One RawMoveSample from two Philox blocks keyed by the run seed with
 * counter (step_lo, step_hi, chain, block).  The field meanings follow
 * src/RawMoveDistribution.hpp:97-155: move type by cumulative '<='
 * thresholds; v uniform in [0, n-2], w uniform in [0, n-3] then w++ if
 * w >= v; three uniforms in [0,1); one N(0, sd) jump (Box-Muller).
 * The device sampler uses the same words; the jump goes through the
 * device's log/cos, so replays that need bit-exact beta use recorded
 * moves.
 */
void orc_sample_move(const orc_move_probs *mp, uint32_t n_nodes,
                     uint64_t seed, uint32_t chain, uint64_t step,
                     orc_raw_move *out) {
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t c0[4] = {(uint32_t)step, (uint32_t)(step >> 32), chain, 0u};
  uint32_t c1[4] = {(uint32_t)step, (uint32_t)(step >> 32), chain, 1u};
  uint32_t a[4], b[4];
  orc_philox4x32_10(c0, key, a);
  orc_philox4x32_10(c1, key, b);
  float ut = u01_24(a[0]);
  int32_t type;
  if (ut <= mp->cum_beta)
    type = ORC_CHANGE_BETA;
  else if (ut <= mp->cum_prune)
    type = ORC_PRUNE_REATTACH;
  else if (ut <= mp->cum_swap)
    type = ORC_SWAP_NODES;
  else
    type = ORC_SWAP_SUBTREES;
  uint32_t v = uniform_below(a[1], n_nodes - 1);
  uint32_t w = uniform_below(a[2], n_nodes - 2);
  if (w >= v)
    w++;
  out->move_type = type;
  out->raw_v = v;
  out->raw_w = w;
  out->raw_descendant_of_v = u01_24(a[3]);
  out->raw_nondescendant_of_v = u01_24(b[0]);
  out->acceptance_level = u01_24(b[1]);
  float u1 = ((float)(b[2] >> 8) + 1.0f) * (1.0f / 16777216.0f);
  float u2 = u01_24(b[3]);
  float z = sqrtf(-2.0f * logf(u1)) * cosf(6.2831853071795864769f * u2);
  out->beta_jump = z * mp->beta_jump_sd;
  out->pad_ = 0;
}

/* ------------------------------------------------------------------ */
/* Multi-threaded plain run (CPU baseline)                             */
/* ------------------------------------------------------------------ */

typedef struct {
  const orc_chain_params *cp;
  const orc_move_probs *mp;
  uint64_t seed;
  uint32_t n_nodes, n_cells, n_chains, n_steps, n_threads, tid;
  const uint64_t *mut, *known;
  const uint32_t *parents;
  float *final_scores, *best_scores;
} orc_mt_job;

static void *orc_mt_worker(void *arg) {
  orc_mt_job *j = (orc_mt_job *)arg;
  uint32_t W = orc_words(j->n_nodes);
  size_t nw = (size_t)W * j->n_nodes;
  uint64_t *am = (uint64_t *)malloc(sizeof(uint64_t) * nw);
  uint64_t *dm = (uint64_t *)malloc(sizeof(uint64_t) * nw);
  orc_raw_move *moves = (orc_raw_move *)malloc(sizeof(orc_raw_move) * 1024);
  orc_scorer sc;
  orc_scorer_init(&sc, j->cp->alpha_mean, j->cp->beta_mean, j->cp->beta_sd);
  for (uint32_t c = j->tid; c < j->n_chains; c += j->n_threads) {
    orc_parent_vector_to_matrix(j->parents + (size_t)c * j->n_nodes,
                                j->n_nodes, am, dm);
    float beta = j->cp->beta_mean;
    float st;
    float sref = orc_logscore_tree(&sc, dm, j->n_nodes, j->mut, j->known,
                                   j->n_cells, beta, NULL, &st, NULL);
    float score = j->cp->score_mode ? st : sref;
    int best_valid = 0;
    float best_beta = 0, best_score = -INFINITY;
    for (uint32_t s0 = 0; s0 < j->n_steps; s0 += 1024) {
      uint32_t n = j->n_steps - s0 < 1024 ? j->n_steps - s0 : 1024;
      for (uint32_t i = 0; i < n; i++)
        orc_sample_move(j->mp, j->n_nodes, j->seed, c, (uint64_t)s0 + i,
                        &moves[i]);
      orc_run_chain(j->cp, j->n_nodes, j->mut, j->known, j->n_cells, moves,
                    n, am, dm, &beta, &score, &best_valid, NULL, NULL,
                    &best_beta, &best_score, NULL, NULL, 0.0f);
    }
    if (j->final_scores)
      j->final_scores[c] = score;
    j->best_scores[c] = best_score;
  }
  free(am);
  free(dm);
  free(moves);
  return NULL;
}

float orc_run_chains_mt(const orc_chain_params *cp,
                        const orc_move_probs *mp, uint64_t seed,
                        uint32_t n_nodes, const uint64_t *mut,
                        const uint64_t *known, uint32_t n_cells,
                        const uint32_t *parents, uint32_t n_chains,
                        uint32_t n_steps, uint32_t n_threads,
                        float *final_scores) {
  if (n_threads < 1)
    n_threads = 1;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * n_threads);
  orc_mt_job *jobs = (orc_mt_job *)malloc(sizeof(orc_mt_job) * n_threads);
  float *best = (float *)malloc(sizeof(float) * n_chains);
  for (uint32_t t = 0; t < n_threads; t++) {
    orc_mt_job j = {cp,       mp,        seed,    n_nodes, n_cells,
                    n_chains, n_steps,   n_threads, t,     mut,
                    known,    parents,   final_scores, best};
    jobs[t] = j;
    pthread_create(&th[t], NULL, orc_mt_worker, &jobs[t]);
  }
  for (uint32_t t = 0; t < n_threads; t++)
    pthread_join(th[t], NULL);
  float b = best[0];
  for (uint32_t c = 1; c < n_chains; c++)
    if (best[c] > b)
      b = best[c];
  free(th);
  free(jobs);
  free(best);
  return b;
}

/* ------------------------------------------------------------------ */
/* CPUTreeScorer proxy                                                 */
/* ------------------------------------------------------------------ */

typedef struct {
  float L[2][2];
  const uint64_t *mutq, *knownq, *dmq;
  uint32_t n_trees, reps, n_threads, tid;
  double sum;
} orc_proxy_job;

/* cpu_scoring_benchmark/CPUTreeScorer.hpp:165-213 (AVX2 variant): for
 * every node, the maximum over cells of the four-class score over two
 * quadwords, summed over nodes.  noipa: the compiler may not learn that
 * the function is pure, so the benchmark's repeated scorings of a tree
 * are not hoisted out of their loop and done once. */
static float __attribute__((noipa)) orc_proxy_score(const float L[2][2],
                                                    const uint64_t *mutq,
                             const uint64_t *knownq, const uint64_t *dm) {
  float tree_score = 0.0f;
  for (uint32_t node = 0; node < 128; node++) {
    float node_score = -INFINITY;
    for (uint32_t cell = 0; cell < 128; cell++) {
      float s = 0.0f;
      for (int o = 0; o < 2; o++)
        for (int t = 0; t < 2; t++) {
          uint32_t n = 0;
          for (int q = 0; q < 2; q++) {
            uint64_t occ = knownq[q * 128 + cell];
            occ &= o ? mutq[q * 128 + cell] : ~mutq[q * 128 + cell];
            occ &= t ? dm[q * 128 + node] : ~dm[q * 128 + node];
            n += (uint32_t)popc64(occ);
          }
          s += (float)n * L[o][t];
        }
      node_score = node_score < s ? s : node_score;  /* std::max(node_score, s) */
    }
    tree_score += node_score;
  }
  return tree_score;
}

static void *orc_proxy_worker(void *arg) {
  orc_proxy_job *j = (orc_proxy_job *)arg;
  double sum = 0.0;
  for (uint32_t t = j->tid; t < j->n_trees; t += j->n_threads)
    for (uint32_t r = 0; r < j->reps; r++)
      sum += orc_proxy_score(j->L, j->mutq, j->knownq, j->dmq + t * 256);
  j->sum = sum;
  return NULL;
}

/* The scores of n_trees trees (dmq: n_trees x 2 x 128 words), one by one:
 * the per-tree values the benchmark loop sums. */
void orc_cpu_proxy_scores(float alpha, float beta, const uint64_t *mutq,
                          const uint64_t *knownq, const uint64_t *dmq,
                          uint32_t n_trees, float *out) {
  float L[2][2];
  L[0][0] = (float)log(1.0 - (double)alpha);
  L[1][0] = logf(alpha);
  L[0][1] = logf(beta);
  L[1][1] = (float)log(1.0 - (double)beta);
  for (uint32_t t = 0; t < n_trees; t++)
    out[t] = orc_proxy_score(L, mutq, knownq, dmq + t * 256);
}

double orc_cpu_scoring_proxy(float alpha, float beta, const uint64_t *mutq,
                             const uint64_t *knownq, const uint64_t *dmq,
                             uint32_t n_trees, uint32_t reps,
                             uint32_t n_threads) {
  if (n_threads < 1)
    n_threads = 1;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * n_threads);
  orc_proxy_job *jobs =
      (orc_proxy_job *)malloc(sizeof(orc_proxy_job) * n_threads);
  for (uint32_t t = 0; t < n_threads; t++) {
    jobs[t].L[0][0] = (float)log(1.0 - (double)alpha);
    jobs[t].L[1][0] = logf(alpha);
    jobs[t].L[0][1] = logf(beta);
    jobs[t].L[1][1] = (float)log(1.0 - (double)beta);
    jobs[t].mutq = mutq;
    jobs[t].knownq = knownq;
    jobs[t].dmq = dmq;
    jobs[t].n_trees = n_trees;
    jobs[t].reps = reps;
    jobs[t].n_threads = n_threads;
    jobs[t].tid = t;
    pthread_create(&th[t], NULL, orc_proxy_worker, &jobs[t]);
  }
  double s = 0.0;
  for (uint32_t t = 0; t < n_threads; t++) {
    pthread_join(th[t], NULL);
    s += jobs[t].sum;
  }
  free(th);
  free(jobs);
  return s;
}
