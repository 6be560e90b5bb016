/*
 * bbscite_gb300.hpp -- the reference's C++ surface (Parameters,
 * MutationTree, TreeScorer, Application) as header-only wrappers over the C
 * ABI in bbscite_gb300.h.
 *
 * Differences from the reference's templates (src/MutationTree.hpp,
 * src/TreeScorer.hpp, src/Application.hpp, src/Parameters.hpp):
 *   - sizes are runtime values (up to BBS_MAX_GENES genes and BBS_MAX_CELLS
 *     cells) instead of template caps; an AncestorMatrix is a vector of
 *     n_nodes rows of bbs_words(n_nodes) uint64 words, bit y of row x;
 *   - a failed C-ABI call throws bbSCITE::Error carrying bbs_last_error();
 *   - Application takes host bit rows instead of SYCL buffers and a queue,
 *     keeps any chain count (no rounding up to a pipeline capacity) and
 *     draws moves on the device from a Philox stream keyed by the -seed
 *     value, so runs are reproducible.
 */
#ifndef BBSCITE_GB300_HPP
#define BBSCITE_GB300_HPP

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <map>
#include <memory>
#include <optional>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "bbscite_gb300.h"

namespace bbSCITE {

struct Error : std::runtime_error {
  int status;
  Error(int status, const char *what) : std::runtime_error(what), status(status) {}
};

inline void check(int status) {
  if (status != BBS_OK) throw Error(status, bbs_last_error());
}

/* src/MoveType.hpp:23-42 */
enum class MoveType : int32_t {
  ChangeBeta = BBS_MOVE_CHANGE_BETA,
  PruneReattach = BBS_MOVE_PRUNE_REATTACH,
  SwapNodes = BBS_MOVE_SWAP_NODES,
  SwapSubtrees = BBS_MOVE_SWAP_SUBTREES,
};

using RawMoveSample = bbs_raw_move;             // src/RawMoveDistribution.hpp:44-50
using ModificationParameters = bbs_move_params;  // src/MutationTree.hpp:84-89
using AncestorMatrix = std::vector<uint64_t>;

/* ------------------------------------------------------------------ */
/* src/Parameters.hpp: the SCITE-compatible command line.               */
class Parameters {
 public:
  Parameters() = default;

  /* Same flags, warnings, errors and result as
   * src/Parameters.hpp:61-281.  Extensions: -seed <n> is used (the
   * reference ignores it), -score max|sum, -error_move beta|rw|langevin and
   * -error_step <x> select the score and the error-rate move. */
  bool load_and_verify_args(int argc, char **argv) {
    bool error = false;
    auto missing = [&](const char *flag) {
      std::cerr << "Error: Missing argument to parameter " << flag << "."
                << std::endl;
      error = true;
    };
    auto warn_ignored = [](const char *flag) {
      std::cerr << "Warning: The " << flag
                << " parameter is not supported by bbSCITE (yet). Ignoring "
                   "the "
                << flag << " parameter." << std::endl;
    };
    auto nonneg = [&](float v) {
      if (v < 0.0f) {
        std::cerr << "Error: Move probabilities may not be negative."
                  << std::endl;
        error = true;
      }
      return v;
    };
    for (int i = 1; i < argc; ++i) {
      const char *a = argv[i];
      if (a[0] != '-') continue;
      const bool has_next = i + 1 < argc;
      if (!std::strcmp(a, "-i")) {
        if (has_next) input_path = argv[++i]; else missing(a);
      } else if (!std::strcmp(a, "-t")) {
        warn_ignored("-t");
      } else if (!std::strcmp(a, "-o")) {
        if (has_next) output_path_base = argv[++i]; else missing(a);
      } else if (!std::strcmp(a, "-n")) {
        std::cerr << "Warning: The number of genes is inferred from the "
                     "input file. Ignoring parameter -n."
                  << std::endl;
      } else if (!std::strcmp(a, "-m")) {
        std::cerr << "Warning: The number of cells is inferred from the "
                     "input file. Ignoring parameter -m."
                  << std::endl;
      } else if (!std::strcmp(a, "-r")) {
        if (has_next) n_chains = (uint32_t)std::atoi(argv[++i]); else missing(a);
      } else if (!std::strcmp(a, "-l")) {
        if (has_next) chain_length = (uint32_t)std::atoi(argv[++i]); else missing(a);
      } else if (!std::strcmp(a, "-g")) {
        if (has_next) gamma = (float)std::atof(argv[++i]); else missing(a);
      } else if (!std::strcmp(a, "-fd")) {
        if (has_next) alpha_mean = (float)std::atof(argv[++i]); else missing(a);
      } else if (!std::strcmp(a, "-ad")) {
        if (has_next) beta_mean = (float)std::atof(argv[++i]); else missing(a);
        if (i + 1 < argc && argv[i + 1][0] != '-') {
          beta_mean = (float)((double)beta_mean + std::atof(argv[++i]));
          std::cerr << "Warning: homo- and heterocygous mutations are not "
                       "supported by bbSCITE (yet). Summing false negative "
                       "probabilites."
                    << std::endl;
        }
      } else if (!std::strcmp(a, "-cc")) {
        std::cerr << "Warning: homo- and heterocygous mutations are not "
                     "supported by bbSCITE (yet). -cc argument ignored."
                  << std::endl;
      } else if (!std::strcmp(a, "-e")) {
        if (has_next) prob_beta_change = nonneg((float)std::atof(argv[++i]));
        else missing(a);
      } else if (!std::strcmp(a, "-x")) {
        if (has_next) beta_jump_scaling_chi = (float)std::atof(argv[++i]);
        else missing(a);
      } else if (!std::strcmp(a, "-sd")) {
        if (has_next) beta_sd = (float)std::atof(argv[++i]); else missing(a);
      } else if (!std::strcmp(a, "-a")) {
        warn_ignored("-a");
      } else if (!std::strcmp(a, "-p")) {
        warn_ignored("-p");
      } else if (!std::strcmp(a, "-names")) {
        std::cerr << "The -names parameter is not supported by bbSCITE (yet). "
                     "Ignoring the -names parameter."
                  << std::endl;
      } else if (!std::strcmp(a, "-move_probs")) {
        float *dst[3] = {&prob_prune_n_reattach, &prob_swap_nodes,
                         &prob_swap_subtrees};
        for (float *d : dst) {
          if (i + 1 < argc) *d = nonneg((float)std::atof(argv[++i]));
          else missing("-move_probs");
        }
      } else if (!std::strcmp(a, "-seed")) {
        if (has_next) seed = std::strtoull(argv[++i], nullptr, 10); else missing(a);
      } else if (!std::strcmp(a, "-max_treelist_size")) {
        if (has_next) max_n_best_trees = (uint32_t)std::atoi(argv[++i]);
        else missing(a);
      } else if (!std::strcmp(a, "-no_tree_list")) {
        warn_ignored("-no_tree_list");
      } else if (!std::strcmp(a, "-s")) {
        warn_ignored("-s");
      } else if (!std::strcmp(a, "-transpose")) {
        warn_ignored("-transpose");
      } else if (!std::strcmp(a, "-score")) {
        if (!has_next) {
          missing(a);
        } else if (!std::strcmp(argv[++i], "max")) {
          score_mode = BBS_SCORE_MAX;
        } else if (!std::strcmp(argv[i], "sum")) {
          score_mode = BBS_SCORE_SUM;
        } else {
          std::cerr << "Error: Unknown score " << argv[i] << "." << std::endl;
          error = true;
        }
      } else if (!std::strcmp(a, "-error_move")) {
        if (!has_next) {
          missing(a);
        } else if (!std::strcmp(argv[++i], "beta")) {
          error_move = BBS_ERROR_BETA_WALK;
        } else if (!std::strcmp(argv[i], "rw")) {
          error_move = BBS_ERROR_RANDOM_WALK;
        } else if (!std::strcmp(argv[i], "langevin")) {
          error_move = BBS_ERROR_LANGEVIN;
        } else {
          std::cerr << "Error: Unknown error move " << argv[i] << "."
                    << std::endl;
          error = true;
        }
      } else if (!std::strcmp(a, "-error_step")) {
        if (has_next) error_step = (float)std::atof(argv[++i]); else missing(a);
      } else {
        std::cerr << "Error: Unknown parameter " << a << "." << std::endl;
        error = true;
      }
    }
    if (!input_path) {
      std::cerr << "Error: Missing input file path. Did you forget to set "
                   "the -i paramater?"
                << std::endl;
      error = true;
    }
    if (!n_chains) {
      std::cerr << "Error: Missing number of markov chains to simulate. Did "
                   "you forget to set the -r parameter?"
                << std::endl;
      error = true;
    }
    if (!chain_length) {
      std::cerr << "Error: Missing markov chain length. Did you forget to "
                   "set the -l parameter?"
                << std::endl;
      error = true;
    }
    if (prob_beta_change + prob_prune_n_reattach + prob_swap_nodes +
            prob_swap_subtrees ==
        0) {
      std::cerr << "Error: The sum of the move type probabilities is zero."
                << std::endl;
      error = true;
    }
    return !error;
  }

  std::string get_input_path() const { return input_path.value(); }
  void set_input_path(std::string p) { input_path = std::move(p); }
  /* src/Parameters.hpp:306-313: the input path without its last suffix
   * unless -o was given. */
  std::string get_output_path_base() const {
    if (output_path_base) return *output_path_base;
    return input_path->substr(0, input_path->find_last_of('.'));
  }
  void set_output_path_base(std::string p) { output_path_base = std::move(p); }
  uint32_t get_n_chains() const { return n_chains.value(); }
  void set_n_chains(uint32_t v) { n_chains = v; }
  uint32_t get_chain_length() const { return chain_length.value(); }
  void set_chain_length(uint32_t v) { chain_length = v; }
  uint32_t get_max_n_best_trees() const { return max_n_best_trees; }
  void set_max_n_best_trees(uint32_t v) { max_n_best_trees = v; }
  float get_alpha_mean() const { return alpha_mean; }
  void set_alpha_mean(float v) { alpha_mean = v; }
  float get_beta_mean() const { return beta_mean; }
  void set_beta_mean(float v) { beta_mean = v; }
  float get_beta_sd() const { return beta_sd; }
  void set_beta_sd(float v) { beta_sd = v; }
  /* src/Parameters.hpp:451-612: probabilities normalised by their sum */
  float get_prob_beta_change() const { return prob_beta_change / sum_of_move_probs(); }
  float get_prob_prune_n_reattach() const {
    return prob_prune_n_reattach / sum_of_move_probs();
  }
  float get_prob_swap_nodes() const { return prob_swap_nodes / sum_of_move_probs(); }
  float get_prob_swap_subtrees() const {
    return prob_swap_subtrees / sum_of_move_probs();
  }
  float get_beta_jump_sd() const { return beta_sd / beta_jump_scaling_chi; }
  void set_move_probs(float beta_change, float prune, float swap_nodes,
                      float swap_subtrees) {
    prob_beta_change = beta_change;
    prob_prune_n_reattach = prune;
    prob_swap_nodes = swap_nodes;
    prob_swap_subtrees = swap_subtrees;
  }
  float get_beta_jump_scaling_chi() const { return beta_jump_scaling_chi; }
  float get_gamma() const { return gamma; }
  void set_gamma(float v) { gamma = v; }
  uint64_t get_seed() const { return seed; }
  void set_seed(uint64_t v) { seed = v; }

  /* The C-ABI parameter block of these settings (raw move weights: the
   * library normalises them the same way). */
  bbs_params to_bbs_params() const {
    bbs_params p;
    bbs_params_default(&p);
    p.alpha_mean = alpha_mean;
    p.beta_mean = beta_mean;
    p.beta_sd = beta_sd;
    p.prob_beta_change = prob_beta_change;
    p.prob_prune_n_reattach = prob_prune_n_reattach;
    p.prob_swap_nodes = prob_swap_nodes;
    p.prob_swap_subtrees = prob_swap_subtrees;
    p.beta_jump_scaling_chi = beta_jump_scaling_chi;
    p.gamma = gamma;
    p.seed = seed;
    p.treelist_size = std::max<uint32_t>(
        1u, std::min<uint32_t>(max_n_best_trees, BBS_MAX_TREELIST_PER_CHAIN));
    p.score_mode = score_mode;
    p.error_move = error_move;
    if (error_step > 0.0f) p.error_step = error_step;
    return p;
  }

 private:
  float sum_of_move_probs() const {
    return prob_beta_change + prob_prune_n_reattach + prob_swap_nodes +
           prob_swap_subtrees;
  }
  // defaults: src/Parameters.hpp:39-45
  std::optional<std::string> input_path, output_path_base;
  std::optional<uint32_t> n_chains, chain_length;
  uint32_t max_n_best_trees = 128;
  float alpha_mean = 6.04e-5f, beta_mean = 0.4309f, beta_sd = 0.1f;
  float prob_beta_change = 0.0f, prob_prune_n_reattach = 0.55f,
        prob_swap_nodes = 0.4f, prob_swap_subtrees = 0.05f;
  float beta_jump_scaling_chi = 10.0f, gamma = 1.0f;
  uint64_t seed = 0;
  uint32_t score_mode = BBS_SCORE_MAX, error_move = BBS_ERROR_BETA_WALK;
  float error_step = 0.0f;
};

/* ------------------------------------------------------------------ */
namespace detail {
/* A context over one empty cell of n_genes genes: the device handle that
 * the move entry points (realize + update) need, one per thread and size. */
inline bbs_ctx *move_context(uint32_t n_genes) {
  struct Holder {
    std::map<uint32_t, bbs_ctx *> ctx;
    ~Holder() {
      for (auto &kv : ctx) bbs_destroy(kv.second);
    }
  };
  thread_local Holder h;
  auto it = h.ctx.find(n_genes);
  if (it != h.ctx.end()) return it->second;
  std::vector<uint64_t> zero(bbs_words(n_genes + 1), 0);
  bbs_params p;
  bbs_params_default(&p);
  bbs_ctx *c = nullptr;
  check(bbs_create(&c, zero.data(), zero.data(), 1, n_genes, &p));
  h.ctx[n_genes] = c;
  return c;
}
}  // namespace detail

/* ------------------------------------------------------------------ */
/* src/MutationTree.hpp: a tree over caller-owned ancestor matrices.    */
class MutationTree {
 public:
  /* src/MutationTree.hpp:104-107 */
  MutationTree(AncestorMatrix &ancestor, AncestorMatrix &descendant,
               uint32_t n_genes, float beta)
      : ancestor(ancestor), descendant(descendant), n_nodes(n_genes + 1),
        W(bbs_words(n_genes + 1)), beta(beta) {}

  /* Update constructor, src/MutationTree.hpp:123-307: the proposed tree of
   * `old_tree` under `parameters`, computed by the library's move kernel. */
  MutationTree(AncestorMatrix &am, AncestorMatrix &dm,
               MutationTree const &old_tree, ModificationParameters parameters)
      : ancestor(am), descendant(dm), n_nodes(old_tree.n_nodes),
        W(old_tree.W), beta(old_tree.beta) {
    descendant.assign((size_t)n_nodes * W, 0);
    float nb = 0.0f;
    check(bbs_apply_moves(detail::move_context(n_nodes - 1),
                          old_tree.descendant.data(), &old_tree.beta, 1,
                          nullptr, &parameters, nullptr, descendant.data(),
                          &nb));
    beta = nb;
    ancestor.assign((size_t)n_nodes * W, 0);
    check(bbs_dm_to_am(descendant.data(), n_nodes, ancestor.data()));
  }

  MutationTree(MutationTree const &other) = default;

  /* src/MutationTree.hpp:323-363 */
  ModificationParameters realize_raw_move_sample(RawMoveSample raw) const {
    ModificationParameters out{};
    std::vector<uint64_t> scratch((size_t)n_nodes * W);
    float nb = 0.0f;
    check(bbs_apply_moves(detail::move_context(n_nodes - 1), descendant.data(),
                          &beta, 1, &raw, nullptr, &out, scratch.data(), &nb));
    return out;
  }

  /* src/MutationTree.hpp:379-425 */
  static std::tuple<AncestorMatrix, AncestorMatrix>
  parent_vector_to_matrix(std::vector<uint32_t> const &parent) {
    const uint32_t n = (uint32_t)parent.size();
    AncestorMatrix am((size_t)n * bbs_words(n)), dm(am.size());
    check(bbs_parent_vector_to_matrix(parent.data(), n, am.data(), dm.data()));
    return {am, dm};
  }

  /* src/MutationTree.hpp:427-476 */
  static std::vector<uint32_t>
  pruefer_code_to_parent_vector(std::vector<uint32_t> const &code) {
    std::vector<uint32_t> parent(code.size() + 2);
    check(bbs_pruefer_to_parent_vector(code.data(), (uint32_t)code.size(),
                                       parent.data()));
    return parent;
  }

  uint32_t get_n_nodes() const { return n_nodes; }
  uint32_t get_root() const { return n_nodes - 1; }
  float get_beta() const { return beta; }

  /* src/MutationTree.hpp:549-596: the parent of x is the y != x whose
   * ancestor set is that of x without x; the root is its own parent. */
  uint32_t get_parent(uint32_t x) const {
    if (x == get_root()) return x;
    uint32_t best = get_root(), best_n = 0;
    for (uint32_t y = 0; y < n_nodes; y++) {
      if (y == x || !bit(descendant, x, y)) continue;
      const uint32_t k = get_n_ancestors(y);
      if (k > best_n) {
        best_n = k;
        best = y;
      }
    }
    return best;
  }
  bool is_parent(uint32_t parent, uint32_t child) const {
    return get_parent(child) == parent;
  }
  /* src/MutationTree.hpp:609-640 */
  bool is_ancestor(uint32_t a, uint32_t b) const { return bit(ancestor, a, b); }
  bool is_descendant(uint32_t a, uint32_t b) const { return bit(ancestor, b, a); }
  /* src/MutationTree.hpp:661-674, 733-746 */
  uint32_t get_n_descendants(uint32_t x) const { return popc_row(ancestor, x); }
  uint32_t get_n_ancestors(uint32_t x) const { return popc_row(descendant, x); }
  /* src/MutationTree.hpp:686-716, 840-878: the k-th (non-)descendant,
   * 0 when k is out of range. */
  uint32_t get_descendant(uint32_t x, uint32_t k) const { return kth(x, k, true); }
  uint32_t get_nondescendant(uint32_t x, uint32_t k) const { return kth(x, k, false); }

  /* src/MutationTree.hpp:760-792 */
  bool operator==(MutationTree const &o) const {
    if (n_nodes != o.n_nodes || beta != o.beta) return false;
    for (uint32_t x = 0; x < n_nodes; x++)
      for (uint32_t y = 0; y < n_nodes; y++)
        if (bit(ancestor, x, y) != bit(o.ancestor, x, y)) return false;
    return true;
  }
  bool operator!=(MutationTree const &o) const { return !(*this == o); }

  std::vector<uint32_t> parent_vector() const {
    std::vector<uint32_t> p(n_nodes);
    check(bbs_matrix_to_parent_vector(descendant.data(), n_nodes, p.data()));
    return p;
  }
  /* src/MutationTree.hpp:799-837 (byte-identical output) */
  std::string to_graphviz() const { return render(bbs_tree_to_graphviz); }
  std::string to_newick() const { return render(bbs_tree_to_newick); }

  AncestorMatrix const &get_ancestor_matrix() const { return ancestor; }
  AncestorMatrix const &get_descendant_matrix() const { return descendant; }

 private:
  bool bit(AncestorMatrix const &m, uint32_t row, uint32_t col) const {
    return (m[(size_t)row * W + col / 64] >> (col % 64)) & 1;
  }
  uint32_t popc_row(AncestorMatrix const &m, uint32_t row) const {
    uint32_t k = 0;
    for (uint32_t y = 0; y < n_nodes; y++) k += bit(m, row, y);
    return k;
  }
  uint32_t kth(uint32_t x, uint32_t k, bool desc) const {
    for (uint32_t y = 0; y < n_nodes; y++)
      if (bit(ancestor, x, y) == desc && k-- == 0) return y;
    return 0;
  }
  template <class F>
  std::string render(F f) const {
    const std::vector<uint32_t> p = parent_vector();
    size_t len = 0;
    check(f(p.data(), n_nodes, nullptr, 0, &len));
    std::string s(len + 1, '\0');
    check(f(p.data(), n_nodes, s.data(), s.size(), &len));
    s.resize(len);
    return s;
  }

  AncestorMatrix &ancestor, &descendant;
  uint32_t n_nodes, W;
  float beta;
};

/* ------------------------------------------------------------------ */
/* src/TreeScorer.hpp: scores trees of one dataset on the device.       */
class TreeScorer {
 public:
  /* src/TreeScorer.hpp:92-117; is_mutated / is_known hold n_cells rows of
   * bbs_words(n_genes + 1) words (bit g = gene g). */
  TreeScorer(float alpha_mean, float beta_mean, float beta_sd,
             uint32_t n_cells, uint32_t n_genes,
             std::vector<uint64_t> const &is_mutated,
             std::vector<uint64_t> const &is_known)
      : n_genes(n_genes) {
    bbs_params p;
    bbs_params_default(&p);
    p.alpha_mean = alpha_mean;
    p.beta_mean = beta_mean;
    p.beta_sd = beta_sd;
    bbs_ctx *c = nullptr;
    check(bbs_create(&c, is_mutated.data(), is_known.data(), n_cells, n_genes,
                     &p));
    ctx.reset(c);
  }

  /* src/TreeScorer.hpp:122-126 */
  float logscore_beta(float beta) const {
    float r = 0.0f;
    check(bbs_logscore_beta(ctx.get(), beta, &r));
    return r;
  }

  /* src/TreeScorer.hpp:131-210: max over attachments, plus the prior. */
  float logscore_tree(MutationTree const &tree) {
    float beta = tree.get_beta(), s = 0.0f;
    check(bbs_score_trees(ctx.get(), tree.get_descendant_matrix().data(), &beta,
                          1, &s, nullptr, nullptr));
    return s;
  }

  /* Many trees in one launch; dm holds n_trees stacked descendant
   * matrices. */
  std::vector<float> logscore_trees(std::vector<uint64_t> const &dm,
                                    std::vector<float> const &betas) {
    std::vector<float> s(betas.size());
    check(bbs_score_trees(ctx.get(), dm.data(), betas.data(),
                          (uint32_t)betas.size(), s.data(), nullptr, nullptr));
    return s;
  }

 private:
  struct Free {
    void operator()(bbs_ctx *c) const { bbs_destroy(c); }
  };
  std::unique_ptr<bbs_ctx, Free> ctx;
  uint32_t n_genes;
};

/* ------------------------------------------------------------------ */
/* src/Application.hpp: the chains of one dataset.                      */
class Application {
 public:
  /* src/Application.hpp:88-186.  Initial trees: uniform random Pruefer
   * codes from the -seed stream (src/Application.hpp:149-164). */
  Application(std::vector<uint64_t> const &is_mutated,
              std::vector<uint64_t> const &is_known,
              Parameters const &parameters, uint32_t n_cells, uint32_t n_genes)
      : parameters(parameters), n_genes(n_genes) {
    const auto t0 = std::chrono::steady_clock::now();
    const bbs_params p = parameters.to_bbs_params();
    bbs_ctx *c = nullptr;
    check(bbs_create(&c, is_mutated.data(), is_known.data(), n_cells, n_genes,
                     &p));
    ctx.reset(c);
    check(bbs_init_chains(c, parameters.get_n_chains(), nullptr));
    setup_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0)
                  .count();
  }

  /* Host time of creating the context and the initial chains (the moves
   * themselves are drawn inside the chain kernel). */
  double get_setup_seconds() const { return setup_s; }

  /* src/Application.hpp:197-219: runs every chain for -l steps; returns
   * the device makespan in ms. */
  float run_simulation() {
    check(bbs_run(ctx.get(), parameters.get_chain_length(), nullptr, nullptr));
    float ms = 0.0f;
    check(bbs_last_run_ms(ctx.get(), &ms));
    fetched = false;
    return ms;
  }

  /* src/Application.hpp:224-256 */
  AncestorMatrix get_best_am() { return fetch(), best_am; }
  AncestorMatrix get_best_dm() { return fetch(), best_dm; }
  float get_best_beta() { return fetch(), best_beta; }
  float get_best_score() { return fetch(), best_score; }
  float get_best_alpha() {
    float a = 0.0f;
    check(bbs_get_best_alpha(ctx.get(), &a));
    return a;
  }
  /* The co-optimal tree list (SCITE's -max_treelist_size): up to
   * max_trees distinct trees tied with the best, the best first, as
   * descendant matrices with their betas. */
  std::vector<std::pair<AncestorMatrix, float>> get_treelist(uint32_t max_trees) {
    const uint32_t n = n_genes + 1, W = bbs_words(n);
    std::vector<uint64_t> dm((size_t)max_trees * n * W);
    std::vector<float> betas(max_trees);
    float score = 0.0f;
    uint32_t k = 0;
    check(bbs_get_treelist(ctx.get(), max_trees, dm.data(), betas.data(),
                           &score, &k));
    std::vector<std::pair<AncestorMatrix, float>> out;
    for (uint32_t i = 0; i < k; i++)
      out.emplace_back(AncestorMatrix(dm.begin() + (size_t)i * n * W,
                                      dm.begin() + (size_t)(i + 1) * n * W),
                       betas[i]);
    return out;
  }
  /* Chain checkpoints (bbs_save_chains / bbs_load_chains): the image of
   * every chain's state, and its restoration into an Application made with
   * the same data and parameters, after which run_simulation continues the
   * chains exactly. */
  std::vector<uint8_t> save_chains() {
    size_t size = 0;
    check(bbs_save_chains(ctx.get(), nullptr, &size));
    std::vector<uint8_t> image(size);
    check(bbs_save_chains(ctx.get(), image.data(), &size));
    return image;
  }
  void load_chains(std::vector<uint8_t> const &image) {
    check(bbs_load_chains(ctx.get(), image.data(), image.size()));
    fetched = false;
  }
  bbs_ctx *handle() { return ctx.get(); }

 private:
  void fetch() {
    if (fetched) return;
    const uint32_t n = n_genes + 1, W = bbs_words(n);
    best_am.assign((size_t)n * W, 0);
    best_dm.assign((size_t)n * W, 0);
    check(bbs_get_best(ctx.get(), best_am.data(), best_dm.data(), nullptr,
                       &best_beta, &best_score, nullptr, nullptr));
    fetched = true;
  }
  struct Free {
    void operator()(bbs_ctx *c) const { bbs_destroy(c); }
  };
  std::unique_ptr<bbs_ctx, Free> ctx;
  Parameters parameters;
  uint32_t n_genes;
  double setup_s = 0.0;
  bool fetched = false;
  AncestorMatrix best_am, best_dm;
  float best_beta = 0.0f, best_score = 0.0f;
};

}  // namespace bbSCITE

#endif
