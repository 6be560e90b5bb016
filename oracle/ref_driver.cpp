// ref_driver.cpp -- extern "C" entry points over the reference's OWN
// classes (src/MutationTree.hpp, src/TreeScorer.hpp,
// src/RawMoveDistribution.hpp, src/Parameters.hpp), compiled unmodified
// from the reference tree against the host shim in oracle/shim/.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile into
// oracle/_ref/libbbs_ref.so when the reference sources are present; used
// by tests/golden/make_golden.py and tests/test_oracle.py to pin the C
// restatement in oracle/bbs_oracle.c.  The chain loop below restates
// src/Application.hpp:408-487 (the only part of Application.hpp that needs
// the FPGA runtime) around the reference's classes.
#include <MutationTree.hpp>
#include <Parameters.hpp>
#include <RawMoveDistribution.hpp>
#include <TreeScorer.hpp>

#include <cmath>
#include <random>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

using namespace bbSCITE;

namespace {

template <uint32_t G> using Tree = MutationTree<G>;

template <uint32_t G>
void to_words(typename Tree<G>::AncestorMatrix const &m, uint32_t n_nodes,
              uint64_t *out) {
  uint32_t W = (n_nodes + 63) / 64;
  for (uint32_t x = 0; x < n_nodes; x++)
    for (uint32_t k = 0; k < W; k++) {
      uint64_t v = 0;
      for (uint32_t b = 0; b < 64; b++) {
        uint32_t y = k * 64 + b;
        if (y < Tree<G>::max_n_nodes && m[x][y])
          v |= 1ull << b;
      }
      out[x * W + k] = v;
    }
}

template <uint32_t G>
void from_words(const uint64_t *in, uint32_t n_nodes,
                typename Tree<G>::AncestorMatrix &m) {
  uint32_t W = (n_nodes + 63) / 64;
  for (uint32_t x = 0; x < Tree<G>::max_n_nodes; x++) {
    m[x] = 0;
    if (x >= n_nodes)
      continue;
    for (uint32_t y = 0; y < n_nodes; y++)
      m[x][y] = (in[x * W + y / 64] >> (y % 64)) & 1u;
  }
}

struct RawC {
  int32_t move_type;
  uint32_t raw_v, raw_w;
  float d, nd, jump, acc;
  uint32_t pad;
};
struct ParamsC {
  int32_t move_type;
  uint32_t v, w, pv, pw, dv, ndv;
  float new_beta;
};

RawMoveSample to_raw(const RawC &r) {
  return RawMoveSample{.move_type = (MoveType)r.move_type,
                       .raw_v = r.raw_v,
                       .raw_w = r.raw_w,
                       .raw_descendant_of_v = r.d,
                       .raw_nondescendant_of_v = r.nd,
                       .beta_jump = r.jump,
                       .acceptance_level = r.acc};
}

template <uint32_t G> int realize(const uint64_t *am, const uint64_t *dm,
                                  uint32_t n_nodes, float beta,
                                  const RawC *raw, ParamsC *out) {
  typename Tree<G>::AncestorMatrix a, d;
  from_words<G>(am, n_nodes, a);
  from_words<G>(dm, n_nodes, d);
  Tree<G> t(a, d, n_nodes - 1, beta);
  auto p = t.realize_raw_move_sample(to_raw(*raw));
  *out = ParamsC{(int32_t)p.move_type, p.v, p.w, p.parent_of_v,
                 p.parent_of_w, p.descendant_of_v, p.nondescendant_of_v,
                 p.new_beta};
  return 0;
}

template <uint32_t G> float apply(const uint64_t *am, const uint64_t *dm,
                                  uint32_t n_nodes, float beta,
                                  const ParamsC *p, uint64_t *nam,
                                  uint64_t *ndm) {
  typename Tree<G>::AncestorMatrix a, d, pa, pd;
  from_words<G>(am, n_nodes, a);
  from_words<G>(dm, n_nodes, d);
  Tree<G> t(a, d, n_nodes - 1, beta);
  typename Tree<G>::ModificationParameters mp{
      .move_type = (MoveType)p->move_type,
      .v = p->v,
      .w = p->w,
      .parent_of_v = p->pv,
      .parent_of_w = p->pw,
      .descendant_of_v = p->dv,
      .nondescendant_of_v = p->ndv,
      .new_beta = p->new_beta};
  for (auto &r : pa) r = 0;
  for (auto &r : pd) r = 0;
  Tree<G> nt(pa, pd, t, mp);
  to_words<G>(pa, n_nodes, nam);
  to_words<G>(pd, n_nodes, ndm);
  return nt.get_beta();
}

template <uint32_t C, uint32_t G> struct Scoring {
  using Sc = TreeScorer<C, G>;
  using MDM = typename Sc::MutationDataMatrix;
  MDM mut_in{}, known_in{}, mut_loc{}, known_loc{};
  Sc *sc = nullptr;
  Scoring(float alpha, float beta_mean, float beta_sd, uint32_t n_cells,
          uint32_t n_genes, const uint64_t *mut, const uint64_t *known) {
    uint32_t W = (n_genes + 1 + 63) / 64;
    for (uint32_t c = 0; c < C; c++) {
      mut_in[c] = 0;
      known_in[c] = 0;
      if (c >= n_cells)
        continue;
      for (uint32_t g = 0; g < n_genes + 1; g++) {
        mut_in[c][g] = (mut[c * W + g / 64] >> (g % 64)) & 1u;
        known_in[c][g] = (known[c * W + g / 64] >> (g % 64)) & 1u;
      }
    }
    typename Sc::MutationDataAccessor ma{mut_in.data()}, ka{known_in.data()};
    sc = new Sc(alpha, beta_mean, beta_sd, n_cells, n_genes, ma, ka, mut_loc,
                known_loc);
  }
  ~Scoring() { delete sc; }
};

template <uint32_t C, uint32_t G>
float score(float alpha, float beta_mean, float beta_sd, uint32_t n_cells,
            uint32_t n_genes, const uint64_t *mut, const uint64_t *known,
            const uint64_t *dm, float beta) {
  Scoring<C, G> s(alpha, beta_mean, beta_sd, n_cells, n_genes, mut, known);
  typename Tree<G>::AncestorMatrix a, d;
  from_words<G>(dm, n_genes + 1, d);
  for (auto &r : a) r = 0;
  Tree<G> t(a, d, n_genes, beta);
  return s.sc->logscore_tree(t);
}

// src/Application.hpp:408-487 around the reference's classes, one chain,
// recorded moves; forced decisions inside the ambiguity band.
template <uint32_t C, uint32_t G>
void run_chain(float alpha, float beta_mean, float beta_sd, float gamma,
               uint32_t n_cells, uint32_t n_genes, const uint64_t *mut,
               const uint64_t *known, const RawC *moves, uint32_t n_steps,
               uint64_t *am_io, uint64_t *dm_io, float *beta_io,
               float *score_io, float *best_score, uint64_t *best_dm,
               float *prop_scores, uint8_t *accepted,
               const uint8_t *forced, float ambiguity, uint32_t *n_ambig) {
  Scoring<C, G> s(alpha, beta_mean, beta_sd, n_cells, n_genes, mut, known);
  uint32_t n_nodes = n_genes + 1;
  typename Tree<G>::AncestorMatrix cam, cdm, pam, pdm, bam, bdm;
  from_words<G>(am_io, n_nodes, cam);
  from_words<G>(dm_io, n_nodes, cdm);
  for (auto &r : bam) r = 0;
  for (auto &r : bdm) r = 0;
  float cur_beta = *beta_io, cur_score = *score_io;
  float bscore = -std::numeric_limits<float>::infinity();
  uint32_t ambig = 0;
  for (uint32_t i = 0; i < n_steps; i++) {
    Tree<G> cur(cam, cdm, n_genes, cur_beta);
    RawMoveSample raw = to_raw(moves[i]);
    auto mp = cur.realize_raw_move_sample(raw);
    for (auto &r : pam) r = 0;
    for (auto &r : pdm) r = 0;
    Tree<G> prop(pam, pdm, cur, mp);
    float pbeta = prop.get_beta();
    float pscore = s.sc->logscore_tree(prop);
    float corr;
    if (raw.move_type == MoveType::SwapSubtrees && cur.is_ancestor(mp.w, mp.v))
      corr = float(cur.get_n_descendants(mp.v)) /
             float(cur.get_n_descendants(mp.w));
    else
      corr = 1.0;
    float ratio = corr * std::exp((pscore - cur_score) * gamma);
    bool accept = ratio > raw.acceptance_level;
    if (forced) {
      float u = raw.acceptance_level, dd = std::fabs(ratio - u);
      if (dd <= ambiguity * std::fabs(u) || dd <= ambiguity * std::fabs(ratio)) {
        if (accept != bool(forced[i]))
          ambig++;
        accept = forced[i];
      }
    }
    bool new_max = i == 0 || pscore > bscore;
    if (new_max) {
      bscore = pscore;
      bam = pam;
      bdm = pdm;
    }
    if (prop_scores)
      prop_scores[i] = pscore;
    if (accepted)
      accepted[i] = accept;
    if (accept) {
      cam = pam;
      cdm = pdm;
      cur_beta = pbeta;
      cur_score = pscore;
    }
  }
  to_words<G>(cam, n_nodes, am_io);
  to_words<G>(cdm, n_nodes, dm_io);
  *beta_io = cur_beta;
  *score_io = cur_score;
  *best_score = bscore;
  if (best_dm)
    to_words<G>(bdm, n_nodes, best_dm);
  if (n_ambig)
    *n_ambig = ambig;
}

template <class F> auto by_genes(uint32_t n_genes, F &&f) {
  if (n_genes <= 31) return f(std::integral_constant<uint32_t, 31>{});
  if (n_genes <= 63) return f(std::integral_constant<uint32_t, 63>{});
  if (n_genes <= 95) return f(std::integral_constant<uint32_t, 95>{});
  if (n_genes <= 127) return f(std::integral_constant<uint32_t, 127>{});
  return f(std::integral_constant<uint32_t, 255>{});
}
template <class F> auto by_cells(uint32_t n_cells, F &&f) {
  if (n_cells <= 32) return f(std::integral_constant<uint32_t, 32>{});
  if (n_cells <= 64) return f(std::integral_constant<uint32_t, 64>{});
  if (n_cells <= 96) return f(std::integral_constant<uint32_t, 96>{});
  if (n_cells <= 128) return f(std::integral_constant<uint32_t, 128>{});
  if (n_cells <= 256) return f(std::integral_constant<uint32_t, 256>{});
  return f(std::integral_constant<uint32_t, 512>{});
}

} // namespace

extern "C" {

int ref_max_genes() { return 255; }
int ref_max_cells() { return 512; }

void ref_pruefer_to_parent(const uint32_t *code, uint32_t len,
                           uint32_t *parent) {
  std::vector<uint32_t> c(code, code + len);
  auto pv = by_genes(len + 1, [&](auto g) {
    return Tree<decltype(g)::value>::pruefer_code_to_parent_vector(c);
  });
  std::memcpy(parent, pv.data(), sizeof(uint32_t) * pv.size());
}

void ref_parent_to_matrix(const uint32_t *parent, uint32_t n_nodes,
                          uint64_t *am, uint64_t *dm) {
  std::vector<uint32_t> pv(parent, parent + n_nodes);
  by_genes(n_nodes - 1, [&](auto g) {
    constexpr uint32_t G = decltype(g)::value;
    auto t = Tree<G>::parent_vector_to_matrix(pv);
    to_words<G>(std::get<0>(t), n_nodes, am);
    to_words<G>(std::get<1>(t), n_nodes, dm);
    return 0;
  });
}

uint32_t ref_get_parent(const uint64_t *am, const uint64_t *dm,
                        uint32_t n_nodes, uint32_t x) {
  return by_genes(n_nodes - 1, [&](auto g) {
    constexpr uint32_t G = decltype(g)::value;
    typename Tree<G>::AncestorMatrix a, d;
    from_words<G>(am, n_nodes, a);
    from_words<G>(dm, n_nodes, d);
    Tree<G> t(a, d, n_nodes - 1, 0.5f);
    return t.get_parent(x);
  });
}

int ref_realize(const uint64_t *am, const uint64_t *dm, uint32_t n_nodes,
                float beta, const void *raw, void *out) {
  return by_genes(n_nodes - 1, [&](auto g) {
    return realize<decltype(g)::value>(am, dm, n_nodes, beta,
                                       (const RawC *)raw, (ParamsC *)out);
  });
}

float ref_apply(const uint64_t *am, const uint64_t *dm, uint32_t n_nodes,
                float beta, const void *params, uint64_t *nam,
                uint64_t *ndm) {
  return by_genes(n_nodes - 1, [&](auto g) {
    return apply<decltype(g)::value>(am, dm, n_nodes, beta,
                                     (const ParamsC *)params, nam, ndm);
  });
}

float ref_score(float alpha, float beta_mean, float beta_sd, uint32_t n_cells,
                uint32_t n_genes, const uint64_t *mut, const uint64_t *known,
                const uint64_t *dm, float beta) {
  return by_cells(n_cells, [&](auto c) {
    return by_genes(n_genes, [&](auto g) {
      return score<decltype(c)::value, decltype(g)::value>(
          alpha, beta_mean, beta_sd, n_cells, n_genes, mut, known, dm, beta);
    });
  });
}

float ref_logscore_beta(float alpha, float beta_mean, float beta_sd,
                        float beta) {
  Scoring<32, 31> s(alpha, beta_mean, beta_sd, 0, 1, nullptr, nullptr);
  return s.sc->logscore_beta(beta);
}

void ref_run_chain(float alpha, float beta_mean, float beta_sd, float gamma,
                   uint32_t n_cells, uint32_t n_genes, const uint64_t *mut,
                   const uint64_t *known, const void *moves, uint32_t n_steps,
                   uint64_t *am_io, uint64_t *dm_io, float *beta_io,
                   float *score_io, float *best_score, uint64_t *best_dm,
                   float *prop_scores, uint8_t *accepted,
                   const uint8_t *forced, float ambiguity,
                   uint32_t *n_ambig) {
  by_cells(n_cells, [&](auto c) {
    return by_genes(n_genes, [&](auto g) {
      run_chain<decltype(c)::value, decltype(g)::value>(
          alpha, beta_mean, beta_sd, gamma, n_cells, n_genes, mut, known,
          (const RawC *)moves, n_steps, am_io, dm_io, beta_io, score_io,
          best_score, best_dm, prop_scores, accepted, forced, ambiguity,
          n_ambig);
      return 0;
    });
  });
}

// Tree text formats (src/MutationTree.hpp:799-837); returns the length.
int ref_to_graphviz(const uint64_t *am, const uint64_t *dm, uint32_t n_nodes,
                    char *buf, int cap) {
  std::string s = by_genes(n_nodes - 1, [&](auto g) {
    constexpr uint32_t G = decltype(g)::value;
    typename Tree<G>::AncestorMatrix a, d;
    from_words<G>(am, n_nodes, a);
    from_words<G>(dm, n_nodes, d);
    Tree<G> t(a, d, n_nodes - 1, 0.5f);
    return t.to_graphviz();
  });
  std::strncpy(buf, s.c_str(), cap);
  return (int)s.size();
}

int ref_to_newick(const uint64_t *am, const uint64_t *dm, uint32_t n_nodes,
                  char *buf, int cap) {
  std::string s = by_genes(n_nodes - 1, [&](auto g) {
    constexpr uint32_t G = decltype(g)::value;
    typename Tree<G>::AncestorMatrix a, d;
    from_words<G>(am, n_nodes, a);
    from_words<G>(dm, n_nodes, d);
    Tree<G> t(a, d, n_nodes - 1, 0.5f);
    return t.to_newick();
  });
  std::strncpy(buf, s.c_str(), cap);
  return (int)s.size();
}

// src/Parameters.hpp:61-281 on an argv; returns 1 if valid and fills
// out[] = {alpha, beta, beta_sd, p_beta, p_prune, p_swap, p_subtrees,
//          chi, gamma, n_chains, chain_length, max_treelist}.
// One chain's initial tree and move stream from the reference's own
// samplers and URNG: MutationTree::sample_random_pruefer_code
// (src/MutationTree.hpp:492-510) decoded by pruefer_code_to_parent_vector,
// RawMoveDistribution::operator() (src/RawMoveDistribution.hpp:97-155)
// with the probabilities normalised by Parameters (src/Parameters.hpp:
// 451-612), all drawn from std::minstd_rand (src/main.cpp:34) seeded with
// `seed`.  The reference seeds one generator for all chains from
// random_device; here each chain gets its own seed so runs repeat.
void ref_sample_chain(uint32_t n_genes, float prob_beta_change,
                      float prob_prune, float prob_swap, float prob_subtrees,
                      float beta_sd, float chi, uint32_t seed,
                      uint32_t n_steps, uint32_t *parent_out,
                      void *moves_out) {
  std::minstd_rand rng(seed);
  const std::vector<uint32_t> code =
      Tree<255>::sample_random_pruefer_code(rng, n_genes);
  const std::vector<uint32_t> parent =
      Tree<255>::pruefer_code_to_parent_vector(code);
  std::memcpy(parent_out, parent.data(), sizeof(uint32_t) * parent.size());
  Parameters p;
  p.set_prob_beta_change(prob_beta_change);
  p.set_prob_prune_n_reattach(prob_prune);
  p.set_prob_swap_nodes(prob_swap);
  p.set_prob_swap_subtrees(prob_subtrees);
  p.set_beta_sd(beta_sd);
  p.set_beta_jump_scaling_chi(chi);
  RawMoveDistribution dist(n_genes + 1, p);
  RawC *out = (RawC *)moves_out;
  for (uint32_t i = 0; i < n_steps; i++) {
    const RawMoveSample r = dist(rng);
    out[i] = RawC{(int32_t)r.move_type, r.raw_v, r.raw_w,
                  r.raw_descendant_of_v, r.raw_nondescendant_of_v,
                  r.beta_jump, r.acceptance_level, 0u};
  }
}

int ref_parse_args(int argc, char **argv, float *out) {
  Parameters p;
  bool ok = p.load_and_verify_args(argc, argv);
  out[0] = p.get_alpha_mean();
  out[1] = p.get_beta_mean();
  out[2] = p.get_beta_sd();
  if (ok) {
    out[3] = p.get_prob_beta_change();
    out[4] = p.get_prob_prune_n_reattach();
    out[5] = p.get_prob_swap_nodes();
    out[6] = p.get_prob_swap_subtrees();
    out[9] = (float)p.get_n_chains();
    out[10] = (float)p.get_chain_length();
  }
  out[7] = p.get_beta_jump_scaling_chi();
  out[8] = p.get_gamma();
  out[11] = (float)p.get_max_n_best_trees();
  return ok ? 1 : 0;
}

} // extern "C"
