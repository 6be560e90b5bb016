// ref_proxy.cpp -- extern "C" entry points over the reference's OWN CPU
// scoring benchmark class (cpu_scoring_benchmark/CPUTreeScorer.hpp),
// compiled unmodified from the reference tree against the host shim in
// oracle/shim/ (2-D accessor, vec<T, N>).
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile into
// oracle/_ref/libbbs_ref.so when the reference sources are present; used
// by tests/test_oracle.py to pin orc_cpu_scoring_proxy in
// oracle/bbs_oracle.c, the restatement that the CPU baseline runs.
#include <CPUTreeScorer.hpp>

#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

using Scorer = bbSCITE::CPUTreeScorer;

// One tree at the class's fixed 128 cells x 127 genes: mutq / knownq are
// [quadword][cell] words, dm is [quadword][node] words (2 x 128 each).
float score_one(const Scorer &s, const uint64_t *dm) {
  Scorer::AncestorMatrix am;
  for (uint32_t q = 0; q < Scorer::n_quadwords; q++)
    std::memcpy(am[q].data(), dm + q * Scorer::n_nodes,
                sizeof(uint64_t) * Scorer::n_nodes);
  return s.logscore_tree(am);
}

Scorer make_scorer(float alpha, float beta, const uint64_t *mutq,
                   const uint64_t *knownq) {
  Scorer::MutationDataAccessor m{mutq, Scorer::n_cells};
  Scorer::MutationDataAccessor k{knownq, Scorer::n_cells};
  // the beta prior sd is unused by this class
  return Scorer(alpha, beta, 0.1f, m, k);
}

}  // namespace

extern "C" {

// Scores of n_trees trees (dmq: n_trees x 2 x 128 words) into out.
void ref_proxy_scores(float alpha, float beta, const uint64_t *mutq,
                      const uint64_t *knownq, const uint64_t *dmq,
                      uint32_t n_trees, float *out) {
  const Scorer s = make_scorer(alpha, beta, mutq, knownq);
  for (uint32_t t = 0; t < n_trees; t++) out[t] = score_one(s, dmq + t * 256);
}

// The benchmark loop: every tree scored `reps` times, trees spread over
// n_threads host threads; returns the sum of all scores.
double ref_cpu_scoring_proxy(float alpha, float beta, const uint64_t *mutq,
                             const uint64_t *knownq, const uint64_t *dmq,
                             uint32_t n_trees, uint32_t reps,
                             uint32_t n_threads) {
  if (n_threads < 1) n_threads = 1;
  const Scorer s = make_scorer(alpha, beta, mutq, knownq);
  std::vector<double> sums(n_threads, 0.0);
  std::vector<std::thread> th;
  for (uint32_t i = 0; i < n_threads; i++)
    th.emplace_back([&, i] {
      double acc = 0.0;
      for (uint32_t t = i; t < n_trees; t += n_threads)
        for (uint32_t r = 0; r < reps; r++) acc += score_one(s, dmq + t * 256);
      sums[i] = acc;
    });
  double total = 0.0;
  for (uint32_t i = 0; i < n_threads; i++) {
    th[i].join();
    total += sums[i];
  }
  return total;
}

}  // extern "C"
