// wrapper_probe.cpp -- line-driven harness over the C++ wrappers of
// include/bbscite_gb300.hpp, for the Python tests.  One command per input
// line; one result per output line.
//   params <argv...>            Parameters::load_and_verify_args
//   pruefer <code...>           MutationTree::pruefer_code_to_parent_vector
//   tree <beta> <parent...>     sets the current tree, prints its queries
//   update <type> <v> <w> <pv> <pw> <dv> <ndv> <new_beta>   (device)
//   realize <type> <v> <w> <u_desc> <u_nondesc> <jump>      (device)
//   scorer <alpha> <beta> <sd> <n_cells> <n_genes> <mut words...> <known words...>
//   score                       logscore_tree of the current tree (device)
//   prior <beta>                logscore_beta (context on the device)
//   resume <n_cells> <n_genes> <steps1> <steps2> <mut words...> <known words...> <argv...>
//                               Application run for steps1 + steps2 vs run
//                               for steps1, saved, restored and run for steps2
#include <iomanip>
#include <iostream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "bbscite_gb300.hpp"

using namespace bbSCITE;

namespace {

std::string escape(const std::string &s) {
  std::string o;
  for (char c : s) o += c == '\n' ? std::string("\\n") : std::string(1, c);
  return o;
}

struct State {
  AncestorMatrix am, dm;
  std::unique_ptr<MutationTree> tree;
  std::unique_ptr<TreeScorer> scorer;
  uint32_t n_genes = 0;
};

void print_tree(MutationTree const &t) {
  const uint32_t n = t.get_n_nodes();
  std::cout << "parent";
  for (uint32_t x = 0; x < n; x++) std::cout << ' ' << t.get_parent(x);
  std::cout << " | n_desc";
  for (uint32_t x = 0; x < n; x++) std::cout << ' ' << t.get_n_descendants(x);
  std::cout << " | n_anc";
  for (uint32_t x = 0; x < n; x++) std::cout << ' ' << t.get_n_ancestors(x);
  std::cout << " | anc";
  for (uint32_t x = 0; x < n; x++) {
    std::cout << ' ';
    for (uint32_t y = 0; y < n; y++) std::cout << (t.is_ancestor(x, y) ? '1' : '0');
  }
  std::cout << " | desc";
  for (uint32_t x = 0; x < n; x++) {
    std::cout << ' ';
    for (uint32_t y = 0; y < n; y++) std::cout << (t.is_descendant(x, y) ? '1' : '0');
  }
  std::cout << " | is_parent";
  for (uint32_t x = 0; x < n; x++) {
    std::cout << ' ';
    for (uint32_t y = 0; y < n; y++) std::cout << (t.is_parent(x, y) ? '1' : '0');
  }
  std::cout << " | kth_desc";
  for (uint32_t x = 0; x < n; x++)
    for (uint32_t k = 0; k <= t.get_n_descendants(x); k++)
      std::cout << ' ' << t.get_descendant(x, k);
  std::cout << " | kth_nondesc";
  for (uint32_t x = 0; x < n; x++)
    for (uint32_t k = 0; k <= n - t.get_n_descendants(x); k++)
      std::cout << ' ' << t.get_nondescendant(x, k);
  std::cout << " | gv " << escape(t.to_graphviz()) << " | newick "
            << escape(t.to_newick()) << " | beta " << t.get_beta() << "\n";
}

void run(const std::string &line, State &st) {
  std::istringstream in(line);
  std::string cmd;
  in >> cmd;
  if (cmd == "params") {
    std::vector<std::string> tok{"bbscite"};
    std::string t;
    while (in >> t) tok.push_back(t);
    std::vector<char *> argv;
    for (auto &s : tok) argv.push_back(s.data());
    Parameters p;
    const bool ok = p.load_and_verify_args((int)argv.size(), argv.data());
    std::cout << std::setprecision(9) << "ok " << ok << " alpha "
              << p.get_alpha_mean() << " beta " << p.get_beta_mean() << " sd "
              << p.get_beta_sd() << " e " << p.get_prob_beta_change()
              << " prune " << p.get_prob_prune_n_reattach() << " swap "
              << p.get_prob_swap_nodes() << " subtrees "
              << p.get_prob_swap_subtrees() << " chi "
              << p.get_beta_jump_scaling_chi() << " gamma " << p.get_gamma()
              << " max_trees " << p.get_max_n_best_trees() << " seed "
              << p.get_seed();
    if (ok)
      std::cout << " chains " << p.get_n_chains() << " length "
                << p.get_chain_length() << " out " << p.get_output_path_base();
    std::cout << "\n";
  } else if (cmd == "pruefer") {
    std::vector<uint32_t> code;
    uint32_t v;
    while (in >> v) code.push_back(v);
    for (uint32_t x : MutationTree::pruefer_code_to_parent_vector(code))
      std::cout << x << ' ';
    std::cout << "\n";
  } else if (cmd == "tree") {
    float beta;
    in >> beta;
    std::vector<uint32_t> parent;
    uint32_t v;
    while (in >> v) parent.push_back(v);
    std::tie(st.am, st.dm) = MutationTree::parent_vector_to_matrix(parent);
    st.n_genes = (uint32_t)parent.size() - 1;
    st.tree = std::make_unique<MutationTree>(st.am, st.dm, st.n_genes, beta);
    print_tree(*st.tree);
  } else if (cmd == "update") {
    ModificationParameters mp{};
    in >> mp.move_type >> mp.v >> mp.w >> mp.parent_of_v >> mp.parent_of_w >>
        mp.descendant_of_v >> mp.nondescendant_of_v >> mp.new_beta;
    AncestorMatrix am, dm;
    MutationTree t(am, dm, *st.tree, mp);
    print_tree(t);
  } else if (cmd == "realize") {
    RawMoveSample r{};
    in >> r.move_type >> r.raw_v >> r.raw_w >> r.raw_descendant_of_v >>
        r.raw_nondescendant_of_v >> r.beta_jump;
    const ModificationParameters m = st.tree->realize_raw_move_sample(r);
    std::cout << std::setprecision(9) << m.move_type << ' ' << m.v << ' '
              << m.w << ' ' << m.parent_of_v << ' ' << m.parent_of_w << ' '
              << m.descendant_of_v << ' ' << m.nondescendant_of_v << ' '
              << m.new_beta << "\n";
  } else if (cmd == "scorer") {
    float a, b, sd;
    uint32_t nc, ng;
    in >> a >> b >> sd >> nc >> ng;
    const size_t words = (size_t)nc * bbs_words(ng + 1);
    std::vector<uint64_t> mut(words), known(words);
    for (auto &w : mut) in >> w;
    for (auto &w : known) in >> w;
    st.scorer = std::make_unique<TreeScorer>(a, b, sd, nc, ng, mut, known);
    std::cout << "ok\n";
  } else if (cmd == "score") {
    std::cout << std::setprecision(9) << st.scorer->logscore_tree(*st.tree)
              << "\n";
  } else if (cmd == "prior") {
    float b;
    in >> b;
    std::cout << std::setprecision(9) << st.scorer->logscore_beta(b) << "\n";
  } else if (cmd == "resume") {
    uint32_t nc, ng, s1, s2;
    in >> nc >> ng >> s1 >> s2;
    const size_t words = (size_t)nc * bbs_words(ng + 1);
    std::vector<uint64_t> mut(words), known(words);
    for (auto &w : mut) in >> w;
    for (auto &w : known) in >> w;
    std::vector<std::string> rest;
    std::string t;
    while (in >> t) rest.push_back(t);
    auto params_for = [&](uint32_t steps) {
      std::vector<std::string> tok{"bbscite"};
      tok.insert(tok.end(), rest.begin(), rest.end());
      tok.push_back("-l");
      tok.push_back(std::to_string(steps));
      std::vector<char *> argv;
      for (auto &s : tok) argv.push_back(s.data());
      Parameters p;
      if (!p.load_and_verify_args((int)argv.size(), argv.data()))
        throw std::runtime_error("bad arguments");
      return p;
    };
    Application whole(mut, known, params_for(s1 + s2), nc, ng);
    whole.run_simulation();
    Application first(mut, known, params_for(s1), nc, ng);
    first.run_simulation();
    const std::vector<uint8_t> image = first.save_chains();
    Application second(mut, known, params_for(s2), nc, ng);
    second.load_chains(image);
    second.run_simulation();
    std::cout << std::setprecision(9) << "whole " << whole.get_best_score()
              << " resumed " << second.get_best_score() << " same_tree "
              << (whole.get_best_dm() == second.get_best_dm()) << " bytes "
              << image.size() << "\n";
  } else {
    std::cout << "unknown command\n";
  }
}

}  // namespace

int main() {
  State st;
  std::string line;
  while (std::getline(std::cin, line)) {
    if (line.empty()) continue;
    try {
      run(line, st);
    } catch (Error const &e) {
      std::cout << "error " << e.status << ' ' << e.what() << "\n";
    }
    std::cout.flush();
  }
  return 0;
}
