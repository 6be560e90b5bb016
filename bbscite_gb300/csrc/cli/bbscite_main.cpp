// bbscite_main.cpp -- the SCITE-compatible command line of the GB300 path.
//
// Same flags, messages, exit codes and output files as src/main.cpp:42-214
// of the reference:
//   <base>_ml0.gv, <base>_ml0.newick, <base>_ml0_beta.txt,
//   <base>_ml0_am.txt, <base>_ml0_dm.txt
// with <base> from -o or the input path without its suffix.  Trees tied
// with the best (SCITE's tree list, -max_treelist_size, which the
// reference parses but does not use) follow as _ml1, _ml2, ...  The size
// limits are BBS_MAX_CELLS cells and BBS_MAX_GENES genes instead of the
// FPGA builds' 64/96.  "Move generation makespan" reports the host setup
// time (context and initial trees): the moves are drawn inside the chain
// kernel.
#include <algorithm>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "bbscite_gb300.hpp"

using namespace bbSCITE;

namespace {

// First pass over the input, src/main.cpp:50-101: counts cells (entries of
// the first line) and genes (lines) and rejects other characters.
int scan_input(const std::string &path, uint32_t &n_cells, uint32_t &n_genes) {
  std::ifstream in(path);
  n_cells = n_genes = 0;
  uint32_t in_line = 0;
  int ch;
  while ((ch = in.get()) != EOF) {
    const char c = (char)ch;
    if (c == '0' || c == '1' || c == '2' || c == '3') {
      in_line++;
    } else if (c == '\n') {
      if (n_cells == 0) {
        n_cells = in_line;
      } else if (n_cells != in_line) {
        std::cerr << "Error: Inconsistent rows in the input file!" << std::endl;
        return 1;
      }
      n_genes++;
      in_line = 0;
    } else if (c == ' ') {
      continue;
    } else {
      std::cerr << "Error: Illegal character " << c << " in the input file!"
                << std::endl;
      return 1;
    }
  }
  // a last line without a newline counts when it is complete; an
  // incomplete one is reported and left out, as the reference does
  if (in_line == n_cells) {
    n_genes++;
  } else if (in_line != 0) {
    std::cerr << "Error: Inconsistent rows in the input file!" << std::endl;
  }
  return 0;
}

// Second pass, src/main.cpp:106-144: gene rows, cell columns; 0 known
// unmutated, 1 and 2 mutated, 3 unknown.
int load_input(const std::string &path, uint32_t n_cells, uint32_t n_genes,
               std::vector<uint64_t> &mut, std::vector<uint64_t> &known) {
  const uint32_t W = bbs_words(n_genes + 1);
  mut.assign((size_t)n_cells * W, 0);
  known.assign((size_t)n_cells * W, 0);
  std::ifstream in(path);
  for (uint32_t g = 0; g < n_genes; g++) {
    for (uint32_t c = 0; c < n_cells; c++) {
      int entry;
      in >> entry;
      const uint64_t bit = uint64_t{1} << (g % 64);
      uint64_t &m = mut[(size_t)c * W + g / 64];
      uint64_t &k = known[(size_t)c * W + g / 64];
      switch (entry) {
        case 0:
          m &= ~bit;
          k |= bit;
          break;
        case 1:
        case 2:
          m |= bit;
          k |= bit;
          break;
        case 3:
          k &= ~bit;
          break;
        default:
          std::cerr << "Error: The input file contains the invalid entry "
                    << entry << std::endl;
          return 1;
      }
    }
  }
  // an unknown entry carries no mutation bit (the kernels require M within K)
  for (size_t i = 0; i < mut.size(); i++) mut[i] &= known[i];
  return 0;
}

void write_matrix(const std::string &path, AncestorMatrix const &m,
                  uint32_t n) {
  const uint32_t W = bbs_words(n);
  std::ofstream out(path);
  std::string line(n, '0');
  for (uint32_t i = 0; i < n; i++) {
    for (uint32_t j = 0; j < n; j++)
      line[j] = ((m[(size_t)i * W + j / 64] >> (j % 64)) & 1) ? '1' : '0';
    out << line << "\n";
  }
}

}  // namespace

int main(int argc, char **argv) {
  Parameters parameters;
  if (!parameters.load_and_verify_args(argc, argv)) {
    std::cerr << "Quitting due to CLI argument errors." << std::endl;
    return 1;
  }

  uint32_t n_cells = 0, n_genes = 0;
  if (scan_input(parameters.get_input_path(), n_cells, n_genes)) return 1;
  if (n_cells == 0 || n_genes == 0) {
    std::cerr << "Error: Empty input file!" << std::endl;
    return 1;
  }
  if (n_cells > BBS_MAX_CELLS) {
    std::cerr << "Error: This build of bbSCITE only supports up "
              << BBS_MAX_CELLS << " cells. The input data contains " << n_cells
              << " cells." << std::endl;
    return 1;
  }
  if (n_genes > BBS_MAX_GENES) {
    std::cerr << "Error: This build of bbSCITE only supports up "
              << BBS_MAX_GENES << " genes. The input data contains " << n_genes
              << " genes." << std::endl;
    return 1;
  }
  std::vector<uint64_t> mut, known;
  if (load_input(parameters.get_input_path(), n_cells, n_genes, mut, known))
    return 1;

  try {
    Application app(mut, known, parameters, n_cells, n_genes);
    std::cout << "Move generation makespan: " << app.get_setup_seconds()
              << " s" << std::endl;
    const float runtime = app.run_simulation();
    std::cout << "Time elapsed: " << runtime << " ms" << std::endl;

    // <base>_ml<i> for every co-optimal tree (SCITE's tree list; the
    // reference writes only _ml0, which is the best tree here too)
    const std::string base = parameters.get_output_path_base();
    auto list = app.get_treelist(
        std::max<uint32_t>(1u, parameters.get_max_n_best_trees()));
    for (size_t i = 0; i < list.size(); i++) {
      AncestorMatrix best_dm = list[i].first;
      const float best_beta = list[i].second;
      AncestorMatrix best_am(best_dm.size());
      check(bbs_dm_to_am(best_dm.data(), n_genes + 1, best_am.data()));
      MutationTree tree(best_am, best_dm, n_genes, best_beta);
      const std::string ml = base + "_ml" + std::to_string(i);
      {
        std::ofstream out(ml + ".gv");
        out << tree.to_graphviz();
      }
      {
        std::ofstream out(ml + ".newick");
        out << tree.to_newick();
      }
      {
        std::ofstream out(ml + "_beta.txt");
        out << best_beta << std::endl;
      }
      write_matrix(ml + "_am.txt", best_am, n_genes + 1);
      write_matrix(ml + "_dm.txt", best_dm, n_genes + 1);
    }
  } catch (Error const &e) {
    std::cerr << "Error: " << e.what() << std::endl;
    return 1;
  }
  return 0;
}
