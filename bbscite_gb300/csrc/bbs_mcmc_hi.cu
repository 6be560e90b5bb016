// Persistent chain kernels for trees of 129..256 nodes (W32 = 5..8).
#include "bbs_launch.cuh"

namespace bbs {

#define BBS_Q_CASES(W)                                        \
  case W * 10 + 1: return launch_mcmc_t<W, 1>(a, cpb, n_sms, s); \
  case W * 10 + 2: return launch_mcmc_t<W, 2>(a, cpb, n_sms, s);

int launch_mcmc_hi(const RunArgs &a, int w32, int q, int cpb, int n_sms,
                   cudaStream_t s) {
  switch (w32 * 10 + q) {
    BBS_Q_CASES(5)
    BBS_Q_CASES(6)
    BBS_Q_CASES(7)
    BBS_Q_CASES(8)
    default: return (int)cudaErrorInvalidValue;
  }
}

}  // namespace bbs
