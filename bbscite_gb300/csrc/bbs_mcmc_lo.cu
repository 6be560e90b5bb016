// Persistent chain kernels for trees of up to 128 nodes (W32 = 1..4).
#include "bbs_launch.cuh"

namespace bbs {

#define BBS_Q_CASES(W)                                        \
  case W * 10 + 1: return launch_mcmc_t<W, 1>(a, cpb, n_sms, s); \
  case W * 10 + 2: return launch_mcmc_t<W, 2>(a, cpb, n_sms, s); \
  case W * 10 + 3: return launch_mcmc_t<W, 3>(a, cpb, n_sms, s); \
  case W * 10 + 4: return launch_mcmc_t<W, 4>(a, cpb, n_sms, s);

int launch_mcmc_lo(const RunArgs &a, int w32, int q, int cpb, int n_sms,
                   cudaStream_t s) {
  switch (w32 * 10 + q) {
    BBS_Q_CASES(1)
    BBS_Q_CASES(2)
    BBS_Q_CASES(3)
    BBS_Q_CASES(4)
    default: return (int)cudaErrorInvalidValue;
  }
}

}  // namespace bbs
