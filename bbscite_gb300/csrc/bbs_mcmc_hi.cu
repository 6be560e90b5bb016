// Persistent chain kernels for trees of 129..256 nodes (W32 = 5..8).
#include "bbs_launch.cuh"

namespace bbs {

#define BBS_CASE(W, QQ)                                                   \
  case W * 10 + QQ:                                                       \
    return sum ? launch_mcmc_t<W, QQ, true>(a, cpb, n_sms, s)             \
               : launch_mcmc_t<W, QQ, false>(a, cpb, n_sms, s);
#define BBS_Q_CASES(W) BBS_CASE(W, 1) BBS_CASE(W, 2)

int launch_mcmc_hi(const RunArgs &a, int w32, int q, bool sum, int cpb,
                   int n_sms, cudaStream_t s) {
  switch (w32 * 10 + q) {
    BBS_Q_CASES(5)
    BBS_Q_CASES(6)
    BBS_Q_CASES(7)
    BBS_Q_CASES(8)
    default: return (int)cudaErrorInvalidValue;
  }
}

}  // namespace bbs
