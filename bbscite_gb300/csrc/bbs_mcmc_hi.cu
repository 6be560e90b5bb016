// Persistent chain kernels for trees of 129..256 nodes (W32 = 5..8).
#include "bbs_launch.cuh"

// This unit builds the launches without recording; bbs_mcmc_hi_rec.cu
// includes it again with recorded moves and step traces compiled in.
#ifndef BBS_REC
#define BBS_REC false
#define BBS_MCMC_HI launch_mcmc_hi
#endif

namespace bbs {

#define BBS_CASE(W, QQ)                                                   \
  case W * 10 + QQ:                                                       \
    return sum ? launch_mcmc_t<W, QQ, true, BBS_REC>(a, cpb, n_sms, s)    \
               : launch_mcmc_t<W, QQ, false, BBS_REC>(a, cpb, n_sms, s);
#define BBS_Q_CASES(W) BBS_CASE(W, 1) BBS_CASE(W, 2)

int BBS_MCMC_HI(const RunArgs &a, int w32, int q, bool sum, int cpb,
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
