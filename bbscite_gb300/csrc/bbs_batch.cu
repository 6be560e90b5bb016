// Work-list kernels for many datasets in one launch, one instantiation per
// row width W32 (trees of up to 32 W32 nodes) and cells per lane.
#include "bbs_launch.cuh"

// This unit builds the launches of one-warp chains; bbs_batch_multi.cu
// includes it again for chains of several warps.
#ifndef BBS_MULTI
#define BBS_MULTI false
#define BBS_BATCH_LO launch_batch_lo
#define BBS_BATCH_HI launch_batch_hi
#endif

namespace bbs {

#define BBS_BCASE(W, QQ)                                                  \
  case W * 10 + QQ:                                                       \
    return sum ? launch_batch_t<W, QQ, true, BBS_MULTI>(b, wpb, n_sms, s) \
               : launch_batch_t<W, QQ, false, BBS_MULTI>(b, wpb, n_sms, s);

int BBS_BATCH_LO(const BatchArgs &b, int w32, int q, bool sum, int wpb,
                 int n_sms, cudaStream_t s) {
  switch (w32 * 10 + q) {
    BBS_BCASE(1, 1)
    BBS_BCASE(1, 2)
    BBS_BCASE(1, 3)
    BBS_BCASE(1, 4)
    BBS_BCASE(2, 1)
    BBS_BCASE(2, 2)
    BBS_BCASE(2, 3)
    BBS_BCASE(2, 4)
    BBS_BCASE(3, 1)
    BBS_BCASE(3, 2)
    BBS_BCASE(3, 3)
    BBS_BCASE(3, 4)
    BBS_BCASE(4, 1)
    BBS_BCASE(4, 2)
    BBS_BCASE(4, 3)
    BBS_BCASE(4, 4)
    default: return (int)cudaErrorInvalidValue;
  }
}

int BBS_BATCH_HI(const BatchArgs &b, int w32, int q, bool sum, int wpb,
                 int n_sms, cudaStream_t s) {
  switch (w32 * 10 + q) {
    BBS_BCASE(5, 1)
    BBS_BCASE(5, 2)
    BBS_BCASE(6, 1)
    BBS_BCASE(6, 2)
    BBS_BCASE(7, 1)
    BBS_BCASE(7, 2)
    BBS_BCASE(8, 1)
    BBS_BCASE(8, 2)
    default: return (int)cudaErrorInvalidValue;
  }
}

}  // namespace bbs
