// Work-list kernels for chains of several warps (one chain per block).
#define BBS_MULTI true
#define BBS_BATCH_LO launch_batch_lo_multi
#define BBS_BATCH_HI launch_batch_hi_multi
#include "bbs_batch.cu"
