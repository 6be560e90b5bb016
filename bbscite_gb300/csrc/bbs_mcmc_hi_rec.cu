// Recording launches (recorded moves and/or a step trace) of
// bbs_mcmc_hi.cu.
#define BBS_REC true
#define BBS_MCMC_HI launch_mcmc_hi_rec
#include "bbs_mcmc_hi.cu"
