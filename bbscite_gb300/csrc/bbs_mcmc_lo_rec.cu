// Recording launches (recorded moves and/or a step trace) of
// bbs_mcmc_lo.cu.
#define BBS_REC true
#define BBS_MCMC_LO launch_mcmc_lo_rec
#include "bbs_mcmc_lo.cu"
