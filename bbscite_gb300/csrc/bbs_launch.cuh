// bbs_launch.cuh -- templated host launchers shared by the kernel TUs.
#pragma once
#include <algorithm>

#include "bbs_kernels.cuh"

namespace bbs {

template <typename K>
inline cudaError_t prepare_smem(K kernel, size_t smem) {
  if (smem > 48 * 1024)
    return cudaFuncSetAttribute(kernel,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem);
  return cudaSuccess;
}

// Persistent launch: as many warps as chains, capped at what stays
// resident, so each warp walks chain, chain + total_warps, ...
template <int W32, int Q>
int launch_mcmc_t(const RunArgs &a, int wpb, int n_sms, cudaStream_t s) {
  constexpr int RS = rs_of_w32(W32);
  const size_t smem = (size_t)wpb * 2 * a.ds.n_nodes * RS * sizeof(uint32_t);
  cudaError_t e = prepare_smem(mcmc_kernel<W32, Q>, smem);
  if (e != cudaSuccess) return (int)e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mcmc_kernel<W32, Q>,
                                                    wpb * 32, smem);
  if (e != cudaSuccess) return (int)e;
  if (per_sm < 1) return (int)cudaErrorInvalidConfiguration;
  const int want = (a.n_chains + wpb - 1) / wpb;
  const int blocks = std::max(1, std::min(want, per_sm * n_sms));
  mcmc_kernel<W32, Q><<<blocks, wpb * 32, smem, s>>>(a);
  return (int)cudaGetLastError();
}

int launch_mcmc_lo(const RunArgs &a, int w32, int q, int wpb, int n_sms,
                   cudaStream_t s);
int launch_mcmc_hi(const RunArgs &a, int w32, int q, int wpb, int n_sms,
                   cudaStream_t s);

}  // namespace bbs
