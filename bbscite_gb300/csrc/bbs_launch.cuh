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

// Persistent launch.  wpc == 1: blocks of `cpb` one-warp chains; wpc > 1:
// blocks of one chain of wpc warps.  As many blocks as chains need, capped
// at what stays resident; each block then walks its chain slots.
template <int W32, int Q, bool SUM, bool REC>
int launch_mcmc_t(const RunArgs &a, int cpb, int n_sms, cudaStream_t s) {
  constexpr int RS = rs_of_w32(W32);
  if (a.wpc > 1) cpb = 1;
  const int threads = 32 * a.wpc * cpb;
  if (threads > chain_max_threads(Q)) return (int)cudaErrorInvalidConfiguration;
  const bool counts = inherits_counts(W32, a.ds.n_cells, 32 * a.wpc * Q);
  const size_t smem =
      (size_t)cpb * slot_bytes(a.ds.n_nodes, RS, a.wpc, SUM || counts, W32, Q,
                               counts) +
      table_bytes(a.ds.n_nodes, W32, Q, a.wpc, counts);
  auto kern = mcmc_kernel<W32, Q, SUM, REC>;
  cudaError_t e = prepare_smem(kern, smem);
  if (e != cudaSuccess) return (int)e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
  if (e != cudaSuccess) return (int)e;
  if (per_sm < 1) return (int)cudaErrorInvalidConfiguration;
  const int want = (a.n_chains + cpb - 1) / cpb;
  const int blocks = std::max(1, std::min(want, per_sm * n_sms));
  kern<<<blocks, threads, smem, s>>>(a);
  return (int)cudaGetLastError();
}

// Work-list launch: enough resident slots to fill the GPU, never more than
// there are units.  Blocks of wpb one-warp slots (b.wpc == 1), or of one
// slot of wpb == b.wpc warps.
template <int W32, int Q, bool SUM, bool MULTI>
int launch_batch_t(const BatchArgs &b, int wpb, int n_sms, cudaStream_t s) {
  constexpr int RS = rs_of_w32(W32);
  const int threads = 32 * wpb;
  if (threads > chain_max_threads(Q)) return (int)cudaErrorInvalidConfiguration;
  if (b.wpc < 1 || b.wpc > 4 || (b.wpc > 1) != MULTI ||
      (MULTI && wpb != b.wpc))
    return (int)cudaErrorInvalidValue;
  const int slots = wpb / b.wpc;
  const bool counts = b.with_counts != 0;
  if (counts && W32 <= 4 && b.table_ds < 0)
    return (int)cudaErrorInvalidValue;  // count tables need one dataset's rows
  const size_t smem =
      (size_t)slots * slot_bytes(b.max_nodes, RS, b.wpc, SUM || counts, W32,
                                 Q, counts) +
      table_bytes(b.max_nodes, W32, Q, b.wpc, counts);
  auto kern = batch_kernel<W32, Q, SUM, MULTI>;
  cudaError_t e = prepare_smem(kern, smem);
  if (e != cudaSuccess) return (int)e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
  if (e != cudaSuccess) return (int)e;
  if (per_sm < 1) return (int)cudaErrorInvalidConfiguration;
  const int want = (b.n_units + slots - 1) / slots;
  const int blocks = std::max(1, std::min(want, per_sm * n_sms));
  kern<<<blocks, threads, smem, s>>>(b);
  return (int)cudaGetLastError();
}

// Recording launches (recorded moves or a trace) go to the _rec units.
int launch_mcmc_lo(const RunArgs &a, int w32, int q, bool sum, int cpb,
                   int n_sms, cudaStream_t s);
int launch_mcmc_hi(const RunArgs &a, int w32, int q, bool sum, int cpb,
                   int n_sms, cudaStream_t s);
int launch_mcmc_lo_rec(const RunArgs &a, int w32, int q, bool sum, int cpb,
                       int n_sms, cudaStream_t s);
int launch_mcmc_hi_rec(const RunArgs &a, int w32, int q, bool sum, int cpb,
                       int n_sms, cudaStream_t s);
int launch_batch_lo(const BatchArgs &b, int w32, int q, bool sum, int wpb,
                    int n_sms, cudaStream_t s);
int launch_batch_hi(const BatchArgs &b, int w32, int q, bool sum, int wpb,
                    int n_sms, cudaStream_t s);
// (chains of several warps: their own units)
int launch_batch_lo_multi(const BatchArgs &b, int w32, int q, bool sum,
                          int wpb, int n_sms, cudaStream_t s);
int launch_batch_hi_multi(const BatchArgs &b, int w32, int q, bool sum,
                          int wpb, int n_sms, cudaStream_t s);

}  // namespace bbs
