// bbs_aux.cu -- dispatch of the chain kernels, batch scorer / mover /
// adjoint launchers and the integer-pipe calibration kernel.
#include "bbs_launch.cuh"

namespace bbs {

int pick_q(int n_cells) {
  // Keep every cell in registers when 32*Q covers the dataset; otherwise
  // the widest chunk.
  return std::min(kMaxQ, std::max(1, (n_cells + 31) / 32));
}

int launch_mcmc(const RunArgs &a, int q, int cpb, int n_sms, void *stream) {
  const int w32 = w32_of_nodes(a.ds.n_nodes);
  cudaStream_t s = (cudaStream_t)stream;
  const bool sum = a.md.score_mode == 1;
  if (w32 > 4) q = std::min(q, 2);
  const bool rec = a.moves != nullptr || a.trace != nullptr;
  if (w32 <= 4)
    return rec ? launch_mcmc_lo_rec(a, w32, q, sum, cpb, n_sms, s)
               : launch_mcmc_lo(a, w32, q, sum, cpb, n_sms, s);
  return rec ? launch_mcmc_hi_rec(a, w32, q, sum, cpb, n_sms, s)
             : launch_mcmc_hi(a, w32, q, sum, cpb, n_sms, s);
}

int launch_batch(const BatchArgs &b, int w32, int q, bool sum, int wpb,
                 int n_sms, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  if (b.wpc > 1)
    return w32 <= 4 ? launch_batch_lo_multi(b, w32, q, sum, wpb, n_sms, s)
                    : launch_batch_hi_multi(b, w32, q, sum, wpb, n_sms, s);
  if (w32 <= 4) return launch_batch_lo(b, w32, q, sum, wpb, n_sms, s);
  return launch_batch_hi(b, w32, q, sum, wpb, n_sms, s);
}

template <int W32, bool SUM>
static int launch_init_t(const InitArgs &a, cudaStream_t s) {
  constexpr int RS = rs_of_w32(W32), WPB = 4, Q = 2;
  // per warp: the rows and (sum score) the canonical order and histogram,
  // as init_kernel lays them out
  const int n = a.max_nodes;
  const size_t per_warp = (size_t)4 * n * RS +
      (SUM ? align16(2 * n) + align16(4 * 32 * ((n + 31) / 32)) : 0);
  const size_t smem = (size_t)WPB * per_warp;
  auto kern = init_kernel<W32, Q, SUM>;
  cudaError_t e = prepare_smem(kern, smem);
  if (e != cudaSuccess) return (int)e;
  kern<<<(a.n_chains + WPB - 1) / WPB, WPB * 32, smem, s>>>(a);
  return (int)cudaGetLastError();
}

// Random initial trees (TreeArgs): one warp per chain.  The lanes draw
// the code and count node degrees; lane 0 decodes it in linear time,
// always taking the smallest leaf (the order of src/MutationTree.hpp:
// 454-463); the lanes then write each node's ancestor row (the node, its
// ancestors and the root, as parent_vector_to_matrix does).
inline constexpr int kTreeWords = 3 * 256;  // shared words per warp

__global__ void __launch_bounds__(128) tree_kernel(const TreeArgs a) {
  extern __shared__ __align__(16) uint32_t smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int chain = blockIdx.x * (blockDim.x >> 5) + wib;
  if (chain >= a.n_chains) return;
  const uint32_t d = a.chain_ds != nullptr ? a.chain_ds[chain] : 0u;
  const int n = a.ds[d].n_nodes;
  const uint64_t seed = a.md[d].seed;
  const uint32_t local =
      (uint32_t)chain - d * (uint32_t)a.chains_per_dataset;
  uint32_t *code = smem + (size_t)wib * kTreeWords;
  uint32_t *deg = code + 256;
  uint32_t *par = deg + 256;
  const int len = n - 2;
  for (int i = lane; i < n; i += 32) deg[i] = 1u;
  __syncwarp();
  const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
  for (int i4 = 4 * lane; i4 < len; i4 += 128) {
    const uint4 r = philox4x32_10(make_uint4((uint32_t)i4, local, 0x7265u, 0u),
                                  key);
    const uint32_t rr[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
    for (int k = 0; k < 4; k++)
      if (i4 + k < len) {
        const uint32_t v = __umulhi(rr[k], (uint32_t)n);
        code[i4 + k] = v;
        atomicAdd(&deg[v], 1u);
      }
  }
  __syncwarp();
  if (lane == 0) {
    // deg counts the remaining edges of every node not yet removed; every
    // node below ptr with degree 1 has been removed already
    int ptr = 0;
    while (ptr < n && deg[ptr] != 1u) ptr++;
    int leaf = ptr;
    for (int i = 0; i < len; i++) {
      const uint32_t v = code[i];
      par[leaf] = v;
      if (--deg[v] == 1u && (int)v < ptr) {
        leaf = (int)v;
      } else {
        ptr++;
        while (ptr < n && deg[ptr] != 1u) ptr++;
        leaf = ptr;
      }
    }
    par[leaf < n ? leaf : 0] = (uint32_t)(n - 1);
    par[n - 1] = (uint32_t)(n - 1);
  }
  __syncwarp();
  const int RS = 2 * ((n + 63) / 64), root = n - 1;
  uint32_t *out = a.chain_off != nullptr ? a.rows + a.chain_off[chain]
                                         : a.rows + (size_t)chain * n * RS;
  for (int x = lane; x < n; x += 32)
    for (int k = 0; k < RS; k++) {
      uint32_t v = 0;
      int y = x;
      for (int step = 0; step <= n; step++) {
        if ((y >> 5) == k) v |= 1u << (y & 31);
        if (y == root) break;
        y = (int)par[y];
      }
      out[(size_t)x * RS + k] = v;
    }
}

int launch_trees(const TreeArgs &a, void *stream) {
  constexpr int WPB = 4;
  const size_t smem = (size_t)WPB * kTreeWords * sizeof(uint32_t);
  cudaError_t e = prepare_smem(tree_kernel, smem);
  if (e != cudaSuccess) return (int)e;
  tree_kernel<<<(a.n_chains + WPB - 1) / WPB, WPB * 32, smem,
                (cudaStream_t)stream>>>(a);
  return (int)cudaGetLastError();
}

int launch_init(const InitArgs &a, int w32, bool sum, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  switch (w32 * 2 + (sum ? 1 : 0)) {
#define BBS_INIT_CASE(W)                          \
  case W * 2: return launch_init_t<W, false>(a, s); \
  case W * 2 + 1: return launch_init_t<W, true>(a, s);
    BBS_INIT_CASE(1)
    BBS_INIT_CASE(2)
    BBS_INIT_CASE(3)
    BBS_INIT_CASE(4)
    BBS_INIT_CASE(5)
    BBS_INIT_CASE(6)
    BBS_INIT_CASE(7)
    BBS_INIT_CASE(8)
#undef BBS_INIT_CASE
    default: return (int)cudaErrorInvalidValue;
  }
}

template <int W32, bool ATTACH>
static int launch_score_t(const ScoreArgs &a, cudaStream_t s) {
  constexpr int RS = rs_of_w32(W32), WPB = 4, Q = 2;
  const size_t smem = (size_t)WPB * a.ds.n_nodes * RS * sizeof(uint32_t);
  cudaError_t e = prepare_smem(score_kernel<W32, Q, ATTACH>, smem);
  if (e != cudaSuccess) return (int)e;
  const int blocks = (a.n_trees + WPB - 1) / WPB;
  score_kernel<W32, Q, ATTACH><<<blocks, WPB * 32, smem, s>>>(a);
  return (int)cudaGetLastError();
}

int launch_score(const ScoreArgs &a, int, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  const bool att = a.attach != nullptr;
  switch (w32_of_nodes(a.ds.n_nodes)) {
#define BBS_SCORE_CASE(W) \
  case W: return att ? launch_score_t<W, true>(a, s) : launch_score_t<W, false>(a, s);
    BBS_SCORE_CASE(1)
    BBS_SCORE_CASE(2)
    BBS_SCORE_CASE(3)
    BBS_SCORE_CASE(4)
    BBS_SCORE_CASE(5)
    BBS_SCORE_CASE(6)
    BBS_SCORE_CASE(7)
    BBS_SCORE_CASE(8)
#undef BBS_SCORE_CASE
    default: return (int)cudaErrorInvalidValue;
  }
}

template <int W32>
static int launch_apply_t(const ApplyArgs &a, cudaStream_t s) {
  constexpr int RS = rs_of_w32(W32), WPB = 4;
  const size_t smem = (size_t)WPB * a.n_nodes * RS * sizeof(uint32_t);
  cudaError_t e = prepare_smem(apply_kernel<W32>, smem);
  if (e != cudaSuccess) return (int)e;
  apply_kernel<W32><<<(a.n_trees + WPB - 1) / WPB, WPB * 32, smem, s>>>(a);
  return (int)cudaGetLastError();
}

int launch_apply(const ApplyArgs &a, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  switch (w32_of_nodes(a.n_nodes)) {
    case 1: return launch_apply_t<1>(a, s);
    case 2: return launch_apply_t<2>(a, s);
    case 3: return launch_apply_t<3>(a, s);
    case 4: return launch_apply_t<4>(a, s);
    case 5: return launch_apply_t<5>(a, s);
    case 6: return launch_apply_t<6>(a, s);
    case 7: return launch_apply_t<7>(a, s);
    case 8: return launch_apply_t<8>(a, s);
    default: return (int)cudaErrorInvalidValue;
  }
}

template <int W32>
static int launch_grad_t(const GradArgs &a, cudaStream_t s) {
  constexpr int RS = rs_of_w32(W32), WPB = 4, Q = 2;
  const size_t smem = (size_t)WPB * a.ds.n_nodes * RS * sizeof(uint32_t);
  cudaError_t e = prepare_smem(grad_kernel<W32, Q>, smem);
  if (e != cudaSuccess) return (int)e;
  grad_kernel<W32, Q><<<(a.n_trees + WPB - 1) / WPB, WPB * 32, smem, s>>>(a);
  return (int)cudaGetLastError();
}

int launch_grad(const GradArgs &a, int, void *stream) {
  cudaStream_t s = (cudaStream_t)stream;
  switch (w32_of_nodes(a.ds.n_nodes)) {
    case 1: return launch_grad_t<1>(a, s);
    case 2: return launch_grad_t<2>(a, s);
    case 3: return launch_grad_t<3>(a, s);
    case 4: return launch_grad_t<4>(a, s);
    case 5: return launch_grad_t<5>(a, s);
    case 6: return launch_grad_t<6>(a, s);
    case 7: return launch_grad_t<7>(a, s);
    case 8: return launch_grad_t<8>(a, s);
    default: return (int)cudaErrorInvalidValue;
  }
}

// ------------------------------------------------------------------------
// Integer-pipe calibration: 8 independent popcounts per iteration per
// thread (LOP3 + POPC + IADD each); the SM clock is read with clock64().
// ------------------------------------------------------------------------
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__global__ void __launch_bounds__(256) popc_bench_kernel(int iters,
                                                         uint32_t *sink,
                                                         long long *clock_probe) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t x[8], acc[8];
#pragma unroll
  for (int i = 0; i < 8; i++) {
    x[i] = t * 2654435761u + 40503u * (uint32_t)i;
    acc[i] = 0;
  }
  const long long c0 = clock64();
  const uint64_t g0 = global_ns();
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int i = 0; i < 8; i++) acc[i] += __popc(x[i] ^ (uint32_t)it);
  }
  const long long c1 = clock64();
  const uint64_t g1 = global_ns();
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) s += acc[i];
  if (s == 0xffffffffu) sink[t] = s;
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    clock_probe[0] = c1 - c0;
    clock_probe[1] = (long long)(g1 - g0);
  }
}

// A check that fails on purpose: the index 7 is compared with the limit
// 5 and nothing is read or written at it.
__global__ void check_selftest_kernel(int *status) {
  const uint32_t index = 7, limit = 5;
  if (!device_check(index < limit, status, kCheckSelfTest, index, limit)) return;
}

int run_check_selftest(int *status_device, int *enabled) {
#ifdef BBS_CHECKED
  *enabled = 1;
#else
  *enabled = 0;
#endif
  check_selftest_kernel<<<1, 32>>>(status_device);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return (int)e;
}

int run_popc_bench(double *popc_per_s, double *clock_hz) {
  int dev = 0, n_sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess)
    e = cudaDeviceGetAttribute(&n_sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return (int)e;
  const int threads = 256, blocks = n_sms * 8, iters = 1 << 16;
  uint32_t *sink = nullptr;
  long long *cyc = nullptr;
  e = cudaMalloc(&sink, sizeof(uint32_t) * threads * blocks);
  if (e == cudaSuccess) e = cudaMalloc(&cyc, 2 * sizeof(long long));
  cudaEvent_t a = nullptr, b = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  float best_ms = 1e30f;
  long long probe[2] = {0, 1};
  for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {
    cudaEventRecord(a);
    popc_bench_kernel<<<blocks, threads>>>(iters, sink, cyc);
    cudaEventRecord(b);
    e = cudaEventSynchronize(b);
    float ms = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    if (e == cudaSuccess && rep > 0 && ms < best_ms) {
      best_ms = ms;
      e = cudaMemcpy(probe, cyc, 2 * sizeof(long long), cudaMemcpyDeviceToHost);
    }
  }
  if (e == cudaSuccess) {
    const double ops = (double)threads * blocks * iters * 8.0;
    *popc_per_s = ops / (best_ms * 1e-3);
    // SM cycles over global-timer nanoseconds of one block
    *clock_hz = (double)probe[0] / ((double)probe[1] * 1e-9);
  }
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  cudaFree(sink);
  cudaFree(cyc);
  return (int)e;
}

}  // namespace bbs
