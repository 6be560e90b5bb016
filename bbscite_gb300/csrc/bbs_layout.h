// bbs_layout.h -- shared-memory layout of the chain kernels: the sizes the
// kernels carve their dynamic shared memory by and the host launchers
// request (host and device code).
#pragma once
#include "bbs_internal.h"

namespace bbs {

// Bytes of a packed count table of n nodes x 32 lanes for q cells per
// lane: (q + 1) / 2 32-bit words per entry.
__host__ __device__ inline int pack_table_bytes(int n, int q) {
  return 4 * ((q + 1) / 2) * n * 32;
}

// Shared memory of the chain kernels, in bytes (16-byte aligned pieces).
__host__ __device__ inline int align16(int b) { return (b + 15) & ~15; }

// Rows of five to eight words: a warp's ring of the packed counts of the
// last kRing nodes in the canonical order, and its gene table, one entry
// of NW words per 8 genes and lane laid out as the counts are packed (word
// h: byte 0 the D bits of the 8 genes for cell slot 2h, byte 1 their M
// bits, bytes 2 and 3 the same for cell slot 2h + 1).
__host__ __device__ inline int ring_bytes(int q) {
  return 4 * ((q + 1) / 2) * kRing * 32;
}
__host__ __device__ inline int gene_table_bytes(int n, int q) {
  return 4 * ((q + 1) / 2) * ((n + 7) / 8) * 32;
}

// Per warp of a chain with the node-order scratch (every sum-score chain:
// its order is canonical; every chain that inherits counts): the canonical
// node order, its depth histogram and, with `counts`, the packed counts of
// every node for the lane's cells (rows of up to four words) or the ring
// and gene table (wider rows).
__host__ __device__ inline int sum_warp_bytes(int n, int w32, int q,
                                              bool counts) {
  int b = align16(2 * n) + align16(4 * 32 * ((n + 31) / 32));
  if (counts)
    b += w32 <= 4 ? align16(pack_table_bytes(n, q))
                  : align16(ring_bytes(q)) + align16(gene_table_bytes(n, q));
  return b;
}

// Each warp's Philox blocks of 16 steps: 32 x 16 bytes.
inline constexpr int kPhiloxBytes = 512;

// The head of a chain slot: two row buffers, the partial sums of both step
// parities (2 x wpc x 12 words), a flag word (16 bytes) and each warp's
// Philox blocks.
__host__ __device__ inline int slot_head_bytes(int n, int rs, int wpc) {
  return 4 * (2 * n * rs + 24 * wpc + 4) + kPhiloxBytes * wpc;
}

// One chain slot: its head and, with the scratch, the current and proposed
// parent vectors and each warp's scratch.
__host__ __device__ inline int slot_bytes(int n, int rs, int wpc, bool scratch,
                                          int w32, int q, bool counts) {
  int b = slot_head_bytes(n, rs, wpc);
  if (scratch) b += align16(2 * n) + wpc * sum_warp_bytes(n, w32, q, counts);
  return b;
}

// After the slots, with `counts`: the block's tables of per-gene
// increments, one per warp part of a chain (wpc), each for that warp's
// 32 q cell slots.
__host__ __device__ inline int inc_table_bytes(int n, int q) {
  return align16(pack_table_bytes(n, q));
}
__host__ __device__ inline int table_bytes(int n, int w32, int q, int wpc,
                                           bool counts) {
  return counts && w32 <= 4 ? wpc * inc_table_bytes(n, q) : 0;
}

// Chain-kernel blocks: one-warp chains of one dataset share the block's
// increment table.  The launch bounds of each cells-per-lane variant aim
// at 16, 12 and 8 resident warps per SM for 1, 2 and 3-4 cells per lane
// (registers per thread 128, 168, 255), in blocks of up to 4, 4 and 8
// warps: eight warps of three or four cells per lane fill an SM alone.
// (The batched kernel for rows of five to eight words takes up to 255
// registers: shared memory limits those launches first.)
inline constexpr int kMaxBlockThreads = 256;
__host__ __device__ constexpr int chain_max_threads(int q) {
  return q >= 3 ? 256 : 128;
}
__host__ __device__ constexpr int chain_min_blocks(int q) {
  return q == 1 ? 4 : (q == 2 ? 3 : 1);
}
__host__ __device__ constexpr int chain_regs(int q) {
  return q == 1 ? 128 : (q == 2 ? 168 : 255);
}

// Dynamic shared memory of a chain-kernel launch: `slots` chain slots of
// `wpc` warps and, with inherited counts, the increment tables.
__host__ __device__ inline int chain_launch_smem(int n, int n_cells, int q,
                                                 int wpc, int slots,
                                                 bool sum) {
  const int w32 = w32_of_nodes(n);
  const bool counts = inherits_counts(w32, n_cells, 32 * wpc * q);
  return slots * slot_bytes(n, rs_of_w32(w32), wpc, sum || counts, w32, q,
                            counts) +
         table_bytes(n, w32, q, wpc, counts);
}

// Resident warps per SM of such a launch (blocks of warps_per_block
// warps), from the SM's shared memory (smem_sm bytes, reserved_per_block
// of them taken by each block, at most smem_block per block) and registers.
inline int chain_resident_warps(int smem, int warps_per_block, int q,
                                int smem_sm, int smem_block,
                                int reserved_per_block) {
  if (smem > smem_block) return 0;
  const int by_smem = smem_sm / (smem + reserved_per_block);
  const int regs = (chain_regs(q) + 7) & ~7;
  const int by_regs = 65536 / (regs * 32 * warps_per_block);
  const int blocks = by_smem < by_regs ? by_smem : by_regs;
  return blocks * warps_per_block;
}

}  // namespace bbs
