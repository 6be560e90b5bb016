// bbs_device.cuh -- warp-level building blocks of the chain step on sm_103a.
//
// One warp owns one chain.  The tree is kept only as its ancestor rows
// (dm[x] = ancestors of x, src/MutationTree.hpp:718-723) in shared memory;
// descendant sets are rebuilt on demand with one __ballot_sync per 32
// nodes, so no transposed copy has to be updated.  Lane l owns nodes
// x = 32 r + l (r < W32) for the update and cells c = 32 q + l for scoring.
#pragma once
#include <cstdint>

#include "bbs_internal.h"
#include "bbs_layout.h"

namespace bbs {

#define BBS_FULL_MASK 0xffffffffu

// ------------------------------------------------------------------------
// Device checks.  A build with BBS_CHECKED defined tests the indices that
// come from data rather than from loop bounds (the nodes of a realised
// move, work-list entries, dataset numbers); the first failure sets bit 1
// of status[0] and stores its code, value and limit in status[1..3], and
// the caller skips what the index would have reached.  Without
// BBS_CHECKED every check is true at compile time and costs nothing.
// ------------------------------------------------------------------------
__device__ __forceinline__ bool device_check(bool ok, int *status, int code,
                                             uint32_t value, uint32_t limit) {
#ifdef BBS_CHECKED
  if (!ok && status != nullptr && (atomicOr(status, 2) & 2) == 0) {
    status[1] = code;
    status[2] = (int)value;
    status[3] = (int)limit;
  }
  return ok;
#else
  (void)ok;
  (void)status;
  (void)code;
  (void)value;
  (void)limit;
  return true;
#endif
}

// ------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11) and the move sampler.  The word
// assignment matches orc_sample_move in the CPU oracle.
// ------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}

__device__ __forceinline__ float u01_24(uint32_t x) {
  return __uint2float_rn(x >> 8) * 5.9604644775390625e-08f;
}

// The move of one step from its two Philox blocks a = Philox(step, chain,
// 0) and b = Philox(step, chain, 1) under the key (seed).  The normal jump
// is only drawn when it is used (beta moves) or recorded.
__device__ __forceinline__ bbs_raw_move move_from_words(const MoveProbs &mp,
                                                        uint32_t n_nodes,
                                                        const uint4 a,
                                                        const uint4 b,
                                                        bool always_jump) {
  bbs_raw_move m;
  const float ut = u01_24(a.x);
  m.move_type = ut <= mp.cum_beta    ? BBS_MOVE_CHANGE_BETA
                : ut <= mp.cum_prune ? BBS_MOVE_PRUNE_REATTACH
                : ut <= mp.cum_swap  ? BBS_MOVE_SWAP_NODES
                                     : BBS_MOVE_SWAP_SUBTREES;
  uint32_t v = __umulhi(a.y, n_nodes - 1u);
  uint32_t w = __umulhi(a.z, n_nodes - 2u);
  if (w >= v) w++;
  m.raw_v = v;
  m.raw_w = w;
  m.raw_descendant_of_v = u01_24(a.w);
  m.raw_nondescendant_of_v = u01_24(b.x);
  m.acceptance_level = u01_24(b.y);
  m.beta_jump = 0.0f;
  if (always_jump || m.move_type == BBS_MOVE_CHANGE_BETA) {
    const float u1 =
        (__uint2float_rn(b.z >> 8) + 1.0f) * 5.9604644775390625e-08f;
    const float u2 = u01_24(b.w);
    const float z = __fmul_rn(sqrtf(__fmul_rn(-2.0f, logf(u1))),
                              cosf(__fmul_rn(6.2831853071795864769f, u2)));
    m.beta_jump = __fmul_rn(z, mp.beta_jump_sd);
  }
  m.reserved = 0;
  return m;
}

// The Philox blocks of 16 consecutive steps, computed by the whole warp at
// once: lane l computes block (l & 1) of step step0 + (l >> 1) into
// buf[l] (a warp's kPhiloxBytes of shared memory).  Step step0 + k then
// reads its two blocks buf[2k] and buf[2k + 1]: one Philox evaluation per
// lane for 16 steps instead of two per step.
__device__ __forceinline__ void philox_fill(uint4 *buf, uint64_t seed,
                                            uint32_t chain, uint64_t step0,
                                            int lane) {
  const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
  const uint64_t step = step0 + (uint64_t)(lane >> 1);
  buf[lane] = philox4x32_10(make_uint4((uint32_t)step, (uint32_t)(step >> 32),
                                       chain, (uint32_t)(lane & 1)),
                            key);
}

// ------------------------------------------------------------------------
// Bit rows
// ------------------------------------------------------------------------
template <int W32>
__device__ __forceinline__ void ld_row(const uint32_t *p, uint32_t (&a)[W32]) {
  if constexpr (W32 == 1) {
    a[0] = p[0];
  } else if constexpr (W32 == 2) {
    const uint2 t = *reinterpret_cast<const uint2 *>(p);
    a[0] = t.x;
    a[1] = t.y;
  } else if constexpr (W32 <= 4) {
    const uint4 t = *reinterpret_cast<const uint4 *>(p);
    a[0] = t.x;
    a[1] = t.y;
    a[2] = t.z;
    if constexpr (W32 == 4) a[3] = t.w;
  } else if constexpr (W32 <= 6) {
    const uint2 t0 = reinterpret_cast<const uint2 *>(p)[0];
    const uint2 t1 = reinterpret_cast<const uint2 *>(p)[1];
    const uint2 t2 = reinterpret_cast<const uint2 *>(p)[2];
    a[0] = t0.x;
    a[1] = t0.y;
    a[2] = t1.x;
    a[3] = t1.y;
    a[4] = t2.x;
    if constexpr (W32 == 6) a[5] = t2.y;
  } else {
    const uint4 t0 = reinterpret_cast<const uint4 *>(p)[0];
    const uint4 t1 = reinterpret_cast<const uint4 *>(p)[1];
    a[0] = t0.x;
    a[1] = t0.y;
    a[2] = t0.z;
    a[3] = t0.w;
    a[4] = t1.x;
    a[5] = t1.y;
    a[6] = t1.z;
    if constexpr (W32 == 8) a[7] = t1.w;
  }
}

// Stores all RS words of a row (padding words zero).
template <int W32>
__device__ __forceinline__ void st_row(uint32_t *p, const uint32_t (&a)[W32]) {
  constexpr int RS = rs_of_w32(W32);
  uint32_t t[RS];
#pragma unroll
  for (int k = 0; k < RS; k++) t[k] = k < W32 ? a[k] : 0u;
  if constexpr (RS == 2) {
    *reinterpret_cast<uint2 *>(p) = make_uint2(t[0], t[1]);
  } else if constexpr (RS == 4) {
    *reinterpret_cast<uint4 *>(p) = make_uint4(t[0], t[1], t[2], t[3]);
  } else if constexpr (RS == 6) {
    reinterpret_cast<uint2 *>(p)[0] = make_uint2(t[0], t[1]);
    reinterpret_cast<uint2 *>(p)[1] = make_uint2(t[2], t[3]);
    reinterpret_cast<uint2 *>(p)[2] = make_uint2(t[4], t[5]);
  } else {
    reinterpret_cast<uint4 *>(p)[0] = make_uint4(t[0], t[1], t[2], t[3]);
    reinterpret_cast<uint4 *>(p)[1] = make_uint4(t[4], t[5], t[6], t[7]);
  }
}

// a[idx] without dynamic register indexing.
template <int W32>
__device__ __forceinline__ uint32_t pick(const uint32_t (&a)[W32], uint32_t idx) {
  uint32_t r = 0;
#pragma unroll
  for (int k = 0; k < W32; k++) r = (k == (int)idx) ? a[k] : r;
  return r;
}

template <int W32>
__device__ __forceinline__ uint32_t has_bit(const uint32_t (&a)[W32], uint32_t y) {
  return (pick<W32>(a, y >> 5) >> (y & 31u)) & 1u;
}

// Bits of node group r (nodes 32r .. 32r+31) that exist in an n-node tree.
__device__ __forceinline__ uint32_t group_mask(int r, int n) {
  const int left = n - 32 * r;
  return left >= 32 ? BBS_FULL_MASK : (left <= 0 ? 0u : ((1u << left) - 1u));
}

// k-th (0-based) set bit of a warp-uniform bit set S over W32 groups, or 0
// if there is none (src/MutationTree.hpp:840-878).
template <int W32>
__device__ __forceinline__ uint32_t select_bit(const uint32_t (&S)[W32],
                                               uint32_t k, int lane) {
  uint32_t before = 0, result = 0;
  bool found = false;
#pragma unroll
  for (int r = 0; r < W32; r++) {
    const uint32_t c = __popc(S[r]);
    if (!found && k < before + c) {  // warp-uniform branch
      const uint32_t kk = k - before;
      const bool hit = ((S[r] >> lane) & 1u) &&
                       (uint32_t)__popc(S[r] & ((1u << lane) - 1u)) == kk;
      const uint32_t b = __ballot_sync(BBS_FULL_MASK, hit);
      result = 32u * r + (uint32_t)(__ffs(b) - 1);
      found = true;
    }
    before += c;
  }
  return result;
}

// ------------------------------------------------------------------------
// Move realisation and the proposed tree
// ------------------------------------------------------------------------
struct Realized {
  bbs_move_params p;
  int ndv, ndw;   // descendant counts of v and w (v, w included)
  bool related;   // w is an ancestor of v
  bool fallback;  // a k-th (non)descendant index reached its count: the
                  // reference's rule then takes node 0
};

// Descendant sets of v and w as warp-uniform bit sets (one ballot per node
// group: node x has v in its ancestor row <=> x is a descendant of v).
template <int W32>
__device__ __forceinline__ void descendant_sets(const uint32_t *rows, int n,
                                                uint32_t v, uint32_t w,
                                                int lane, uint32_t (&Dv)[W32],
                                                uint32_t (&Dw)[W32]) {
  constexpr int RS = rs_of_w32(W32);
#pragma unroll
  for (int r = 0; r < W32; r++) {
    const int x = 32 * r + lane;
    bool bv = false, bw = false;
    if (x < n) {
      const uint32_t *row = rows + x * RS;
      bv = (row[v >> 5] >> (v & 31u)) & 1u;
      bw = (row[w >> 5] >> (w & 31u)) & 1u;
    }
    Dv[r] = __ballot_sync(BBS_FULL_MASK, bv);
    Dw[r] = __ballot_sync(BBS_FULL_MASK, bw);
  }
}

// realize_raw_move_sample, src/MutationTree.hpp:323-363.  v, w must be
// < n (the caller validates recorded moves; they are clamped here).
template <int W32>
__device__ __forceinline__ Realized realize_move(const uint32_t *rows, int n,
                                                 float beta,
                                                 const bbs_raw_move &raw,
                                                 int lane, uint32_t (&Dv)[W32],
                                                 uint32_t (&Dw)[W32]) {
  constexpr int RS = rs_of_w32(W32);
  Realized R;
  uint32_t v = min(raw.raw_v, (uint32_t)(n - 1));
  uint32_t w = min(raw.raw_w, (uint32_t)(n - 1));
  // is_ancestor(v, w) <=> v is in w's ancestor row
  if ((rows[w * RS + (v >> 5)] >> (v & 31u)) & 1u) {
    const uint32_t t = v;
    v = w;
    w = t;
  }
  uint32_t Av[W32], Aw[W32];
  ld_row<W32>(rows + v * RS, Av);
  ld_row<W32>(rows + w * RS, Aw);
  // Parents: the deepest proper ancestor (depth = ancestor count).
  uint32_t kv = 0, kw = 0;
#pragma unroll
  for (int r = 0; r < W32; r++) {
    const int x = 32 * r + lane;
    bool bv = false, bw = false;
    uint32_t depth = 0;
    if (x < n) {
      uint32_t a[W32];
      ld_row<W32>(rows + x * RS, a);
#pragma unroll
      for (int k = 0; k < W32; k++) depth += __popc(a[k]);
      bv = has_bit<W32>(a, v);
      bw = has_bit<W32>(a, w);
    }
    Dv[r] = __ballot_sync(BBS_FULL_MASK, bv);
    Dw[r] = __ballot_sync(BBS_FULL_MASK, bw);
    const uint32_t key = (depth << 16) | (uint32_t)x;
    if (x < n && ((Av[r] >> lane) & 1u) && (uint32_t)x != v) kv = max(kv, key);
    if (x < n && ((Aw[r] >> lane) & 1u) && (uint32_t)x != w) kw = max(kw, key);
  }
  kv = __reduce_max_sync(BBS_FULL_MASK, kv);
  kw = __reduce_max_sync(BBS_FULL_MASK, kw);
  // A node without a proper ancestor is the root, its own parent.
  R.p.parent_of_v = kv ? (kv & 0xffffu) : v;
  R.p.parent_of_w = kw ? (kw & 0xffffu) : w;
  int ndv = 0, ndw = 0;
#pragma unroll
  for (int r = 0; r < W32; r++) {
    ndv += __popc(Dv[r]);
    ndw += __popc(Dw[r]);
  }
  const int nnd = n - ndv;
  const float fd = floorf(__fmul_rn(raw.raw_descendant_of_v, (float)ndv));
  const float fn = floorf(__fmul_rn(raw.raw_nondescendant_of_v, (float)nnd));
  const uint32_t i_desc = __float2uint_rz(fd);
  const uint32_t i_nondesc = __float2uint_rz(fn);
  uint32_t ND[W32];
#pragma unroll
  for (int r = 0; r < W32; r++) ND[r] = ~Dv[r] & group_mask(r, n);
  R.p.move_type = raw.move_type;
  R.p.v = v;
  R.p.w = w;
  R.p.descendant_of_v = select_bit<W32>(Dv, i_desc, lane);
  R.p.nondescendant_of_v = select_bit<W32>(ND, i_nondesc, lane);
  float nb = __fadd_rn(beta, raw.beta_jump);
  if (nb < 0.0f) nb = fabsf(nb);
  if (nb > 1.0f) nb = __fsub_rn(nb, __fmul_rn(2.0f, __fsub_rn(nb, 1.0f)));
  R.p.new_beta = nb;
  R.ndv = ndv;
  R.ndw = ndw;
  R.related = has_bit<W32>(Dw, v);
  R.fallback = i_desc >= (uint32_t)ndv || i_nondesc >= (uint32_t)nnd;
  return R;
}

// The update constructor, src/MutationTree.hpp:123-307, on ancestor rows
// only.  Lane l writes rows x = 32 r + l of `out`.  With D(x) the
// descendant set and A(x) the ancestor row:
//   SwapNodes(v,w):    A'(x) = swap_bits_vw(A(s(x))), s swaps v and w
//   PruneReattach(v,t): x in D(v): A'(x) = A(t) | (A(x) & D(v))
//   SwapSubtrees unrelated: x in D(v): A(pw) | (A(x) & D(v));
//                           x in D(w): A(pv) | (A(x) & D(w))
//   SwapSubtrees related (w above v, d = descendant_of_v):
//                           x in D(v): A(x) & ~(D(w) & ~D(v));
//                           x in D(w) \ D(v): A(x) | (A(d) & D(v))
//   ChangeBeta: unchanged.
// The same rules are checked bit-exactly against the reference's
// per-bit rules by the tests.
// Warp `wic` of `wpc` writes the node groups r with r % wpc == wic.
template <int W32>
__device__ __forceinline__ void build_proposal(const uint32_t *rows,
                                               uint32_t *out, int n,
                                               const bbs_move_params &p,
                                               const uint32_t (&Dv)[W32],
                                               const uint32_t (&Dw)[W32],
                                               bool related, int wpc, int wic,
                                               int lane) {
  constexpr int RS = rs_of_w32(W32);
  const uint32_t v = p.v, w = p.w;
  uint32_t T1[W32], T2[W32];
  const int type = p.move_type;
  // Target rows (warp-uniform broadcast loads).
  uint32_t t1 = 0, t2 = 0;
  if (type == BBS_MOVE_PRUNE_REATTACH) {
    t1 = p.nondescendant_of_v;
  } else if (type == BBS_MOVE_SWAP_SUBTREES) {
    t1 = p.parent_of_w;
    t2 = related ? p.descendant_of_v : p.parent_of_v;
  }
  t1 = min(t1, (uint32_t)(n - 1));
  t2 = min(t2, (uint32_t)(n - 1));
  ld_row<W32>(rows + t1 * RS, T1);
  ld_row<W32>(rows + t2 * RS, T2);
#pragma unroll
  for (int r = 0; r < W32; r++) {
    const int x = 32 * r + lane;
    if (x >= n || r % wpc != wic) continue;
    const bool in_v = (Dv[r] >> lane) & 1u;
    const bool in_w = (Dw[r] >> lane) & 1u;
    uint32_t a[W32];
    if (type == BBS_MOVE_SWAP_NODES) {
      const uint32_t src = (uint32_t)x == v ? w : ((uint32_t)x == w ? v : (uint32_t)x);
      ld_row<W32>(rows + src * RS, a);
      const uint32_t bv = has_bit<W32>(a, v), bw = has_bit<W32>(a, w);
#pragma unroll
      for (int k = 0; k < W32; k++) {
        const uint32_t mv = (k == (int)(v >> 5)) ? (1u << (v & 31u)) : 0u;
        const uint32_t mw = (k == (int)(w >> 5)) ? (1u << (w & 31u)) : 0u;
        a[k] = (a[k] & ~(mv | mw)) | (bw ? mv : 0u) | (bv ? mw : 0u);
      }
    } else {
      ld_row<W32>(rows + x * RS, a);
      if (type == BBS_MOVE_PRUNE_REATTACH) {
        if (in_v) {
#pragma unroll
          for (int k = 0; k < W32; k++) a[k] = T1[k] | (a[k] & Dv[k]);
        }
      } else if (type == BBS_MOVE_SWAP_SUBTREES) {
        if (!related) {
          if (in_v) {
#pragma unroll
            for (int k = 0; k < W32; k++) a[k] = T1[k] | (a[k] & Dv[k]);
          } else if (in_w) {
#pragma unroll
            for (int k = 0; k < W32; k++) a[k] = T2[k] | (a[k] & Dw[k]);
          }
        } else {
          if (in_v) {
#pragma unroll
            for (int k = 0; k < W32; k++) a[k] = a[k] & ~(Dw[k] & ~Dv[k]);
          } else if (in_w) {
#pragma unroll
            for (int k = 0; k < W32; k++) a[k] = a[k] | (T2[k] & Dv[k]);
          }
        }
      }
    }
    st_row<W32>(out + x * RS, a);
  }
}

// ------------------------------------------------------------------------
// Paired single precision (sm_100 and later): one instruction applies the
// same IEEE round-to-nearest operation to both halves of a register pair,
// with the results of two scalar instructions (no flush-to-zero), in half
// the issue slots.  The node loops run two nodes of a cell side by side in
// the two halves.  There is no paired multiply here: the compiler fuses a
// paired multiply into a paired add that uses it, even with explicit
// round-to-nearest modifiers (measured on GB300: the results equal the
// fused form), so exact products are taken as fused multiply-adds of a
// -0.0 addend that the compiler cannot see (pair_score_b2).
// ------------------------------------------------------------------------
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "mov.b64 rc, {%6, %7};\n\tfma.rn.f32x2 rd, ra, rb, rc;\n\t"
      "mov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return d;
}
__device__ __forceinline__ float2 fadd2(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 fsub2(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
// max(a, b, c) in one instruction (sm_100 and later); exact, like fmaxf.
__device__ __forceinline__ float fmax3(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
__device__ __forceinline__ float2 dup2(float x) { return make_float2(x, x); }

// ------------------------------------------------------------------------
// Packed counts.  A lane's Q cells' counts of one node, d | m << 8 per cell
// (d, m <= 255: a count of genes), two cells per 32-bit word: NW = (Q+1)/2
// words, word q/2 holding cell q in bits 16 (q & 1) upwards.  Adding two
// packed words adds every field at once (no field can carry into the
// next).  A field becomes the exact biased float 2^23 + count with one byte
// permute into the bit pattern 0x4B0000xx.  In shared memory a table of
// entries [node][lane] keeps an entry's NW words together: one 32- or
// 64-bit access per entry (for three cells the fourth field is unused).
// ------------------------------------------------------------------------
template <int Q>
inline constexpr int kPackWords = (Q + 1) / 2;

template <int Q>
__device__ __forceinline__ void ld_pack(const uint32_t *t, int idx,
                                        uint32_t (&k)[kPackWords<Q>]) {
  if constexpr (kPackWords<Q> == 1) {
    k[0] = t[idx];
  } else {
    const uint2 v = reinterpret_cast<const uint2 *>(t)[idx];
    k[0] = v.x;
    k[1] = v.y;
  }
}

template <int Q>
__device__ __forceinline__ void st_pack(uint32_t *t, int idx,
                                        const uint32_t (&k)[kPackWords<Q>]) {
  if constexpr (kPackWords<Q> == 1) {
    t[idx] = k[0];
  } else {
    reinterpret_cast<uint2 *>(t)[idx] = make_uint2(k[0], k[1]);
  }
}

// Biased floats 2^23 + d and 2^23 + m of cell slot q (its word w = the
// entry's word q / 2; q is a constant after unrolling).
__device__ __forceinline__ float pack_d_biased(uint32_t w, int q) {
  return __int_as_float((int)__byte_perm(w, 0x4B000000u, 0x7540u + 2u * (q & 1)));
}
__device__ __forceinline__ float pack_m_biased(uint32_t w, int q) {
  return __int_as_float((int)__byte_perm(w, 0x4B000000u, 0x7541u + 2u * (q & 1)));
}
// The 16-bit field d | m << 8 of cell slot q.
template <int NW>
__device__ __forceinline__ uint32_t pack_field(const uint32_t (&k)[NW], int q) {
  return (k[q >> 1] >> (16 * (q & 1))) & 0xFFFFu;
}

// ------------------------------------------------------------------------
// Scoring (src/TreeScorer.hpp:131-210)
// ------------------------------------------------------------------------
// Population count of (X & A) over W32 words.  Groups of three words go
// through a full adder (ones = a^b^c, twos = maj(a,b,c); both single LOP3
// operations), so three words cost two POPC instead of three.
template <int W32>
__device__ __forceinline__ int masked_popc(const uint32_t (&X)[W32],
                                          const uint32_t (&A)[W32]) {
  int s = 0;
  constexpr int G3 = W32 / 3;
#pragma unroll
  for (int g = 0; g < G3; g++) {
    const uint32_t a = X[3 * g] & A[3 * g], b = X[3 * g + 1] & A[3 * g + 1],
                   c = X[3 * g + 2] & A[3 * g + 2];
    const uint32_t ones = a ^ b ^ c;
    const uint32_t twos = (a & b) | (c & (a ^ b));
    s += __popc(ones) + 2 * __popc(twos);
  }
#pragma unroll
  for (int w = 3 * G3; w < W32; w++) s += __popc(X[w] & A[w]);
  return s;
}

// The per-(cell,node) score in the reference's order
//   (((n00*l00 + n01*l01) + n10*l10) + n11*l11), no contraction,
// with the four counts as exact floats.  With D = K & ~M (observed 0) and
// M (observed 1), d = popc(D & A) and m = popc(M & A) give
// n01 = d, n11 = m, n00 = popc(D) - d, n10 = popc(M) - m.  Biased floats
// 2^23 + i (bit pattern 0x4B000000 + i) make every difference exact:
//   pdb = 2^23 + popc(D),  pmb = 2^23 + popc(M).
__device__ __forceinline__ float pair_score_b(float db, float mb, float pdb,
                                              float pmb, float l00, float l01,
                                              float l10, float l11) {
  const float f01 = __fsub_rn(db, 8388608.0f);
  const float f11 = __fsub_rn(mb, 8388608.0f);
  const float f00 = __fsub_rn(pdb, db);
  const float f10 = __fsub_rn(pmb, mb);
  float s = __fmul_rn(f00, l00);
  s = __fadd_rn(s, __fmul_rn(f01, l01));
  s = __fadd_rn(s, __fmul_rn(f10, l10));
  s = __fadd_rn(s, __fmul_rn(f11, l11));
  return s;
}

// The same from the integer counts.
__device__ __forceinline__ float pair_score(int d, int m, float pdb,
                                            float pmb, float l00, float l01,
                                            float l10, float l11) {
  return pair_score_b(__int_as_float(0x4B000000 + d),
                      __int_as_float(0x4B000000 + m), pdb, pmb, l00, l01, l10,
                      l11);
}

// The log table duplicated into both halves of paired registers, with a
// pair of -0.0 read from memory (DatasetDev::neg_zero).
struct LogTable2 {
  float2 l00, l01, l10, l11, nz;
};

// pair_score_b of two (cell, node) pairs side by side: the same four
// products and three sums in the same order, rounded as the scalar form
// rounds them.  Each product is a fused multiply-add of -0.0 (exactly the
// rounded product); with the addend unknown at compile time the compiler
// cannot fuse the product into the sum that follows, which it does with a
// paired multiply and add whatever their rounding modifiers.
__device__ __forceinline__ float2 pair_score_b2(float2 db, float2 mb,
                                                float2 pdb, float2 pmb,
                                                const LogTable2 &L) {
  const float2 bias = dup2(8388608.0f);
  const float2 f01 = fsub2(db, bias);
  const float2 f11 = fsub2(mb, bias);
  const float2 f00 = fsub2(pdb, db);
  const float2 f10 = fsub2(pmb, mb);
  float2 s = ffma2(f00, L.l00, L.nz);
  s = fadd2(s, ffma2(f01, L.l01, L.nz));
  s = fadd2(s, ffma2(f10, L.l10, L.nz));
  s = fadd2(s, ffma2(f11, L.l11, L.nz));
  return s;
}

// 64-bit hash of a tree's ancestor rows, the same in every lane: a mix of
// each word with its position, summed and xor-ed over the warp.  Only
// co-optimal tree lists use it, so it is kept out of line.
template <int W32>
__device__ __noinline__ uint64_t tree_hash(const uint32_t *rows, int n,
                                              int lane) {
  constexpr int RS = rs_of_w32(W32);
  uint32_t h0 = 0, h1 = 0;
#pragma unroll
  for (int r = 0; r < W32; r++) {
    const int x = 32 * r + lane;
    if (x < n) {
      uint32_t a[W32];
      ld_row<W32>(rows + x * RS, a);
#pragma unroll
      for (int k = 0; k < W32; k++) {
        uint32_t v = a[k] ^ (0x9E3779B9u * (uint32_t)(x * W32 + k + 1));
        v *= 0x85EBCA6Bu;
        v ^= v >> 13;
        v *= 0xC2B2AE35u;
        v ^= v >> 16;
        h0 += v;
        h1 ^= v * 0x27D4EB2Fu + (uint32_t)x;
      }
    }
  }
  h0 = __reduce_add_sync(BBS_FULL_MASK, h0);
  h1 = __reduce_xor_sync(BBS_FULL_MASK, h1);
  return ((uint64_t)h1 << 32) | h0;
}

// Per lane: Q cells as observed-0 rows D = K & ~M and observed-1 rows M.
template <int W32, int Q>
struct Cells {
  uint32_t D[Q][W32], M[Q][W32];
  float pdb[Q], pmb[Q];
};

// Loads cells c = c0 + stride * q + lane (zero rows past n_cells: such a
// cell has no counts and adds nothing).
template <int W32, int Q>
__device__ __forceinline__ void load_cells(Cells<W32, Q> &cb,
                                           const DatasetDev &ds, int c0,
                                           int stride, int lane) {
  constexpr int RS = rs_of_w32(W32);
#pragma unroll
  for (int q = 0; q < Q; q++) {
    const int c = c0 + stride * q + lane;
    int pd = 0, pm = 0;
#pragma unroll
    for (int k = 0; k < W32; k++) {
      uint32_t kw = 0, mw = 0;
      if (c < ds.n_cells) {
        kw = __ldg(ds.K + (size_t)c * RS + k);
        mw = __ldg(ds.M + (size_t)c * RS + k);
      }
      cb.D[q][k] = kw & ~mw;
      cb.M[q][k] = mw;
      pd += __popc(kw & ~mw);
      pm += __popc(mw);
    }
    cb.pdb[q] = __int_as_float(0x4B000000 + pd);
    cb.pmb[q] = __int_as_float(0x4B000000 + pm);
  }
}

// First-max attachment node of each of the lane's Q cells against all n
// ancestor rows (ties keep the lower node: std::max in
// src/TreeScorer.hpp:187-193; node 0 always initialises).  Nodes are taken
// two at a time for instruction-level parallelism, in order.
template <int W32, int Q>
__device__ __forceinline__ void best_nodes(const uint32_t *rows, int n,
                                           const Cells<W32, Q> &cb, float l00,
                                           float l01, float l10, float l11,
                                           float nz, int (&bj)[Q]) {
  constexpr int RS = rs_of_w32(W32);
  float best[Q];
  {
    uint32_t a[W32];
    ld_row<W32>(rows, a);
#pragma unroll
    for (int q = 0; q < Q; q++) {
      const int d = masked_popc<W32>(cb.D[q], a);
      const int m = masked_popc<W32>(cb.M[q], a);
      best[q] = pair_score(d, m, cb.pdb[q], cb.pmb[q], l00, l01, l10, l11);
      bj[q] = 0;
    }
  }
  int j = 1;
  const LogTable2 L2{dup2(l00), dup2(l01), dup2(l10), dup2(l11), dup2(nz)};
#pragma unroll 1
  for (; j + 1 < n; j += 2) {
    uint32_t a[W32], b[W32];
    ld_row<W32>(rows + j * RS, a);
    ld_row<W32>(rows + (j + 1) * RS, b);
#pragma unroll
    for (int q = 0; q < Q; q++) {
      const float2 db = make_float2(
          __int_as_float(0x4B000000 + masked_popc<W32>(cb.D[q], a)),
          __int_as_float(0x4B000000 + masked_popc<W32>(cb.D[q], b)));
      const float2 mb = make_float2(
          __int_as_float(0x4B000000 + masked_popc<W32>(cb.M[q], a)),
          __int_as_float(0x4B000000 + masked_popc<W32>(cb.M[q], b)));
      const float2 s2 = pair_score_b2(db, mb, dup2(cb.pdb[q]),
                                      dup2(cb.pmb[q]), L2);
      const float s0 = s2.x, s1 = s2.y;
      const bool up0 = s0 > best[q];
      best[q] = up0 ? s0 : best[q];
      bj[q] = up0 ? j : bj[q];
      const bool up1 = s1 > best[q];
      best[q] = up1 ? s1 : best[q];
      bj[q] = up1 ? j + 1 : bj[q];
    }
  }
  if (j < n) {
    uint32_t a[W32];
    ld_row<W32>(rows + j * RS, a);
#pragma unroll
    for (int q = 0; q < Q; q++) {
      const float s = pair_score(masked_popc<W32>(cb.D[q], a),
                                 masked_popc<W32>(cb.M[q], a), cb.pdb[q],
                                 cb.pmb[q], l00, l01, l10, l11);
      const bool up = s > best[q];
      best[q] = up ? s : best[q];
      bj[q] = up ? j : bj[q];
    }
  }
}

// Lane sums of k and m at the chosen nodes.
template <int W32, int Q>
__device__ __forceinline__ void counts_at(const uint32_t *rows,
                                          const Cells<W32, Q> &cb,
                                          const int (&bj)[Q], int &k, int &m) {
  constexpr int RS = rs_of_w32(W32);
#pragma unroll
  for (int q = 0; q < Q; q++) {
    uint32_t a[W32];
    ld_row<W32>(rows + bj[q] * RS, a);
    const int mm = masked_popc<W32>(cb.M[q], a);
    k += masked_popc<W32>(cb.D[q], a) + mm;
    m += mm;
  }
}

// The log table of one (alpha, beta) state.
struct LogTable {
  float l00, l10, l01, l11;
};

__device__ __forceinline__ LogTable2 log_table2(const LogTable &L, float nz) {
  return LogTable2{dup2(L.l00), dup2(L.l01), dup2(L.l10), dup2(L.l11),
                   dup2(nz)};
}

// Sum-over-attachments pass with its adjoint, for the lane's Q cells.
// Per cell the scores s_j are summed as exp(s_j - r) against a reference r
// that depends only on the cell and the log table: r = ub - 72 with ub =
// pd max(l00, l01) + pm max(l10, l11) >= every s_j, so no term overflows.
// A cell whose maximum lies more than 80 below r is summed once more
// against its maximum.  In base-2 units t_j = (s_j - r) log2(e) is affine
// in (d, m) = (popc(D & A), popc(M & A)), two FMAs per pair.  Adds to
// acc[6], in fixed point (2^-16 units for scores, 2^-20 for counts, so the
// result does not depend on how cells are split over lanes and warps):
// [0] sum_c lse_c, [2] E[n01] and [4] E[n11] (the expected class counts
// of observed-0 and observed-1 bits under the attachment posterior) and
// [5] sum_c max_j s_cj (the max score).  [1] and [3], E[n00] and E[n10],
// are left to the caller: with every cell counted they are the dataset's
// totals of observed-0 and observed-1 bits less [2] and [4]
// (complete_expected_counts).
inline constexpr float kFixScale = 1048576.0f;  // 2^20, class counts
inline constexpr float kScoreScale = 65536.0f;  // 2^16, scores: a cell's
  // |log-likelihood| stays below 2^15 for any float alpha, beta (at most
  // 255 genes of |log p| <= 104), so each cell's term fits in 32 bits

// E[n00] and E[n10] of a whole chain's sums (every cell counted once):
// the dataset's observed-0 and observed-1 bits less E[n01] and E[n11].
__device__ __forceinline__ void complete_expected_counts(const DatasetDev &ds,
                                                         long long (&acc)[6]) {
  acc[1] = (long long)(ds.sum_k - ds.sum_m) * 1048576ll - acc[2];
  acc[3] = (long long)ds.sum_m * 1048576ll - acc[4];
}

// The warp's sum of an int64 per lane (|x| < 2^40) with three 32-bit
// warp reductions: the high word and two 16-bit pieces of the low word,
// whose 32-lane sums cannot overflow; the same total in every lane.
__device__ __forceinline__ long long warp_sum_ll(long long x) {
  const int hi = (int)(x >> 32);
  const unsigned lo = (unsigned)(x & 0xFFFFFFFFll);
  const long long h = (long long)__reduce_add_sync(BBS_FULL_MASK, hi);
  const long long m = (long long)__reduce_add_sync(BBS_FULL_MASK, lo >> 16);
  const long long l = (long long)__reduce_add_sync(BBS_FULL_MASK, lo & 0xFFFFu);
  return h * 4294967296ll + m * 65536ll + l;
}

// An int64 fixed-point total as a float without double-precision
// arithmetic: x = hi * 2^24 + lo with 0 <= lo < 2^24, both exact in float
// for |x| < 2^48, and one rounding in the fused multiply-add.
__device__ __forceinline__ float ll_to_float(long long x) {
  const int hi = (int)(x >> 24);
  const int lo = (int)(x & 0xFFFFFFll);
  return fmaf((float)hi, 16777216.0f, (float)lo);
}
inline constexpr float kLog2E = 1.44269504088896341f;
inline constexpr float kLn2 = 0.693147180559945309f;

__device__ __forceinline__ float ex2_approx(float t) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(t));
  return r;
}

// ------------------------------------------------------------------------
// The sum score's node order.  Every sum-score evaluation adds its per-node
// terms in one canonical order of the tree -- by depth, ties by node index:
// the root first, every node after its parent -- and in the same pairs, so
// that a cell's sum does not depend on where it is computed (cells held in
// registers or streamed, any launch shape, batched or alone) nor on how its
// counts are found.  Two count sources give the same integers:
//   - masked popcounts of the node's ancestor row (any tree);
//   - inherited counts: a node's ancestors are its parent's plus itself,
//     so (d, m) of node j = (d, m) of its parent + (D, M) bits of gene j.
//     This needs the tree's parent vector, a per-warp table of every
//     node's packed counts and a block table of per-gene increments, and
//     issues no POPC; it serves cells held in registers with rows of up to
//     four words.
// ------------------------------------------------------------------------
struct SumCtx {
  uint16_t *ord;        // [n]: node | parent << 8, in canonical order
  int *hist;            // [32 * ceil(n / 32)]: depth histogram, scratch
  uint32_t *cnt;        // [n][32][NW]: every node's packed counts of the
                        // lane's cells, or null
  const uint32_t *inc;  // [n][32][NW]: per-gene packed increments of the
                        // warp's cells, or null
  const uint8_t *par;   // parent vector of the evaluated tree, or null
  // Rows of five to eight words (inherited counts without a table of every
  // node): the packed counts of the last kRing order positions (position i
  // in entry i % kRing) and the gene table of the cells being scored, or
  // null.
  uint32_t *ring;       // [kRing][32][NW]
  uint32_t *gt;         // [ceil(n / 8)][32][NW]
};

// ord and hist of the tree with ancestor rows `rows`; the parent of each
// node from `par` (0 where par is null).  Depth = ancestors - 1 = the
// popcount of the node's row less one (a row holds the node and the root).
template <int W32>
__device__ __forceinline__ void canonical_order(const uint32_t *rows, int n,
                                                const uint8_t *par,
                                                uint16_t *ord, int *hist,
                                                int lane) {
  constexpr int RS = rs_of_w32(W32);
  const int B = (n + 31) >> 5;  // node groups; bins per lane in the scan
  for (int i = lane; i < 32 * B; i += 32) hist[i] = 0;
  __syncwarp();
  int dep[W32];
#pragma unroll
  for (int g = 0; g < W32; g++) {
    const int x = 32 * g + lane;
    dep[g] = -1;
    if (x < n) {
      uint32_t a[W32];
      ld_row<W32>(rows + x * RS, a);
      int pc = 0;
#pragma unroll
      for (int k = 0; k < W32; k++) pc += __popc(a[k]);
      dep[g] = pc - 1;
      atomicAdd(&hist[pc - 1], 1);
    }
  }
  __syncwarp();
  // exclusive scan of the bins, lane l owning bins l*B .. l*B + B - 1
  int loc[W32], s = 0;
#pragma unroll
  for (int k = 0; k < W32; k++) {
    loc[k] = k < B ? hist[lane * B + k] : 0;
    s += loc[k];
  }
  int incl = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(BBS_FULL_MASK, incl, o);
    if (lane >= o) incl += v;
  }
  int run = incl - s;
  __syncwarp();
#pragma unroll
  for (int k = 0; k < W32; k++)
    if (k < B) {
      hist[lane * B + k] = run;
      run += loc[k];
    }
  __syncwarp();
  const unsigned below = (1u << lane) - 1u;
#pragma unroll
  for (int g = 0; g < W32; g++) {
    const int x = 32 * g + lane;
    const bool valid = x < n;
    const unsigned same = __match_any_sync(BBS_FULL_MASK, valid ? dep[g] : -1);
    if (valid) {
      const int pos = hist[dep[g]] + __popc(same & below);
      ord[pos] = (uint16_t)(x | ((par != nullptr ? (int)par[x] : 0) << 8));
    }
    __syncwarp();
    if (valid && (same & below) == 0) hist[dep[g]] += __popc(same);
    __syncwarp();
  }
}

// The canonical order for counts inherited through a ring (rows of five to
// eight words): the positions of canonical_order, each entry node | ppos
// << 8 with ppos the order position of the node's parent, from `par`, the
// tree's parent vector (the root, at position 0, gets 0).  Returns whether
// every node lies fewer than kRing positions after its parent, so that the
// parent's counts are still in the ring when the node is reached; where
// not, ord still holds the canonical node order in its low bytes.  hist
// doubles as the node -> position map (32 ceil(n / 32) >= n ints).
template <int W32>
__device__ __forceinline__ bool ring_order(const uint32_t *rows, int n,
                                           const uint8_t *par, uint16_t *ord,
                                           int *hist, int lane) {
  constexpr int RS = rs_of_w32(W32);
  const int B = (n + 31) >> 5;
  for (int i = lane; i < 32 * B; i += 32) hist[i] = 0;
  __syncwarp();
  int dep[W32], at[W32];
#pragma unroll
  for (int g = 0; g < W32; g++) {
    const int x = 32 * g + lane;
    dep[g] = -1;
    at[g] = 0;
    if (x < n) {
      uint32_t a[W32];
      ld_row<W32>(rows + x * RS, a);
      int pc = 0;
#pragma unroll
      for (int k = 0; k < W32; k++) pc += __popc(a[k]);
      dep[g] = pc - 1;
      atomicAdd(&hist[pc - 1], 1);
    }
  }
  __syncwarp();
  int loc[W32], s = 0;
#pragma unroll
  for (int k = 0; k < W32; k++) {
    loc[k] = k < B ? hist[lane * B + k] : 0;
    s += loc[k];
  }
  int incl = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(BBS_FULL_MASK, incl, o);
    if (lane >= o) incl += v;
  }
  int run = incl - s;
  __syncwarp();
#pragma unroll
  for (int k = 0; k < W32; k++)
    if (k < B) {
      hist[lane * B + k] = run;
      run += loc[k];
    }
  __syncwarp();
  const unsigned below = (1u << lane) - 1u;
#pragma unroll
  for (int g = 0; g < W32; g++) {
    const int x = 32 * g + lane;
    const bool valid = x < n;
    const unsigned same = __match_any_sync(BBS_FULL_MASK, valid ? dep[g] : -1);
    if (valid) at[g] = hist[dep[g]] + __popc(same & below);
    __syncwarp();
    if (valid && (same & below) == 0) hist[dep[g]] += __popc(same);
    __syncwarp();
  }
  // node -> position, then the entries with their parents' positions
#pragma unroll
  for (int g = 0; g < W32; g++) {
    const int x = 32 * g + lane;
    if (x < n) hist[x] = at[g];
  }
  __syncwarp();
  bool ok = true;
#pragma unroll
  for (int g = 0; g < W32; g++) {
    const int x = 32 * g + lane;
    if (x < n) {
      const int pp = x == n - 1 ? 0 : hist[min((int)par[x], n - 1)];
      ord[at[g]] = (uint16_t)(x | (pp << 8));
      ok = ok && at[g] - pp < kRing;
    }
  }
  __syncwarp();
  return __all_sync(BBS_FULL_MASK, ok);
}

// The gene table of the lane's Q cells (layout in bbs_layout.h): gene j's
// increment of every cell is then (entry >> (j & 7)) & 0x01010101, word by
// word.  Each lane writes, and later reads, only its own column.
template <int W32, int Q>
__device__ __forceinline__ void build_gene_table(const Cells<W32, Q> &cb,
                                                 uint32_t *gt, int n,
                                                 int lane) {
  constexpr int NW = kPackWords<Q>;
#pragma unroll
  for (int w = 0; w < W32; w++) {
#pragma unroll
    for (int b = 0; b < 4; b++) {
      const int g8 = 4 * w + b;
      if (8 * g8 < n) {
        // byte b of D, then byte b of M, in the two low bytes
        const uint32_t sel = (uint32_t)b | ((uint32_t)(4 + b) << 4);
        uint32_t y[NW];
#pragma unroll
        for (int h = 0; h < NW; h++) {
          constexpr int top = Q - 1;
          const int qa = 2 * h, qb = 2 * h + 1 < Q ? 2 * h + 1 : top;
          const uint32_t lo = __byte_perm(cb.D[qa][w], cb.M[qa][w], sel);
          const uint32_t hi = 2 * h + 1 < Q
                                  ? __byte_perm(cb.D[qb][w], cb.M[qb][w], sel)
                                  : 0u;
          y[h] = __byte_perm(lo, hi, 0x5410u);
        }
        st_pack<Q>(gt, g8 * 32 + lane, y);
      }
    }
  }
}

// Gene j's packed increments of the lane's cells, from the gene table.
template <int Q>
__device__ __forceinline__ void gene_inc(const uint32_t *gt, int j, int lane,
                                         uint32_t (&g)[kPackWords<Q>]) {
  ld_pack<Q>(gt, (j >> 3) * 32 + lane, g);
  const uint32_t sh = (uint32_t)j & 7u;
#pragma unroll
  for (int w = 0; w < kPackWords<Q>; w++) g[w] = (g[w] >> sh) & 0x01010101u;
}

// The parent vector of the tree with ancestor rows `rows`: each node's
// deepest proper ancestor (the root is its own parent).  depth_tmp: n ints.
// Once per launch, so out of line.
template <int W32>
__device__ __noinline__ void derive_parents(const uint32_t *rows, int n,
                                               uint8_t *par, int *depth_tmp,
                                               int lane) {
  constexpr int RS = rs_of_w32(W32);
  for (int x = lane; x < n; x += 32) {
    uint32_t a[W32];
    ld_row<W32>(rows + x * RS, a);
    int pc = 0;
#pragma unroll
    for (int k = 0; k < W32; k++) pc += __popc(a[k]);
    depth_tmp[x] = pc;
  }
  __syncwarp();
  for (int x = lane; x < n; x += 32) {
    uint32_t a[W32];
    ld_row<W32>(rows + x * RS, a);
    int best = x, bd = -1;
#pragma unroll
    for (int k = 0; k < W32; k++) {
      uint32_t w = k == (x >> 5) ? a[k] & ~(1u << (x & 31)) : a[k];
      while (w != 0u) {  // at most 32 set bits
        const int y = 32 * k + __ffs(w) - 1;
        w &= w - 1u;
        if (depth_tmp[y] > bd) {
          bd = depth_tmp[y];
          best = y;
        }
      }
    }
    par[x] = (uint8_t)best;
  }
  __syncwarp();
}

// The proposal's parent vector from the current one and the realised move,
// as the reference's own test restates each move on parent vectors
// (test/MutationTree.cpp:697-735).  `related`: w is an ancestor of v.
__device__ __forceinline__ void propose_parents(const uint8_t *cur,
                                                uint8_t *prop, int n,
                                                const bbs_move_params &p,
                                                bool related, int lane) {
  const uint32_t v = p.v, w = p.w;
  const bool swap_nodes = p.move_type == BBS_MOVE_SWAP_NODES;
  for (int x = lane; x < n; x += 32) {
    uint32_t q = cur[x];
    if (swap_nodes && (uint32_t)x != v && (uint32_t)x != w)
      q = q == v ? w : (q == w ? v : q);
    prop[x] = (uint8_t)q;
  }
  __syncwarp();
  if (lane == 0) {
    if (p.move_type == BBS_MOVE_PRUNE_REATTACH) {
      prop[v] = (uint8_t)p.nondescendant_of_v;
    } else if (swap_nodes) {
      const uint32_t pv = cur[v], pw = cur[w];
      if (pv == w) {
        prop[v] = (uint8_t)pw;
        prop[w] = (uint8_t)v;
      } else if (pw == v) {
        prop[w] = (uint8_t)pv;
        prop[v] = (uint8_t)w;
      } else {
        prop[v] = (uint8_t)pw;
        prop[w] = (uint8_t)pv;
      }
    } else if (p.move_type == BBS_MOVE_SWAP_SUBTREES) {
      prop[v] = (uint8_t)p.parent_of_w;
      prop[w] = (uint8_t)(related ? p.descendant_of_v : p.parent_of_v);
    }
  }
  __syncwarp();
}

// Whether `par` is the parent vector of the rows: every non-root node's row
// is its parent's row plus the node itself.  Once per evaluation, so out of
// line.
template <int W32>
__device__ __noinline__ bool parents_match_rows(const uint32_t *rows, int n,
                                                   const uint8_t *par,
                                                   int lane) {
  constexpr int RS = rs_of_w32(W32);
  bool ok = true;
  for (int x = lane; x < n - 1; x += 32) {
    const int p = par[x];
    if (p >= n) {
      ok = false;
      continue;
    }
    uint32_t a[W32], b[W32];
    ld_row<W32>(rows + x * RS, a);
    ld_row<W32>(rows + p * RS, b);
#pragma unroll
    for (int k = 0; k < W32; k++) {
      const uint32_t own = k == (x >> 5) ? 1u << (x & 31) : 0u;
      ok = ok && a[k] == (b[k] | own) && (b[k] & own) == 0u;
    }
  }
  return __all_sync(BBS_FULL_MASK, ok);
}

// Inherited counts of the nodes at order positions i and i + 1, all Q
// cells at once (packed), stored in the count table.  All four loads come
// first; when node i + 1 is node i's child, its parent's counts are taken
// from the register instead of the table (whose entry is not stored yet).
template <int Q, int NW = kPackWords<Q>>
__device__ __forceinline__ void inherit_pair(const SumCtx &sx, int i, int lane,
                                             uint32_t (&k0)[NW],
                                             uint32_t (&k1)[NW], int &j0,
                                             int &j1) {
  const uint32_t o0 = sx.ord[i], o1 = sx.ord[i + 1];
  j0 = (int)(o0 & 0xFF);
  j1 = (int)(o1 & 0xFF);
  const int p0 = (int)(o0 >> 8), p1 = (int)(o1 >> 8);
  uint32_t a0[NW], a1[NW], g0[NW], g1[NW];
  ld_pack<Q>(sx.cnt, p0 * 32 + lane, a0);
  ld_pack<Q>(sx.cnt, p1 * 32 + lane, a1);
  ld_pack<Q>(sx.inc, j0 * 32 + lane, g0);
  ld_pack<Q>(sx.inc, j1 * 32 + lane, g1);
#pragma unroll
  for (int w = 0; w < NW; w++) {
    k0[w] = a0[w] + g0[w];
    k1[w] = (p1 == j0 ? k0[w] : a1[w]) + g1[w];
  }
  st_pack<Q>(sx.cnt, j0 * 32 + lane, k0);
  st_pack<Q>(sx.cnt, j1 * 32 + lane, k1);
}

// The same for the node at order position i alone.
template <int Q, int NW = kPackWords<Q>>
__device__ __forceinline__ void inherit_one(const SumCtx &sx, int i, int lane,
                                            uint32_t (&k)[NW], int &j) {
  const uint32_t o = sx.ord[i];
  j = (int)(o & 0xFF);
  const int p = (int)(o >> 8);
  uint32_t a[NW], g[NW];
  ld_pack<Q>(sx.cnt, p * 32 + lane, a);
  ld_pack<Q>(sx.inc, j * 32 + lane, g);
#pragma unroll
  for (int w = 0; w < NW; w++) k[w] = a[w] + g[w];
  st_pack<Q>(sx.cnt, j * 32 + lane, k);
}

// inherit_pair for rows of five to eight words: the parents' counts come
// from the ring (entries hold the parents' order positions, ring_order),
// the increments from the gene table, and positions i and i + 1 are stored
// in the ring.  Why no load reads an overwritten entry: when the loads run,
// positions up to i - 1 are stored (each lane reads and writes only its own
// column, in program order).  A parent at position p < i was stored at
// entry p % kRing, and the positions stored since, p + 1 .. i - 1, are
// fewer than kRing (ring_order checked i + 1 - p < kRing), so none of them
// maps to that entry.  A parent at position i, not stored yet, is taken
// from the register.
template <int Q, int NW = kPackWords<Q>>
__device__ __forceinline__ void inherit_pair_ring(const SumCtx &sx, int i,
                                                  int lane,
                                                  uint32_t (&k0)[NW],
                                                  uint32_t (&k1)[NW], int &j0,
                                                  int &j1) {
  const uint32_t o0 = sx.ord[i], o1 = sx.ord[i + 1];
  j0 = (int)(o0 & 0xFF);
  j1 = (int)(o1 & 0xFF);
  const int p0 = (int)(o0 >> 8), p1 = (int)(o1 >> 8);
  uint32_t a0[NW], a1[NW], g0[NW], g1[NW];
  ld_pack<Q>(sx.ring, (p0 & (kRing - 1)) * 32 + lane, a0);
  ld_pack<Q>(sx.ring, (p1 & (kRing - 1)) * 32 + lane, a1);
  gene_inc<Q>(sx.gt, j0, lane, g0);
  gene_inc<Q>(sx.gt, j1, lane, g1);
#pragma unroll
  for (int w = 0; w < NW; w++) {
    k0[w] = a0[w] + g0[w];
    k1[w] = (p1 == i ? k0[w] : a1[w]) + g1[w];
  }
  st_pack<Q>(sx.ring, (i & (kRing - 1)) * 32 + lane, k0);
  st_pack<Q>(sx.ring, ((i + 1) & (kRing - 1)) * 32 + lane, k1);
}

template <int Q, int NW = kPackWords<Q>>
__device__ __forceinline__ void inherit_one_ring(const SumCtx &sx, int i,
                                                 int lane, uint32_t (&k)[NW],
                                                 int &j) {
  const uint32_t o = sx.ord[i];
  j = (int)(o & 0xFF);
  const int p = (int)(o >> 8);
  uint32_t a[NW], g[NW];
  ld_pack<Q>(sx.ring, (p & (kRing - 1)) * 32 + lane, a);
  gene_inc<Q>(sx.gt, j, lane, g);
#pragma unroll
  for (int w = 0; w < NW; w++) k[w] = a[w] + g[w];
  st_pack<Q>(sx.ring, (i & (kRing - 1)) * 32 + lane, k);
}

// The two count sources by inheritance: the table of every node (rows of
// up to four words) or the ring.
template <int Q, bool RING, int NW = kPackWords<Q>>
__device__ __forceinline__ void inherit2(const SumCtx &sx, int i, int lane,
                                         uint32_t (&k0)[NW],
                                         uint32_t (&k1)[NW], int &j0,
                                         int &j1) {
  if constexpr (RING)
    inherit_pair_ring<Q>(sx, i, lane, k0, k1, j0, j1);
  else
    inherit_pair<Q>(sx, i, lane, k0, k1, j0, j1);
}

template <int Q, bool RING, int NW = kPackWords<Q>>
__device__ __forceinline__ void inherit1(const SumCtx &sx, int i, int lane,
                                         uint32_t (&k)[NW], int &j) {
  if constexpr (RING)
    inherit_one_ring<Q>(sx, i, lane, k, j);
  else
    inherit_one<Q>(sx, i, lane, k, j);
}

// The root's zero counts, at order position 0.
template <int Q, bool RING, int NW = kPackWords<Q>>
__device__ __forceinline__ void store_root(const SumCtx &sx, int lane) {
  uint32_t zero[NW];
#pragma unroll
  for (int w = 0; w < NW; w++) zero[w] = 0u;
  if constexpr (RING)
    st_pack<Q>(sx.ring, lane, zero);
  else
    st_pack<Q>(sx.cnt, (int)(sx.ord[0] & 0xFF) * 32 + lane, zero);
}

// The sum score's float work of two nodes, side by side in the halves of
// paired registers, for the lane's Q cells: t = base + d c1 + m c2, its
// power of two, the running maximum of t, and the sums of 2^t, 2^t d and
// 2^t m, each kept as two partial sums (the nodes in the .x halves and
// those in the .y halves) that are added at the end.  Both count sources
// call this, so the sums are the same whichever found the counts.
template <int Q>
__device__ __forceinline__ void sum_pair2(const float2 (&fd)[Q],
                                          const float2 (&fm)[Q], float2 c1,
                                          float2 c2, const float2 (&base)[Q],
                                          float (&mx)[Q], float2 (&z)[Q],
                                          float2 (&ed)[Q], float2 (&em)[Q]) {
#pragma unroll
  for (int q = 0; q < Q; q++) {
    const float2 t = ffma2(fd[q], c1, ffma2(fm[q], c2, base[q]));
    const float2 e = make_float2(ex2_approx(t.x), ex2_approx(t.y));
    mx[q] = fmax3(mx[q], t.x, t.y);
    z[q] = fadd2(z[q], e);
    ed[q] = ffma2(e, fd[q], ed[q]);
    em[q] = ffma2(e, fm[q], em[q]);
  }
}

// The exact float counts (d, m) of the lane's Q cells at two nodes from
// their packed entries (node 0 in .x, node 1 in .y).
template <int Q, int NW>
__device__ __forceinline__ void pack_to_float2(const uint32_t (&k0)[NW],
                                               const uint32_t (&k1)[NW],
                                               float2 (&fd)[Q],
                                               float2 (&fm)[Q]) {
  const float2 bias = dup2(8388608.0f);
#pragma unroll
  for (int q = 0; q < Q; q++) {
    fd[q] = fsub2(make_float2(pack_d_biased(k0[q >> 1], q),
                              pack_d_biased(k1[q >> 1], q)), bias);
    fm[q] = fsub2(make_float2(pack_m_biased(k0[q >> 1], q),
                              pack_m_biased(k1[q >> 1], q)), bias);
  }
}

// sum_pair2 on two nodes' packed counts.
template <int Q, int NW>
__device__ __forceinline__ void sum_counts2(const uint32_t (&k0)[NW],
                                            const uint32_t (&k1)[NW],
                                            float2 c1, float2 c2,
                                            const float2 (&base)[Q],
                                            float (&mx)[Q], float2 (&z)[Q],
                                            float2 (&ed)[Q], float2 (&em)[Q]) {
  float2 fd[Q], fm[Q];
  pack_to_float2<Q, NW>(k0, k1, fd, fm);
  sum_pair2<Q>(fd, fm, c1, c2, base, mx, z, ed, em);
}

// Q floats, passed and returned by value.
template <int Q>
struct QF {
  float v[Q];
};

template <int Q>
struct QI {
  int v[Q];
};

template <int Q>
struct Resum {
  QF<Q> z, ed, em;
};

// The second pass of the cells in `bad` (bit q: cell slot q), each against
// its own maximum (base already shifted), one node at a time in the
// canonical order.  Rarely taken, so kept out of line: the node loop's code
// stays small, and the cells come by value.
template <int W32, int Q, bool INHERIT>
__device__ __noinline__ Resum<Q> resum_cells(const uint32_t *rows, int n,
                                             const Cells<W32, Q> cb,
                                             const SumCtx sx, int lane,
                                             float c1, float c2,
                                             const QF<Q> base, unsigned bad) {
  constexpr int RS = rs_of_w32(W32);
  constexpr int NW = kPackWords<Q>;
  Resum<Q> o;
#pragma unroll
  for (int q = 0; q < Q; q++) o.z.v[q] = o.ed.v[q] = o.em.v[q] = 0.0f;
#pragma unroll 1
  for (int i2 = 0; i2 < n; i2++) {
    const int j = (int)(sx.ord[i2] & 0xFF);
    uint32_t a[W32], k[NW];
    if constexpr (!INHERIT) ld_row<W32>(rows + j * RS, a);
    if constexpr (INHERIT) ld_pack<Q>(sx.cnt, j * 32 + lane, k);
#pragma unroll
    for (int q = 0; q < Q; q++) {
      if (!((bad >> q) & 1u)) continue;
      float fd, fm;
      if constexpr (INHERIT) {
        fd = pack_d_biased(k[q >> 1], q) - 8388608.0f;
        fm = pack_m_biased(k[q >> 1], q) - 8388608.0f;
      } else {
        fd = __int_as_float(0x4B000000 + masked_popc<W32>(cb.D[q], a)) - 8388608.0f;
        fm = __int_as_float(0x4B000000 + masked_popc<W32>(cb.M[q], a)) - 8388608.0f;
      }
      const float e = ex2_approx(fmaf(fd, c1, fmaf(fm, c2, base.v[q])));
      o.z.v[q] += e;
      o.ed.v[q] = fmaf(e, fd, o.ed.v[q]);
      o.em.v[q] = fmaf(e, fm, o.em.v[q]);
    }
  }
  return o;
}

// resum_cells for the ring: the counts inherited once more along the
// order (the chunk's gene table is still in place), the same terms summed
// in the same order as resum_cells, so the sums are those of the other
// count sources.
template <int Q>
__device__ __noinline__ Resum<Q> resum_cells_ring(int n, const SumCtx sx,
                                                  int lane, float c1,
                                                  float c2, const QF<Q> base,
                                                  unsigned bad) {
  constexpr int NW = kPackWords<Q>;
  Resum<Q> o;
#pragma unroll
  for (int q = 0; q < Q; q++) o.z.v[q] = o.ed.v[q] = o.em.v[q] = 0.0f;
  store_root<Q, true>(sx, lane);
#pragma unroll 1
  for (int i2 = 0; i2 < n; i2++) {
    uint32_t k[NW];
    if (i2 == 0) {
#pragma unroll
      for (int w = 0; w < NW; w++) k[w] = 0u;
    } else {
      int j;
      inherit_one_ring<Q>(sx, i2, lane, k, j);
    }
#pragma unroll
    for (int q = 0; q < Q; q++) {
      if (!((bad >> q) & 1u)) continue;
      const float fd = pack_d_biased(k[q >> 1], q) - 8388608.0f;
      const float fm = pack_m_biased(k[q >> 1], q) - 8388608.0f;
      const float e = ex2_approx(fmaf(fd, c1, fmaf(fm, c2, base.v[q])));
      o.z.v[q] += e;
      o.ed.v[q] = fmaf(e, fd, o.ed.v[q]);
      o.em.v[q] = fmaf(e, fm, o.em.v[q]);
    }
  }
  return o;
}

// Lane sums of k and m at the chosen nodes of cells it loads itself.
template <int W32, int Q>
__device__ __noinline__ int2 counts_at_reload(const uint32_t *rows,
                                              const DatasetDev *ds, int c0,
                                              int stride, const QI<Q> bj,
                                              int lane) {
  Cells<W32, Q> cb;
  load_cells<W32, Q>(cb, *ds, c0, stride, lane);
  int k = 0, m = 0;
  counts_at<W32, Q>(rows, cb, bj.v, k, m);
  return make_int2(k, m);
}

template <int W32, int Q, bool INHERIT, bool RING = false>
__device__ __forceinline__ void sum_cells(const uint32_t *rows, int n,
                                          const Cells<W32, Q> &cb,
                                          const LogTable &L, int c0, int stride,
                                          int lane, int n_cells,
                                          long long (&acc)[6],
                                          const SumCtx &sx) {
  constexpr int RS = rs_of_w32(W32);
  constexpr int NW = kPackWords<Q>;
  const float c1 = (L.l01 - L.l00) * kLog2E;  // per counted observed-0 bit
  const float c2 = (L.l11 - L.l10) * kLog2E;  // per counted observed-1 bit
  const float2 c1p = dup2(c1), c2p = dup2(c2);
  const float u0 = fmaxf(L.l00, L.l01), u1 = fmaxf(L.l10, L.l11);
  float r[Q], base[Q], mx[Q];
  float2 base2[Q], z2[Q], ed2[Q], em2[Q];
#pragma unroll
  for (int q = 0; q < Q; q++) {
    const float pd = cb.pdb[q] - 8388608.0f, pm = cb.pmb[q] - 8388608.0f;
    r[q] = fmaf(pd, u0, pm * u1) - 72.0f;
    base[q] = (fmaf(pd, L.l00, pm * L.l10) - r[q]) * kLog2E;
    base2[q] = dup2(base[q]);
  }
  // the root (ord[0]) has no counted bits: t = base
  if constexpr (INHERIT) store_root<Q, RING>(sx, lane);
#pragma unroll
  for (int q = 0; q < Q; q++) {
    mx[q] = base[q];
    z2[q] = make_float2(ex2_approx(base[q]), 0.0f);
    ed2[q] = em2[q] = make_float2(0.0f, 0.0f);
  }
  // the other nodes two at a time, in the two halves of paired registers
  int i = 1;
  if constexpr (INHERIT) {
    // counts one pair ahead of the float work, which hides the table's
    // load latency behind the previous pair's arithmetic; two pairs per
    // iteration, alternating between two register sets
    if (i + 1 < n) {
      uint32_t kA0[NW], kA1[NW], kB0[NW], kB1[NW];
      int jA0, jA1, jB0, jB1;  // node numbers (the max score uses them)
      inherit2<Q, RING>(sx, i, lane, kA0, kA1, jA0, jA1);
#pragma unroll 1
      for (; i + 5 < n; i += 4) {
        inherit2<Q, RING>(sx, i + 2, lane, kB0, kB1, jB0, jB1);
        sum_counts2<Q, NW>(kA0, kA1, c1p, c2p, base2, mx, z2, ed2, em2);
        inherit2<Q, RING>(sx, i + 4, lane, kA0, kA1, jA0, jA1);
        sum_counts2<Q, NW>(kB0, kB1, c1p, c2p, base2, mx, z2, ed2, em2);
      }
      if (i + 3 < n) {
        inherit2<Q, RING>(sx, i + 2, lane, kB0, kB1, jB0, jB1);
        sum_counts2<Q, NW>(kA0, kA1, c1p, c2p, base2, mx, z2, ed2, em2);
        sum_counts2<Q, NW>(kB0, kB1, c1p, c2p, base2, mx, z2, ed2, em2);
        i += 4;
      } else {
        sum_counts2<Q, NW>(kA0, kA1, c1p, c2p, base2, mx, z2, ed2, em2);
        i += 2;
      }
    }
  } else {
    // the order entries one pair ahead: the rows' addresses are known when
    // an iteration starts
    uint32_t o0 = 0, o1 = 0;
    if (i + 1 < n) {
      o0 = sx.ord[i];
      o1 = sx.ord[i + 1];
    }
#pragma unroll 1
    for (; i + 1 < n; i += 2) {
      const int j0 = (int)(o0 & 0xFF), j1 = (int)(o1 & 0xFF);
      if (i + 3 < n) {
        o0 = sx.ord[i + 2];
        o1 = sx.ord[i + 3];
      }
      float2 fd[Q], fm[Q];
      uint32_t a[W32], b[W32];
      ld_row<W32>(rows + j0 * RS, a);
      ld_row<W32>(rows + j1 * RS, b);
#pragma unroll
      for (int q = 0; q < Q; q++) {
        fd[q] = make_float2(
            __int_as_float(0x4B000000 + masked_popc<W32>(cb.D[q], a)) - 8388608.0f,
            __int_as_float(0x4B000000 + masked_popc<W32>(cb.D[q], b)) - 8388608.0f);
        fm[q] = make_float2(
            __int_as_float(0x4B000000 + masked_popc<W32>(cb.M[q], a)) - 8388608.0f,
            __int_as_float(0x4B000000 + masked_popc<W32>(cb.M[q], b)) - 8388608.0f);
      }
      sum_pair2<Q>(fd, fm, c1p, c2p, base2, mx, z2, ed2, em2);
    }
  }
  if (i < n) {
    float fd[Q], fm[Q];
    if constexpr (INHERIT) {
      uint32_t k[NW];
      int j;
      inherit1<Q, RING>(sx, i, lane, k, j);
#pragma unroll
      for (int q = 0; q < Q; q++) {
        fd[q] = pack_d_biased(k[q >> 1], q) - 8388608.0f;
        fm[q] = pack_m_biased(k[q >> 1], q) - 8388608.0f;
      }
    } else {
      const int j = (int)(sx.ord[i] & 0xFF);
      uint32_t a[W32];
      ld_row<W32>(rows + j * RS, a);
#pragma unroll
      for (int q = 0; q < Q; q++) {
        fd[q] = __int_as_float(0x4B000000 + masked_popc<W32>(cb.D[q], a)) - 8388608.0f;
        fm[q] = __int_as_float(0x4B000000 + masked_popc<W32>(cb.M[q], a)) - 8388608.0f;
      }
    }
#pragma unroll
    for (int q = 0; q < Q; q++) {
      const float t = fmaf(fd[q], c1, fmaf(fm[q], c2, base[q]));
      const float e = ex2_approx(t);
      mx[q] = fmaxf(mx[q], t);
      z2[q].x += e;
      ed2[q].x = fmaf(e, fd[q], ed2[q].x);
      em2[q].x = fmaf(e, fm[q], em2[q].x);
    }
  }
  float z[Q], ed[Q], em[Q];
  bool bad[Q], any = false;
#pragma unroll
  for (int q = 0; q < Q; q++) {
    z[q] = z2[q].x + z2[q].y;
    ed[q] = ed2[q].x + ed2[q].y;
    em[q] = em2[q].x + em2[q].y;
    bad[q] = !(mx[q] >= -80.0f * kLog2E);
    any |= bad[q];
  }
  if (__any_sync(BBS_FULL_MASK, any)) {
    // cells summed once more against their maximum, one node at a time in
    // the same order
    QF<Q> b2;
    unsigned badm = 0;
#pragma unroll
    for (int q = 0; q < Q; q++) {
      if (bad[q]) {
        r[q] = fmaf(mx[q], kLn2, r[q]);
        base[q] -= mx[q];
        mx[q] = 0.0f;
        badm |= 1u << q;
      }
      b2.v[q] = base[q];
    }
    // (the ring no longer holds every node: the counts are inherited once
    // more)
    Resum<Q> o;
    if constexpr (RING)
      o = resum_cells_ring<Q>(n, sx, lane, c1, c2, b2, badm);
    else
      o = resum_cells<W32, Q, INHERIT>(rows, n, cb, sx, lane, c1, c2, b2,
                                       badm);
#pragma unroll
    for (int q = 0; q < Q; q++)
      if (bad[q]) {
        z[q] = o.z.v[q];
        ed[q] = o.ed.v[q];
        em[q] = o.em.v[q];
      }
  }
#pragma unroll
  for (int q = 0; q < Q; q++) {
    const int c = c0 + stride * q + lane;
    if (c >= n_cells) continue;
    const float inv = __frcp_rn(z[q]);  // 1 / z, correctly rounded
    const float Ed = ed[q] * inv, Em = em[q] * inv;
    acc[0] += (long long)__float2int_rn((r[q] + logf(z[q])) * kScoreScale);
    // E[n00] and E[n10] follow from the chain's totals (class_sums)
    acc[2] += (long long)__float2int_rn(Ed * kFixScale);         // E[n01]
    acc[4] += (long long)__float2int_rn(Em * kFixScale);         // E[n11]
    acc[5] += (long long)__float2int_rn(fmaf(mx[q], kLn2, r[q]) * kScoreScale);
  }
}

// This warp's part of the sum score and expected counts (fixed point,
// warp-reduced), its terms added in the canonical order (sx.ord, built
// here).  Inherited counts serve cells held in registers when sx brings the
// parent vector, the count table and the increment table.
// The masked-popcount node loop, out of line: it serves only streamed cells
// and mixed launch groups (rows of up to four words), trees whose order
// does not fit the ring or whose parent vector is not known (wider rows),
// and keeping one copy of it outside the chain kernels leaves the
// inherited-count loops and the step code small.
struct Acc6 {
  long long v[6];
};

template <int W32, int Q>
__device__ __noinline__ Acc6 sum_cells_popc(const uint32_t *rows, int n,
                                            const Cells<W32, Q> cb,
                                            const LogTable L, int c0,
                                            int stride, int lane, int n_cells,
                                            const SumCtx sx) {
  long long acc[6] = {0, 0, 0, 0, 0, 0};
  sum_cells<W32, Q, false>(rows, n, cb, L, c0, stride, lane, n_cells, acc, sx);
  Acc6 o;
#pragma unroll
  for (int i = 0; i < 6; i++) o.v[i] = acc[i];
  return o;
}

template <int W32, int Q>
__device__ __forceinline__ void sum_part(const uint32_t *rows, int n,
                                         const DatasetDev &ds,
                                         Cells<W32, Q> &cb, bool resident,
                                         const LogTable &L, int wpc, int wic,
                                         int lane, long long (&acc)[6],
                                         const SumCtx &sx) {
#pragma unroll
  for (int i = 0; i < 6; i++) acc[i] = 0;
  if constexpr (W32 > 4) {
    // rows of five to eight words: counts through the ring where the
    // tree's parent vector is known and its order fits the ring, the cells
    // streamed in chunks with a gene table built per chunk
    bool ring = false;
    if (sx.ring != nullptr && sx.par != nullptr)
      ring = ring_order<W32>(rows, n, sx.par, sx.ord, sx.hist, lane);
    else
      canonical_order<W32>(rows, n, sx.par, sx.ord, sx.hist, lane);
    if (ring) {
      const int span = 32 * wpc * Q;
      for (int c0 = 0; c0 < ds.n_cells; c0 += span) {
        Cells<W32, Q> cc;
        load_cells<W32, Q>(cc, ds, c0 + 32 * wic, 32 * wpc, lane);
        build_gene_table<W32, Q>(cc, sx.gt, n, lane);
        sum_cells<W32, Q, true, true>(rows, n, cc, L, c0 + 32 * wic, 32 * wpc,
                                      lane, ds.n_cells, acc, sx);
      }
      acc[0] = warp_sum_ll(acc[0]);
      acc[2] = warp_sum_ll(acc[2]);
      acc[4] = warp_sum_ll(acc[4]);
      acc[5] = warp_sum_ll(acc[5]);
      return;
    }
  } else {
    canonical_order<W32>(rows, n, sx.par, sx.ord, sx.hist, lane);
  }
  if (resident) {
    bool inherit = false;
    if constexpr (W32 <= 4)
      inherit = sx.cnt != nullptr && sx.inc != nullptr && sx.par != nullptr;
    if (inherit) {
      if constexpr (W32 <= 4)
        sum_cells<W32, Q, true>(rows, n, cb, L, 32 * wic, 32 * wpc, lane,
                                ds.n_cells, acc, sx);
    } else {
      const Acc6 o = sum_cells_popc<W32, Q>(rows, n, cb, L, 32 * wic,
                                            32 * wpc, lane, ds.n_cells, sx);
#pragma unroll
      for (int k = 0; k < 6; k++) acc[k] += o.v[k];
    }
  } else {
    const int span = 32 * wpc * Q;
    for (int c0 = 0; c0 < ds.n_cells; c0 += span) {
      load_cells<W32, Q>(cb, ds, c0 + 32 * wic, 32 * wpc, lane);
      const Acc6 o = sum_cells_popc<W32, Q>(rows, n, cb, L, c0 + 32 * wic,
                                            32 * wpc, lane, ds.n_cells, sx);
#pragma unroll
      for (int k = 0; k < 6; k++) acc[k] += o.v[k];
    }
  }
  acc[0] = warp_sum_ll(acc[0]);
  acc[2] = warp_sum_ll(acc[2]);
  acc[4] = warp_sum_ll(acc[4]);
  acc[5] = warp_sum_ll(acc[5]);
}

// Max score with inherited counts (rows of up to four words, cells in
// registers): the nodes in the canonical order with their counts found one
// pair ahead as for the sum score, each node's score in the reference's
// order, and the first maximum in node-index order -- an equal score at a
// lower index wins, which is what std::max over the nodes in index order
// keeps (src/TreeScorer.hpp:187-193) -- so the chosen nodes, and the class
// counts at them, are those of best_nodes.
__device__ __forceinline__ void max_select(float s, int j, float &best,
                                           int &bj) {
  const bool up = s > best || (s == best && j < bj);
  best = up ? s : best;
  bj = up ? j : bj;
}

// Two nodes' reference-order scores (node j0 in .x, j1 in .y) of the
// lane's Q cells from their packed counts, then the selection, j0 first.
template <int Q, int NW>
__device__ __forceinline__ void max_update2(const uint32_t (&k0)[NW], int j0,
                                            const uint32_t (&k1)[NW], int j1,
                                            const float2 (&pdb)[Q],
                                            const float2 (&pmb)[Q],
                                            const LogTable2 &L2,
                                            float (&best)[Q], int (&bj)[Q]) {
#pragma unroll
  for (int q = 0; q < Q; q++) {
    const float2 db = make_float2(pack_d_biased(k0[q >> 1], q),
                                  pack_d_biased(k1[q >> 1], q));
    const float2 mb = make_float2(pack_m_biased(k0[q >> 1], q),
                                  pack_m_biased(k1[q >> 1], q));
    const float2 s = pair_score_b2(db, mb, pdb[q], pmb[q], L2);
    max_select(s.x, j0, best[q], bj[q]);
    max_select(s.y, j1, best[q], bj[q]);
  }
}

template <int W32, int Q, bool RING = false>
__device__ __forceinline__ void max_cells_inherit(const uint32_t *rows, int n,
                                                  const Cells<W32, Q> &cb,
                                                  const LogTable &L, float nz,
                                                  int lane, const SumCtx &sx,
                                                  int &k, int &m,
                                                  QI<Q> *chosen = nullptr) {
  constexpr int NW = kPackWords<Q>;
  const LogTable2 L2 = log_table2(L, nz);
  float best[Q];
  int bj[Q];
  float2 pdb[Q], pmb[Q];
  {
    const int root = (int)(sx.ord[0] & 0xFF);
    store_root<Q, RING>(sx, lane);
#pragma unroll
    for (int q = 0; q < Q; q++) {
      best[q] = pair_score(0, 0, cb.pdb[q], cb.pmb[q], L.l00, L.l01, L.l10,
                           L.l11);
      bj[q] = root;
      pdb[q] = dup2(cb.pdb[q]);
      pmb[q] = dup2(cb.pmb[q]);
    }
  }
  int i = 1;
  if (i + 1 < n) {
    uint32_t kA0[NW], kA1[NW], kB0[NW], kB1[NW];
    int jA0, jA1, jB0, jB1;
    inherit2<Q, RING>(sx, i, lane, kA0, kA1, jA0, jA1);
#pragma unroll 1
    for (; i + 5 < n; i += 4) {
      inherit2<Q, RING>(sx, i + 2, lane, kB0, kB1, jB0, jB1);
      max_update2<Q, NW>(kA0, jA0, kA1, jA1, pdb, pmb, L2, best, bj);
      inherit2<Q, RING>(sx, i + 4, lane, kA0, kA1, jA0, jA1);
      max_update2<Q, NW>(kB0, jB0, kB1, jB1, pdb, pmb, L2, best, bj);
    }
    if (i + 3 < n) {
      inherit2<Q, RING>(sx, i + 2, lane, kB0, kB1, jB0, jB1);
      max_update2<Q, NW>(kA0, jA0, kA1, jA1, pdb, pmb, L2, best, bj);
      max_update2<Q, NW>(kB0, jB0, kB1, jB1, pdb, pmb, L2, best, bj);
      i += 4;
    } else {
      max_update2<Q, NW>(kA0, jA0, kA1, jA1, pdb, pmb, L2, best, bj);
      i += 2;
    }
  }
  if (i < n) {
    uint32_t kk[NW];
    int j;
    inherit1<Q, RING>(sx, i, lane, kk, j);
#pragma unroll
    for (int q = 0; q < Q; q++) {
      const float s = pair_score_b(pack_d_biased(kk[q >> 1], q),
                                   pack_m_biased(kk[q >> 1], q), cb.pdb[q],
                                   cb.pmb[q], L.l00, L.l01, L.l10, L.l11);
      max_select(s, j, best[q], bj[q]);
    }
  }
  // the counts at the chosen nodes: k = popc(K & A) = d + m (the ring no
  // longer holds every node: the caller takes masked popcounts then)
  if constexpr (RING) {
#pragma unroll
    for (int q = 0; q < Q; q++) chosen->v[q] = bj[q];
  } else {
#pragma unroll
    for (int q = 0; q < Q; q++) {
      uint32_t c[NW];
      ld_pack<Q>(sx.cnt, bj[q] * 32 + lane, c);
      const uint32_t f = pack_field<NW>(c, q);
      k += (int)(f & 0xFFu) + (int)(f >> 8);
      m += (int)(f >> 8);
    }
  }
}

// The max score's masked-popcount pass over one chunk of cells it loads
// itself: lane sums of k and m at the chosen nodes.
template <int W32, int Q>
__device__ __noinline__ int2 max_chunk_popc(const uint32_t *rows, int n,
                                            const DatasetDev *ds, int c0,
                                            int stride, const LogTable L,
                                            int lane) {
  Cells<W32, Q> cb;
  load_cells<W32, Q>(cb, *ds, c0, stride, lane);
  int bj[Q], k = 0, m = 0;
  best_nodes<W32, Q>(rows, n, cb, L.l00, L.l01, L.l10, L.l11, ds->neg_zero,
                     bj);
  counts_at<W32, Q>(rows, cb, bj, k, m);
  return make_int2(k, m);
}

// This warp's part of the class sums over its cells (max score).  Cells
// are split over the `wpc` warps of a chain: cell = c0 + 32*wpc*q +
// 32*wic + lane.  With `resident`, cb already holds the warp's cells.
template <int W32, int Q>
__device__ __forceinline__ void score_part(const uint32_t *rows, int n,
                                           const DatasetDev &ds,
                                           Cells<W32, Q> &cb, bool resident,
                                           const LogTable &L, int wpc,
                                           int wic, int lane, int &sk,
                                           int &sm, const SumCtx &sx) {
  int k = 0, m = 0, bj[Q];
  if constexpr (W32 > 4) {
    // rows of five to eight words: counts through the ring, as for the sum
    // score
    if (sx.ring != nullptr && sx.par != nullptr &&
        ring_order<W32>(rows, n, sx.par, sx.ord, sx.hist, lane)) {
      const int span = 32 * wpc * Q;
      for (int c0 = 0; c0 < ds.n_cells; c0 += span) {
        QI<Q> chosen;
        {
          Cells<W32, Q> cc;
          load_cells<W32, Q>(cc, ds, c0 + 32 * wic, 32 * wpc, lane);
          build_gene_table<W32, Q>(cc, sx.gt, n, lane);
          max_cells_inherit<W32, Q, true>(rows, n, cc, L, ds.neg_zero, lane,
                                          sx, k, m, &chosen);
        }
        const int2 km = counts_at_reload<W32, Q>(rows, &ds, c0 + 32 * wic,
                                                 32 * wpc, chosen, lane);
        k += km.x;
        m += km.y;
      }
      sk = (int)__reduce_add_sync(BBS_FULL_MASK, (uint32_t)k);
      sm = (int)__reduce_add_sync(BBS_FULL_MASK, (uint32_t)m);
      return;
    }
  }
  bool inherit = false;
  if constexpr (W32 <= 4)
    inherit = resident && sx.cnt != nullptr && sx.inc != nullptr &&
              sx.par != nullptr;
  if (inherit) {
    if constexpr (W32 <= 4) {
      canonical_order<W32>(rows, n, sx.par, sx.ord, sx.hist, lane);
      max_cells_inherit<W32, Q>(rows, n, cb, L, ds.neg_zero, lane, sx, k,
                                  m);
    }
  } else if (resident) {
    best_nodes<W32, Q>(rows, n, cb, L.l00, L.l01, L.l10, L.l11, ds.neg_zero, bj);
    counts_at<W32, Q>(rows, cb, bj, k, m);
  } else {
    const int span = 32 * wpc * Q;
    for (int c0 = 0; c0 < ds.n_cells; c0 += span) {
      if constexpr (W32 > 4) {
        // (out of line: wider rows take their counts through the ring)
        const int2 km = max_chunk_popc<W32, Q>(rows, n, &ds, c0 + 32 * wic,
                                               32 * wpc, L, lane);
        k += km.x;
        m += km.y;
      } else {
        load_cells<W32, Q>(cb, ds, c0 + 32 * wic, 32 * wpc, lane);
        best_nodes<W32, Q>(rows, n, cb, L.l00, L.l01, L.l10, L.l11,
                           ds.neg_zero, bj);
        counts_at<W32, Q>(rows, cb, bj, k, m);
      }
    }
  }
  sk = (int)__reduce_add_sync(BBS_FULL_MASK, (uint32_t)k);
  sm = (int)__reduce_add_sync(BBS_FULL_MASK, (uint32_t)m);
}

// Class totals (n00, n01, n10, n11) from the sums.
__device__ __forceinline__ void class_totals(const DatasetDev &ds, int sk,
                                             int sm, int (&N)[4]) {
  N[0] = ds.sum_k - ds.sum_m - sk + sm;
  N[1] = sk - sm;
  N[2] = ds.sum_m - sm;
  N[3] = sm;
}

// ((l00*N00 + l01*N01) + l10*N10) + l11*N11 + prior, no contraction.
__device__ __forceinline__ float tree_score(const DatasetDev &ds, int sk,
                                           int sm, const LogTable &L,
                                           float prior) {
  int N[4];
  class_totals(ds, sk, sm, N);
  float t = __fmul_rn((float)N[0], L.l00);
  t = __fadd_rn(t, __fmul_rn((float)N[1], L.l01));
  t = __fadd_rn(t, __fmul_rn((float)N[2], L.l10));
  t = __fadd_rn(t, __fmul_rn((float)N[3], L.l11));
  return __fadd_rn(t, prior);
}

// The beta-dependent table entries (src/TreeScorer.hpp:136-137) and
// logscore_beta (src/TreeScorer.hpp:122-126) for a new beta.
__device__ __forceinline__ void beta_terms(const DatasetDev &ds, float beta,
                                           float &l01, float &l11,
                                           float &prior) {
  l01 = logf(beta);
  l11 = (float)log(1.0 - (double)beta);
  float r = __fadd_rn(ds.lg_ab, __fmul_rn(__fsub_rn(ds.bpa, 1.0f), logf(beta)));
  r = __fadd_rn(r, __fmul_rn(__fsub_rn(ds.bpb, 1.0f), logf(__fsub_rn(1.0f, beta))));
  r = __fsub_rn(r, ds.lg_a);
  prior = __fsub_rn(r, ds.lg_b);
}

// The same entries in single precision for the learned error moves (no
// reference counterpart to match, so no double-precision logs): the log
// table of a proposed (alpha, beta) and logscore_beta.
__device__ __forceinline__ void alpha_terms_f(float alpha, float &l00,
                                              float &l10) {
  l00 = log1pf(-alpha);
  l10 = logf(alpha);
}
__device__ __forceinline__ void beta_terms_f(const DatasetDev &ds, float beta,
                                             float &l01, float &l11,
                                             float &prior) {
  l01 = logf(beta);
  l11 = log1pf(-beta);
  float r = __fadd_rn(ds.lg_ab, __fmul_rn(__fsub_rn(ds.bpa, 1.0f), l01));
  r = __fadd_rn(r, __fmul_rn(__fsub_rn(ds.bpb, 1.0f), logf(__fsub_rn(1.0f, beta))));
  r = __fsub_rn(r, ds.lg_a);
  prior = __fsub_rn(r, ds.lg_b);
}

// ------------------------------------------------------------------------
// Error-rate moves in (a, b) = (logit alpha, logit beta).  The target is
//   gamma * S(alpha, beta) + log(alpha (1-alpha)) + log(beta (1-beta)),
// S = data term + log Beta prior(beta), the Jacobian terms making it the
// density of (a, b).  Expected (or, for the max score, exact) class counts
// e[4] = (n00, n01, n10, n11) give the gradient and a diagonal
// preconditioner M = 1 / (1 + curvature) from the same counts.
// ------------------------------------------------------------------------
struct ErrorGeom {
  float grad_a, grad_b, prec_a, prec_b;
};

__device__ __forceinline__ ErrorGeom error_geometry(const DatasetDev &ds,
                                                    float alpha, float beta,
                                                    float gamma,
                                                    const float (&e)[4]) {
  ErrorGeom g;
  const float va = alpha * (1.0f - alpha), vb = beta * (1.0f - beta);
  const float dS_da = -e[0] / (1.0f - alpha) + e[2] / alpha;
  const float dS_db = e[1] / beta - e[3] / (1.0f - beta) +
                      (ds.bpa - 1.0f) / beta - (ds.bpb - 1.0f) / (1.0f - beta);
  g.grad_a = gamma * va * dS_da + (1.0f - 2.0f * alpha);
  g.grad_b = gamma * vb * dS_db + (1.0f - 2.0f * beta);
  g.prec_a = 1.0f / (1.0f + gamma * (e[0] + e[2]) * va);
  g.prec_b = 1.0f / (1.0f + gamma * (e[1] + e[3] + fmaxf(ds.bpa + ds.bpb - 2.0f, 0.0f)) * vb);
  return g;
}

__device__ __forceinline__ float logit(float p) { return logf(p) - log1pf(-p); }
__device__ __forceinline__ float sigmoid(float x) { return 1.0f / (1.0f + __expf(-x)); }

// log q(to | from) of the (preconditioned, optionally gradient-drifted)
// Gaussian proposal, up to the constant shared by both directions.
__device__ __forceinline__ float log_q(float ta, float tb, float fa, float fb,
                                       const ErrorGeom &g, float eps,
                                       bool drift) {
  const float h = drift ? 0.5f * eps * eps : 0.0f;
  const float ra = ta - fa - h * g.prec_a * g.grad_a;
  const float rb = tb - fb - h * g.prec_b * g.grad_b;
  const float e2 = eps * eps;
  return -(ra * ra) / (2.0f * e2 * g.prec_a) - (rb * rb) / (2.0f * e2 * g.prec_b) -
         0.5f * (logf(g.prec_a) + logf(g.prec_b));
}

// Two standard normals from the move's two uniforms (Box-Muller); the
// record's raw_descendant_of_v / raw_nondescendant_of_v are unused by
// error moves, so recorded streams fix these draws too.
__device__ __forceinline__ void error_normals(const bbs_raw_move &raw,
                                              float &z0, float &z1) {
  const float u1 = fmaxf(1.0f - raw.raw_descendant_of_v, 1.0e-30f);
  const float r = sqrtf(-2.0f * logf(u1));
  float s, c;
  sincospif(2.0f * raw.raw_nondescendant_of_v, &s, &c);
  z0 = r * c;
  z1 = r * s;
}

}  // namespace bbs
