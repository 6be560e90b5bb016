// Shared-memory layout of the chain kernels, walked on the host over every
// shape the launchers accept: node counts 2..256, 1..4 cells per lane,
// 1..4 warps per chain (one-warp chains 1..8 per block), both scores.  For
// each chain slot the pieces the kernels address -- the two row buffers,
// both parities of the per-warp partial sums, the flag word, the parent
// vectors, each warp's Philox blocks, node order, depth histogram and count
// table (or ring and gene table) --
// must lie inside the slot, be disjoint and be aligned for their element
// type; the block's increment tables (one per warp of a chain) must lie
// after the slots and inside the launch's dynamic shared memory, and the
// launch's size must be the one the host asks for (chain_launch_smem).  Prints "layout ok <cases>" or the first
// violation (exit status 1).
#include <cstdint>
#include <cstdio>
#include <vector>

#include "bbs_kernels.cuh"

namespace {

struct Piece {
  const char *name;
  size_t lo, hi;  // byte offsets [lo, hi) from the block's base
  size_t align;
};

long g_cases = 0;

bool fail(const char *what, int n, int q, int wpc, int cpb, bool sum,
          const char *a, const char *b = "") {
  std::printf("FAIL %s: n=%d q=%d wpc=%d cpb=%d sum=%d %s %s\n", what, n, q,
              wpc, cpb, (int)sum, a, b);
  return false;
}

// A packed table of n nodes x 32 lanes for q cells per lane at byte
// offset w: (q + 1) / 2 words per entry, read as one 32- or 64-bit access.
void add_table(std::vector<Piece> &all, const char *name, size_t w, int n,
               int q) {
  all.push_back({name, w, w + (size_t)bbs::pack_table_bytes(n, q),
                 (size_t)4 * ((q + 1) / 2)});
}

// One launch: cpb slots of wpc warps, the tables after them.  `counts`
// says whether the chains inherit counts: with rows of up to four words
// (cells in registers) the slots then carry count tables and the launch its
// increment tables; with wider rows (always) each warp carries a ring of
// kRing entries and a gene table of ceil(n / 8) entries.
bool check(int n, int q, int wpc, int cpb, bool sum, bool counts) {
  const int w32 = bbs::w32_of_nodes(n);
  const int rs = bbs::rs_of_w32(w32);
  const bool scratch = sum || counts;
  const int sb = bbs::slot_bytes(n, rs, wpc, scratch, w32, q, counts);
  const size_t tb = (size_t)bbs::table_bytes(n, w32, q, wpc, counts);
  const size_t total = (size_t)cpb * sb + tb;
  // the launchers' size, for the cell counts that give this `counts`
  const int cells = counts ? 32 * wpc * q : 32 * wpc * q + 1;
  if (bbs::inherits_counts(w32, cells, 32 * wpc * q) == counts &&
      (size_t)bbs::chain_launch_smem(n, cells, q, wpc, cpb, sum) != total)
    return fail("launch size differs from chain_launch_smem", n, q, wpc, cpb,
                sum, "");
  std::vector<uint8_t> smem(total + 16);
  uint8_t *base = smem.data();
  std::vector<Piece> all;
  if (sb % 16 != 0) return fail("slot size not a multiple of 16", n, q, wpc, cpb, sum, "");
  for (int s = 0; s < cpb; s++) {
    const size_t o = (size_t)s * sb;
    const size_t first = all.size();  // this slot's pieces start here
    const size_t rows = (size_t)4 * 2 * n * rs;
    const size_t part = o + rows;
    all.push_back({"rows", o, o + rows, 16});
    // partial sums: max score 12 words per warp and parity, read as ints
    // at [12 w] and [12 w + 1]; sum score 6 long longs per warp and parity
    const size_t pmax = (size_t)4 * (12 * wpc + 12 * (wpc - 1) + 2);
    const size_t psum = (size_t)8 * (6 * wpc + 6 * (wpc - 1) + 6);
    all.push_back({"partials", part, part + (sum ? psum : pmax), sum ? 8u : 4u});
    const size_t flag = part + (size_t)4 * 24 * wpc;
    if ((sum ? part + psum : part + pmax) > flag)
      return fail("partials overrun the flag", n, q, wpc, cpb, sum, "");
    all.push_back({"flag", flag, flag + 4, 4});
    // the batched kernel's unit word of a multi-warp slot
    all.push_back({"unit", flag + 4, flag + 8, 4});
    // each warp's Philox blocks (32 x 16 bytes) after the flag words
    for (int wic = 0; wic < wpc; wic++) {
      const size_t ph = flag + 16 + (size_t)bbs::kPhiloxBytes * wic;
      all.push_back({"philox", ph, ph + bbs::kPhiloxBytes, 16});
    }
    if (scratch) {
      for (int wic = 0; wic < wpc; wic++) {
        const bbs::SlotSum ss =
            bbs::slot_sum(base + o, n, rs, wpc, wic, w32, q, counts);
        auto off = [&](const void *p) {
          return (size_t)(static_cast<const uint8_t *>(p) - base);
        };
        if (wic == 0) {
          all.push_back({"par0", off(ss.par0), off(ss.par0) + n, 1});
          all.push_back({"par1", off(ss.par1), off(ss.par1) + n, 1});
        }
        all.push_back({"ord", off(ss.sx.ord), off(ss.sx.ord) + 2 * n, 2});
        // the histogram doubles as the depth scratch of the parent
        // derivation: n ints at least
        const size_t hist = (size_t)4 * 32 * ((n + 31) / 32);
        if (hist < (size_t)4 * n)
          return fail("histogram smaller than n ints", n, q, wpc, cpb, sum, "");
        all.push_back({"hist", off(ss.sx.hist), off(ss.sx.hist) + hist, 4});
        if (counts && w32 <= 4) {
          if (ss.sx.cnt == nullptr || ss.sx.ring != nullptr)
            return fail("no count table", n, q, wpc, cpb, sum, "");
          add_table(all, "cnt", off(ss.sx.cnt), n, q);
        } else if (counts) {
          if (ss.sx.ring == nullptr || ss.sx.gt == nullptr ||
              ss.sx.cnt != nullptr)
            return fail("no ring or gene table", n, q, wpc, cpb, sum, "");
          // entries [kRing][32] and [ceil(n / 8)][32], packed like counts
          add_table(all, "ring", off(ss.sx.ring), bbs::kRing, q);
          add_table(all, "gene table", off(ss.sx.gt), (n + 7) / 8, q);
        } else if (ss.sx.cnt != nullptr || ss.sx.ring != nullptr ||
                   ss.sx.gt != nullptr) {
          return fail("count table without inherited counts", n, q, wpc,
                      cpb, sum, "");
        }
      }
    }
    for (size_t i = first; i < all.size(); i++)
      if (all[i].lo < o || all[i].hi > o + sb)
        return fail("piece outside its slot", n, q, wpc, cpb, sum, all[i].name);
  }
  if (counts && w32 <= 4) {
    const size_t lo = (size_t)cpb * sb;
    if (tb != (size_t)wpc * bbs::inc_table_bytes(n, q))
      return fail("increment tables sized wrongly", n, q, wpc, cpb, sum, "");
    for (int wic = 0; wic < wpc; wic++)
      add_table(all, "inc", lo + (size_t)wic * bbs::inc_table_bytes(n, q), n,
                q);
  }
  for (size_t i = 0; i < all.size(); i++) {
    if (all[i].hi > total)
      return fail("piece past the launch's shared memory", n, q, wpc, cpb,
                  sum, all[i].name);
    if (all[i].lo % all[i].align != 0)
      return fail("misaligned piece", n, q, wpc, cpb, sum, all[i].name);
    for (size_t j = i + 1; j < all.size(); j++)
      if (all[i].lo < all[j].hi && all[j].lo < all[i].hi)
        return fail("overlapping pieces", n, q, wpc, cpb, sum, all[i].name,
                    all[j].name);
  }
  g_cases++;
  return true;
}

}  // namespace

int main() {
  for (int n = 2; n <= 256; n++)
    for (int q = 1; q <= bbs::kMaxQ; q++)
      for (int sum = 0; sum < 2; sum++)
        for (int counts = 0; counts < 2; counts++) {
          // plain kernel: one-warp chains 1..8 per block, or one chain of
          // 2..4 warps
          for (int cpb = 1; 32 * cpb <= bbs::kMaxBlockThreads; cpb++)
            if (!check(n, q, 1, cpb, sum != 0, counts != 0)) return 1;
          for (int wpc = 2; wpc <= 4; wpc++)
            if (!check(n, q, wpc, 1, sum != 0, counts != 0)) return 1;
        }
  // (the batched kernel's launches are one-warp slots, 1..8 per block, or
  // one slot of 2..4 warps: the cases of the plain kernel)
  std::printf("layout ok %ld\n", g_cases);
  return 0;
}
