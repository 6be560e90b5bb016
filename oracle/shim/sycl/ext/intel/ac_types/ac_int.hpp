// Host-only stand-in for the subset of Intel's unsigned ac_int<W,false>
// that the reference's MutationTree/TreeScorer headers use: bit storage
// in 64-bit words, bit references, complement, AND, 64-bit slices,
// counter arithmetic and comparisons.  Test infrastructure: used only to
// compile the reference's own headers into oracle/_ref for pinning the
// oracle.
#pragma once
#include <array>
#include <cstdint>

template <int W, bool S> class ac_int {
  static_assert(!S, "only unsigned ac_int is provided");
  static constexpr int NW = (W + 63) / 64;
  std::array<uint64_t, NW> w_{};
  void trim() {
    if constexpr (W % 64 != 0)
      w_[NW - 1] &= (~0ull >> (64 - W % 64));
  }

public:
  ac_int() = default;
  ac_int(unsigned long long v) { w_[0] = v; trim(); }
  ac_int(unsigned long v) { w_[0] = v; trim(); }
  ac_int(unsigned v) { w_[0] = v; trim(); }
  ac_int(long long v) { fill_signed(v); }
  ac_int(long v) { fill_signed(v); }
  ac_int(int v) { fill_signed(v); }

  struct bit_ref {
    ac_int *a;
    int i;
    operator bool() const { return (a->w_[i / 64] >> (i % 64)) & 1u; }
    bit_ref &operator=(bool b) {
      uint64_t m = 1ull << (i % 64);
      if (b) a->w_[i / 64] |= m; else a->w_[i / 64] &= ~m;
      return *this;
    }
    bit_ref &operator=(const bit_ref &o) { return *this = bool(o); }
  };
  bit_ref operator[](unsigned i) { return bit_ref{this, (int)i}; }
  bool operator[](unsigned i) const { return (w_[i / 64] >> (i % 64)) & 1u; }

  ac_int bit_complement() const {
    ac_int r;
    for (int k = 0; k < NW; k++) r.w_[k] = ~w_[k];
    r.trim();
    return r;
  }
  ac_int operator&(const ac_int &o) const {
    ac_int r;
    for (int k = 0; k < NW; k++) r.w_[k] = w_[k] & o.w_[k];
    return r;
  }
  template <int SW> ac_int<SW, false> slc(int off) const {
    static_assert(SW == 64, "only 64-bit slices are provided");
    if (off % 64 == 0 && off / 64 < NW)
      return ac_int<SW, false>((unsigned long long)w_[off / 64]);
    unsigned long long r = 0;
    for (int b = 0; b < 64 && off + b < W; b++)
      if ((*this)[off + b]) r |= 1ull << b;
    return ac_int<SW, false>(r);
  }
  ac_int &operator+=(unsigned long long v) { w_[0] += v; trim(); return *this; }
  ac_int &operator+=(int v) { w_[0] += (uint64_t)(int64_t)v; trim(); return *this; }
  explicit operator float() const { return (float)w_[0]; }
  uint64_t to_uint64() const { return w_[0]; }
  uint64_t word(int k) const { return w_[k]; }
  void set_word(int k, uint64_t v) { w_[k] = v; trim(); }
  bool operator==(const ac_int &o) const { return w_ == o.w_; }
  bool operator!=(const ac_int &o) const { return !(w_ == o.w_); }
  bool operator==(long long v) const { return *this == ac_int(v); }
  bool operator==(int v) const { return *this == ac_int(v); }
  ac_int operator%(long long m) const { ac_int r; r.w_[0] = w_[0] % (uint64_t)m; return r; }

private:
  void fill_signed(long long v) {
    w_[0] = (uint64_t)v;
    for (int k = 1; k < NW; k++) w_[k] = v < 0 ? ~0ull : 0ull;
    trim();
  }
};
