// bbs_api.cu -- the C ABI (include/bbscite_gb300.h): contexts, argument
// checks, host tree helpers and the SCITE input format.  Every entry point
// catches everything and returns a status; nothing aborts across the ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <mutex>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "bbs_internal.h"
#include "bbs_layout.h"

using namespace bbs;

namespace {

thread_local std::string g_error;

int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_error = buf;
  return code;
}

int cuda_fail(int err, const char *what) {
  return fail(BBS_ERR_CUDA, "%s: %s", what,
              cudaGetErrorString((cudaError_t)err));
}

// A run's status words: a failed device check (bit 1, with its code, value
// and limit; BBS_CHECKED builds) or a cancelled run (bit 0).
int status_result(const int (&st)[kStatusWords]) {
  if (st[0] & 2)
    return fail(BBS_ERR_DEVICE_CHECK, "device check %d failed: %u is not below %u",
                st[1], (unsigned)st[2], (unsigned)st[3]);
  if (st[0] & 1) return fail(BBS_ERR_TIMEOUT, "the run was cancelled");
  return BBS_OK;
}

#define BBS_CUDA(call, what)                                   \
  do {                                                         \
    cudaError_t e_ = (call);                                   \
    if (e_ != cudaSuccess) return cuda_fail((int)e_, (what));  \
  } while (0)

inline uint32_t words64(uint32_t n) { return (n + 63u) / 64u; }
inline bool getb(const uint64_t *row, uint32_t i) {
  return (row[i >> 6] >> (i & 63u)) & 1u;
}
inline void setb(uint64_t *row, uint32_t i) { row[i >> 6] |= 1ull << (i & 63u); }

// Host Philox4x32-10 (same algorithm as the device sampler).
void philox(const uint32_t c_in[4], const uint32_t k_in[2], uint32_t out[4]) {
  uint32_t c0 = c_in[0], c1 = c_in[1], c2 = c_in[2], c3 = c_in[3];
  uint32_t k0 = k_in[0], k1 = k_in[1];
  for (int r = 0; r < 10; r++) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    c0 = n0;
    c1 = (uint32_t)p1;
    c2 = n2;
    c3 = (uint32_t)p0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

// Parent vector checks: entries < n, root (n-1) is its own parent, every
// node reaches the root.
int check_parent_vector(const uint32_t *pv, uint32_t n) {
  if (n < 2) return fail(BBS_ERR_INPUT, "a tree needs at least 2 nodes");
  if (pv[n - 1] != n - 1)
    return fail(BBS_ERR_INPUT, "the root %u must be its own parent", n - 1);
  for (uint32_t x = 0; x < n; x++) {
    if (pv[x] >= n)
      return fail(BBS_ERR_INPUT, "parent of node %u is %u >= %u", x, pv[x], n);
    uint32_t y = x, steps = 0;
    while (y != n - 1) {
      y = pv[y];
      if (++steps > n)
        return fail(BBS_ERR_INPUT, "the parent vector has a cycle at node %u", x);
    }
  }
  return BBS_OK;
}

// src/MutationTree.hpp:379-409 (after check_parent_vector).
void parent_to_matrix(const uint32_t *pv, uint32_t n, uint64_t *am,
                      uint64_t *dm) {
  const uint32_t W = words64(n), root = n - 1;
  if (am) std::memset(am, 0, sizeof(uint64_t) * W * n);
  if (dm) std::memset(dm, 0, sizeof(uint64_t) * W * n);
  for (uint32_t i = 0; i < n; i++) {
    uint32_t anc = i;
    while (anc != root) {
      if (am) setb(am + (size_t)anc * W, i);
      if (dm) setb(dm + (size_t)i * W, anc);
      anc = pv[anc];
    }
    if (am) {
      setb(am + (size_t)i * W, i);
      setb(am + (size_t)root * W, i);
    }
    if (dm) {
      setb(dm + (size_t)i * W, i);
      setb(dm + (size_t)i * W, root);
    }
  }
}

// Parent = the deepest proper ancestor; the root is its own parent.
void matrix_to_parent(const uint64_t *dm, uint32_t n, uint32_t *pv) {
  const uint32_t W = words64(n);
  std::vector<int> depth(n);
  for (uint32_t x = 0; x < n; x++) {
    int d = 0;
    for (uint32_t k = 0; k < W; k++) d += __builtin_popcountll(dm[x * W + k]);
    depth[x] = d;
  }
  for (uint32_t x = 0; x < n; x++) {
    uint32_t best = x;
    int bd = -1;
    for (uint32_t y = 0; y < n; y++)
      if (y != x && getb(dm + (size_t)x * W, y) && depth[y] > bd) {
        bd = depth[y];
        best = y;
      }
    pv[x] = best;
  }
}

void pruefer_decode(const uint32_t *code, uint32_t len, uint32_t *parent) {
  const uint32_t n = len + 2;
  std::vector<uint32_t> degree(n, 1);
  for (uint32_t i = 0; i < n; i++) parent[i] = n - 1;
  for (uint32_t i = 0; i < len; i++) degree[code[i]]++;
  // The smallest degree-1 node each step (src/MutationTree.hpp:454-463).
  std::vector<uint32_t> heap;
  for (uint32_t j = 0; j < n; j++)
    if (degree[j] == 1) heap.push_back(j);
  std::make_heap(heap.begin(), heap.end(), std::greater<uint32_t>());
  for (uint32_t i = 0; i < len; i++) {
    std::pop_heap(heap.begin(), heap.end(), std::greater<uint32_t>());
    const uint32_t j = heap.back();
    heap.pop_back();
    parent[j] = code[i];
    degree[code[i]]--;
    degree[j]--;
    if (degree[code[i]] == 1) {
      heap.push_back(code[i]);
      std::push_heap(heap.begin(), heap.end(), std::greater<uint32_t>());
    }
  }
  for (uint32_t i = 0; i < n; i++)
    if (degree[i] == 1) {
      parent[i] = n - 1;
      break;
    }
}

void random_parents(uint64_t seed, uint32_t n_genes, uint32_t n_trees,
                    uint32_t *out) {
  const uint32_t n = n_genes + 1;
  std::vector<uint32_t> code(n >= 2 ? n - 2 : 0);
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  for (uint32_t t = 0; t < n_trees; t++) {
    for (uint32_t i = 0; i < code.size(); i += 4) {
      const uint32_t ctr[4] = {i, t, 0x7265u /* tree stream */, 0u};
      uint32_t r[4];
      philox(ctr, key, r);
      for (uint32_t k = 0; k < 4 && i + k < code.size(); k++)
        code[i + k] = (uint32_t)(((uint64_t)r[k] * n) >> 32);
    }
    pruefer_decode(code.data(), (uint32_t)code.size(), out + (size_t)t * n);
  }
}

void newick_rec(const std::vector<std::vector<uint32_t>> &ch, uint32_t x,
                std::string &s) {
  if (!ch[x].empty()) {
    s += '(';
    for (size_t i = 0; i < ch[x].size(); i++) {
      newick_rec(ch, ch[x][i], s);
      if (i + 1 != ch[x].size()) s += ',';
    }
    s += ')';
  }
  s += std::to_string(x);
}

int put_string(const std::string &s, char *buf, size_t cap, size_t *len) {
  if (len) *len = s.size();
  if (buf && cap > 0) {
    const size_t k = std::min(cap - 1, s.size());
    std::memcpy(buf, s.data(), k);
    buf[k] = '\0';
  }
  return BBS_OK;
}

}  // namespace

// ------------------------------------------------------------------------
// Context
// ------------------------------------------------------------------------
struct bbs_ctx {
  int device = 0, n_sms = 0;
  int smem_sm = 0, smem_block = 0, smem_reserved = 0;  // per SM / block
  cudaStream_t stream = nullptr;
  uint32_t n_cells = 0, n_genes = 0, n_nodes = 0, W64 = 0, RS = 0;
  bbs_params params{};
  DatasetDev ds{};
  ModelDev md{};
  float terms[8] = {};  // (alpha_mean, beta_mean) log-table terms, host libm
  uint32_t *d_K = nullptr, *d_M = nullptr;
  DatasetDev *d_ds = nullptr;  // one-entry tables for the init kernel
  ModelDev *d_md = nullptr;
  float *d_terms = nullptr;
  uint32_t n_chains = 0;
  uint32_t *d_rows = nullptr, *d_best = nullptr;  // d_best: K slots per chain
  uint32_t K = 1;                  // co-optimal trees kept per chain
  uint64_t *d_lhash = nullptr;     // [n_chains][K] when K > 1
  float *d_lbeta = nullptr;
  ChainState *d_states = nullptr;
  int *d_status = nullptr;
  int *h_cancel = nullptr;        // mapped pinned flag
  int *d_cancel = nullptr;
  int q = 1, wpc = 1, cpb = 1;  // chain-kernel launch shape
  bool running = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0.0f;
  // scratch of the host-buffer scoring calls and its pinned host mirror,
  // scratch_cap bytes each; grows, never shrinks
  uint8_t *d_scratch = nullptr, *h_scratch = nullptr;
  size_t scratch_cap = 0;
  uint64_t fingerprint = 0;  // of the dataset and parameters (checkpoints)
};

namespace {

void free_chains(bbs_ctx *c) {
  cudaFree(c->d_rows);
  cudaFree(c->d_best);
  cudaFree(c->d_states);
  cudaFree(c->d_lhash);
  cudaFree(c->d_lbeta);
  c->d_rows = c->d_best = nullptr;
  c->d_states = nullptr;
  c->d_lhash = nullptr;
  c->d_lbeta = nullptr;
  c->n_chains = 0;
}

// Host values of the beta-dependent log-table entries and logscore_beta,
// exactly as src/TreeScorer.hpp:104-106, 122-126, 136-137 compute them.
void host_beta_terms(const DatasetDev &ds, float beta, float *l01, float *l11,
                     float *prior) {
  *l01 = logf(beta);
  *l11 = (float)std::log(1.0 - (double)beta);
  float r = ds.lg_ab;
  r = r + (ds.bpa - 1.0f) * logf(beta);
  r = r + (ds.bpb - 1.0f) * logf(1.0f - beta);
  r = r - ds.lg_a;
  r = r - ds.lg_b;
  *prior = r;
}

int check_params(const bbs_params *p) {
  if (!p) return fail(BBS_ERR_INPUT, "params is NULL");
  const float probs[4] = {p->prob_beta_change, p->prob_prune_n_reattach,
                          p->prob_swap_nodes, p->prob_swap_subtrees};
  for (float v : probs)
    if (!(v >= 0.0f)) return fail(BBS_ERR_INPUT, "Move probabilities may not be negative.");
  if (probs[0] + probs[1] + probs[2] + probs[3] == 0.0f)
    return fail(BBS_ERR_INPUT, "The sum of the move type probabilities is zero.");
  if (!(p->alpha_mean > 0.0f && p->alpha_mean < 1.0f))
    return fail(BBS_ERR_INPUT, "alpha must lie in (0, 1), got %g", p->alpha_mean);
  if (!(p->beta_mean > 0.0f && p->beta_mean < 1.0f))
    return fail(BBS_ERR_INPUT, "beta must lie in (0, 1), got %g", p->beta_mean);
  if (!(p->beta_sd > 0.0f)) return fail(BBS_ERR_INPUT, "beta_sd must be positive");
  if (p->score_mode > BBS_SCORE_SUM)
    return fail(BBS_ERR_INPUT, "unknown score mode %u", p->score_mode);
  if (p->error_move > BBS_ERROR_LANGEVIN)
    return fail(BBS_ERR_INPUT, "unknown error move %u", p->error_move);
  if (p->error_move != BBS_ERROR_BETA_WALK && !(p->error_step > 0.0f))
    return fail(BBS_ERR_INPUT, "error_step must be positive");
  if (p->treelist_size > BBS_MAX_TREELIST_PER_CHAIN)
    return fail(BBS_ERR_INPUT, "treelist_size %u above %d", p->treelist_size,
                BBS_MAX_TREELIST_PER_CHAIN);
  return BBS_OK;
}

// Host side of one dataset: cell rows (genes only, mutated within known),
// the scorer constants of src/TreeScorer.hpp:99-111, the move thresholds of
// src/Parameters.hpp:451-584 / src/RawMoveDistribution.hpp:119-131 and the
// log-table terms of (alpha_mean, beta_mean).  Device pointers are filled
// in by the caller.
struct HostDataset {
  std::vector<uint64_t> K, M;
  DatasetDev ds{};
  ModelDev md{};
  float terms[8] = {};
};

void prepare_dataset(const bbs_params *params, uint32_t n_cells,
                     uint32_t n_genes, const uint64_t *is_mutated,
                     const uint64_t *is_known, HostDataset &h) {
  const uint32_t n_nodes = n_genes + 1, W64 = words64(n_nodes);
  h.K.assign((size_t)n_cells * W64, 0);
  h.M.assign(h.K.size(), 0);
  int64_t sum_k = 0, sum_m = 0;
  for (uint32_t cell = 0; cell < n_cells; cell++)
    for (uint32_t k = 0; k < W64; k++) {
      uint64_t mask = ~0ull;
      const uint32_t lo = 64 * k;
      if (lo >= n_genes) mask = 0;
      else if (n_genes - lo < 64) mask = (1ull << (n_genes - lo)) - 1ull;
      const size_t i = (size_t)cell * W64 + k;
      h.K[i] = is_known[i] & mask;
      h.M[i] = is_mutated[i] & h.K[i];
      sum_k += __builtin_popcountll(h.K[i]);
      sum_m += __builtin_popcountll(h.M[i]);
    }
  const float alpha = params->alpha_mean, bm = params->beta_mean,
              sd = params->beta_sd;
  DatasetDev &ds = h.ds;
  ds.n_cells = (int)n_cells;
  ds.n_nodes = (int)n_nodes;
  ds.sum_k = (int)sum_k;
  ds.sum_m = (int)sum_m;
  ds.l00 = (float)std::log(1.0 - (double)alpha);
  ds.l10 = logf(alpha);
  ds.bpa = (float)(((double)(1.0f - bm) * std::pow((double)bm, 2.0) /
                    std::pow((double)sd, 2.0)) - (double)bm);
  ds.bpb = ds.bpa * ((1.0f / bm) - 1.0f);
  ds.lg_ab = logf(tgammaf(ds.bpa + ds.bpb));
  ds.lg_a = logf(tgammaf(ds.bpa));
  ds.lg_b = logf(tgammaf(ds.bpb));
  ds.neg_zero = -0.0f;
  const float sum = params->prob_beta_change + params->prob_prune_n_reattach +
                    params->prob_swap_nodes + params->prob_swap_subtrees;
  const float pb = params->prob_beta_change / sum;
  const float pp = params->prob_prune_n_reattach / sum;
  const float ps = params->prob_swap_nodes / sum;
  ModelDev &md = h.md;
  md.mp.cum_beta = pb;
  md.mp.cum_prune = pb + pp;
  md.mp.cum_swap = pb + pp + ps;
  md.mp.beta_jump_sd = sd / params->beta_jump_scaling_chi;
  md.gamma = params->gamma;
  md.score_mode = (int32_t)params->score_mode;
  md.error_move = (int32_t)params->error_move;
  md.error_step = params->error_step;
  md.treelist = (int32_t)std::max(1u, params->treelist_size);
  md.seed = params->seed;
  h.terms[0] = alpha;
  h.terms[1] = bm;
  h.terms[2] = ds.l00;
  h.terms[3] = ds.l10;
  host_beta_terms(ds, bm, &h.terms[4], &h.terms[5], &h.terms[6]);
  h.terms[7] = 0.0f;
}

int sync_stream(bbs_ctx *c, const char *what) {
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail((int)e, what);
  return BBS_OK;
}

template <typename T>
struct DevBuf {
  T *p = nullptr;
  ~DevBuf() { cudaFree(p); }
  cudaError_t alloc(size_t n) { return cudaMalloc((void **)&p, sizeof(T) * std::max<size_t>(n, 1)); }
};

// A piece of the context's scratch: its device address and the same
// offset in the pinned host mirror.
template <typename T>
struct Piece {
  T *d;
  T *h;
};

// Pieces of the context's scratch for one call of a host-buffer entry point
// (bbs_score_trees, bbs_apply_moves, bbs_sumscore_grad).  The call adds up
// its pieces with add(), reserves once, then takes them in the same order
// with take(); inputs come first and outputs last, so that each call moves
// one contiguous range each way between the pinned mirror and the device.
// The scratch only moves while nothing is taken, and a caller that scores
// one tree at a time allocates on its first call only.
class ScratchPlan {
 public:
  template <typename T>
  void add(size_t n) { bytes_ += piece(sizeof(T) * n); }
  int reserve(bbs_ctx *c) {
    c_ = c;
    off_ = 0;
    if (bytes_ <= c->scratch_cap) return BBS_OK;
    // every entry point drains the stream before it returns, so no copy or
    // kernel of an earlier call still uses the old scratch
    cudaFree(c->d_scratch);
    if (c->h_scratch) cudaFreeHost(c->h_scratch);
    c->d_scratch = c->h_scratch = nullptr;
    c->scratch_cap = 0;
    // half again as much, so that a slowly growing caller reallocates
    // rarely; the exact size when that much is not free
    for (const size_t cap : {bytes_ + bytes_ / 2, bytes_}) {
      cudaError_t e = cudaMalloc(&c->d_scratch, cap);
      if (e == cudaSuccess) e = cudaHostAlloc(&c->h_scratch, cap, cudaHostAllocDefault);
      if (e == cudaSuccess) {
        c->scratch_cap = cap;
        return BBS_OK;
      }
      (void)cudaGetLastError();
      cudaFree(c->d_scratch);
      if (c->h_scratch) cudaFreeHost(c->h_scratch);
      c->d_scratch = c->h_scratch = nullptr;
      if (cap == bytes_) return cuda_fail((int)e, "scratch allocation");
    }
    return BBS_OK;
  }
  template <typename T>
  Piece<T> take(size_t n) {
    Piece<T> p{reinterpret_cast<T *>(c_->d_scratch + off_),
               reinterpret_cast<T *>(c_->h_scratch + off_)};
    off_ += piece(sizeof(T) * n);
    return p;
  }
  // Offset of the next piece: the end of the inputs, the start of the outputs.
  size_t mark() const { return off_; }
  // One copy of the mirror's bytes [from, to) to the device or back, on the
  // context's stream.
  cudaError_t to_device(size_t from, size_t to) const {
    return cudaMemcpyAsync(c_->d_scratch + from, c_->h_scratch + from, to - from,
                           cudaMemcpyHostToDevice, c_->stream);
  }
  cudaError_t to_host(size_t from, size_t to) const {
    return cudaMemcpyAsync(c_->h_scratch + from, c_->d_scratch + from, to - from,
                           cudaMemcpyDeviceToHost, c_->stream);
  }

 private:
  // 256-byte aligned; an empty piece takes no room, so a piece that add()
  // left out may still be taken with n = 0
  static size_t piece(size_t bytes) { return (bytes + 255) & ~size_t(255); }
  bbs_ctx *c_ = nullptr;
  size_t bytes_ = 0;
  size_t off_ = 0;
};

// FNV-1a, 64 bit.
uint64_t fnv1a(uint64_t h, const void *p, size_t n) {
  const uint8_t *b = static_cast<const uint8_t *>(p);
  for (size_t i = 0; i < n; i++) {
    h ^= b[i];
    h *= 0x100000001B3ull;
  }
  return h;
}

template <typename T>
uint64_t fnv1a_of(uint64_t h, const T &v) {
  return fnv1a(h, &v, sizeof(T));
}

// The dataset as the kernels see it and every parameter field (not the
// struct's padding).
uint64_t context_fingerprint(const bbs_params &p, uint32_t n_cells,
                             uint32_t n_genes, const std::vector<uint64_t> &K,
                             const std::vector<uint64_t> &M) {
  uint64_t h = 0xCBF29CE484222325ull;
  h = fnv1a_of(h, n_cells);
  h = fnv1a_of(h, n_genes);
  h = fnv1a(h, K.data(), sizeof(uint64_t) * K.size());
  h = fnv1a(h, M.data(), sizeof(uint64_t) * M.size());
  for (const float f : {p.alpha_mean, p.beta_mean, p.beta_sd, p.prob_beta_change,
                        p.prob_prune_n_reattach, p.prob_swap_nodes,
                        p.prob_swap_subtrees, p.beta_jump_scaling_chi, p.gamma,
                        p.error_step})
    h = fnv1a_of(h, f);
  for (const uint32_t u : {p.treelist_size, p.score_mode, p.error_move})
    h = fnv1a_of(h, u);
  return fnv1a_of(h, p.seed);
}

// True when dm (n rows of W words) is the descendant matrix of a tree
// rooted at n-1: its parent vector is valid and gives back the same rows.
bool valid_tree_rows(const uint64_t *dm, uint32_t n, std::vector<uint32_t> &pv,
                     std::vector<uint64_t> &tmp) {
  const uint32_t W = words64(n);
  pv.resize(n);
  tmp.resize((size_t)n * W);
  matrix_to_parent(dm, n, pv.data());
  if (check_parent_vector(pv.data(), n) != BBS_OK) return false;
  parent_to_matrix(pv.data(), n, nullptr, tmp.data());
  return std::memcmp(tmp.data(), dm, sizeof(uint64_t) * tmp.size()) == 0;
}

// Layout of a chain checkpoint: this header, then the current rows
// (n_chains x n_nodes x W words), the best rows (n_chains x treelist x
// n_nodes x W), the chain states (n_chains x 128 bytes) and, with
// treelist > 1, the tree hashes (n_chains x treelist) and betas of the
// co-optimal lists, padded to 8 bytes.
struct CheckpointHeader {
  char magic[8];
  uint32_t version, header_bytes;
  uint64_t fingerprint;
  uint32_t n_nodes, n_cells, words, n_chains;
  uint32_t treelist, state_bytes;
  uint64_t total_bytes;
  uint64_t reserved[3];
};
static_assert(sizeof(CheckpointHeader) == 80, "checkpoint header layout");
constexpr char kCheckpointMagic[8] = {'B', 'B', 'S', 'C', 'H', 'K', 'P', 'T'};
constexpr uint32_t kCheckpointVersion = 1;

struct CheckpointSizes {
  size_t rows, best, states, hashes, betas, total;
};

CheckpointSizes checkpoint_sizes(uint32_t n_nodes, uint32_t n_chains,
                                 uint32_t K) {
  CheckpointSizes z{};
  const size_t tw = (size_t)n_nodes * words64(n_nodes);
  z.rows = sizeof(uint64_t) * tw * n_chains;
  z.best = z.rows * K;
  z.states = sizeof(ChainState) * n_chains;
  z.hashes = K > 1 ? sizeof(uint64_t) * n_chains * K : 0;
  z.betas = K > 1 ? (sizeof(float) * n_chains * K + 7) / 8 * 8 : 0;
  z.total = sizeof(CheckpointHeader) + z.rows + z.best + z.states + z.hashes +
            z.betas;
  return z;
}

}  // namespace

extern "C" {

const char *bbs_last_error(void) { return g_error.c_str(); }
const char *bbs_version(void) { return "bbscite_gb300 0.1 (sm_103a)"; }
uint32_t bbs_words(uint32_t n_nodes) { return words64(n_nodes); }

void bbs_params_default(bbs_params *p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->alpha_mean = 6.04e-5f;
  p->beta_mean = 0.4309f;
  p->beta_sd = 0.1f;
  p->prob_beta_change = 0.0f;
  p->prob_prune_n_reattach = 0.55f;
  p->prob_swap_nodes = 0.4f;
  p->prob_swap_subtrees = 0.05f;
  p->beta_jump_scaling_chi = 10.0f;
  p->gamma = 1.0f;
  p->seed = 0x5eed5eedull;
  p->score_mode = BBS_SCORE_MAX;
  p->error_move = BBS_ERROR_BETA_WALK;
  p->error_step = 1.2f;
  p->treelist_size = 1;
}

int bbs_pruefer_to_parent_vector(const uint32_t *code, uint32_t code_len,
                                 uint32_t *parent) {
  if (!parent || (code_len && !code)) return fail(BBS_ERR_INPUT, "NULL buffer");
  if (code_len + 2 > BBS_MAX_GENES + 1)
    return fail(BBS_ERR_SIZE, "at most %d nodes", BBS_MAX_GENES + 1);
  for (uint32_t i = 0; i < code_len; i++)
    if (code[i] >= code_len + 2)
      return fail(BBS_ERR_INPUT, "code entry %u out of range", code[i]);
  pruefer_decode(code, code_len, parent);
  return BBS_OK;
}

int bbs_parent_vector_to_matrix(const uint32_t *parent, uint32_t n_nodes,
                                uint64_t *am, uint64_t *dm) {
  if (!parent) return fail(BBS_ERR_INPUT, "NULL parent vector");
  if (n_nodes > BBS_MAX_GENES + 1) return fail(BBS_ERR_SIZE, "too many nodes");
  const int r = check_parent_vector(parent, n_nodes);
  if (r != BBS_OK) return r;
  parent_to_matrix(parent, n_nodes, am, dm);
  return BBS_OK;
}

int bbs_matrix_to_parent_vector(const uint64_t *dm, uint32_t n_nodes,
                                uint32_t *parent) {
  if (!dm || !parent) return fail(BBS_ERR_INPUT, "NULL buffer");
  if (n_nodes < 1 || n_nodes > BBS_MAX_GENES + 1)
    return fail(BBS_ERR_SIZE, "node count %u out of range", n_nodes);
  matrix_to_parent(dm, n_nodes, parent);
  return BBS_OK;
}

int bbs_dm_to_am(const uint64_t *dm, uint32_t n_nodes, uint64_t *am) {
  if (!dm || !am) return fail(BBS_ERR_INPUT, "NULL buffer");
  const uint32_t W = words64(n_nodes);
  std::memset(am, 0, sizeof(uint64_t) * W * n_nodes);
  for (uint32_t x = 0; x < n_nodes; x++)
    for (uint32_t y = 0; y < n_nodes; y++)
      if (getb(dm + (size_t)x * W, y)) setb(am + (size_t)y * W, x);
  return BBS_OK;
}

int bbs_tree_to_graphviz(const uint32_t *parent, uint32_t n_nodes, char *buf,
                         size_t cap, size_t *len) {
  if (!parent) return fail(BBS_ERR_INPUT, "NULL parent vector");
  std::string s = "digraph G {\nnode [color=deeppink4, style=filled, fontcolor=white];\n";
  for (uint32_t x = 0; x + 1 < n_nodes; x++)
    s += std::to_string(parent[x]) + " -> " + std::to_string(x) + ";\n";
  s += "}\n";
  return put_string(s, buf, cap, len);
}

int bbs_tree_to_newick(const uint32_t *parent, uint32_t n_nodes, char *buf,
                       size_t cap, size_t *len) {
  if (!parent) return fail(BBS_ERR_INPUT, "NULL parent vector");
  const int r = check_parent_vector(parent, n_nodes);
  if (r != BBS_OK) return r;
  std::vector<std::vector<uint32_t>> ch(n_nodes);
  for (uint32_t x = 0; x + 1 < n_nodes; x++) ch[parent[x]].push_back(x);
  std::string s;
  newick_rec(ch, n_nodes - 1, s);
  s += '\n';
  return put_string(s, buf, cap, len);
}

int bbs_random_parent_vectors(uint64_t seed, uint32_t n_genes,
                              uint32_t n_trees, uint32_t *parents) {
  if (!parents) return fail(BBS_ERR_INPUT, "NULL buffer");
  if (n_genes < 1 || n_genes > BBS_MAX_GENES)
    return fail(BBS_ERR_SIZE, "gene count %u out of range", n_genes);
  random_parents(seed, n_genes, n_trees, parents);
  return BBS_OK;
}

// src/main.cpp:50-144: first pass counts cells per line and lines, second
// pass reads the entries.
int bbs_read_csv(const char *path, uint32_t *n_cells, uint32_t *n_genes,
                 uint64_t *is_mutated, uint64_t *is_known) {
  if (!path || !n_cells || !n_genes) return fail(BBS_ERR_INPUT, "NULL argument");
  std::ifstream in(path, std::ios::binary);
  if (!in) return fail(BBS_ERR_IO, "Error: could not open the input file %s", path);
  uint32_t cells = 0, genes = 0, in_line = 0;
  int ch;
  while ((ch = in.get()) != EOF) {
    const char c = (char)ch;
    if (c == '0' || c == '1' || c == '2' || c == '3') {
      in_line++;
    } else if (c == '\n') {
      if (cells == 0) {
        cells = in_line;
      } else if (cells != in_line) {
        return fail(BBS_ERR_INPUT, "Error: Inconsistent rows in the input file!");
      }
      genes++;
      in_line = 0;
    } else if (c == ' ') {
      continue;
    } else {
      return fail(BBS_ERR_INPUT, "Error: Illegal character %c in the input file!", c);
    }
  }
  if (in_line == cells) {
    genes++;
  } else if (in_line != 0) {
    return fail(BBS_ERR_INPUT, "Error: Inconsistent rows in the input file!");
  }
  if (cells == 0 || genes == 0) return fail(BBS_ERR_INPUT, "Error: Empty input file!");
  if (cells > BBS_MAX_CELLS)
    return fail(BBS_ERR_SIZE,
                "Error: This build of bbSCITE only supports up %u cells. The "
                "input data contains %u cells.",
                (unsigned)BBS_MAX_CELLS, cells);
  if (genes > BBS_MAX_GENES)
    return fail(BBS_ERR_SIZE,
                "Error: This build of bbSCITE only supports up %u genes. The "
                "input data contains %u genes.",
                (unsigned)BBS_MAX_GENES, genes);
  *n_cells = cells;
  *n_genes = genes;
  if (!is_mutated || !is_known) return BBS_OK;
  const uint32_t W = words64(genes + 1);
  std::memset(is_mutated, 0, sizeof(uint64_t) * W * cells);
  std::memset(is_known, 0, sizeof(uint64_t) * W * cells);
  in.clear();
  in.seekg(0);
  for (uint32_t g = 0; g < genes; g++)
    for (uint32_t c = 0; c < cells; c++) {
      int entry = -1;
      if (!(in >> entry))
        return fail(BBS_ERR_INPUT, "Error: The input file contains the invalid entry %d", entry);
      switch (entry) {
        case 0: setb(is_known + (size_t)c * W, g); break;
        case 1:
        case 2:
          setb(is_known + (size_t)c * W, g);
          setb(is_mutated + (size_t)c * W, g);
          break;
        case 3: break;
        default:
          return fail(BBS_ERR_INPUT, "Error: The input file contains the invalid entry %d", entry);
      }
    }
  return BBS_OK;
}

int bbs_create(bbs_ctx **out, const uint64_t *is_mutated,
               const uint64_t *is_known, uint32_t n_cells, uint32_t n_genes,
               const bbs_params *params) {
  try {
    if (!out || !is_mutated || !is_known)
      return fail(BBS_ERR_INPUT, "NULL argument to bbs_create");
    *out = nullptr;
    if (n_genes < 2 || n_genes > BBS_MAX_GENES)
      return fail(BBS_ERR_SIZE, "gene count %u outside [2, %d]", n_genes, BBS_MAX_GENES);
    if (n_cells < 1 || n_cells > BBS_MAX_CELLS)
      return fail(BBS_ERR_SIZE, "cell count %u outside [1, %d]", n_cells, BBS_MAX_CELLS);
    int r = check_params(params);
    if (r != BBS_OK) return r;
    int n_dev = 0;
    if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev < 1)
      return fail(BBS_ERR_CUDA, "no CUDA device is available");
    bbs_ctx *c = new (std::nothrow) bbs_ctx();
    if (!c) return fail(BBS_ERR_ALLOC, "out of host memory");
    c->params = *params;
    c->n_cells = n_cells;
    c->n_genes = n_genes;
    c->n_nodes = n_genes + 1;
    c->W64 = words64(c->n_nodes);
    c->RS = 2 * c->W64;
    cudaGetDevice(&c->device);
    cudaDeviceGetAttribute(&c->n_sms, cudaDevAttrMultiProcessorCount, c->device);
    cudaDeviceGetAttribute(&c->smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor,
                           c->device);
    cudaDeviceGetAttribute(&c->smem_block, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                           c->device);
    cudaDeviceGetAttribute(&c->smem_reserved, cudaDevAttrReservedSharedMemoryPerBlock,
                           c->device);
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    HostDataset h;
    prepare_dataset(params, n_cells, n_genes, is_mutated, is_known, h);
    const size_t bytes = sizeof(uint64_t) * h.K.size();
    if (e == cudaSuccess) e = cudaMalloc(&c->d_K, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_M, bytes);
    if (e == cudaSuccess) e = cudaMemcpy(c->d_K, h.K.data(), bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c->d_M, h.M.data(), bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_status, sizeof(int) * kStatusWords);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    if (e == cudaSuccess) e = cudaHostAlloc(&c->h_cancel, sizeof(int), cudaHostAllocMapped);
    if (e == cudaSuccess) {
      *c->h_cancel = 0;
      e = cudaHostGetDevicePointer((void **)&c->d_cancel, c->h_cancel, 0);
    }
    h.ds.K = c->d_K;
    h.ds.M = c->d_M;
    if (e == cudaSuccess) e = cudaMalloc(&c->d_ds, sizeof(DatasetDev));
    if (e == cudaSuccess) e = cudaMalloc(&c->d_md, sizeof(ModelDev));
    if (e == cudaSuccess) e = cudaMalloc(&c->d_terms, sizeof(h.terms));
    if (e == cudaSuccess) e = cudaMemcpy(c->d_ds, &h.ds, sizeof(DatasetDev), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c->d_md, &h.md, sizeof(ModelDev), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c->d_terms, h.terms, sizeof(h.terms), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      const int rr = cuda_fail((int)e, "bbs_create");
      bbs_destroy(c);
      return rr;
    }
    c->ds = h.ds;
    c->md = h.md;
    std::memcpy(c->terms, h.terms, sizeof(h.terms));
    c->fingerprint = context_fingerprint(*params, n_cells, n_genes, h.K, h.M);
    c->q = pick_q((int)n_cells);
    *out = c;
    return BBS_OK;
  } catch (...) {
    return fail(BBS_ERR_ALLOC, "allocation failed in bbs_create");
  }
}

void bbs_destroy(bbs_ctx *c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_chains(c);
  cudaFree(c->d_scratch);
  if (c->h_scratch) cudaFreeHost(c->h_scratch);
  cudaFree(c->d_K);
  cudaFree(c->d_M);
  cudaFree(c->d_ds);
  cudaFree(c->d_md);
  cudaFree(c->d_terms);
  cudaFree(c->d_status);
  if (c->h_cancel) cudaFreeHost(c->h_cancel);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

int bbs_get_sizes(const bbs_ctx *c, uint32_t *n_cells, uint32_t *n_genes,
                  uint32_t *n_chains) {
  if (!c) return fail(BBS_ERR_INPUT, "NULL context");
  if (n_cells) *n_cells = c->n_cells;
  if (n_genes) *n_genes = c->n_genes;
  if (n_chains) *n_chains = c->n_chains;
  return BBS_OK;
}

namespace {

// One-warp chains per block (1-8; they share the block's increment table)
// that keep the most warps resident on an SM; ties keep the smaller block.
int pick_chains_per_block(const bbs_ctx *c, int q) {
  const bool sum = c->md.score_mode != 0;
  int best = 1, best_warps = 0;
  for (int cpb = 1; cpb * 32 <= chain_max_threads(q); cpb++) {
    const int smem = chain_launch_smem((int)c->n_nodes, (int)c->n_cells, q, 1,
                                       cpb, sum);
    const int w = chain_resident_warps(smem, cpb, q, c->smem_sm, c->smem_block,
                                       c->smem_reserved);
    if (w > best_warps) {
      best_warps = w;
      best = cpb;
    }
  }
  return best;
}

// Launch shape without timing: split the cells over up to four warps per
// chain when there are too few chains to give every scheduler ~3 warps,
// preferring shapes that leave no cell slots empty.
void default_launch(bbs_ctx *c) {
  const int groups = (int)((c->n_cells + 31) / 32);
  const int qmax = w32_of_nodes((int)c->n_nodes) > 4 ? 2 : kMaxQ;
  double best = 1e30;
  for (int wpc = 1; wpc <= 4; wpc++) {
    const int q = std::max(1, (groups + wpc - 1) / wpc);
    if (q > qmax) continue;
    const double waste = (double)(wpc * q) / groups;
    const double warps = (double)c->n_chains * wpc;
    const double occ = std::min(1.0, warps / (12.0 * c->n_sms));
    const double est = waste / occ * (1.0 + 0.1 * (wpc - 1));
    if (est < best) {
      best = est;
      c->wpc = wpc;
      c->q = q;
    }
  }
  if (best >= 1e30) {  // very wide datasets: chunks of qmax per lane
    c->wpc = 4;
    c->q = qmax;
  }
  c->cpb = c->wpc == 1 ? pick_chains_per_block(c, c->q) : 1;
}

size_t tree_words(const bbs_ctx *c, uint32_t n_trees) {
  return (size_t)n_trees * c->n_nodes * c->W64;
}

}  // namespace

int bbs_init_chains(bbs_ctx *c, uint32_t n_chains, const uint32_t *parents) {
  try {
    if (!c) return fail(BBS_ERR_INPUT, "NULL context");
    if (c->running) return fail(BBS_ERR_STATE, "a run is in progress");
    if (n_chains < 1) return fail(BBS_ERR_INPUT, "need at least one chain");
    const uint32_t n = c->n_nodes;
    const size_t tw = (size_t)n * c->W64;
    std::vector<uint64_t> dm;
    if (parents) {
      for (uint32_t t = 0; t < n_chains; t++) {
        const int r = check_parent_vector(parents + (size_t)t * n, n);
        if (r != BBS_OK) return r;
      }
      dm.resize(tw * n_chains);
      for (uint32_t t = 0; t < n_chains; t++)
        parent_to_matrix(parents + (size_t)t * n, n, nullptr, dm.data() + t * tw);
    }
    free_chains(c);
    const size_t words = tw * n_chains;
    c->K = (uint32_t)c->md.treelist;
    cudaError_t e = cudaMalloc(&c->d_rows, sizeof(uint64_t) * words);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_best, sizeof(uint64_t) * words * c->K);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_states, sizeof(ChainState) * n_chains);
    if (e == cudaSuccess && c->K > 1)
      e = cudaMalloc(&c->d_lhash, sizeof(uint64_t) * n_chains * c->K);
    if (e == cudaSuccess && c->K > 1)
      e = cudaMalloc(&c->d_lbeta, sizeof(float) * n_chains * c->K);
    if (e == cudaSuccess && parents)
      e = cudaMemcpyAsync(c->d_rows, dm.data(), sizeof(uint64_t) * words,
                          cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess && !parents) {
      // random initial trees drawn on the device (the host helper
      // bbs_random_parent_vectors gives the same trees)
      TreeArgs ta{};
      ta.ds = c->d_ds;
      ta.md = c->d_md;
      ta.n_chains = (int)n_chains;
      ta.rows = reinterpret_cast<uint32_t *>(c->d_rows);
      ta.max_nodes = (int)n;
      e = (cudaError_t)launch_trees(ta, c->stream);
    }
    if (e == cudaSuccess)
      e = cudaMemsetAsync(c->d_best, 0, sizeof(uint64_t) * words * c->K,
                          c->stream);
    if (e != cudaSuccess) {
      free_chains(c);
      return cuda_fail((int)e, "bbs_init_chains");
    }
    c->n_chains = n_chains;
    InitArgs ia{};
    ia.ds = c->d_ds;
    ia.md = c->d_md;
    ia.chain_ds = nullptr;
    ia.chain_off = nullptr;
    ia.terms = c->d_terms;
    ia.n_chains = (int)n_chains;
    ia.rows = c->d_rows;
    ia.states = c->d_states;
    ia.max_nodes = (int)n;
    const int le = launch_init(ia, w32_of_nodes((int)n),
                               c->md.score_mode == BBS_SCORE_SUM, c->stream);
    int r = le != 0 ? cuda_fail(le, "init kernel launch")
                    : sync_stream(c, "init kernel");
    if (r != BBS_OK) free_chains(c);
    default_launch(c);
    return r;
  } catch (...) {
    return fail(BBS_ERR_ALLOC, "allocation failed in bbs_init_chains");
  }
}

namespace {

int start_run(bbs_ctx *c, uint32_t n_steps, const bbs_raw_move *d_moves,
              bbs_step_trace *d_trace) {
  {
    const int cpb = c->wpc > 1 ? 1 : c->cpb;
    const int smem = chain_launch_smem((int)c->n_nodes, (int)c->n_cells, c->q,
                                       c->wpc, cpb, c->md.score_mode != 0);
    if (32 * c->wpc * cpb > chain_max_threads(c->q) || smem > c->smem_block)
      return fail(BBS_ERR_SIZE,
                  "launch shape (%d cells per lane, %d warps per chain, %d "
                  "chains per block) needs %d bytes of shared memory and %d "
                  "threads per block; the kernel and device allow %d and %d",
                  c->q, c->wpc, cpb, smem, 32 * c->wpc * cpb, c->smem_block,
                  chain_max_threads(c->q));
  }
  RunArgs a{};
  a.ds = c->ds;
  a.md = c->md;
  a.n_chains = (int)c->n_chains;
  a.n_steps = (int)n_steps;
  a.rows = c->d_rows;
  a.best_rows = c->d_best;
  a.list_hash = c->K > 1 ? c->d_lhash : nullptr;
  a.list_beta = c->K > 1 ? c->d_lbeta : nullptr;
  a.states = c->d_states;
  a.moves = d_moves;
  a.trace = d_trace;
  a.cancel = c->d_cancel;
  a.status = c->d_status;
  a.wpc = c->wpc;
  *c->h_cancel = 0;
  BBS_CUDA(cudaMemsetAsync(c->d_status, 0, sizeof(int) * kStatusWords, c->stream),
           "cudaMemset");
  BBS_CUDA(cudaEventRecord(c->ev0, c->stream), "cudaEventRecord");
  const int e = launch_mcmc(a, c->q, c->cpb, c->n_sms, c->stream);
  if (e != 0) return cuda_fail(e, "chain kernel launch");
  BBS_CUDA(cudaEventRecord(c->ev1, c->stream), "cudaEventRecord");
  return BBS_OK;
}

int finish_run(bbs_ctx *c) {
  cudaError_t e = cudaStreamSynchronize(c->stream);
  c->running = false;
  if (e != cudaSuccess) return cuda_fail((int)e, "chain kernel");
  e = cudaEventElapsedTime(&c->last_ms, c->ev0, c->ev1);
  if (e != cudaSuccess) return cuda_fail((int)e, "event timing");
  int status[kStatusWords] = {};
  e = cudaMemcpy(status, c->d_status, sizeof(status), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail((int)e, "status read");
  return status_result(status);
}

}  // namespace

int bbs_run(bbs_ctx *c, uint32_t n_steps, const bbs_raw_move *moves,
            bbs_step_trace *trace) {
  try {
    if (!c) return fail(BBS_ERR_INPUT, "NULL context");
    if (c->running) return fail(BBS_ERR_STATE, "a run is in progress");
    if (c->n_chains == 0) return fail(BBS_ERR_STATE, "bbs_init_chains was not called");
    if (n_steps == 0) return BBS_OK;
    if (n_steps > 0x7fffffffu) return fail(BBS_ERR_SIZE, "too many steps");
    const size_t total = (size_t)c->n_chains * n_steps;
    DevBuf<bbs_raw_move> d_moves;
    DevBuf<bbs_step_trace> d_trace;
    if (moves) {
      for (size_t i = 0; i < total; i++) {
        const bbs_raw_move &m = moves[i];
        if (m.move_type < 0 || m.move_type > 3)
          return fail(BBS_ERR_INPUT, "move %zu has type %d", i, m.move_type);
        if (m.raw_v >= c->n_nodes || m.raw_w >= c->n_nodes)
          return fail(BBS_ERR_INPUT, "move %zu names a node >= %u", i, c->n_nodes);
      }
      BBS_CUDA(d_moves.alloc(total), "cudaMalloc");
      BBS_CUDA(cudaMemcpyAsync(d_moves.p, moves, sizeof(bbs_raw_move) * total,
                               cudaMemcpyHostToDevice, c->stream), "cudaMemcpy");
    }
    if (trace) BBS_CUDA(d_trace.alloc(total), "cudaMalloc");
    c->running = true;
    int r = start_run(c, n_steps, d_moves.p, d_trace.p);
    if (r != BBS_OK) {
      c->running = false;
      return r;
    }
    r = finish_run(c);
    if (r == BBS_OK && trace)
      BBS_CUDA(cudaMemcpy(trace, d_trace.p, sizeof(bbs_step_trace) * total,
                          cudaMemcpyDeviceToHost), "trace copy");
    return r;
  } catch (...) {
    c->running = false;
    return fail(BBS_ERR_ALLOC, "allocation failed in bbs_run");
  }
}

int bbs_run_async(bbs_ctx *c, uint32_t n_steps) {
  if (!c) return fail(BBS_ERR_INPUT, "NULL context");
  if (c->running) return fail(BBS_ERR_STATE, "a run is in progress");
  if (c->n_chains == 0) return fail(BBS_ERR_STATE, "bbs_init_chains was not called");
  if (n_steps == 0) return BBS_OK;
  c->running = true;
  const int r = start_run(c, n_steps, nullptr, nullptr);
  if (r != BBS_OK) c->running = false;
  return r;
}

int bbs_sync(bbs_ctx *c) {
  if (!c) return fail(BBS_ERR_INPUT, "NULL context");
  if (!c->running) return BBS_OK;
  return finish_run(c);
}

int bbs_cancel(bbs_ctx *c) {
  if (!c) return fail(BBS_ERR_INPUT, "NULL context");
  if (c->h_cancel) *(volatile int *)c->h_cancel = 1;
  return BBS_OK;
}

int bbs_set_launch(bbs_ctx *c, int cells_per_lane, int warps_per_chain,
                   int chains_per_block) {
  if (!c) return fail(BBS_ERR_INPUT, "NULL context");
  const int qmax = w32_of_nodes((int)c->n_nodes) > 4 ? 2 : kMaxQ;
  if (cells_per_lane < 0 || cells_per_lane > qmax)
    return fail(BBS_ERR_INPUT, "cells per lane must be in [1, %d]", qmax);
  if (warps_per_chain < 0 || warps_per_chain > 4)
    return fail(BBS_ERR_INPUT, "warps per chain must be in [1, 4]");
  if (chains_per_block < 0 || 32 * chains_per_block > kMaxBlockThreads)
    return fail(BBS_ERR_INPUT, "chains per block must be in [1, %d]",
                kMaxBlockThreads / 32);
  if (cells_per_lane) c->q = cells_per_lane;
  if (warps_per_chain) c->wpc = warps_per_chain;
  if (chains_per_block) c->cpb = chains_per_block;
  if (c->wpc > 1) c->cpb = 1;
  return BBS_OK;
}

int bbs_get_launch(const bbs_ctx *c, int *cells_per_lane,
                   int *warps_per_chain, int *chains_per_block) {
  if (!c) return fail(BBS_ERR_INPUT, "NULL context");
  if (cells_per_lane) *cells_per_lane = c->q;
  if (warps_per_chain) *warps_per_chain = c->wpc;
  if (chains_per_block) *chains_per_block = c->cpb;
  return BBS_OK;
}

int bbs_autotune(bbs_ctx *c, uint32_t probe_steps, float *best_ms) {
  try {
    if (!c) return fail(BBS_ERR_INPUT, "NULL context");
    if (c->running) return fail(BBS_ERR_STATE, "a run is in progress");
    if (c->n_chains == 0) return fail(BBS_ERR_STATE, "bbs_init_chains was not called");
    if (probe_steps == 0) probe_steps = 64;
    // Keep the chains as they are: save, probe, restore.
    const size_t rows_bytes = sizeof(uint64_t) * c->n_chains * c->n_nodes * c->W64;
    const size_t best_bytes = rows_bytes * c->K;
    const size_t list_bytes = c->K > 1 ? (size_t)c->n_chains * c->K : 0;
    DevBuf<uint8_t> save_rows, save_best, save_states, save_lh, save_lb;
    BBS_CUDA(save_rows.alloc(rows_bytes), "cudaMalloc");
    BBS_CUDA(save_best.alloc(best_bytes), "cudaMalloc");
    BBS_CUDA(save_states.alloc(sizeof(ChainState) * c->n_chains), "cudaMalloc");
    if (list_bytes) {
      BBS_CUDA(save_lh.alloc(list_bytes * sizeof(uint64_t)), "cudaMalloc");
      BBS_CUDA(save_lb.alloc(list_bytes * sizeof(float)), "cudaMalloc");
    }
    auto copy = [&](void *dst, const void *src, size_t b) {
      return cudaMemcpyAsync(dst, src, b, cudaMemcpyDeviceToDevice, c->stream);
    };
    BBS_CUDA(copy(save_rows.p, c->d_rows, rows_bytes), "save");
    BBS_CUDA(copy(save_best.p, c->d_best, best_bytes), "save");
    BBS_CUDA(copy(save_states.p, c->d_states, sizeof(ChainState) * c->n_chains), "save");
    if (list_bytes) {
      BBS_CUDA(copy(save_lh.p, c->d_lhash, list_bytes * sizeof(uint64_t)), "save");
      BBS_CUDA(copy(save_lb.p, c->d_lbeta, list_bytes * sizeof(float)), "save");
    }
    const int groups = (int)((c->n_cells + 31) / 32);
    const int qmax = w32_of_nodes((int)c->n_nodes) > 4 ? 2 : kMaxQ;
    const int q0 = c->q, w0 = c->wpc, b0 = c->cpb;
    float best = 1e30f;
    int bq = q0, bw = w0, bb = b0;
    for (int wpc = 1; wpc <= 4; wpc++)
      for (int q = 1; q <= qmax; q++) {
        if (wpc * q > groups + 1) continue;  // mostly empty cell slots
        for (int cpb : {1, 2, 4, 7, 8}) {
          if (wpc > 1 && cpb > 1) continue;
          if (32 * wpc * cpb > chain_max_threads(q)) continue;
          if (chain_launch_smem((int)c->n_nodes, (int)c->n_cells, q, wpc, cpb,
                                c->md.score_mode != 0) > c->smem_block)
            continue;  // too large a block
          c->q = q;
          c->wpc = wpc;
          c->cpb = cpb;
          c->running = true;
          int r = start_run(c, probe_steps, nullptr, nullptr);
          if (r == BBS_OK) r = finish_run(c);
          c->running = false;
          if (r == BBS_OK && c->last_ms < best) {
            best = c->last_ms;
            bq = q;
            bw = wpc;
            bb = cpb;
          }
          BBS_CUDA(copy(c->d_rows, save_rows.p, rows_bytes), "restore");
          BBS_CUDA(copy(c->d_best, save_best.p, best_bytes), "restore");
          BBS_CUDA(copy(c->d_states, save_states.p,
                        sizeof(ChainState) * c->n_chains), "restore");
          if (list_bytes) {
            BBS_CUDA(copy(c->d_lhash, save_lh.p, list_bytes * sizeof(uint64_t)),
                     "restore");
            BBS_CUDA(copy(c->d_lbeta, save_lb.p, list_bytes * sizeof(float)),
                     "restore");
          }
        }
      }
    c->q = bq;
    c->wpc = bw;
    c->cpb = bb;
    const int r = sync_stream(c, "autotune restore");
    if (best_ms) *best_ms = best;
    return r;
  } catch (...) {
    c->running = false;
    return fail(BBS_ERR_ALLOC, "allocation failed in bbs_autotune");
  }
}

int bbs_last_run_ms(const bbs_ctx *c, float *ms) {
  if (!c || !ms) return fail(BBS_ERR_INPUT, "NULL argument");
  *ms = c->last_ms;
  return BBS_OK;
}

int bbs_get_best(bbs_ctx *c, uint64_t *am, uint64_t *dm, uint32_t *parent,
                 float *beta, float *score, uint64_t *counts,
                 uint32_t *chain) {
  try {
    if (!c) return fail(BBS_ERR_INPUT, "NULL context");
    if (c->running) return fail(BBS_ERR_STATE, "a run is in progress");
    if (c->n_chains == 0) return fail(BBS_ERR_STATE, "no chains");
    std::vector<ChainState> st(c->n_chains);
    BBS_CUDA(cudaMemcpy(st.data(), c->d_states, sizeof(ChainState) * st.size(),
                        cudaMemcpyDeviceToHost), "state copy");
    // First chain in index order holding the maximum (the emulator's
    // chain-major order, strict '>' as src/Application.hpp:456).
    int best = -1;
    for (uint32_t i = 0; i < c->n_chains; i++) {
      if (!st[i].has_best) continue;
      if (best < 0 || st[i].best_score > st[best].best_score) best = (int)i;
    }
    if (best < 0) return fail(BBS_ERR_STATE, "no steps have been run");
    const uint32_t n = c->n_nodes;
    const size_t tw = (size_t)n * c->W64;
    std::vector<uint64_t> rows(tw);
    BBS_CUDA(cudaMemcpy(rows.data(), c->d_best + (size_t)best * c->K * tw * 2,
                        sizeof(uint64_t) * tw, cudaMemcpyDeviceToHost), "best copy");
    if (dm) std::memcpy(dm, rows.data(), sizeof(uint64_t) * tw);
    if (am) bbs_dm_to_am(rows.data(), n, am);
    if (parent) matrix_to_parent(rows.data(), n, parent);
    if (beta) *beta = st[best].best_beta;
    if (score) *score = st[best].best_score;
    if (counts) {
      const int sk = st[best].best_sk, sm = st[best].best_sm;
      counts[0] = (uint64_t)(c->ds.sum_k - c->ds.sum_m - sk + sm);
      counts[1] = (uint64_t)(sk - sm);
      counts[2] = (uint64_t)(c->ds.sum_m - sm);
      counts[3] = (uint64_t)sm;
    }
    if (chain) *chain = (uint32_t)best;
    return BBS_OK;
  } catch (...) {
    return fail(BBS_ERR_ALLOC, "allocation failed in bbs_get_best");
  }
}

int bbs_get_chains(bbs_ctx *c, uint64_t *dm, float *alpha, float *beta,
                   float *score, uint64_t *counts, uint32_t *err_stats) {
  try {
    if (!c) return fail(BBS_ERR_INPUT, "NULL context");
    if (c->running) return fail(BBS_ERR_STATE, "a run is in progress");
    if (c->n_chains == 0) return fail(BBS_ERR_STATE, "no chains");
    const size_t tw = (size_t)c->n_nodes * c->W64;
    if (dm)
      BBS_CUDA(cudaMemcpy(dm, c->d_rows, sizeof(uint64_t) * tw * c->n_chains,
                          cudaMemcpyDeviceToHost), "row copy");
    std::vector<ChainState> st(c->n_chains);
    BBS_CUDA(cudaMemcpy(st.data(), c->d_states, sizeof(ChainState) * st.size(),
                        cudaMemcpyDeviceToHost), "state copy");
    for (uint32_t i = 0; i < c->n_chains; i++) {
      if (alpha) alpha[i] = st[i].alpha;
      if (beta) beta[i] = st[i].beta;
      if (score) score[i] = st[i].score;
      if (counts) {
        const int sk = st[i].sk, sm = st[i].sm;
        counts[4 * i + 0] = (uint64_t)(c->ds.sum_k - c->ds.sum_m - sk + sm);
        counts[4 * i + 1] = (uint64_t)(sk - sm);
        counts[4 * i + 2] = (uint64_t)(c->ds.sum_m - sm);
        counts[4 * i + 3] = (uint64_t)sm;
      }
      if (err_stats) {
        err_stats[2 * i] = st[i].err_proposed;
        err_stats[2 * i + 1] = st[i].err_accepted;
      }
    }
    return BBS_OK;
  } catch (...) {
    return fail(BBS_ERR_ALLOC, "allocation failed in bbs_get_chains");
  }
}

int bbs_get_treelist(bbs_ctx *c, uint32_t max_trees, uint64_t *dm,
                     float *betas, float *score, uint32_t *n_trees) {
  try {
    if (!c || !dm || !n_trees) return fail(BBS_ERR_INPUT, "NULL argument");
    if (c->running) return fail(BBS_ERR_STATE, "a run is in progress");
    if (c->n_chains == 0) return fail(BBS_ERR_STATE, "no chains");
    *n_trees = 0;
    std::vector<ChainState> st(c->n_chains);
    BBS_CUDA(cudaMemcpy(st.data(), c->d_states, sizeof(ChainState) * st.size(),
                        cudaMemcpyDeviceToHost), "state copy");
    int best = -1;
    for (uint32_t i = 0; i < c->n_chains; i++) {
      if (!st[i].has_best) continue;
      if (best < 0 || st[i].best_score > st[best].best_score) best = (int)i;
    }
    if (best < 0) return fail(BBS_ERR_STATE, "no steps have been run");
    const float top = st[best].best_score;
    if (score) *score = top;
    const size_t tw = (size_t)c->n_nodes * c->W64;
    std::vector<uint64_t> rows(tw * c->K);
    std::vector<float> lb(c->K);
    uint32_t found = 0;
    // the bbs_get_best chain first, then the others in index order
    for (uint32_t k = 0; k <= c->n_chains && found < max_trees; k++) {
      const uint32_t i = k == 0 ? (uint32_t)best : k - 1;
      if (k > 0 && i == (uint32_t)best) continue;
      if (!st[i].has_best || st[i].best_score != top) continue;
      const uint32_t cnt = c->K > 1 ? std::min(st[i].list_count, c->K) : 1u;
      BBS_CUDA(cudaMemcpy(rows.data(), c->d_best + (size_t)i * c->K * tw * 2,
                          sizeof(uint64_t) * tw * cnt, cudaMemcpyDeviceToHost),
               "tree list copy");
      if (c->K > 1)
        BBS_CUDA(cudaMemcpy(lb.data(), c->d_lbeta + (size_t)i * c->K,
                            sizeof(float) * cnt, cudaMemcpyDeviceToHost),
                 "tree list copy");
      else
        lb[0] = st[i].best_beta;
      for (uint32_t j = 0; j < cnt && found < max_trees; j++) {
        const uint64_t *t = rows.data() + j * tw;
        bool dup = false;
        for (uint32_t u = 0; u < found && !dup; u++)
          dup = std::memcmp(dm + u * tw, t, sizeof(uint64_t) * tw) == 0;
        if (dup) continue;
        std::memcpy(dm + found * tw, t, sizeof(uint64_t) * tw);
        if (betas) betas[found] = lb[j];
        found++;
      }
    }
    *n_trees = found;
    return BBS_OK;
  } catch (...) {
    return fail(BBS_ERR_ALLOC, "allocation failed in bbs_get_treelist");
  }
}

int bbs_save_chains(bbs_ctx *c, void *buf, size_t *size) {
  try {
    if (!c || !size) return fail(BBS_ERR_INPUT, "NULL argument");
    if (c->running) return fail(BBS_ERR_STATE, "a run is in progress");
    if (c->n_chains == 0) return fail(BBS_ERR_STATE, "no chains");
    const CheckpointSizes z = checkpoint_sizes(c->n_nodes, c->n_chains, c->K);
    if (!buf) {
      *size = z.total;
      return BBS_OK;
    }
    if (*size < z.total) {
      const size_t have = *size;
      *size = z.total;
      return fail(BBS_ERR_SIZE, "checkpoint needs %zu bytes, buffer has %zu",
                  z.total, have);
    }
    CheckpointHeader hd{};
    std::memcpy(hd.magic, kCheckpointMagic, sizeof(hd.magic));
    hd.version = kCheckpointVersion;
    hd.header_bytes = sizeof(CheckpointHeader);
    hd.fingerprint = c->fingerprint;
    hd.n_nodes = c->n_nodes;
    hd.n_cells = c->n_cells;
    hd.words = c->W64;
    hd.n_chains = c->n_chains;
    hd.treelist = c->K;
    hd.state_bytes = sizeof(ChainState);
    hd.total_bytes = z.total;
    uint8_t *p = static_cast<uint8_t *>(buf);
    std::memcpy(p, &hd, sizeof(hd));
    p += sizeof(hd);
    BBS_CUDA(cudaMemcpy(p, c->d_rows, z.rows, cudaMemcpyDeviceToHost), "checkpoint copy");
    p += z.rows;
    BBS_CUDA(cudaMemcpy(p, c->d_best, z.best, cudaMemcpyDeviceToHost), "checkpoint copy");
    p += z.best;
    BBS_CUDA(cudaMemcpy(p, c->d_states, z.states, cudaMemcpyDeviceToHost), "checkpoint copy");
    p += z.states;
    if (c->K > 1) {
      BBS_CUDA(cudaMemcpy(p, c->d_lhash, z.hashes, cudaMemcpyDeviceToHost), "checkpoint copy");
      p += z.hashes;
      std::memset(p, 0, z.betas);
      BBS_CUDA(cudaMemcpy(p, c->d_lbeta, sizeof(float) * c->n_chains * c->K,
                          cudaMemcpyDeviceToHost), "checkpoint copy");
    }
    *size = z.total;
    return BBS_OK;
  } catch (...) {
    return fail(BBS_ERR_ALLOC, "allocation failed in bbs_save_chains");
  }
}

int bbs_load_chains(bbs_ctx *c, const void *buf, size_t size) {
  try {
    if (!c || !buf) return fail(BBS_ERR_INPUT, "NULL argument");
    if (c->running) return fail(BBS_ERR_STATE, "a run is in progress");
    CheckpointHeader hd;
    if (size < sizeof(hd)) return fail(BBS_ERR_INPUT, "checkpoint too short");
    std::memcpy(&hd, buf, sizeof(hd));
    if (std::memcmp(hd.magic, kCheckpointMagic, sizeof(hd.magic)) != 0)
      return fail(BBS_ERR_INPUT, "not a chain checkpoint");
    if (hd.version != kCheckpointVersion || hd.header_bytes != sizeof(hd) ||
        hd.state_bytes != sizeof(ChainState))
      return fail(BBS_ERR_INPUT, "checkpoint version %u is not supported",
                  hd.version);
    if (hd.fingerprint != c->fingerprint || hd.n_nodes != c->n_nodes ||
        hd.n_cells != c->n_cells || hd.words != c->W64 ||
        hd.treelist != (uint32_t)c->md.treelist)
      return fail(BBS_ERR_INPUT,
                  "the checkpoint was made with another dataset or other "
                  "parameters");
    if (hd.n_chains < 1) return fail(BBS_ERR_INPUT, "checkpoint has no chains");
    const uint32_t n = c->n_nodes, K = hd.treelist;
    const CheckpointSizes z = checkpoint_sizes(n, hd.n_chains, K);
    if (hd.total_bytes != z.total || size < z.total)
      return fail(BBS_ERR_INPUT, "checkpoint size %zu, expected %zu", size,
                  z.total);
    const uint8_t *p = static_cast<const uint8_t *>(buf) + sizeof(hd);
    const uint64_t *rows = reinterpret_cast<const uint64_t *>(p);
    const uint64_t *best = reinterpret_cast<const uint64_t *>(p + z.rows);
    std::vector<ChainState> st(hd.n_chains);
    std::memcpy(st.data(), p + z.rows + z.best, z.states);
    // every tree the kernels will read must be a tree: moves walk its rows
    const size_t tw = (size_t)n * c->W64;
    std::vector<uint32_t> pv;
    std::vector<uint64_t> tmp;
    for (uint32_t i = 0; i < hd.n_chains; i++) {
      if (!valid_tree_rows(rows + i * tw, n, pv, tmp))
        return fail(BBS_ERR_INPUT, "checkpoint chain %u holds no valid tree", i);
      if (st[i].list_count > K || st[i].has_best > 1)
        return fail(BBS_ERR_INPUT, "checkpoint chain %u has a bad state", i);
      const uint32_t listed = st[i].has_best ? (K > 1 ? st[i].list_count : 1u) : 0u;
      for (uint32_t j = 0; j < listed; j++)
        if (!valid_tree_rows(best + ((size_t)i * K + j) * tw, n, pv, tmp))
          return fail(BBS_ERR_INPUT, "checkpoint chain %u holds no valid best tree", i);
    }
    free_chains(c);
    c->K = K;
    cudaError_t e = cudaMalloc(&c->d_rows, z.rows);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_best, z.best);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_states, z.states);
    if (e == cudaSuccess && K > 1) e = cudaMalloc(&c->d_lhash, z.hashes);
    if (e == cudaSuccess && K > 1)
      e = cudaMalloc(&c->d_lbeta, sizeof(float) * hd.n_chains * K);
    if (e == cudaSuccess) e = cudaMemcpy(c->d_rows, rows, z.rows, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c->d_best, best, z.best, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(c->d_states, st.data(), z.states, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && K > 1)
      e = cudaMemcpy(c->d_lhash, p + z.rows + z.best + z.states, z.hashes,
                     cudaMemcpyHostToDevice);
    if (e == cudaSuccess && K > 1)
      e = cudaMemcpy(c->d_lbeta, p + z.rows + z.best + z.states + z.hashes,
                     sizeof(float) * hd.n_chains * K, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      free_chains(c);
      return cuda_fail((int)e, "bbs_load_chains");
    }
    c->n_chains = hd.n_chains;
    default_launch(c);
    return BBS_OK;
  } catch (...) {
    return fail(BBS_ERR_ALLOC, "allocation failed in bbs_load_chains");
  }
}

int bbs_get_best_alpha(bbs_ctx *c, float *alpha) {
  if (!c || !alpha) return fail(BBS_ERR_INPUT, "NULL argument");
  uint32_t chain = 0;
  const int r = bbs_get_best(c, nullptr, nullptr, nullptr, nullptr, nullptr,
                             nullptr, &chain);
  if (r != BBS_OK) return r;
  ChainState st;
  BBS_CUDA(cudaMemcpy(&st, c->d_states + chain, sizeof(ChainState),
                      cudaMemcpyDeviceToHost), "state copy");
  *alpha = st.best_alpha;
  return BBS_OK;
}

int bbs_score_trees(bbs_ctx *c, const uint64_t *dm, const float *betas,
                    uint32_t n_trees, float *scores, uint64_t *counts,
                    uint32_t *attach) {
  try {
    if (!c || !dm || !betas || !scores) return fail(BBS_ERR_INPUT, "NULL argument");
    if (c->running) return fail(BBS_ERR_STATE, "a run is in progress");
    if (n_trees == 0) return BBS_OK;
    for (uint32_t t = 0; t < n_trees; t++)
      if (!(betas[t] > 0.0f && betas[t] < 1.0f))
        return fail(BBS_ERR_INPUT, "beta of tree %u outside (0, 1)", t);
    const size_t words = tree_words(c, n_trees);
    const size_t n_attach = (size_t)n_trees * c->n_cells;
    ScratchPlan plan;
    plan.add<uint64_t>(words);
    plan.add<float>(4 * (size_t)n_trees);
    plan.add<float>(n_trees);
    if (counts) plan.add<uint64_t>(4 * (size_t)n_trees);
    if (attach) plan.add<uint32_t>(n_attach);
    int r = plan.reserve(c);
    if (r != BBS_OK) return r;
    const auto rows = plan.take<uint64_t>(words);
    const auto terms = plan.take<float>(4 * (size_t)n_trees);
    const size_t out_begin = plan.mark();
    const auto d_scores = plan.take<float>(n_trees);
    const auto d_counts = plan.take<uint64_t>(counts ? 4 * (size_t)n_trees : 0);
    const auto d_attach = plan.take<uint32_t>(attach ? n_attach : 0);
    const size_t out_end = plan.mark();
    // inputs: the ancestor rows and the host log-table terms of each beta
    std::memcpy(rows.h, dm, sizeof(uint64_t) * words);
    for (uint32_t t = 0; t < n_trees; t++) {
      float *tt = terms.h + 4 * (size_t)t;
      tt[0] = betas[t];
      host_beta_terms(c->ds, betas[t], &tt[1], &tt[2], &tt[3]);
    }
    BBS_CUDA(plan.to_device(0, out_begin), "scratch upload");
    ScoreArgs a{};
    a.ds = c->ds;
    a.rows = reinterpret_cast<const uint32_t *>(rows.d);
    a.beta_terms = terms.d;
    a.n_trees = (int)n_trees;
    a.scores = d_scores.d;
    a.counts = counts ? d_counts.d : nullptr;
    a.attach = attach ? d_attach.d : nullptr;
    a.states = nullptr;
    const int e = launch_score(a, c->q, c->stream);
    if (e != 0) return cuda_fail(e, "score kernel launch");
    BBS_CUDA(plan.to_host(out_begin, out_end), "result copy");
    r = sync_stream(c, "score kernel");
    if (r != BBS_OK) return r;
    std::memcpy(scores, d_scores.h, sizeof(float) * n_trees);
    if (counts) std::memcpy(counts, d_counts.h, sizeof(uint64_t) * 4 * n_trees);
    if (attach) std::memcpy(attach, d_attach.h, sizeof(uint32_t) * n_attach);
    return BBS_OK;
  } catch (...) {
    return fail(BBS_ERR_ALLOC, "allocation failed in bbs_score_trees");
  }
}

int bbs_logscore_beta(const bbs_ctx *c, float beta, float *out) {
  if (!c || !out) return fail(BBS_ERR_INPUT, "NULL argument");
  float l01, l11;
  host_beta_terms(c->ds, beta, &l01, &l11, out);
  return BBS_OK;
}

int bbs_apply_moves(bbs_ctx *c, const uint64_t *dm, const float *betas,
                    uint32_t n_trees, const bbs_raw_move *raw,
                    const bbs_move_params *params,
                    bbs_move_params *params_out, uint64_t *dm_out,
                    float *beta_out) {
  try {
    if (!c || !dm || !betas || !dm_out) return fail(BBS_ERR_INPUT, "NULL argument");
    if (!raw && !params) return fail(BBS_ERR_INPUT, "need raw moves or move parameters");
    if (n_trees == 0) return BBS_OK;
    const uint32_t n = c->n_nodes;
    for (uint32_t t = 0; t < n_trees; t++) {
      const int type = raw ? raw[t].move_type : params[t].move_type;
      if (type < 0 || type > 3) return fail(BBS_ERR_INPUT, "move %u has type %d", t, type);
      if (raw && (raw[t].raw_v >= n || raw[t].raw_w >= n))
        return fail(BBS_ERR_INPUT, "move %u names a node >= %u", t, n);
      if (params) {
        const bbs_move_params &p = params[t];
        if (p.v >= n || p.w >= n || p.parent_of_v >= n || p.parent_of_w >= n ||
            p.descendant_of_v >= n || p.nondescendant_of_v >= n)
          return fail(BBS_ERR_INPUT, "move %u names a node >= %u", t, n);
      }
    }
    const size_t words = tree_words(c, n_trees);
    ScratchPlan plan;
    plan.add<uint64_t>(words);
    plan.add<float>(n_trees);
    if (raw)
      plan.add<bbs_raw_move>(n_trees);
    else
      plan.add<bbs_move_params>(n_trees);
    plan.add<uint64_t>(words);
    plan.add<float>(n_trees);
    plan.add<bbs_move_params>(n_trees);
    int r = plan.reserve(c);
    if (r != BBS_OK) return r;
    const auto rows = plan.take<uint64_t>(words);
    const auto in_betas = plan.take<float>(n_trees);
    const auto in_raw = plan.take<bbs_raw_move>(raw ? n_trees : 0);
    const auto in_par = plan.take<bbs_move_params>(raw ? 0 : n_trees);
    const size_t out_begin = plan.mark();
    const auto out_rows = plan.take<uint64_t>(words);
    const auto out_beta = plan.take<float>(n_trees);
    const auto out_par = plan.take<bbs_move_params>(n_trees);
    const size_t out_end = plan.mark();
    std::memcpy(rows.h, dm, sizeof(uint64_t) * words);
    std::memcpy(in_betas.h, betas, sizeof(float) * n_trees);
    if (raw)
      std::memcpy(in_raw.h, raw, sizeof(bbs_raw_move) * n_trees);
    else
      std::memcpy(in_par.h, params, sizeof(bbs_move_params) * n_trees);
    BBS_CUDA(plan.to_device(0, out_begin), "scratch upload");
    BBS_CUDA(cudaMemsetAsync(out_rows.d, 0, sizeof(uint64_t) * words, c->stream), "memset");
    ApplyArgs a{};
    a.n_nodes = (int)n;
    a.n_trees = (int)n_trees;
    a.rows = reinterpret_cast<const uint32_t *>(rows.d);
    a.betas = in_betas.d;
    a.raw = raw ? in_raw.d : nullptr;
    a.params = raw ? nullptr : in_par.d;
    a.params_out = out_par.d;
    a.rows_out = reinterpret_cast<uint32_t *>(out_rows.d);
    a.beta_out = out_beta.d;
    const int e = launch_apply(a, c->stream);
    if (e != 0) return cuda_fail(e, "apply kernel launch");
    BBS_CUDA(plan.to_host(out_begin, out_end), "result copy");
    r = sync_stream(c, "apply kernel");
    if (r != BBS_OK) return r;
    std::memcpy(dm_out, out_rows.h, sizeof(uint64_t) * words);
    if (beta_out) std::memcpy(beta_out, out_beta.h, sizeof(float) * n_trees);
    if (params_out)
      std::memcpy(params_out, out_par.h, sizeof(bbs_move_params) * n_trees);
    return BBS_OK;
  } catch (...) {
    return fail(BBS_ERR_ALLOC, "allocation failed in bbs_apply_moves");
  }
}

int bbs_sumscore_grad(bbs_ctx *c, const uint64_t *dm, const float *alphas,
                      const float *betas, uint32_t n_trees, float *logl,
                      float *dalpha, float *dbeta, float *posterior) {
  try {
    if (!c || !dm || !alphas || !betas || !logl)
      return fail(BBS_ERR_INPUT, "NULL argument");
    if (n_trees == 0) return BBS_OK;
    for (uint32_t t = 0; t < n_trees; t++) {
      const double a = alphas[t], b = betas[t];
      if (!(a > 0 && a < 1 && b > 0 && b < 1))
        return fail(BBS_ERR_INPUT, "error rates of tree %u outside (0, 1)", t);
    }
    const size_t words = tree_words(c, n_trees);
    const size_t n_post = (size_t)n_trees * c->n_cells * c->n_nodes;
    ScratchPlan plan;
    plan.add<uint64_t>(words);
    plan.add<float>(6 * (size_t)n_trees);
    plan.add<float>(3 * (size_t)n_trees);
    if (posterior) plan.add<float>(n_post);
    int r = plan.reserve(c);
    if (r != BBS_OK) return r;
    const auto rows = plan.take<uint64_t>(words);
    const auto tab = plan.take<float>(6 * (size_t)n_trees);
    const size_t out_begin = plan.mark();
    const auto out = plan.take<float>(3 * (size_t)n_trees);
    const auto post = plan.take<float>(posterior ? n_post : 0);
    const size_t out_end = plan.mark();
    std::memcpy(rows.h, dm, sizeof(uint64_t) * words);
    // per tree: alpha, beta, log(1-alpha), log beta, log alpha, log(1-beta)
    for (uint32_t t = 0; t < n_trees; t++) {
      const double a = alphas[t], b = betas[t];
      float *tt = tab.h + 6 * (size_t)t;
      tt[0] = alphas[t];
      tt[1] = betas[t];
      tt[2] = (float)std::log1p(-a);
      tt[3] = (float)std::log(b);
      tt[4] = (float)std::log(a);
      tt[5] = (float)std::log1p(-b);
    }
    BBS_CUDA(plan.to_device(0, out_begin), "scratch upload");
    GradArgs a{};
    a.ds = c->ds;
    a.rows = reinterpret_cast<const uint32_t *>(rows.d);
    a.tables = tab.d;
    a.n_trees = (int)n_trees;
    a.logl = out.d;
    a.dalpha = out.d + n_trees;
    a.dbeta = out.d + 2 * (size_t)n_trees;
    a.posterior = posterior ? post.d : nullptr;
    const int e = launch_grad(a, c->q, c->stream);
    if (e != 0) return cuda_fail(e, "adjoint kernel launch");
    BBS_CUDA(plan.to_host(out_begin, out_end), "result copy");
    r = sync_stream(c, "adjoint kernel");
    if (r != BBS_OK) return r;
    std::memcpy(logl, out.h, sizeof(float) * n_trees);
    if (dalpha) std::memcpy(dalpha, out.h + n_trees, sizeof(float) * n_trees);
    if (dbeta) std::memcpy(dbeta, out.h + 2 * (size_t)n_trees, sizeof(float) * n_trees);
    if (posterior) std::memcpy(posterior, post.h, sizeof(float) * n_post);
    return BBS_OK;
  } catch (...) {
    return fail(BBS_ERR_ALLOC, "allocation failed in bbs_sumscore_grad");
  }
}

int bbs_device_check_selftest(int *enabled, uint32_t *code, uint32_t *value,
                              uint32_t *limit) {
  if (!enabled || !code || !value || !limit)
    return fail(BBS_ERR_INPUT, "NULL argument");
  int *d = nullptr;
  BBS_CUDA(cudaMalloc(&d, sizeof(int) * kStatusWords), "cudaMalloc");
  int st[kStatusWords] = {};
  cudaError_t e = cudaMemset(d, 0, sizeof(st));
  if (e == cudaSuccess) e = (cudaError_t)run_check_selftest(d, enabled);
  if (e == cudaSuccess) e = cudaMemcpy(st, d, sizeof(st), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail((int)e, "device check self-test");
  *code = (st[0] & 2) ? (uint32_t)st[1] : 0u;
  *value = (uint32_t)st[2];
  *limit = (uint32_t)st[3];
  return BBS_OK;
}

int bbs_popc_peak(double *popc_per_s, double *sm_clock_hz) {
  if (!popc_per_s || !sm_clock_hz) return fail(BBS_ERR_INPUT, "NULL argument");
  const int e = run_popc_bench(popc_per_s, sm_clock_hz);
  if (e != 0) return cuda_fail(e, "popc benchmark");
  return BBS_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------
// Allocation-free scoring.  The per-tree log-table scratch of
// bbs_score_trees (beta, log beta, log(1-beta), Beta prior) lives in this
// file-scope device array instead of a cudaMalloc'd buffer.  Host code may
// not use the array's name as a device address: the address is looked up
// once per device with cudaGetSymbolAddress, with that device current, and
// passed to the kernel.  Each call overwrites the entries of its own trees
// before the kernel reads them, so nothing in the array has to start at
// zero.
// ------------------------------------------------------------------------
static __device__ __align__(256) float g_noalloc_terms[BBS_NOALLOC_MAX_TREES * 4];

namespace {

constexpr int kNoallocMaxDevices = 64;
std::mutex g_noalloc_mutex;
float *g_noalloc_ptr[kNoallocMaxDevices] = {};

// Device address of g_noalloc_terms on the current device (set up on the
// first call per device).
int noalloc_scratch(int device, float **out) {
  if (device < 0 || device >= kNoallocMaxDevices)
    return fail(BBS_ERR_SIZE, "device ordinal %d is not supported", device);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (g_noalloc_ptr[device] == nullptr) {
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_terms);
    if (e != cudaSuccess)
      return cuda_fail((int)e, "cudaGetSymbolAddress(scratch)");
    g_noalloc_ptr[device] = static_cast<float *>(ptr);
  }
  *out = g_noalloc_ptr[device];
  return BBS_OK;
}

}  // namespace

extern "C" int bbs_score_trees_noalloc(bbs_ctx *c, const uint64_t *dm_device,
                                       const float *betas, uint32_t n_trees,
                                       float *scores_device,
                                       uint64_t *counts_device) {
  if (!c || !dm_device || !betas || !scores_device)
    return fail(BBS_ERR_INPUT, "NULL argument to bbs_score_trees_noalloc");
  if (c->running) return fail(BBS_ERR_STATE, "a run is in progress");
  if (n_trees == 0) return BBS_OK;
  if (n_trees > BBS_NOALLOC_MAX_TREES)
    return fail(BBS_ERR_SIZE,
                "bbs_score_trees_noalloc takes at most %d trees per call "
                "(got %u): its scratch is a fixed %d-entry device array",
                BBS_NOALLOC_MAX_TREES, n_trees, BBS_NOALLOC_MAX_TREES);
  for (uint32_t t = 0; t < n_trees; t++)
    if (!(betas[t] > 0.0f && betas[t] < 1.0f))
      return fail(BBS_ERR_INPUT, "beta of tree %u outside (0, 1)", t);
  int device = -1;
  BBS_CUDA(cudaGetDevice(&device), "cudaGetDevice");
  if (device != c->device)
    return fail(BBS_ERR_STATE, "the context's device %d is not current (%d)",
                c->device, device);
  float *scratch = nullptr;
  int r = noalloc_scratch(device, &scratch);
  if (r != BBS_OK) return r;
  // Host log-table terms, staged through a fixed stack buffer.
  constexpr uint32_t kChunk = 512;
  float chunk[4 * kChunk];
  for (uint32_t t0 = 0; t0 < n_trees; t0 += kChunk) {
    const uint32_t nt = std::min(kChunk, n_trees - t0);
    for (uint32_t t = 0; t < nt; t++) {
      chunk[4 * t] = betas[t0 + t];
      host_beta_terms(c->ds, betas[t0 + t], &chunk[4 * t + 1],
                      &chunk[4 * t + 2], &chunk[4 * t + 3]);
    }
    BBS_CUDA(cudaMemcpyAsync(scratch + 4 * (size_t)t0, chunk,
                             sizeof(float) * 4 * nt, cudaMemcpyHostToDevice,
                             c->stream),
             "scratch upload");
  }
  ScoreArgs a{};
  a.ds = c->ds;
  a.rows = reinterpret_cast<const uint32_t *>(dm_device);
  a.beta_terms = scratch;
  a.n_trees = (int)n_trees;
  a.scores = scores_device;
  a.counts = counts_device;
  a.attach = nullptr;
  a.states = nullptr;
  const int e = launch_score(a, c->q, c->stream);
  if (e != 0) return cuda_fail(e, "score kernel launch");
  return sync_stream(c, "score kernel");
}


// ------------------------------------------------------------------------
// Many datasets in one launch
// ------------------------------------------------------------------------
struct bbs_batch {
  int device = 0, n_sms = 0;
  int smem_block = 0;  // dynamic shared memory a block may have (opt-in)
  cudaStream_t stream = nullptr;
  std::vector<cudaStream_t> side;  // one per launch group (graph branches)
  std::vector<cudaEvent_t> side_ev;
  cudaEvent_t fork = nullptr, ev0 = nullptr, ev1 = nullptr;
  uint32_t n_datasets = 0;
  std::vector<uint32_t> n_cells, n_genes;
  std::vector<DatasetDev> ds;
  std::vector<ModelDev> md;
  std::vector<float> terms;  // [n_datasets][8]
  bool sum = false;
  uint32_t *d_cells = nullptr;
  DatasetDev *d_ds = nullptr;
  ModelDev *d_md = nullptr;
  float *d_terms = nullptr;
  // chains
  uint32_t cpd = 0, n_chains = 0;
  std::vector<uint32_t> chain_ds;
  std::vector<uint64_t> chain_off;
  size_t row_words = 0;
  uint32_t *d_rows = nullptr, *d_best = nullptr;
  ChainState *d_states = nullptr;
  uint32_t *d_chain_ds = nullptr;
  uint64_t *d_chain_off = nullptr;
  // launch groups (row width), rebuilt when the shape changes
  struct Group {
    int w32 = 0, max_nodes = 0;
    int only_ds = -1;  // the group's dataset when it has only one
    std::vector<uint32_t> units;
    uint32_t *d_units = nullptr;
  };
  std::vector<Group> groups;
  unsigned int *d_counters = nullptr;
  int *d_status = nullptr;
  int q = 2, wpb = 4, merge = 0;
  int wpc = 1;  // warps per chain (above 1 a block is one chain)
  // graph of the current shape and step count
  cudaGraphExec_t graph = nullptr;
  uint32_t graph_steps = 0;
  float last_ms = 0.0f;
  uint64_t fingerprint = 0;  // of all datasets and parameters (checkpoints)
};

namespace {

void batch_free_groups(bbs_batch *b) {
  for (auto &g : b->groups) cudaFree(g.d_units);
  b->groups.clear();
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  b->graph_steps = 0;
}

void batch_free_chains(bbs_batch *b) {
  batch_free_groups(b);
  cudaFree(b->d_rows);
  cudaFree(b->d_best);
  cudaFree(b->d_states);
  cudaFree(b->d_chain_ds);
  cudaFree(b->d_chain_off);
  b->d_rows = b->d_best = nullptr;
  b->d_states = nullptr;
  b->d_chain_ds = nullptr;
  b->d_chain_off = nullptr;
  b->n_chains = 0;
}

// The chain layout of a batch with cpd chains per dataset: chain c of
// dataset d is c = d * cpd + k, and its rows start at chain_off[c]
// (32-bit words, 32-byte aligned).  Returns the row words of all chains.
size_t batch_layout(bbs_batch *b, uint32_t cpd) {
  const uint32_t n_chains = cpd * b->n_datasets;
  b->chain_ds.resize(n_chains);
  b->chain_off.resize(n_chains);
  size_t words = 0;
  for (uint32_t d = 0; d < b->n_datasets; d++)
    for (uint32_t k = 0; k < cpd; k++) {
      const uint32_t c = d * cpd + k;
      const uint32_t n = b->n_genes[d] + 1;
      b->chain_ds[c] = d;
      b->chain_off[c] = words;
      words += (size_t)n * 2 * words64(n);
      words = (words + 7) & ~(size_t)7;  // 32-byte aligned rows
    }
  b->row_words = words;
  return words;
}

// Device arrays of the layout batch_layout made (contents not set).
cudaError_t batch_alloc_chains(bbs_batch *b) {
  const size_t n_chains = b->chain_ds.size(), words = b->row_words;
  cudaError_t e = cudaMalloc(&b->d_rows, sizeof(uint32_t) * words);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_best, sizeof(uint32_t) * words);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_states, sizeof(ChainState) * n_chains);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_chain_ds, sizeof(uint32_t) * n_chains);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_chain_off, sizeof(uint64_t) * n_chains);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_chain_ds, b->chain_ds.data(), sizeof(uint32_t) * n_chains,
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_chain_off, b->chain_off.data(), sizeof(uint64_t) * n_chains,
                   cudaMemcpyHostToDevice);
  return e;
}

// Layout of a batch checkpoint: this header, then the current rows and
// the best rows (row_words 32-bit words each, in the batch_layout order)
// and the chain states (128 bytes each).
struct BatchCheckpointHeader {
  char magic[8];
  uint32_t version, header_bytes;
  uint64_t fingerprint;
  uint32_t n_datasets, chains_per_dataset;
  uint32_t state_bytes, reserved0;
  uint64_t row_words;
  uint64_t total_bytes;
  uint64_t reserved[2];
};
static_assert(sizeof(BatchCheckpointHeader) == 72, "batch checkpoint header layout");
constexpr char kBatchCheckpointMagic[8] = {'B', 'B', 'S', 'B', 'A', 'T', 'C', 'H'};

// Launch groups for the current shape: one per row width (exact, or the
// even width of its row stride with merge), chains costliest first.
int batch_build_groups(bbs_batch *b) {
  batch_free_groups(b);
  std::vector<int> key(b->n_datasets);
  for (uint32_t d = 0; d < b->n_datasets; d++) {
    int w = w32_of_nodes((int)b->n_genes[d] + 1);
    if (b->merge) w = rs_of_w32(w);
    key[d] = w;
  }
  for (int w = 1; w <= kMaxW32; w++) {
    bbs_batch::Group g;
    g.w32 = w;
    std::vector<std::pair<double, uint32_t>> cost;
    for (uint32_t c = 0; c < b->n_chains; c++) {
      const uint32_t d = b->chain_ds[c];
      if (key[d] != w) continue;
      const double groups = (b->n_cells[d] + 31) / 32;
      const double nodes = b->n_genes[d] + 1.0;
      cost.push_back({groups * nodes * w + 4.0 * nodes, c});
      g.max_nodes = std::max(g.max_nodes, (int)nodes);
    }
    if (cost.empty()) continue;
    std::stable_sort(cost.begin(), cost.end(),
                     [](const auto &x, const auto &y) { return x.first > y.first; });
    for (auto &p : cost) g.units.push_back(p.second);
    g.only_ds = (int)b->chain_ds[g.units[0]];
    for (const uint32_t u : g.units)
      if ((int)b->chain_ds[u] != g.only_ds) g.only_ds = -1;
    BBS_CUDA(cudaMalloc(&g.d_units, sizeof(uint32_t) * g.units.size()), "cudaMalloc");
    BBS_CUDA(cudaMemcpy(g.d_units, g.units.data(), sizeof(uint32_t) * g.units.size(),
                        cudaMemcpyHostToDevice), "cudaMemcpy");
    b->groups.push_back(std::move(g));
  }
  while (b->side.size() < b->groups.size()) {
    cudaStream_t s;
    cudaEvent_t ev;
    BBS_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
    BBS_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
    b->side.push_back(s);
    b->side_ev.push_back(ev);
  }
  return BBS_OK;
}

// Cells per lane of a launch group: 1 or 2 above 128 nodes.
int group_q(const bbs_batch *b, const bbs_batch::Group &grp) {
  return grp.w32 > 4 ? std::min(b->q, 2) : b->q;
}

// Warps per block of a launch group: with one-warp chains the batch's,
// within the kernel's bounds for the group's cells per lane (groups of
// more than 128 nodes take at most 2 cells per lane and so at most 4 warps
// per block); with several warps per chain the chain's (one per block).
int group_wpb(const bbs_batch *b, const bbs_batch::Group &grp) {
  if (b->wpc > 1) return b->wpc;
  return std::min(b->wpb, chain_max_threads(group_q(b, grp)) / 32);
}

// Whether the chains of a launch group inherit counts: rows of up to four
// words when the group has one dataset whose cells stay in registers (the
// block's increment tables hold that dataset's cells); wider rows always
// (each warp builds its gene table from the cells it scores).
bool group_counts(const bbs_batch *b, const bbs_batch::Group &grp) {
  if (grp.w32 > 4) return true;
  return grp.only_ds >= 0 &&
         inherits_counts(grp.w32, (int)b->n_cells[grp.only_ds],
                         32 * b->wpc * group_q(b, grp));
}

// Whether every launch group of the current shape fits a block: its shared
// memory within the device's limit (threads are clamped to the kernel's
// bounds by group_wpb).  Checked before a run launches anything.
bool batch_shape_fits(const bbs_batch *b) {
  for (const auto &grp : b->groups) {
    const int q = group_q(b, grp);
    const int slots = group_wpb(b, grp) / b->wpc;
    const bool counts = group_counts(b, grp);
    const int smem =
        slots * slot_bytes(grp.max_nodes, rs_of_w32(grp.w32), b->wpc,
                           b->sum || counts, grp.w32, q, counts) +
        table_bytes(grp.max_nodes, grp.w32, q, b->wpc, counts);
    if (smem > b->smem_block) return false;
  }
  return true;
}

// Issues one run: zero the work counters, then one launch per group on its
// own stream (forked from and joined back into b->stream).
int batch_issue(bbs_batch *b, uint32_t n_steps) {
  if (!batch_shape_fits(b))
    return fail(BBS_ERR_SIZE,
                "launch shape (%d cells per lane, %d warps per block) needs "
                "more threads or shared memory per block than the kernel or "
                "device allows",
                b->q, b->wpb);
  // one work counter per launch group (one group per row width)
  if (b->groups.size() > (size_t)kMaxW32)
    return fail(BBS_ERR_STATE, "%zu launch groups, at most %d", b->groups.size(),
                kMaxW32);
  BBS_CUDA(cudaMemsetAsync(b->d_counters, 0, sizeof(unsigned int) * kMaxW32,
                           b->stream), "memset");
  BBS_CUDA(cudaMemsetAsync(b->d_status, 0, sizeof(int) * kStatusWords, b->stream),
           "memset");
  BBS_CUDA(cudaEventRecord(b->fork, b->stream), "event");
  for (size_t g = 0; g < b->groups.size(); g++) {
    const auto &grp = b->groups[g];
    BBS_CUDA(cudaStreamWaitEvent(b->side[g], b->fork, 0), "wait");
    BatchArgs a{};
    a.ds = b->d_ds;
    a.md = b->d_md;
    a.chain_ds = b->d_chain_ds;
    a.chain_off = b->d_chain_off;
    a.units = grp.d_units;
    a.n_units = (int)grp.units.size();
    a.n_chains = (int)b->n_chains;
    a.n_datasets = (int)b->n_datasets;
    a.n_steps = (int)n_steps;
    a.chains_per_dataset = (int)b->cpd;
    a.rows = b->d_rows;
    a.best_rows = b->d_best;
    a.states = b->d_states;
    a.next_unit = b->d_counters + g;
    a.cancel = nullptr;
    a.status = b->d_status;
    a.max_nodes = grp.max_nodes;
    a.table_ds = grp.only_ds;
    const int q = group_q(b, grp);
    a.with_counts = group_counts(b, grp) ? 1 : 0;
    a.wpc = b->wpc;
    const int e = launch_batch(a, grp.w32, q, b->sum, group_wpb(b, grp),
                               b->n_sms, b->side[g]);
    if (e != 0) return cuda_fail(e, "batch kernel launch");
    BBS_CUDA(cudaEventRecord(b->side_ev[g], b->side[g]), "event");
    BBS_CUDA(cudaStreamWaitEvent(b->stream, b->side_ev[g], 0), "wait");
  }
  return BBS_OK;
}

}  // namespace

extern "C" {

int bbs_batch_create(bbs_batch **out, uint32_t n_datasets,
                     const uint32_t *n_cells, const uint32_t *n_genes,
                     const uint64_t *const *is_mutated,
                     const uint64_t *const *is_known,
                     const bbs_params *params) {
  try {
    if (!out || !n_cells || !n_genes || !is_mutated || !is_known || !params)
      return fail(BBS_ERR_INPUT, "NULL argument to bbs_batch_create");
    *out = nullptr;
    if (n_datasets < 1) return fail(BBS_ERR_INPUT, "need at least one dataset");
    bool sum = false;
    for (uint32_t d = 0; d < n_datasets; d++) {
      if (n_genes[d] < 2 || n_genes[d] > BBS_MAX_GENES)
        return fail(BBS_ERR_SIZE, "dataset %u: gene count %u outside [2, %d]", d,
                    n_genes[d], BBS_MAX_GENES);
      if (n_cells[d] < 1 || n_cells[d] > BBS_MAX_CELLS)
        return fail(BBS_ERR_SIZE, "dataset %u: cell count %u outside [1, %d]", d,
                    n_cells[d], BBS_MAX_CELLS);
      if (!is_mutated[d] || !is_known[d])
        return fail(BBS_ERR_INPUT, "dataset %u: NULL cell rows", d);
      const int r = check_params(&params[d]);
      if (r != BBS_OK) return r;
      if (d > 0 && params[d].score_mode != params[0].score_mode)
        return fail(BBS_ERR_INPUT, "all datasets of a batch share one score mode");
      sum = params[d].score_mode == BBS_SCORE_SUM;
    }
    int n_dev = 0;
    if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev < 1)
      return fail(BBS_ERR_CUDA, "no CUDA device is available");
    bbs_batch *b = new (std::nothrow) bbs_batch();
    if (!b) return fail(BBS_ERR_ALLOC, "out of host memory");
    b->n_datasets = n_datasets;
    b->n_cells.assign(n_cells, n_cells + n_datasets);
    b->n_genes.assign(n_genes, n_genes + n_datasets);
    b->sum = sum;
    cudaGetDevice(&b->device);
    cudaDeviceGetAttribute(&b->n_sms, cudaDevAttrMultiProcessorCount, b->device);
    cudaDeviceGetAttribute(&b->smem_block, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                           b->device);
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    std::vector<HostDataset> h(n_datasets);
    size_t words = 0;
    std::vector<size_t> off(n_datasets);
    for (uint32_t d = 0; d < n_datasets; d++) {
      prepare_dataset(&params[d], n_cells[d], n_genes[d], is_mutated[d],
                      is_known[d], h[d]);
      const uint64_t f = context_fingerprint(params[d], n_cells[d], n_genes[d],
                                             h[d].K, h[d].M);
      b->fingerprint = fnv1a_of(d == 0 ? 0xCBF29CE484222325ull : b->fingerprint, f);
      off[d] = words;
      words += 2 * h[d].K.size();  // uint32 words of K, then of M
      words = (words + 7) & ~(size_t)7;
    }
    if (e == cudaSuccess) e = cudaMalloc(&b->d_cells, sizeof(uint32_t) * 2 * std::max<size_t>(words, 1));
    b->ds.resize(n_datasets);
    b->md.resize(n_datasets);
    b->terms.resize(8 * (size_t)n_datasets);
    for (uint32_t d = 0; d < n_datasets && e == cudaSuccess; d++) {
      uint32_t *base = b->d_cells + 2 * off[d];
      const size_t kw = 2 * h[d].K.size();  // uint32 words of K
      e = cudaMemcpy(base, h[d].K.data(), sizeof(uint32_t) * kw, cudaMemcpyHostToDevice);
      if (e == cudaSuccess)
        e = cudaMemcpy(base + kw, h[d].M.data(), sizeof(uint32_t) * kw,
                       cudaMemcpyHostToDevice);
      h[d].ds.K = base;
      h[d].ds.M = base + kw;
      b->ds[d] = h[d].ds;
      b->md[d] = h[d].md;
      std::memcpy(&b->terms[8 * d], h[d].terms, sizeof(h[d].terms));
    }
    if (e == cudaSuccess) e = cudaMalloc(&b->d_ds, sizeof(DatasetDev) * n_datasets);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_md, sizeof(ModelDev) * n_datasets);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_terms, sizeof(float) * b->terms.size());
    if (e == cudaSuccess)
      e = cudaMemcpy(b->d_ds, b->ds.data(), sizeof(DatasetDev) * n_datasets,
                     cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(b->d_md, b->md.data(), sizeof(ModelDev) * n_datasets,
                     cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(b->d_terms, b->terms.data(), sizeof(float) * b->terms.size(),
                     cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_counters, sizeof(unsigned int) * kMaxW32);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_status, sizeof(int) * kStatusWords);
    if (e != cudaSuccess) {
      const int r = cuda_fail((int)e, "bbs_batch_create");
      bbs_batch_destroy(b);
      return r;
    }
    *out = b;
    return BBS_OK;
  } catch (...) {
    return fail(BBS_ERR_ALLOC, "allocation failed in bbs_batch_create");
  }
}

void bbs_batch_destroy(bbs_batch *b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  batch_free_chains(b);
  for (auto s : b->side) cudaStreamDestroy(s);
  for (auto ev : b->side_ev) cudaEventDestroy(ev);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  cudaFree(b->d_cells);
  cudaFree(b->d_ds);
  cudaFree(b->d_md);
  cudaFree(b->d_terms);
  cudaFree(b->d_counters);
  cudaFree(b->d_status);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

int bbs_batch_init_chains(bbs_batch *b, uint32_t cpd) {
  try {
    if (!b) return fail(BBS_ERR_INPUT, "NULL batch");
    if (cpd < 1) return fail(BBS_ERR_INPUT, "need at least one chain per dataset");
    batch_free_chains(b);
    const uint32_t n_chains = cpd * b->n_datasets;
    const size_t words = batch_layout(b, cpd);
    uint32_t max_nodes = 0;
    for (uint32_t d = 0; d < b->n_datasets; d++)
      max_nodes = std::max(max_nodes, b->n_genes[d] + 1);
    cudaError_t e = batch_alloc_chains(b);
    if (e == cudaSuccess)
      e = cudaMemsetAsync(b->d_rows, 0, sizeof(uint32_t) * words, b->stream);
    if (e == cudaSuccess)
      e = cudaMemsetAsync(b->d_best, 0, sizeof(uint32_t) * words, b->stream);
    if (e == cudaSuccess) {
      // every dataset's random initial trees, drawn on the device
      TreeArgs ta{};
      ta.ds = b->d_ds;
      ta.md = b->d_md;
      ta.chain_ds = b->d_chain_ds;
      ta.chain_off = b->d_chain_off;
      ta.chains_per_dataset = (int)cpd;
      ta.n_chains = (int)n_chains;
      ta.rows = b->d_rows;
      ta.max_nodes = (int)max_nodes;
      e = (cudaError_t)launch_trees(ta, b->stream);
    }
    if (e != cudaSuccess) {
      batch_free_chains(b);
      return cuda_fail((int)e, "bbs_batch_init_chains");
    }
    b->cpd = cpd;
    b->n_chains = n_chains;
    int r = batch_build_groups(b);
    if (r != BBS_OK) return r;
    for (const auto &g : b->groups) {
      InitArgs ia{};
      ia.ds = b->d_ds;
      ia.md = b->d_md;
      ia.chain_ds = b->d_chain_ds;
      ia.chain_off = b->d_chain_off;
      ia.terms = b->d_terms;
      ia.chain_list = g.d_units;
      ia.n_chains = (int)g.units.size();
      ia.rows = b->d_rows;
      ia.states = b->d_states;
      ia.max_nodes = g.max_nodes;
      const int le = launch_init(ia, g.w32, b->sum, b->stream);
      if (le != 0) return cuda_fail(le, "init kernel launch");
    }
    BBS_CUDA(cudaStreamSynchronize(b->stream), "init kernel");
    return BBS_OK;
  } catch (...) {
    return fail(BBS_ERR_ALLOC, "allocation failed in bbs_batch_init_chains");
  }
}

int bbs_batch_run(bbs_batch *b, uint32_t n_steps) {
  if (!b) return fail(BBS_ERR_INPUT, "NULL batch");
  if (b->n_chains == 0) return fail(BBS_ERR_STATE, "bbs_batch_init_chains was not called");
  if (n_steps == 0) return BBS_OK;
  if (n_steps > 0x7fffffffu) return fail(BBS_ERR_SIZE, "too many steps");
  if (b->graph == nullptr || b->graph_steps != n_steps) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    cudaGraph_t g = nullptr;
    BBS_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal),
             "begin capture");
    const int r = batch_issue(b, n_steps);
    const cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
    if (r != BBS_OK) {
      if (g) cudaGraphDestroy(g);
      return r;
    }
    BBS_CUDA(ce, "end capture");
    const cudaError_t ie = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    BBS_CUDA(ie, "graph instantiate");
    b->graph_steps = n_steps;
  }
  BBS_CUDA(cudaEventRecord(b->ev0, b->stream), "event");
  BBS_CUDA(cudaGraphLaunch(b->graph, b->stream), "graph launch");
  BBS_CUDA(cudaEventRecord(b->ev1, b->stream), "event");
  BBS_CUDA(cudaStreamSynchronize(b->stream), "batch run");
  BBS_CUDA(cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1), "event timing");
#ifdef BBS_CHECKED
  int status[kStatusWords] = {};
  BBS_CUDA(cudaMemcpy(status, b->d_status, sizeof(status), cudaMemcpyDeviceToHost),
           "status read");
  return status_result(status);
#else
  return BBS_OK;  // a batch run is never cancelled and checks nothing
#endif
}

int bbs_batch_last_run_ms(const bbs_batch *b, float *ms) {
  if (!b || !ms) return fail(BBS_ERR_INPUT, "NULL argument");
  *ms = b->last_ms;
  return BBS_OK;
}

int bbs_batch_set_launch(bbs_batch *b, int q, int wpb, int merge) {
  if (!b) return fail(BBS_ERR_INPUT, "NULL batch");
  if (q < 0 || q > 4)
    return fail(BBS_ERR_INPUT, "cells per lane must be 1, 2, 3 or 4");
  if (wpb < 0 || 32 * wpb > kMaxBlockThreads)
    return fail(BBS_ERR_INPUT, "warps per block must be in [1, %d]",
                kMaxBlockThreads / 32);
  if (q) b->q = q;
  if (wpb) b->wpb = wpb;
  if (merge >= 0 && merge != b->merge) {
    b->merge = merge ? 1 : 0;
    if (b->n_chains) {
      const int r = batch_build_groups(b);
      if (r != BBS_OK) return r;
    }
  }
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  return BBS_OK;
}

int bbs_batch_get_launch(const bbs_batch *b, int *q, int *wpb, int *merge) {
  if (!b) return fail(BBS_ERR_INPUT, "NULL batch");
  if (q) *q = b->q;
  if (wpb) *wpb = b->wpb;
  if (merge) *merge = b->merge;
  return BBS_OK;
}

int bbs_batch_set_chain_warps(bbs_batch *b, int warps_per_chain) {
  if (!b) return fail(BBS_ERR_INPUT, "NULL batch");
  if (warps_per_chain < 1 || warps_per_chain > 4)
    return fail(BBS_ERR_INPUT, "warps per chain must be 1, 2, 3 or 4");
  b->wpc = warps_per_chain;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  return BBS_OK;
}

int bbs_batch_get_chain_warps(const bbs_batch *b, int *warps_per_chain) {
  if (!b || !warps_per_chain) return fail(BBS_ERR_INPUT, "NULL argument");
  *warps_per_chain = b->wpc;
  return BBS_OK;
}

int bbs_batch_autotune(bbs_batch *b, uint32_t probe_steps, float *best_ms) {
  try {
    if (!b) return fail(BBS_ERR_INPUT, "NULL batch");
    if (b->n_chains == 0) return fail(BBS_ERR_STATE, "bbs_batch_init_chains was not called");
    if (probe_steps == 0) probe_steps = 64;
    const size_t rb = sizeof(uint32_t) * b->row_words;
    const size_t sb = sizeof(ChainState) * b->n_chains;
    DevBuf<uint8_t> sr, sbst, sst;
    BBS_CUDA(sr.alloc(rb), "cudaMalloc");
    BBS_CUDA(sbst.alloc(rb), "cudaMalloc");
    BBS_CUDA(sst.alloc(sb), "cudaMalloc");
    auto cp = [&](void *d, const void *s, size_t n) {
      return cudaMemcpyAsync(d, s, n, cudaMemcpyDeviceToDevice, b->stream);
    };
    BBS_CUDA(cp(sr.p, b->d_rows, rb), "save");
    BBS_CUDA(cp(sbst.p, b->d_best, rb), "save");
    BBS_CUDA(cp(sst.p, b->d_states, sb), "save");
    float best = 1e30f;
    int bq = b->q, bw = b->wpb, bm = b->merge, bc = b->wpc;
    // one-warp chains in blocks of 1-8, or one chain of 2 or 4 warps per
    // block (warps per block then = warps per chain)
    struct Shape {
      int wpb, wpc;
    };
    const Shape shapes[] = {{1, 1}, {2, 1}, {4, 1}, {7, 1}, {8, 1},
                            {2, 2}, {4, 4}};
    for (int merge : {0, 1})
      for (int q : {1, 2, 3, 4})
        for (const Shape &sh : shapes) {
          if (32 * sh.wpb > chain_max_threads(q)) continue;
          int r = bbs_batch_set_launch(b, q, sh.wpb, merge);
          if (r != BBS_OK) return r;
          r = bbs_batch_set_chain_warps(b, sh.wpc);
          if (r != BBS_OK) return r;
          if (!batch_shape_fits(b)) continue;  // too large a block
          BBS_CUDA(cudaEventRecord(b->ev0, b->stream), "event");
          r = batch_issue(b, probe_steps);
          if (r != BBS_OK) return r;
          BBS_CUDA(cudaEventRecord(b->ev1, b->stream), "event");
          BBS_CUDA(cudaStreamSynchronize(b->stream), "probe");
          float ms = 0;
          BBS_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1), "timing");
          if (ms < best) {
            best = ms;
            bq = q;
            bw = sh.wpb;
            bm = merge;
            bc = sh.wpc;
          }
          BBS_CUDA(cp(b->d_rows, sr.p, rb), "restore");
          BBS_CUDA(cp(b->d_best, sbst.p, rb), "restore");
          BBS_CUDA(cp(b->d_states, sst.p, sb), "restore");
        }
    int r = bbs_batch_set_launch(b, bq, bw, bm);
    if (r == BBS_OK) r = bbs_batch_set_chain_warps(b, bc);
    BBS_CUDA(cudaStreamSynchronize(b->stream), "restore");
    if (best_ms) *best_ms = best;
    return r;
  } catch (...) {
    return fail(BBS_ERR_ALLOC, "allocation failed in bbs_batch_autotune");
  }
}

int bbs_batch_get_best(bbs_batch *b, uint32_t dataset, uint64_t *dm,
                       uint32_t *parent, float *alpha, float *beta,
                       float *score) {
  try {
    if (!b) return fail(BBS_ERR_INPUT, "NULL batch");
    if (b->n_chains == 0) return fail(BBS_ERR_STATE, "no chains");
    if (dataset >= b->n_datasets) return fail(BBS_ERR_INPUT, "no dataset %u", dataset);
    std::vector<ChainState> st(b->cpd);
    const uint32_t c0 = dataset * b->cpd;
    BBS_CUDA(cudaMemcpy(st.data(), b->d_states + c0, sizeof(ChainState) * b->cpd,
                        cudaMemcpyDeviceToHost), "state copy");
    int best = -1;
    for (uint32_t k = 0; k < b->cpd; k++) {
      if (!st[k].has_best) continue;
      if (best < 0 || st[k].best_score > st[best].best_score) best = (int)k;
    }
    if (best < 0) return fail(BBS_ERR_STATE, "no steps have been run");
    const uint32_t n = b->n_genes[dataset] + 1;
    std::vector<uint64_t> rows((size_t)n * words64(n));
    BBS_CUDA(cudaMemcpy(rows.data(), b->d_best + b->chain_off[c0 + best],
                        sizeof(uint64_t) * rows.size(), cudaMemcpyDeviceToHost),
             "best copy");
    if (dm) std::memcpy(dm, rows.data(), sizeof(uint64_t) * rows.size());
    if (parent) matrix_to_parent(rows.data(), n, parent);
    if (alpha) *alpha = st[best].best_alpha;
    if (beta) *beta = st[best].best_beta;
    if (score) *score = st[best].best_score;
    return BBS_OK;
  } catch (...) {
    return fail(BBS_ERR_ALLOC, "allocation failed in bbs_batch_get_best");
  }
}

int bbs_batch_save_chains(bbs_batch *b, void *buf, size_t *size) {
  try {
    if (!b || !size) return fail(BBS_ERR_INPUT, "NULL argument");
    if (b->n_chains == 0) return fail(BBS_ERR_STATE, "no chains");
    const size_t rows = sizeof(uint32_t) * b->row_words;
    const size_t states = sizeof(ChainState) * b->n_chains;
    const size_t total = sizeof(BatchCheckpointHeader) + 2 * rows + states;
    if (!buf) {
      *size = total;
      return BBS_OK;
    }
    if (*size < total) {
      const size_t have = *size;
      *size = total;
      return fail(BBS_ERR_SIZE, "checkpoint needs %zu bytes, buffer has %zu",
                  total, have);
    }
    BatchCheckpointHeader hd{};
    std::memcpy(hd.magic, kBatchCheckpointMagic, sizeof(hd.magic));
    hd.version = kCheckpointVersion;
    hd.header_bytes = sizeof(hd);
    hd.fingerprint = b->fingerprint;
    hd.n_datasets = b->n_datasets;
    hd.chains_per_dataset = b->cpd;
    hd.state_bytes = sizeof(ChainState);
    hd.row_words = b->row_words;
    hd.total_bytes = total;
    uint8_t *p = static_cast<uint8_t *>(buf);
    std::memcpy(p, &hd, sizeof(hd));
    p += sizeof(hd);
    BBS_CUDA(cudaStreamSynchronize(b->stream), "batch stream");
    BBS_CUDA(cudaMemcpy(p, b->d_rows, rows, cudaMemcpyDeviceToHost), "checkpoint copy");
    BBS_CUDA(cudaMemcpy(p + rows, b->d_best, rows, cudaMemcpyDeviceToHost),
             "checkpoint copy");
    BBS_CUDA(cudaMemcpy(p + 2 * rows, b->d_states, states, cudaMemcpyDeviceToHost),
             "checkpoint copy");
    *size = total;
    return BBS_OK;
  } catch (...) {
    return fail(BBS_ERR_ALLOC, "allocation failed in bbs_batch_save_chains");
  }
}

int bbs_batch_load_chains(bbs_batch *b, const void *buf, size_t size) {
  try {
    if (!b || !buf) return fail(BBS_ERR_INPUT, "NULL argument");
    BatchCheckpointHeader hd;
    if (size < sizeof(hd)) return fail(BBS_ERR_INPUT, "checkpoint too short");
    std::memcpy(&hd, buf, sizeof(hd));
    if (std::memcmp(hd.magic, kBatchCheckpointMagic, sizeof(hd.magic)) != 0)
      return fail(BBS_ERR_INPUT, "not a batch checkpoint");
    if (hd.version != kCheckpointVersion || hd.header_bytes != sizeof(hd) ||
        hd.state_bytes != sizeof(ChainState))
      return fail(BBS_ERR_INPUT, "checkpoint version %u is not supported",
                  hd.version);
    if (hd.fingerprint != b->fingerprint || hd.n_datasets != b->n_datasets)
      return fail(BBS_ERR_INPUT,
                  "the checkpoint was made with other datasets or other "
                  "parameters");
    const uint32_t cpd = hd.chains_per_dataset;
    if (cpd < 1 || (uint64_t)cpd * b->n_datasets * sizeof(ChainState) > size)
      return fail(BBS_ERR_INPUT, "checkpoint of %u chains per dataset does not "
                  "fit in %zu bytes", cpd, size);
    // the layout of cpd chains per dataset, on a scratch copy of the batch's
    // tables so that a refused image leaves the batch as it was
    bbs_batch probe;
    probe.n_datasets = b->n_datasets;
    probe.n_genes = b->n_genes;
    const size_t words = batch_layout(&probe, cpd);
    const uint32_t n_chains = cpd * b->n_datasets;
    const size_t rows = sizeof(uint32_t) * words;
    const size_t states = sizeof(ChainState) * n_chains;
    const size_t total = sizeof(hd) + 2 * rows + states;
    if (hd.row_words != words || hd.total_bytes != total || size < total)
      return fail(BBS_ERR_INPUT, "checkpoint size %zu, expected %zu", size, total);
    const uint8_t *p = static_cast<const uint8_t *>(buf) + sizeof(hd);
    std::vector<ChainState> st(n_chains);
    std::memcpy(st.data(), p + 2 * rows, states);
    std::vector<uint32_t> pv;
    std::vector<uint64_t> tmp;
    for (uint32_t c = 0; c < n_chains; c++) {
      const uint32_t n = b->n_genes[probe.chain_ds[c]] + 1;
      const uint64_t *cur =
          reinterpret_cast<const uint64_t *>(p) + probe.chain_off[c] / 2;
      const uint64_t *bst =
          reinterpret_cast<const uint64_t *>(p + rows) + probe.chain_off[c] / 2;
      if (!valid_tree_rows(cur, n, pv, tmp))
        return fail(BBS_ERR_INPUT, "checkpoint chain %u holds no valid tree", c);
      if (st[c].has_best > 1 || st[c].list_count > 1)
        return fail(BBS_ERR_INPUT, "checkpoint chain %u has a bad state", c);
      if (st[c].has_best && !valid_tree_rows(bst, n, pv, tmp))
        return fail(BBS_ERR_INPUT, "checkpoint chain %u holds no valid best tree", c);
    }
    BBS_CUDA(cudaStreamSynchronize(b->stream), "batch stream");
    batch_free_chains(b);
    batch_layout(b, cpd);
    cudaError_t e = batch_alloc_chains(b);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_rows, p, rows, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_best, p + rows, rows, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy(b->d_states, st.data(), states, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      batch_free_chains(b);
      return cuda_fail((int)e, "bbs_batch_load_chains");
    }
    b->cpd = cpd;
    b->n_chains = n_chains;
    return batch_build_groups(b);
  } catch (...) {
    return fail(BBS_ERR_ALLOC, "allocation failed in bbs_batch_load_chains");
  }
}

}  // extern "C"
