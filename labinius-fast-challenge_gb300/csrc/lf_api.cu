// Host side of the prover: the C ABI, device buffers, the Fiat-Shamir transcript and the phase
// pipeline of one proof (solution/proof_generate/src/main.rs:1692-2009; the checker's
// reference prover verifier/proof_verify/src/reference.rs:137-177 fixes every byte).
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

#include "../../include/labinius_gpu.h"
#include "lf_blake3.cuh"
#include "lf_internal.h"
#include "lf_ring.h"

using namespace lf;

namespace {

// ---------------------------------------------------------------------------------------------
// Shape and modulus rules (verifier/proof_verify/src/main.rs:50-96, rq.rs:17-48)
// ---------------------------------------------------------------------------------------------
const u128 MIN_MODULUS = 34816965049ull;
const u128 MAX_MODULUS = (u128)1 << 96;

u128 q_from_le(const uint8_t* b) {
  u128 q = 0;
  for (int i = 15; i >= 0; --i) q = (q << 8) | b[i];
  return q;
}
uint32_t modulus_bits(u128 q) {
  u128 x = q - 1;
  uint32_t n = 0;
  while (x) ++n, x >>= 1;
  return n;
}
size_t coefficient_bytes(u128 q) { return (modulus_bits(q) + 7) / 8; }

uint64_t fold_cap(const Shape& s) {  // main.rs:62-64, FOLD_CAP = 108 (recursion/mod.rs:81)
  return (uint64_t)std::ceil(108.0 * (double)(((uint64_t)1 << s.lp) / 4 * RING_N));
}
uint64_t isqrt_u64(uint64_t x) {
  uint64_t r = (uint64_t)std::sqrt((double)x);
  while (r * r > x) --r;
  while ((r + 1) * (r + 1) <= x) ++r;
  return r;
}
bool accept_modulus(u128 q, const Shape& s) {
  return q >= MIN_MODULUS && q > (u128)2 * isqrt_u64(fold_cap(s)) && q < MAX_MODULUS;
}

size_t proof_size(u128 q, const Shape& s) {
  return 4 + 16 + 8 + coefficient_bytes(q) * COLUMNS * RING_N + 8 + 16 * 128 + 8 + 48 * (size_t)s.lp + 24 + 8 +
         (COLUMNS * 162 + 7) / 8 + 8 + 4 * RING_N * s.ring_elements;
}

// ---------------------------------------------------------------------------------------------
// Transcript (solution-arm/labinius/crates/pcs/src/challenge.rs:226-341)
// ---------------------------------------------------------------------------------------------
struct Transcript {
  bk::Hasher h;
  uint64_t counter = 0;
  void init(const char* domain) {
    h.init();
    counter = 0;
    absorb_bytes(domain, strlen(domain));
  }
  void absorb_bytes(const void* p, size_t n) {
    h.absorb_u64(n);
    h.absorb((const uint8_t*)p, n);
  }
  void absorb_u64(uint64_t x) { h.absorb_u64(x); }
  void absorb_b128(const b128* xs, size_t n) {
    h.absorb_u64(n);
    for (size_t i = 0; i < n; ++i) {
      h.absorb_u64(xs[i].lo);
      h.absorb_u64(xs[i].hi);
    }
  }
  void absorb_f162(const f162* xs, size_t n) {
    h.absorb_u64(n);
    for (size_t i = 0; i < n; ++i) {
      h.absorb_u64(xs[i].w0);
      h.absorb_u64(xs[i].w1);
      h.absorb_u64(xs[i].w2);
    }
  }
  bk::Pending derive(const char* label) { return bk::derive_root(h, counter++, label, (uint32_t)strlen(label)); }
  void fill(const char* label, uint8_t* out, size_t n) { derive(label).root_bytes(0, out, n); }
  std::vector<b128> sample_b128(const char* label, size_t n) {
    std::vector<uint8_t> b(16 * n);
    fill(label, b.data(), b.size());
    std::vector<b128> o(n);
    memcpy(o.data(), b.data(), b.size());
    return o;
  }
  std::vector<f162> sample_f162(const char* label, size_t n) {
    std::vector<uint8_t> b(24 * n);
    fill(label, b.data(), b.size());
    std::vector<f162> o(n);
    memcpy(o.data(), b.data(), b.size());
    for (auto& x : o) x.w2 &= F162_TOP_MASK;
    return o;
  }
};

std::vector<b128> eq_expand_b128(const std::vector<b128>& r) {  // crossfield.rs:81-137
  std::vector<b128> t((size_t)1 << r.size());
  t[0] = {1, 0};
  for (size_t round = 0; round < r.size(); ++round)
    for (size_t i = ((size_t)1 << round); i-- > 0;) {
      b128 hi = b128_mul(t[i], r[round]);
      t[2 * i + 1] = hi;
      t[2 * i] = b128_add(t[i], hi);
    }
  return t;
}
std::vector<f162> eq_expand_f162(const std::vector<f162>& r) {  // crossfield.rs:67-79
  std::vector<f162> t(1, f162{1, 0, 0});
  for (auto& ri : r) {
    std::vector<f162> n;
    n.reserve(t.size() * 2);
    for (auto& x : t) {
      f162 hi = f162_mul(x, ri);
      n.push_back(f162_add(x, hi));
      n.push_back(hi);
    }
    t.swap(n);
  }
  return t;
}

// pack_f162 (wire/mod.rs:445-452): 162 bits per element, least significant first.
void pack_f162(const std::vector<f162>& v, uint8_t* out) {
  size_t bytes = (v.size() * 162 + 7) / 8;
  memset(out, 0, bytes);
  size_t bit = 0;
  auto put = [&](uint64_t x, int n) {
    for (int i = 0; i < n; ++i, ++bit)
      if ((x >> i) & 1) out[bit >> 3] |= (uint8_t)(1u << (bit & 7));
  };
  for (auto& x : v) put(x.w0, 64), put(x.w1, 64), put(x.w2, 34);
}

// ---------------------------------------------------------------------------------------------
// Device buffers
// ---------------------------------------------------------------------------------------------
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  cudaError_t ensure(size_t n) {
    if (n <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) cap = n;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <class T>
  T* as() const {
    return reinterpret_cast<T*>(p);
  }
};

// Stream-ordered scratch: allocated and freed on one stream from the device's memory pool, so
// freeing it does not wait for the whole device (a cudaFree would, stalling the other lanes and a
// table upload running on the copy stream).
struct StreamBuf {
  void* p = nullptr;
  cudaStream_t s;
  explicit StreamBuf(cudaStream_t st) : s(st) {}
  StreamBuf(const StreamBuf&) = delete;
  StreamBuf& operator=(const StreamBuf&) = delete;
  ~StreamBuf() {
    if (p) cudaFreeAsync(p, s);
  }
  cudaError_t alloc(size_t n) { return cudaMallocAsync(&p, n, s); }
  template <class T>
  T* as() const {
    return reinterpret_cast<T*>(p);
  }
};

// The commitment key of one (Q, ring elements per column): built once on the device, kept.
struct KeyCache {
  u128 q = 0;
  uint64_t elements = 0;
  int extra_bits = 0;  // lift margin beyond a binary witness (the verifier's a_times_v: 15)
  uint64_t last_use = 0;
  ModulusPlan mp;
  DevBuf key;     // u32 [prime][element][leaf][k][l]: the 4x4 base-multiplication matrix per leaf
  DevBuf btiles;  // bf16 [prime][third][64 x 256]: Vandermonde limbs of the commitment kernel
  DevBuf consts;  // PrimeConst [prime]: the plan's per-prime constants, read by every kernel of the key
  size_t bytes() const { return key.cap + btiles.cap + consts.cap; }
};
constexpr size_t MAX_KEYS = 12;  // shapes cached per context (log_vars 19..30 fit)

// The factor-tree plan of one ring modulus for lf_ring_mul, with its prime constants on the device.
struct RingCache {
  u128 q = 0;
  RingPlan plan;
  DevBuf rps;
};
constexpr size_t MAX_RINGS = 8;

}  // namespace

struct lf_ctx {
  int device = 0;
  int sms = 0;
  size_t budget = 0;
  cudaStream_t stream = nullptr;
  std::mutex mu;
  std::mutex errmu;  // err is written by worker threads and read by the caller
  std::string err;
  lf_profile prof{};
  std::vector<std::unique_ptr<KeyCache>> keys;  // per shape, least recently used evicted first
  std::vector<std::unique_ptr<RingCache>> rings;  // lf_ring_mul plans, oldest evicted first
  KeyCache* key = nullptr;                      // the key of the proof in progress
  uint64_t key_clock = 0;
  DevBuf table, stream_buf, partial, sblk, ehi, elo, rhi, vparts, psi, batch, soa, msg, p0, eqt, row,
      hasher, chal, fold, cvs, cvs_scratch, subtrees, status, phase, scratch_small, wbuf, rbuf;
  uint32_t sign_key[8];
  std::vector<uint8_t> host_fold;
  cudaEvent_t ev[16];
  // batches: a second table buffer and a copy stream, so the next table uploads during a proof
  DevBuf table2, fold_strips, fold_part;
  DevBuf kb_ared, kb_leaf, kb_matrix;  // key-build scratch (matrix residues, leaf values, XOF blocks)
  // element splits of the commitment per (log_vars, primes) chosen by lf_tune; the wave-balance
  // heuristic otherwise
  std::map<std::pair<int, int>, int> tuned_splits;
  int split_for(const Shape& sh, int nprimes) const {
    auto it = tuned_splits.find({sh.log_vars, nprimes});
    return it != tuned_splits.end() ? it->second : commit_splits(sh.ring_elements, nprimes, sms);
  }
  // column runs of the fold per log_vars chosen by lf_tune; the wave-balance heuristic otherwise
  std::map<int, int> tuned_fold;
  int fold_split_for(const Shape& sh) const {
    auto it = tuned_fold.find(sh.log_vars);
    return it != tuned_fold.end() ? it->second : fold_splits(sh.ring_elements, sms);
  }
  // switch rounds: msg (device) accumulates a round's message, msg_out (page-locked, mapped) receives
  // it from the last block of the round's kernel
  unsigned long long* msg_out = nullptr;
  unsigned long long* msg_out_dev = nullptr;
  int nlanes = 8;                // proofs in flight at once: this context and nlanes - 1 lanes
  std::vector<lf_ctx*> lanes;    // contexts on the same device (own stream, buffers, keys)
  std::mutex lanemu;             // guards lanes (created on first use, only added to)
  bool is_lane = false;          // this context is another context's lane
  cudaStream_t upload_stream = nullptr;
  cudaEvent_t uploaded[2] = {nullptr, nullptr};
  // lf_prove from host memory: the proof buffer's pages are first touched by the device on this
  // stream (pageable memory on a device that reads it through the host's page tables), while the
  // commitment runs; the first device write into the buffer waits for `touched`.
  cudaStream_t touch_stream = nullptr;
  cudaEvent_t touched = nullptr, up_t0 = nullptr, up_t1 = nullptr;
  int pageable_access = 0;
  // lf_prove from page-locked memory: the table goes up in parts (element ranges of every column)
  // and the copy stream writes the proof's epoch into ready[i] after part i (a stream memory
  // operation: no kernel, so it cannot wait behind the commitment's blocks); the commitment starts
  // at once and each block waits for the part it reads.
  uint32_t* ready = nullptr;  // device, TABLE_PARTS flags
  uint32_t epoch = 0;
  // Test hooks (lf_test_set_point, lf_test_withhold_table_part), used by the next proof only.
  std::vector<b128> test_hi;          // r_hi to use instead of the sampled one (empty: none)
  int test_withhold = -1;             // a streamed table part whose ready flag is not written
  long long test_ready_wait = 0;      // SM cycles the commitment waits for a part (0: its default)
  CUresult (*write_value)(CUstream, CUdeviceptr, cuuint32_t, unsigned int) = nullptr;
  // serving: FIFO of submitted jobs, drained by one worker thread per lane
  struct Queued {
    uint64_t ticket;
    lf_job job;
    std::chrono::steady_clock::time_point submitted;
    size_t need;  // device footprint while in flight
  };
  struct Outcome {
    bool done = false;
    lf_result result{};
  };
  std::vector<std::thread> workers;  // one per lane, this context first
  int inflight = 0;             // requests being proven, and their footprint
  size_t inflight_bytes = 0;
  std::mutex qmu;
  std::condition_variable qcv;
  std::deque<Queued> queue;
  std::map<uint64_t, Outcome> outcomes;
  uint64_t next_ticket = 1;
  bool stopping = false;
};

namespace {

constexpr int TABLE_PARTS = 64;       // at most this many parts of a page-locked host table (lf_prove)
constexpr int TABLE_MIN_PARTS = 16;   // a host table streams when its columns have this many elements
constexpr int TABLE_FIRST_PARTS = 3;  // queued before the commitment's launch

int fail(lf_ctx* c, int code, const std::string& msg) {
  if (c) {
    std::lock_guard<std::mutex> g(c->errmu);
    c->err = msg;
  }
  return code;
}

#define CKL(label)                                                                                 \
  do {                                                                                             \
    cudaError_t e_ = cudaGetLastError();                                                           \
    if (e_ != cudaSuccess) return fail(ctx, LF_E_CUDA, std::string(label) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define CK(expr)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (expr);                                                                       \
    if (e_ != cudaSuccess)                                                                         \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? LF_E_OOM : LF_E_CUDA,                     \
                  std::string(#expr) + ": " + cudaGetErrorString(e_));                             \
  } while (0)

// The phase table of the canonical-embedding test (challenge.rs:525-540):
// PHASE[p][k] = exp(2 pi i p u_k / 243) over the first 81 units u_k, 88 lanes per row.
void phase_tables(std::vector<double>& re, std::vector<double>& im) {
  re.assign(162 * 88, 0.0);
  im.assign(162 * 88, 0.0);
  int units[162], n = 0;
  for (int x = 1; x < 243; ++x)
    if (x % 3) units[n++] = x;
  for (int p = 0; p < 162; ++p)
    for (int k = 0; k < 81; ++k) {
      int m = (p * units[k]) % 243;
      volatile double two_pi = 2.0 * M_PI;
      double angle = two_pi * (double)m;
      angle = angle / 243.0;
      re[p * 88 + k] = cos(angle);
      im[p * 88 + k] = sin(angle);
    }
}

// The challenge sampler's tables in one device buffer: PHASE re and im as f64 (the reference's
// arithmetic) and the same values rounded to f32 (the sampler's fast norm estimate).
cudaError_t upload_phase_tables(void* dst) {
  std::vector<double> re, im;
  phase_tables(re, im);
  std::vector<float> re32(re.begin(), re.end()), im32(im.begin(), im.end());
  uint8_t* d = static_cast<uint8_t*>(dst);
  const size_t n = 162 * 88;
  cudaError_t e = cudaMemcpy(d, re.data(), n * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + n * 8, im.data(), n * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + n * 16, re32.data(), n * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d + n * 20, im32.data(), n * 4, cudaMemcpyHostToDevice);
  return e;
}

// Device bytes one proof at this shape may hold beyond the cached keys: the table (when it is
// copied from the host), the commitment's split partial sums, the partial-sum blocks, the
// transcript stream, the fold output and the smaller work buffers, plus the transient buffers of
// a key build. Used for admission against the context's HBM budget.
size_t proof_footprint(const Shape& sh, bool host_table, int sms, int nprimes) {
  const size_t key = (size_t)nprimes * sh.ring_elements * LEAVES * 64;
  const size_t build = (size_t)nprimes * sh.ring_elements * (RING_N + 4 * LEAVES) * 4 +
                       matrix_scratch_bytes(sh.ring_elements, ~(u128)0 >> 32);  // widest coefficients
  const size_t partial =
      (size_t)commit_splits(sh.ring_elements, nprimes, sms) * nprimes * COLUMNS * LEAVES * 16;
  const size_t blocks = (sh.words / 4096) * (128 * 16 + 16);
  const size_t stream = STREAM_PREFIX + (size_t)12 * COLUMNS * RING_N + 1024;
  const size_t fold = (size_t)4 * RING_N * sh.ring_elements;
  const size_t small = (size_t)16 << 20;
  return (host_table ? sh.words * 16 : 0) + key + build + partial + blocks + stream + fold + small;
}

// Primes of the commitment for modulus q (3 for the baseline, else about one per 14.9 bits of
// the coefficient bound).
int primes_for(u128 q, const Shape& sh) {
  if (q == (u128)3889 * 9721 * 17497) return 3;
  const double bits = std::log2((double)sh.ring_elements) + std::log2(1296.0) + std::log2((double)(q - 1)) + 1.0;
  return std::min(MAX_PRIMES, (int)std::ceil(bits / 14.9));
}

int admit(lf_ctx* ctx, u128 q, const Shape& sh, bool host_table) {
  if (ctx->budget == 0) return LF_OK;
  const size_t need = proof_footprint(sh, host_table, ctx->sms, primes_for(q, sh));
  if (need > ctx->budget)
    return fail(ctx, LF_E_ADMISSION, "request needs " + std::to_string(need >> 20) + " MiB of device memory, budget " +
                                         std::to_string(ctx->budget >> 20) + " MiB");
  return LF_OK;
}

int ensure_key(lf_ctx* ctx, u128 q, const Shape& sh, int extra_bits = 0) {
  ctx->key = nullptr;
  for (auto& k : ctx->keys)
    if (k->q == q && k->elements == sh.ring_elements && (k->extra_bits == extra_bits || !k->mp.exact_lift))
      ctx->key = k.get();
  if (!ctx->key) {
    std::string e;
    ModulusPlan mp;
    if (!make_modulus_plan(q, sh.ring_elements, extra_bits, mp, e)) return fail(ctx, LF_E_MODULUS, e);
    // Evict least recently used shapes: beyond the count limit, or while the cached keys and
    // this proof would exceed the budget.
    auto cached = [&]() {
      size_t b = 0;
      for (auto& k : ctx->keys) b += k->bytes();
      return b;
    };
    const size_t need = proof_footprint(sh, true, ctx->sms, mp.nprimes);
    while (!ctx->keys.empty() &&
           (ctx->keys.size() >= MAX_KEYS || (ctx->budget && cached() + need > ctx->budget))) {
      auto oldest = std::min_element(ctx->keys.begin(), ctx->keys.end(),
                                     [](const std::unique_ptr<KeyCache>& a, const std::unique_ptr<KeyCache>& b) {
                                       return a->last_use < b->last_use;
                                     });
      ctx->keys.erase(oldest);
    }
    std::unique_ptr<KeyCache> kc(new KeyCache());
    const uint64_t E = sh.ring_elements;
    // key-build scratch stays with the context (grown, never freed mid-run: a cudaFree would wait
    // for the whole device, including a table upload on the copy stream and the other lanes)
    DevBuf& ared = ctx->kb_ared;
    DevBuf& leaf = ctx->kb_leaf;
    DevBuf& mscratch = ctx->kb_matrix;
    CK(ared.ensure((size_t)mp.nprimes * E * RING_N * 4));
    CK(leaf.ensure((size_t)mp.nprimes * E * 4 * LEAVES * 4));
    CK(mscratch.ensure(matrix_scratch_bytes(E, q)));
    CK(kc->key.ensure((size_t)mp.nprimes * E * LEAVES * 16 * 4));
    CK(kc->btiles.ensure(mp.btiles.size() * 2));
    CK(cudaMemcpyAsync(kc->btiles.p, mp.btiles.data(), mp.btiles.size() * 2, cudaMemcpyHostToDevice, ctx->stream));
    CK(kc->consts.ensure(sizeof(PrimeConst) * mp.nprimes));
    CK(cudaMemcpyAsync(kc->consts.p, mp.consts.data(), sizeof(PrimeConst) * mp.nprimes, cudaMemcpyHostToDevice,
                       ctx->stream));
    mp.dconsts = kc->consts.as<PrimeConst>();
    launch_matrix_expand(mp, E, ared.as<uint32_t>(), mscratch.p, ctx->stream);
    launch_key_transform(mp, E, ared.as<uint32_t>(), leaf.as<uint32_t>(), kc->key.as<uint32_t>(), ctx->stream);
    CKL("key build");
    CK(cudaStreamSynchronize(ctx->stream));
    kc->mp = mp;
    kc->q = q;
    kc->elements = E;
    kc->extra_bits = extra_bits;
    ctx->keys.push_back(std::move(kc));
    ctx->key = ctx->keys.back().get();
  }
  ctx->key->last_use = ++ctx->key_clock;
  return LF_OK;
}

// Every work buffer a proof of this shape and modulus grows to (the sizes prove_device and the
// functions it calls ask for), grown now: a proof whose buffers are already this large allocates
// nothing, so no cudaFree (a device-wide wait) stalls the other lanes or a table upload mid-batch.
int reserve_buffers(lf_ctx* ctx, u128 q, const Shape& sh, int nprimes, bool host_table) {
  const size_t commit_bytes = coefficient_bytes(q) * COLUMNS * RING_N;
  const uint64_t nblocks = 1ull << (sh.lp - 12), xmax = nblocks;
  const uint64_t nchunks = (STREAM_PREFIX + commit_bytes - 1) / 1024;
  const size_t fold_bytes = 4 * RING_N * sh.ring_elements;
  if (host_table) CK(ctx->table.ensure(sh.words * 16));
  CK(ctx->partial.ensure((size_t)ctx->split_for(sh, nprimes) * nprimes * COLUMNS * LEAVES * 4 * 4));
  CK(ctx->stream_buf.ensure(STREAM_PREFIX + commit_bytes + 1024));
  CK(ctx->status.ensure(16));
  CK(ctx->cvs.ensure(nchunks * 32 + 32));
  CK(ctx->cvs_scratch.ensure(2 * nchunks * 32 + 64));
  CK(ctx->subtrees.ensure(64 * 32));
  CK(ctx->rhi.ensure(64 * 16));
  CK(ctx->elo.ensure(4096 * 16));
  CK(ctx->ehi.ensure(nblocks * 16));
  CK(ctx->sblk.ensure(nblocks * 128 * 16));
  CK(ctx->vparts.ensure(256 * 8));
  CK(ctx->batch.ensure(2 * 128 * 24));
  CK(ctx->psi.ensure(2 * 16 * 256 * 24));
  CK(ctx->soa.ensure(6 * 4096 * 8));
  CK(ctx->wbuf.ensure(2 * xmax * 24 + 48));
  CK(ctx->rbuf.ensure((xmax > 2 ? xmax : 2) * 128 * 16));
  CK(ctx->p0.ensure(64 * 24));
  CK(ctx->eqt.ensure(sh.column_len * 24));
  CK(ctx->row.ensure(COLUMNS * 24));
  CK(ctx->hasher.ensure(sizeof(bk::Hasher)));
  CK(ctx->chal.ensure(COLUMNS * sizeof(Challenge)));
  CK(ctx->fold.ensure(fold_bytes));
  CK(ctx->fold_strips.ensure(COLUMNS * FOLD_STRIP_BYTES));
  CK(ctx->fold_part.ensure((size_t)fold_splits(sh.ring_elements, ctx->sms) * fold_bytes));
  return LF_OK;
}

float ev_ms(lf_ctx* ctx, int a, int b) {
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev[a], ctx->ev[b]);
  return ms;
}

void put_u64(uint8_t* p, uint64_t x) { memcpy(p, &x, 8); }

// v[c] = sum_j bit_c(pi0[j]) eq(r_hi)[j] over the table (crossfield.rs:548-573): GF(2) products
// per block of 4096 words against E_lo on the tensor cores, then 2^(LP-12) GHASH products with
// E_hi. Shared by the prover and the verifier's trusted recomputation (main.rs:308-320).
int device_partials(lf_ctx* ctx, const uint4* table, const Shape& sh, const std::vector<b128>& hi,
                    std::vector<b128>& partials) {
  cudaStream_t st = ctx->stream;
  const int LB = 12, HB = sh.lp - 12;
  const uint64_t nblocks = 1ull << HB;
  CK(ctx->rhi.ensure(64 * 16));
  CK(ctx->elo.ensure(4096 * 16));
  CK(ctx->ehi.ensure(nblocks * 16));
  CK(ctx->sblk.ensure(nblocks * 128 * 16));
  CK(ctx->vparts.ensure(256 * 8));
  CK(ctx->status.ensure(16));
  CK(cudaMemcpyAsync(ctx->rhi.p, hi.data(), 16 * hi.size(), cudaMemcpyHostToDevice, st));
  launch_eq_b128(ctx->rhi.as<b128>() + HB, LB, ctx->elo.as<b128>(), st);
  launch_eq_b128(ctx->rhi.as<b128>(), HB, ctx->ehi.as<b128>(), st);
  launch_sblock(table, nblocks, ctx->elo.as<b128>(), ctx->sblk.as<uint8_t>(), ctx->status.as<int>(), st);
  CK(cudaMemsetAsync(ctx->vparts.p, 0, 256 * 8, st));
  launch_partials_combine(ctx->ehi.as<b128>(), ctx->sblk.as<uint8_t>(), (int)nblocks,
                          ctx->vparts.as<unsigned long long>(), st);
  CKL("partials");
  partials.assign(128, b128{0, 0});
  CK(cudaMemcpyAsync(partials.data(), ctx->vparts.p, 128 * 16, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return LF_OK;
}

// The transcript up to and including the commitment (main.rs:166-174): domain, seed, LOG_VARS,
// COLUMN_LOG, Q and the length are the first STREAM_PREFIX bytes of chunk 0; the commitment's
// chunks are hashed on the device (chaining values, then the complete subtrees) and the stack is
// handed to the host hasher with the last partial chunk. The commitment is either already in
// ctx->stream_buf after the prefix (the prover's K2 wrote it there; commit_host == nullptr) or is
// copied there from commit_host (the checker). commit_out, when set, receives its bytes.
int absorb_commitment(lf_ctx* ctx, Transcript& t, const uint8_t* seed, const Shape& sh, u128 q, uint64_t commit_bytes,
                      const uint8_t* commit_host, uint8_t* commit_out) {
  cudaStream_t st = ctx->stream;
  t.init("labinius-fast/v1");
  t.absorb_bytes(seed, 32);
  t.absorb_u64((uint64_t)sh.log_vars);
  t.absorb_u64((uint64_t)COLUMN_LOG);
  uint8_t qb[16];
  for (int i = 0; i < 16; ++i) qb[i] = (uint8_t)(q >> (8 * i));
  t.absorb_bytes(qb, 16);
  t.absorb_u64(commit_bytes);
  uint8_t prefix[STREAM_PREFIX];
  {
    bk::Hasher probe = t.h;
    if (probe.depth != 0 || probe.chunk.size() != STREAM_PREFIX)
      return fail(ctx, LF_E_INTERNAL, "unexpected transcript prefix length");
    size_t o = 0;
    auto u64 = [&](uint64_t x) { put_u64(prefix + o, x), o += 8; };
    u64(16);
    memcpy(prefix + o, "labinius-fast/v1", 16), o += 16;
    u64(32);
    memcpy(prefix + o, seed, 32), o += 32;
    u64((uint64_t)sh.log_vars);
    u64((uint64_t)COLUMN_LOG);
    u64(16);
    memcpy(prefix + o, qb, 16), o += 16;
    u64(commit_bytes);
  }
  CK(ctx->stream_buf.ensure(STREAM_PREFIX + commit_bytes + 1024));
  CK(cudaMemcpyAsync(ctx->stream_buf.p, prefix, STREAM_PREFIX, cudaMemcpyHostToDevice, st));
  if (commit_host)
    CK(cudaMemcpyAsync(ctx->stream_buf.as<uint8_t>() + STREAM_PREFIX, commit_host, commit_bytes, cudaMemcpyHostToDevice,
                       st));
  const uint64_t total = STREAM_PREFIX + commit_bytes;
  const uint64_t nchunks = (total - 1) / 1024;
  CK(ctx->cvs.ensure(nchunks * 32 + 32));
  CK(ctx->cvs_scratch.ensure(2 * nchunks * 32 + 64));
  CK(ctx->subtrees.ensure(64 * 32));
  launch_chunk_cvs(ctx->stream_buf.as<uint8_t>(), nchunks, t.h.key, t.h.mode, ctx->cvs.as<uint32_t>(), st);
  launch_subtrees(ctx->cvs.as<uint32_t>(), ctx->cvs_scratch.as<uint32_t>(), nchunks, t.h.key, t.h.mode,
                  ctx->subtrees.as<uint32_t>(), st);
  CKL("transcript hashing");
  uint32_t sub[64][8];
  uint8_t tail[1024];
  const int depth = __builtin_popcountll(nchunks);
  const uint64_t tail_len = total - nchunks * 1024;
  CK(cudaMemcpyAsync(sub, ctx->subtrees.p, depth * 32, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(tail, ctx->stream_buf.as<uint8_t>() + nchunks * 1024, tail_len, cudaMemcpyDeviceToHost, st));
  if (commit_out)
    CK(cudaMemcpyAsync(commit_out, ctx->stream_buf.as<uint8_t>() + STREAM_PREFIX, commit_bytes, cudaMemcpyDeviceToHost,
                       st));
  CK(cudaStreamSynchronize(st));
  t.h.depth = depth;
  for (int d = 0; d < depth; ++d) memcpy(t.h.stack[d], sub[d], 32);
  t.h.chunk.start(t.h.key, nchunks, t.h.mode);
  t.h.chunk.absorb(tail, tail_len);
  return LF_OK;
}

// The proof of one table already on the device.
// The copy stream and the touch stream of a context, with their events (created on first use).
int side_streams(lf_ctx* ctx) {
  if (ctx->upload_stream) return LF_OK;
  CK(cudaStreamCreateWithFlags(&ctx->upload_stream, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&ctx->touch_stream, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&ctx->uploaded[0], cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&ctx->uploaded[1], cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&ctx->touched, cudaEventDisableTiming));
  CK(cudaEventCreate(&ctx->up_t0));
  CK(cudaEventCreate(&ctx->up_t1));
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult qr{};
  if (cudaGetDriverEntryPointByVersion("cuStreamWriteValue32", &fn, 12000, cudaEnableDefault, &qr) == cudaSuccess &&
      qr == cudaDriverEntryPointSuccess && fn && cudaMalloc(&ctx->ready, TABLE_PARTS * 4) == cudaSuccess &&
      cudaMemset(ctx->ready, 0, TABLE_PARTS * 4) == cudaSuccess) {
    ctx->write_value = reinterpret_cast<CUresult (*)(CUstream, CUdeviceptr, cuuint32_t, unsigned int)>(fn);
  }
  cudaGetLastError();
  return LF_OK;
}


// A table still being copied in parts (lf_prove from page-locked memory): the commitment reads part
// i once ready[i] holds epoch; every later reader waits for `done`.
struct TableStream {
  const uint32_t* ready;
  uint32_t epoch;
  int part_elems;
  cudaEvent_t done;
  const uint8_t* host;  // the page-locked table
  size_t pitch;         // bytes of one column
  uint64_t elements;    // ring elements per column
  int next;             // parts not yet queued: order[next .. nparts)
  int withhold;         // a part whose flag is left unset (test hook), else -1
  long long wait;       // SM cycles the commitment waits for a part (0: its default)
  int nparts;           // parts of part_elems elements (the last one shorter)
  uint8_t order[TABLE_PARTS];  // the copy order of the parts (order_table_parts)
};

// The parts of a streamed table of `elements` ring elements per column: up to TABLE_PARTS ranges of
// at least 16 elements (1 KB rows of the 2-D copy; shorter rows copy slowly and cost a batch of
// small tables 13 % of its throughput), the last one shorter.
void table_parts(uint64_t elements, int* part_elems, int* nparts) {
  const uint64_t want = std::max<uint64_t>(1, std::min<uint64_t>(TABLE_PARTS, elements / 16));
  *part_elems = (int)((elements + want - 1) / want);
  *nparts = (int)((elements + *part_elems - 1) / *part_elems);
}

// Queues parts order[ts->next .. end) of a streamed table on the copy stream, each followed by its
// ready flag; once every part is queued, `done` (and the upload's end) is recorded after them.
int enqueue_table_parts(lf_ctx* ctx, TableStream* ts, int end) {
  end = std::min(end, ts->nparts);
  for (int n = ts->next; n < end; ++n) {
    const int i = ts->order[n];
    const uint64_t m0 = (uint64_t)i * ts->part_elems, m1 = std::min<uint64_t>(ts->elements, m0 + ts->part_elems);
    if (m0 < m1)
      CK(cudaMemcpy2DAsync(ctx->table.as<uint8_t>() + 64 * m0, ts->pitch, ts->host + 64 * m0, ts->pitch, 64 * (m1 - m0),
                           COLUMNS, cudaMemcpyHostToDevice, ctx->upload_stream));
    if (i == ts->withhold) continue;  // a test hook: the commitment's wait for this part runs out
    if (ctx->write_value(reinterpret_cast<CUstream>(ctx->upload_stream), reinterpret_cast<CUdeviceptr>(ctx->ready + i),
                         ts->epoch, CU_STREAM_WRITE_VALUE_DEFAULT) != CUDA_SUCCESS)
      return fail(ctx, LF_E_CUDA, "stream write of a table part's ready flag failed");
  }
  if (end > ts->next) ts->next = end;
  if (ts->next >= ts->nparts) {
    CK(cudaEventRecord(ctx->uploaded[0], ctx->upload_stream));
    CK(cudaEventRecord(ctx->up_t1, ctx->upload_stream));
  }
  return LF_OK;
}

// A pageable proof buffer on a device that reaches host memory through the host's page tables:
// while the commitment runs, a kernel on the touch stream writes one byte per 4 KB page, so the
// proof's own copies into the buffer find its pages already mapped for the device (a first
// device access to a page is slow). *ready is the event the first device write into the buffer
// must wait for, or stays null (page-locked or otherwise registered memory needs no touch).
int touch_proof_buffer(lf_ctx* ctx, uint8_t* proof, size_t len, cudaEvent_t* ready) {
  *ready = nullptr;
  cudaPointerAttributes pa{};
  if (ctx->pageable_access && len && cudaPointerGetAttributes(&pa, proof) == cudaSuccess &&
      pa.type == cudaMemoryTypeUnregistered) {
    int rc = side_streams(ctx);
    if (rc) return rc;
    launch_touch_pages(proof, len, ctx->touch_stream);
    CKL("proof buffer touch");
    CK(cudaEventRecord(ctx->touched, ctx->touch_stream));
    *ready = ctx->touched;
  }
  cudaGetLastError();  // cudaPointerGetAttributes on plain host memory leaves no error behind
  return LF_OK;
}

// A switch round's message: the round's last block writes the six words into msg_out and then
// sets msg_out[7] (system-scope release). arm_round_message clears the flag before the launch;
// read_round_message spins on it and reads the message as soon as it lands, which saves the
// kernel's and the stream's completion on each of the host's Fiat-Shamir round trips. The spin
// asks the stream every few thousand tries: once the stream has finished (or failed) without the
// flag, the stream's own status decides, so a failed launch never leaves the host spinning.
void arm_round_message(lf_ctx* ctx) {
  __atomic_store_n(ctx->msg_out + 7, 0ull, __ATOMIC_SEQ_CST);
}

cudaError_t read_round_message(lf_ctx* ctx, cudaStream_t st, f162 m[2]) {
  for (unsigned tries = 1;; ++tries) {
    if (__atomic_load_n(ctx->msg_out + 7, __ATOMIC_ACQUIRE)) {
      memcpy(m, ctx->msg_out, 48);
      return cudaSuccess;
    }
    if ((tries & 4095) == 0 && cudaStreamQuery(st) != cudaErrorNotReady) break;
  }
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  if (!__atomic_load_n(ctx->msg_out + 7, __ATOMIC_ACQUIRE)) return cudaErrorUnknown;
  memcpy(m, ctx->msg_out, 48);
  return cudaSuccess;
}

// The copy order of a streamed table's parts: by when the commitment's blocks first read them.
// The commitment's grid runs its element splits in order, blocks_per_split blocks each, about sms
// blocks at a time, and a block reads its split's elements in order at a steady rate, so element m
// of split z is first read about wave(z) + (m - m0(z)) / per waves after the launch. Parts go up
// in the order of their first element's time (part 0 first, already queued): the first wave's
// blocks, which start at several places in the table, all find their first parts early.
void order_table_parts(TableStream* ts, int splits, int blocks_per_split, int sms) {
  const int n = ts->nparts;
  const uint64_t E = ts->elements, per = (E + splits - 1) / splits;
  std::vector<double> need(n, 1e300);
  for (int z = 0; z < splits; ++z) {
    const uint64_t m0 = (uint64_t)z * per, m1 = std::min<uint64_t>(E, m0 + per);
    if (m0 >= m1) continue;
    const double wave = std::floor((double)z * blocks_per_split / std::max(1, sms));
    for (uint64_t p = m0 / ts->part_elems; p < (uint64_t)n && p * ts->part_elems < m1; ++p) {
      const uint64_t e = std::max<uint64_t>(m0, p * ts->part_elems);
      need[p] = std::min(need[p], wave + (double)(e - m0) / (double)per);
    }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin() + ts->next, idx.end(), [&](int a, int b) { return need[a] < need[b]; });
  for (int i = ts->next; i < n; ++i) ts->order[i] = (uint8_t)idx[i];
}

// table_ready (may be null): an event the prover's stream waits for before the first kernel that
// reads the table. With ts, the commitment starts before the table is complete (table_ready is
// then unused). touch: `proof` is host memory that may need touch_proof_buffer (done while the
// commitment runs).
int prove_device(lf_ctx* ctx, const uint8_t seed[32], u128 q, const Shape& sh, const uint4* table, uint8_t* proof,
                 size_t* proof_len, cudaEvent_t table_ready = nullptr, bool touch = false,
                 TableStream* ts = nullptr) {
  cudaStream_t st = ctx->stream;
  const size_t width = coefficient_bytes(q);
  const size_t commit_bytes = width * COLUMNS * RING_N;
  const size_t plen = proof_size(q, sh);
  // Proof layout offsets (main.rs:99-117, bincode fixint).
  const size_t at_commit = 28;
  const size_t at_partials = at_commit + commit_bytes + 8;
  const size_t at_rounds = at_partials + 16 * 128 + 8;
  const size_t at_opened = at_rounds + 48 * sh.lp;
  const size_t at_row = at_opened + 24 + 8;
  const size_t row_bytes = (COLUMNS * 162 + 7) / 8;
  const size_t at_fold = at_row + row_bytes + 8;
  const size_t fold_bytes = 4 * RING_N * sh.ring_elements;

  cudaEventRecord(ctx->ev[1], st);
  int rc = ensure_key(ctx, q, sh);
  if (rc) return rc;
  cudaEventRecord(ctx->ev[2], st);

  // ---- commitment (K1 + K2), written after the 112 transcript prefix bytes of the stream ----
  const int splits = ctx->split_for(sh, ctx->key->mp.nprimes);
  const ModulusPlan& mp = ctx->key->mp;
  CK(ctx->partial.ensure((size_t)splits * mp.nprimes * COLUMNS * LEAVES * 4 * 4));
  CK(ctx->stream_buf.ensure(STREAM_PREFIX + commit_bytes + 1024));
  CK(ctx->status.ensure(16));
  CK(cudaMemsetAsync(ctx->status.p, 0, 16, st));
  // (One commitment launch: splitting it by element ranges, so that each starts as its part of a
  // host table arrives, cost it its wave balance: 4 launches of about 5 splits each ran 1.4 ms
  // longer than one launch at 2^31 bits.)
  if (ts) {
    order_table_parts(ts, splits, commit_blocks_per_split(mp), ctx->sms);
    if ((rc = enqueue_table_parts(ctx, ts, TABLE_FIRST_PARTS))) return rc;
    launch_commit(mp, sh, table, ctx->key->key.as<uint32_t>(), ctx->key->btiles.as<uint16_t>(),
                  ctx->partial.as<uint32_t>(), splits, ctx->status.as<int>(), st, 0, -1, ts->ready, ts->epoch,
                  ts->part_elems, ts->wait);
    // the parts after the first few are queued only now, off the commitment's critical path
    if ((rc = enqueue_table_parts(ctx, ts, ts->nparts))) return rc;
    CK(cudaStreamWaitEvent(st, ts->done, 0));  // every later kernel reads the whole table
  } else {
    if (table_ready) CK(cudaStreamWaitEvent(st, table_ready, 0));
    launch_commit(mp, sh, table, ctx->key->key.as<uint32_t>(), ctx->key->btiles.as<uint16_t>(),
                  ctx->partial.as<uint32_t>(), splits, ctx->status.as<int>(), st);
  }
  cudaEventRecord(ctx->ev[11], st);
  launch_commit_finish(mp, sh, ctx->partial.as<uint32_t>(), splits, ctx->stream_buf.as<uint8_t>() + STREAM_PREFIX, st);
  CKL("commitment");
  cudaEventRecord(ctx->ev[3], st);

  // ---- transcript (main.rs:166-174): the prefix on the host, the commitment's chunks on the device ----
  Transcript t;
  cudaEvent_t proof_ready = nullptr;
  if (touch && (rc = touch_proof_buffer(ctx, proof, plen, &proof_ready))) return rc;
  if (proof_ready) CK(cudaStreamWaitEvent(st, proof_ready, 0));
  rc = absorb_commitment(ctx, t, seed, sh, q, commit_bytes, nullptr, proof + at_commit);
  if (rc) return rc;
  cudaEventRecord(ctx->ev[4], st);

  // ---- point and partials (main.rs:177-189; crossfield.rs:548-573) ----
  std::vector<b128> lo = t.sample_b128("r-lo", 7);
  std::vector<b128> hi = t.sample_b128("r-hi", sh.lp);
  if (!ctx->test_hi.empty()) {  // lf_test_set_point: this proof runs at the given coordinates
    if (ctx->test_hi.size() != hi.size()) return fail(ctx, LF_E_ARGS, "test point has the wrong number of coordinates");
    hi.swap(ctx->test_hi);
    ctx->test_hi.clear();
  }
  const int HB = sh.lp - 12;
  std::vector<b128> partials;
  if ((rc = device_partials(ctx, table, sh, hi, partials))) return rc;
  cudaEventRecord(ctx->ev[5], st);
  b128 claim = {0, 0};
  {
    std::vector<b128> e = eq_expand_b128(lo);
    for (int i = 0; i < 128; ++i) claim = b128_add(claim, b128_mul(partials[i], e[i]));
  }
  t.absorb_b128(&claim, 1);
  t.absorb_b128(partials.data(), 128);
  std::vector<f162> batch = eq_expand_f162(t.sample_f162("switch-batch", 7));

  // ---- switch rounds (reference.rs:150-161; sumcheck.rs:128-251) ----
  // Rounds r < HB from the partials' blocks folded bottom-up (no table read), then one table
  // pass materialises the folded polynomial on the trailing 12 variables, and the last 12 rounds
  // run on those 4096 entries.
  const uint64_t nsmall = 4096;
  const uint64_t xmax = 1ull << HB;
  CK(ctx->batch.ensure(2 * 128 * 24));
  CK(ctx->psi.ensure(2 * 16 * 256 * 24));
  CK(ctx->soa.ensure(6 * nsmall * 8));
  CK(ctx->wbuf.ensure(2 * xmax * 24 + 48));
  CK(ctx->rbuf.ensure((xmax > 2 ? xmax : 2) * 128 * 16));
  f162* G[2] = {ctx->batch.as<f162>(), ctx->batch.as<f162>() + 128};
  f162* W[2] = {ctx->wbuf.as<f162>(), ctx->wbuf.as<f162>() + xmax + 1};
  const f162 one = {1, 0, 0};
  CK(cudaMemcpyAsync(G[0], batch.data(), 128 * 24, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(W[0], &one, 24, cudaMemcpyHostToDevice, st));
  // R_k for k = 1 .. HB - 1 (R_0 is the block array itself).
  std::vector<const b128*> R(HB > 0 ? HB : 1);
  if (HB > 0) R[0] = ctx->sblk.as<b128>();
  {
    size_t off = 0;
    for (int k = 0; k + 1 < HB; ++k) {
      const uint64_t nout = 1ull << (HB - k - 1);
      b128* dst = ctx->rbuf.as<b128>() + off;
      launch_rblock_level(R[k], nout, hi[HB - 1 - k], dst, st);
      R[k + 1] = dst;
      off += nout * 128;
    }
  }
  int launches = HB > 1 ? HB - 1 : 0;
  std::vector<f162> coords, rounds;
  int cur = 0;
  f162* PSI[2] = {ctx->psi.as<f162>(), ctx->psi.as<f162>() + 16 * 256};  // byte tables of Phi_r, Phi_r+1
  launch_psi_tables(G[0], PSI[0], st);
  ++launches;
  for (int r = 0; r < HB; ++r) {
    const uint64_t X = 1ull << r;
    arm_round_message(ctx);
    launch_switch_round_blocks(R[HB - 1 - r], X, hi[r], PSI[cur], W[cur],
                               ctx->msg.as<unsigned long long>(), ctx->msg_out_dev, ctx->sms, st);
    f162 m[2];
    CK(read_round_message(ctx, st, m));
    t.absorb_f162(m, 2);
    f162 rr = t.sample_f162("switch-round", 1)[0];
    rounds.push_back(m[0]);
    rounds.push_back(m[1]);
    coords.push_back(rr);
    launch_round_update(PSI[cur], hi[r], rr, PSI[cur ^ 1], W[cur], X, W[cur ^ 1], st);
    cur ^= 1;
    launches += 2;
  }
  CKL("switch rounds on blocks");
  cudaEventRecord(ctx->ev[14], st);
  uint64_t* sb = ctx->soa.as<uint64_t>();
  Soa A = {sb, sb + nsmall, sb + 2 * nsmall}, P = {sb + 3 * nsmall, sb + 4 * nsmall, sb + 5 * nsmall};
  launch_phi_apply(ctx->elo.as<b128>(), nsmall, PSI[cur], A, st);
  CK(cudaMemsetAsync(P.w0, 0, 3 * nsmall * 8, st));
  launch_materialize(table, W[cur], xmax, P, ctx->sms, st);
  launches += 2;
  CKL("switch materialisation");
  cudaEventRecord(ctx->ev[15], st);
  // The last rounds on the 4096 entries: each launch folds a round and computes the next
  // round's message (the last fold alone).
  uint64_t half = nsmall >> 1;
  if (HB < sh.lp) {
    arm_round_message(ctx);
    launch_switch_msg(A, P, half, ctx->msg.as<unsigned long long>(), ctx->msg_out_dev, ctx->sms, st);
    ++launches;
  }
  for (int r = HB; r < sh.lp; ++r, half >>= 1) {
    f162 m[2];
    CK(read_round_message(ctx, st, m));
    t.absorb_f162(m, 2);
    f162 rr = t.sample_f162("switch-round", 1)[0];
    rounds.push_back(m[0]);
    rounds.push_back(m[1]);
    coords.push_back(rr);
    if (r + 1 < sh.lp) {
      arm_round_message(ctx);
      launch_switch_fold_msg(A, P, half, rr, ctx->msg.as<unsigned long long>(), ctx->msg_out_dev, ctx->sms, st);
    } else {
      launch_switch_fold(A, P, half, rr, ctx->sms, st);
    }
    ++launches;
  }
  CKL("switch rounds");
  f162 opened;
  CK(cudaMemcpyAsync(&opened.w0, P.w0, 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&opened.w1, P.w1, 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&opened.w2, P.w2, 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  cudaEventRecord(ctx->ev[6], st);
  t.absorb_f162(&opened, 1);

  // ---- row evaluation (reference.rs:163-164; main.rs:253-264) ----
  std::vector<f162> p0(coords.rbegin(), coords.rend() - COLUMN_LOG);
  CK(ctx->p0.ensure(64 * 24));
  CK(ctx->eqt.ensure(sh.column_len * 24));
  CK(ctx->row.ensure(COLUMNS * 24));
  CK(cudaMemcpyAsync(ctx->p0.p, p0.data(), 24 * p0.size(), cudaMemcpyHostToDevice, st));
  launch_eq_table_f162(ctx->p0.as<f162>(), sh.rl, ctx->eqt.as<f162>(), st);
  launch_row_eval(table, sh.rl, ctx->eqt.as<f162>(), ctx->row.as<f162>(), ctx->sms, st);
  CKL("row evaluation");
  std::vector<f162> row(COLUMNS);
  CK(cudaMemcpyAsync(row.data(), ctx->row.p, COLUMNS * 24, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  cudaEventRecord(ctx->ev[7], st);
  {  // RowEvaluation::absorb (scheme/commitment.rs:320-331)
    const char* label = "labinius/row-evaluation";
    t.absorb_bytes(label, strlen(label));
    t.absorb_bytes(row.data(), row.size() * 24);
  }

  // ---- folding challenges (main.rs:281-292) on the device ----
  CK(ctx->hasher.ensure(sizeof(bk::Hasher)));
  CK(ctx->chal.ensure(COLUMNS * sizeof(Challenge)));
  CK(ctx->status.ensure(16));
  CK(cudaMemcpyAsync(ctx->hasher.p, &t.h, sizeof(bk::Hasher), cudaMemcpyHostToDevice, st));
  // status[0] was zeroed before the commitment: 3 = commitment pipeline timeout, 1 = sampling
  // bound, 2 = fold range.
  CK(launch_challenges(ctx->hasher.p, t.counter, ctx->sign_key, ctx->phase.p, ctx->chal.as<Challenge>(), COLUMNS,
                       ctx->status.as<int>(), st));
  t.counter += COLUMNS;
  CKL("challenges");
  cudaEventRecord(ctx->ev[8], st);

  // ---- fold (reference.rs:72-133), straight into the proof's i32 region ----
  CK(ctx->fold.ensure(fold_bytes));
  const int fsplits = ctx->fold_split_for(sh);
  CK(ctx->fold_strips.ensure(COLUMNS * FOLD_STRIP_BYTES));
  CK(ctx->fold_part.ensure((size_t)fsplits * fold_bytes));
  launch_fold(table, sh.rl, sh.ring_elements, ctx->chal.as<Challenge>(), ctx->fold_strips.as<uint8_t>(),
              ctx->fold_part.as<int32_t>(), fsplits, ctx->fold.as<int32_t>(), ctx->status.as<int>(), st);
  CKL("fold");
  cudaEventRecord(ctx->ev[9], st);
  CK(cudaMemcpyAsync(proof + at_fold, ctx->fold.p, fold_bytes, cudaMemcpyDeviceToHost, st));
  int status[4];
  CK(cudaMemcpyAsync(status, ctx->status.p, 16, cudaMemcpyDeviceToHost, st));
  cudaEventRecord(ctx->ev[10], st);
  CK(cudaStreamSynchronize(st));
  if (status[0] == 1) return fail(ctx, LF_E_INTERNAL, "challenge sampling exceeded its attempt bound");
  if (status[0] == 2) return fail(ctx, LF_E_INTERNAL, "a fold coefficient does not fit the wire codec");
  if (status[0] == 3) return fail(ctx, LF_E_INTERNAL, "the commitment kernel's pipeline timed out");
  if (status[0] == 4) return fail(ctx, LF_E_INTERNAL, "the partial-sum kernel's pipeline timed out");
  if (status[0] == 5) return fail(ctx, LF_E_INTERNAL, "the fold kernel's pipeline timed out");
  if (status[0] != 0) return fail(ctx, LF_E_INTERNAL, "a device-side check failed");

  // ---- encode (main.rs:98-124) ----
  uint8_t* o = proof;
  o[0] = 1, o[1] = o[2] = o[3] = 0;
  for (int i = 0; i < 16; ++i) o[4 + i] = (uint8_t)(q >> (8 * i));
  put_u64(o + 20, commit_bytes);
  put_u64(o + at_partials - 8, 128);
  memcpy(o + at_partials, partials.data(), 128 * 16);
  put_u64(o + at_rounds - 8, (uint64_t)sh.lp);
  memcpy(o + at_rounds, rounds.data(), 48 * sh.lp);
  memcpy(o + at_opened, &opened, 24);
  put_u64(o + at_row - 8, row_bytes);
  pack_f162(row, o + at_row);
  put_u64(o + at_fold - 8, fold_bytes);
  *proof_len = plen;

  ctx->prof.key_ms = ev_ms(ctx, 1, 2);
  ctx->prof.commit_ms = ev_ms(ctx, 2, 11);
  ctx->prof.finish_ms = ev_ms(ctx, 11, 3);
  // Kernel launches of one proof: commit 2, stream hashing 2, partials 5, switch (counted above),
  // row 2, challenges 1, fold 2.
  ctx->prof.launches = 2 + 2 + 5 + launches + 2 + 1 + 2;
  ctx->prof.transcript_ms = ev_ms(ctx, 3, 4);
  ctx->prof.partials_ms = ev_ms(ctx, 4, 5);
  ctx->prof.switch_ms = ev_ms(ctx, 5, 6);
  ctx->prof.switch_blocks_ms = ev_ms(ctx, 5, 14);
  ctx->prof.switch_materialize_ms = ev_ms(ctx, 14, 15);
  ctx->prof.switch_tail_ms = ev_ms(ctx, 15, 6);
  ctx->prof.row_ms = ev_ms(ctx, 6, 7);
  ctx->prof.challenges_ms = ev_ms(ctx, 7, 8);
  ctx->prof.fold_ms = ev_ms(ctx, 8, 9);
  ctx->prof.download_ms = ev_ms(ctx, 9, 10);
  return LF_OK;
}

int check_request(lf_ctx* ctx, const uint8_t* q_le, uint32_t log_vars, uint8_t* proof, size_t cap, size_t* len, u128& q,
                  Shape& sh) {
  if (!ctx || !q_le || !len) return fail(ctx, LF_E_ARGS, "null argument");
  if (!sh.set(log_vars) || sh.lp < 12) return fail(ctx, LF_E_SHAPE, "unsupported LOG_VARS");
  q = q_from_le(q_le);
  if (!accept_modulus(q, sh)) return fail(ctx, LF_E_MODULUS, "invalid commitment modulus");
  *len = proof_size(q, sh);
  if (!proof || cap < *len) return fail(ctx, LF_E_CAP, "proof buffer too small");
  return LF_OK;
}

// Shape, modulus, buffer and budget checks of one job, before any device work.
int check_job(lf_ctx* ctx, const lf_job& j, u128& q, Shape& sh) {
  if (!j.seed || !j.table || !j.q_le) return fail(ctx, LF_E_ARGS, "null argument");
  size_t len = 0;
  int rc = check_request(ctx, j.q_le, j.log_vars, j.proof, j.proof_cap, &len, q, sh);
  if (rc) return rc;
  if (!j.table_on_device && j.table_bytes != sh.words * 16)
    return fail(ctx, LF_E_TABLE_LEN, "witness table has the wrong length");
  return admit(ctx, q, sh, !j.table_on_device);
}

using clk = std::chrono::steady_clock;
double ms_between(clk::time_point a, clk::time_point b) { return std::chrono::duration<double, std::milli>(b - a).count(); }

// One job with the context lock held; table_dev is the job's table already on the device.
// Starts the copy of a host table into ctx->table on ctx's copy stream. A page-locked table goes up
// in up to TABLE_PARTS element ranges of every column (one 2-D copy each), each followed by a
// stream write of the proof's epoch into its ready flag, and *ts describes them (streamed = true):
// the commitment reads a range as soon as it has arrived. Part 0 is queued here; prove_device
// orders the rest by when the commitment's blocks reach them (order_table_parts), queues the next
// few, launches the commitment and then queues the others (so the host's queueing of them does not
// delay that launch). Any other table goes up in one copy whose completion is ctx->uploaded[0].
int start_table_upload(lf_ctx* ctx, const void* table, size_t table_bytes, const Shape& sh, TableStream* ts,
                       bool* streamed) {
  int rc = side_streams(ctx);
  if (rc) return rc;
  CK(ctx->table.ensure(table_bytes));
  CK(cudaEventRecord(ctx->up_t0, ctx->upload_stream));
  cudaPointerAttributes ta{};
  const bool locked = cudaPointerGetAttributes(&ta, table) == cudaSuccess && ta.type == cudaMemoryTypeHost;
  cudaGetLastError();  // plain host memory leaves an error behind on some drivers
  *streamed = locked && ctx->write_value && sh.ring_elements >= (uint64_t)TABLE_MIN_PARTS;
  if (*streamed) {
    const uint32_t epoch = ++ctx->epoch == 0 ? ++ctx->epoch : ctx->epoch;  // never 0, the flags' initial value
    int part_elems = 0, nparts = 0;
    table_parts(sh.ring_elements, &part_elems, &nparts);
    *ts = TableStream{ctx->ready, epoch, part_elems, ctx->uploaded[0], static_cast<const uint8_t*>(table),
                      (size_t)16 << sh.rl, sh.ring_elements, 0, ctx->test_withhold, ctx->test_ready_wait,
                      nparts, {}};
    for (int i = 0; i < ts->nparts; ++i) ts->order[i] = (uint8_t)i;
    return enqueue_table_parts(ctx, ts, 1);  // the rest once the commitment's layout is known
  }
  CK(cudaMemcpyAsync(ctx->table.p, table, table_bytes, cudaMemcpyHostToDevice, ctx->upload_stream));
  CK(cudaEventRecord(ctx->uploaded[0], ctx->upload_stream));
  CK(cudaEventRecord(ctx->up_t1, ctx->upload_stream));
  return LF_OK;
}

// A job's proof; a host table is copied by start_table_upload (streamed into the commitment when
// it is page-locked); a pageable proof buffer is touched meanwhile (touch_proof_buffer).
int run_job(lf_ctx* ctx, const lf_job& j, size_t* proof_len) {
  u128 q;
  Shape sh;
  int rc = check_job(ctx, j, q, sh);
  if (rc) return rc;
  cudaSetDevice(ctx->device);
  ctx->prof = lf_profile{};
  cudaEventRecord(ctx->ev[0], ctx->stream);
  if (j.table_on_device) {
    rc = prove_device(ctx, j.seed, q, sh, reinterpret_cast<const uint4*>(j.table), j.proof, proof_len, nullptr, true);
    if (ctx->touch_stream) cudaStreamSynchronize(ctx->touch_stream);  // (a proof that failed early)
    return rc;
  }
  if (j.table_bytes != sh.words * 16) return fail(ctx, LF_E_TABLE_LEN, "witness table has the wrong length");
  TableStream ts{};
  bool streamed = false;
  if ((rc = start_table_upload(ctx, j.table, j.table_bytes, sh, &ts, &streamed))) return rc;
  ctx->test_withhold = -1;  // the test hooks apply to one proof
  ctx->test_ready_wait = 0;
  rc = prove_device(ctx, j.seed, q, sh, ctx->table.as<uint4>(), j.proof, proof_len, ctx->uploaded[0], true,
                    streamed ? &ts : nullptr);
  if (streamed && ts.next < ts.nparts) enqueue_table_parts(ctx, &ts, ts.nparts);  // (an early failure)
  // (a proof that failed early may not have waited for the side streams)
  cudaStreamSynchronize(ctx->upload_stream);
  cudaStreamSynchronize(ctx->touch_stream);
  return rc;
}

// The device-side breakdown of a job's run (lf_result): the phases of the proof on its own stream,
// its commitment kernel, and the host table's copy (timed by events on the copy stream).
void result_times(lf_ctx* c, const lf_job& j, lf_result& r) {
  const lf_profile& p = c->prof;
  r.device_ms = p.key_ms + p.commit_ms + p.finish_ms + p.transcript_ms + p.partials_ms + p.switch_ms + p.row_ms +
                p.challenges_ms + p.fold_ms + p.download_ms;
  r.commit_ms = p.commit_ms;
  r.upload_ms = 0;
  float up = 0;
  if (!j.table_on_device && c->up_t0 && cudaEventElapsedTime(&up, c->up_t0, c->up_t1) == cudaSuccess) r.upload_ms = up;
  cudaGetLastError();
}

// One serving lane: `c` (the owner or one of its lanes) proves requests from the owner's FIFO. The front
// request starts when no request is in flight or when the footprints of those in flight and its
// own fit the device-memory budget, so a second request overlaps the first on the device while
// memory allows.
void serve_loop(lf_ctx* owner, lf_ctx* c) {
  for (;;) {
    lf_ctx::Queued item;
    {
      std::unique_lock<std::mutex> lk(owner->qmu);
      owner->qcv.wait(lk, [&] {
        if (owner->stopping) return true;
        if (owner->queue.empty()) return false;
        return owner->inflight == 0 || owner->budget == 0 ||
               owner->inflight_bytes + owner->queue.front().need <= owner->budget;
      });
      if (owner->queue.empty()) return;
      item = owner->queue.front();
      owner->queue.pop_front();
      ++owner->inflight;
      owner->inflight_bytes += item.need;
    }
    lf_result r{};
    const auto start = clk::now();
    r.queue_ms = ms_between(item.submitted, start);
    {
      std::lock_guard<std::mutex> g(c->mu);
      r.status = run_job(c, item.job, &r.proof_len);
      r.run_ms = ms_between(start, clk::now());
      if (r.status == LF_OK) result_times(c, item.job, r);
    }
    {
      std::lock_guard<std::mutex> lk(owner->qmu);
      owner->outcomes[item.ticket] = lf_ctx::Outcome{true, r};
      --owner->inflight;
      owner->inflight_bytes -= item.need;
    }
    owner->qcv.notify_all();
  }
}

// The context's other lanes, created on first use with the same device and budget (fewer when
// one cannot be made; the caller then runs on those there are, the context itself included).
std::vector<lf_ctx*> lanes_of(lf_ctx* ctx) {
  std::lock_guard<std::mutex> g(ctx->lanemu);
  while (!ctx->is_lane && (int)ctx->lanes.size() + 1 < ctx->nlanes) {
    lf_config cfg = {ctx->device, ctx->budget, 1};
    lf_ctx* l = nullptr;
    if (lf_ctx_create(&cfg, &l) != LF_OK) break;
    l->is_lane = true;
    ctx->lanes.push_back(l);
  }
  return ctx->lanes;
}

// ---------------------------------------------------------------------------------------------
// Verifier (verifier/proof_verify/src/main.rs:293-409: check_proof_shape, check_field_switch,
// check_opening). The table passes and ring products run on the device: the trusted partials
// (the prover's partial-sum kernels), a_times_v (K2 over the folded witness's transform) and the
// challenge combination; the transcript replay, the sumcheck recurrence and the small F162 sums
// run on the host.
// ---------------------------------------------------------------------------------------------
struct ProofParts {
  u128 q = 0;
  const uint8_t* commit = nullptr;
  size_t commit_len = 0;
  std::vector<b128> partials;
  std::vector<f162> rounds;  // e0, einf per round
  f162 opened = {0, 0, 0};
  const uint8_t* row = nullptr;
  size_t row_len = 0;
  const uint8_t* folded = nullptr;
  size_t folded_len = 0;
};
uint64_t rd64(const uint8_t* p) {
  uint64_t x;
  memcpy(&x, p, 8);
  return x;
}
// bincode fixint layout of main.rs:98-124, no trailing bytes.
bool decode_proof(const uint8_t* b, size_t len, ProofParts& p, std::string& err) {
  size_t at = 0;
  auto need = [&](uint64_t n) {
    if (at > len || len - at < n) {
      err = "truncated proof";
      return false;
    }
    return true;
  };
  auto vec = [&](const uint8_t*& ptr, size_t& n) {
    if (!need(8)) return false;
    const uint64_t k = rd64(b + at);
    at += 8;
    if (!need(k)) return false;
    ptr = b + at, n = (size_t)k;
    at += k;
    return true;
  };
  if (!need(20)) return false;
  if (b[0] != 1 || b[1] || b[2] || b[3]) {
    err = "unsupported proof version";
    return false;
  }
  p.q = q_from_le(b + 4);
  at = 20;
  if (!vec(p.commit, p.commit_len)) return false;
  if (!need(8)) return false;
  const uint64_t np = rd64(b + at);
  at += 8;
  if (np > (len - at) / 16) return (err = "truncated proof", false);
  p.partials.resize(np);
  for (uint64_t i = 0; i < np; ++i, at += 16) p.partials[i] = {rd64(b + at), rd64(b + at + 8)};
  if (!need(8)) return false;
  const uint64_t nr = rd64(b + at);
  at += 8;
  if (nr > (len - at) / 48) return (err = "truncated proof", false);
  p.rounds.resize(2 * nr);
  for (uint64_t i = 0; i < 2 * nr; ++i, at += 24) p.rounds[i] = {rd64(b + at), rd64(b + at + 8), rd64(b + at + 16)};
  if (!need(24)) return false;
  p.opened = {rd64(b + at), rd64(b + at + 8), rd64(b + at + 16)};
  at += 24;
  if (!vec(p.row, p.row_len) || !vec(p.folded, p.folded_len)) return false;
  if (at != len) return (err = "trailing bytes", false);
  return true;
}

const f162 F_ZERO = {0, 0, 0}, F_ONE = {1, 0, 0};
bool canonical(f162 x) { return (x.w2 >> 34) == 0; }

// eq table (eval.rs:50-64): out[j] = prod_k (bit k of j ? p_k : 1 + p_k).
std::vector<f162> eq_table_host(const std::vector<f162>& ps) {
  std::vector<f162> out(1, F_ONE);
  for (const f162& pk : ps) {
    f162 pk1 = pk;
    pk1.w0 ^= 1;
    std::vector<f162> nx(2 * out.size());
    for (size_t j = 0; j < out.size(); ++j) {
      nx[j] = f162_mul(out[j], pk1);
      nx[j + out.size()] = f162_mul(out[j], pk);
    }
    out.swap(nx);
  }
  return out;
}

// The transparent coefficient (crossfield.rs:10-65, 139-148): prod_i (1 + v_i + h_i) as a
// 128-vector over F162 (coordinate k = coefficient of x^k in GHASH), h_i = r_hi[i] acting by
// GHASH multiplication, folded against batch.
f162 transparent_coeff(const std::vector<b128>& r_hi, const std::vector<f162>& r_pp, const std::vector<f162>& batch) {
  std::vector<f162> t(128, F_ZERO), hs(128), vs(128);
  t[0] = F_ONE;
  for (size_t i = 0; i < r_pp.size(); ++i) {
    for (int k = 0; k < 128; ++k) vs[k] = f162_mul(t[k], r_pp[i]);
    std::fill(hs.begin(), hs.end(), F_ZERO);
    for (int k = 127; k >= 0; --k) {
      // hs <- hs * x in GHASH (x^128 = x^7 + x^2 + x + 1), then + t if bit k of r_hi[i]
      const f162 top = hs[127];
      for (int x = 127; x > 0; --x) hs[x] = hs[x - 1];
      hs[0] = F_ZERO;
      for (int x : {0, 1, 2, 7}) hs[x] = f162_add(hs[x], top);
      if (b128_bit(r_hi[i], k))
        for (int x = 0; x < 128; ++x) hs[x] = f162_add(hs[x], t[x]);
    }
    for (int k = 0; k < 128; ++k) t[k] = f162_add(f162_add(t[k], vs[k]), hs[k]);
  }
  f162 acc = F_ZERO;
  for (int k = 0; k < 128; ++k) acc = f162_add(acc, f162_mul(t[k], batch[k]));
  return acc;
}

// slice_sum (crossfield.rs:637-649): sum_k lift(u_k) batch[k], bit i of u_k = bit k of v[i].
f162 slice_sum(const std::vector<b128>& v, const std::vector<f162>& batch) {
  f162 s = F_ZERO;
  for (int k = 0; k < 128; ++k) {
    b128 u = {0, 0};
    for (int i = 0; i < 128; ++i)
      if (b128_bit(v[i], k)) (i < 64 ? u.lo : u.hi) |= 1ull << (i & 63);
    s = f162_add(s, f162_mul(f162_lift(u), batch[k]));
  }
  return s;
}

b128 claim_of(const std::vector<b128>& partials, const std::vector<b128>& lo) {  // main.rs:184-189
  std::vector<b128> e = eq_expand_b128(lo);
  b128 acc = {0, 0};
  for (int i = 0; i < 128; ++i) acc = b128_add(acc, b128_mul(partials[i], e[i]));
  return acc;
}

bool unpack_row(const uint8_t* b, size_t len, std::vector<f162>& out) {  // wire/mod.rs:96-140
  if (len != ((size_t)COLUMNS * 162 + 7) / 8) return false;
  out.assign(COLUMNS, F_ZERO);
  size_t bit = 0;
  auto get = [&](int n) {
    uint64_t x = 0;
    for (int i = 0; i < n; ++i, ++bit) x |= (uint64_t)((b[bit >> 3] >> (bit & 7)) & 1) << i;
    return x;
  };
  for (int i = 0; i < COLUMNS; ++i) out[i] = {get(64), get(64), get(34)};
  return true;
}

f162 challenge_f162(const Challenge& c) {  // challenge.rs:454-461
  f162 x = F_ZERO;
  for (uint32_t i = 0; i < c.weight; ++i) {
    const int pos = c.positions[i];
    (pos < 64 ? x.w0 : pos < 128 ? x.w1 : x.w2) |= 1ull << (pos & 63);
  }
  return x;
}

u128 rem_euclid(__int128 a, u128 q) {
  const __int128 m = (__int128)q;
  __int128 r = a % m;
  return (u128)(r < 0 ? r + m : r);
}

// The whole check of one proof against a table already on the device (main.rs:293-409).
int verify_device(lf_ctx* ctx, const uint8_t seed[32], const Shape& sh, const uint4* table, const uint8_t* proof,
                  size_t len) {
  cudaStream_t st = ctx->stream;
  auto reject = [&](const std::string& why) { return fail(ctx, LF_E_REJECT, why); };
  if (len > (size_t)64 << 20) return reject("proof too large");
  ProofParts pr;
  std::string e;
  if (!decode_proof(proof, len, pr, e)) return reject(e);
  if (pr.partials.size() != 128) return reject("128 partial evaluations");
  if (pr.rounds.size() != 2 * (size_t)sh.lp) return reject("one switch round per packed coordinate");
  const u128 q = pr.q;
  if (!accept_modulus(q, sh)) return reject("invalid commitment modulus");
  Transcript t;  // main.rs:166-174, the commitment's chunks hashed on the device
  int rc = absorb_commitment(ctx, t, seed, sh, q, pr.commit_len, pr.commit, nullptr);
  if (rc) return rc;
  // ---- check_field_switch ----
  std::vector<b128> lo = t.sample_b128("r-lo", 7);
  std::vector<b128> hi = t.sample_b128("r-hi", sh.lp);
  std::vector<b128> trusted;
  rc = device_partials(ctx, table, sh, hi, trusted);
  if (rc) return rc;
  const b128 value = claim_of(trusted, lo);
  t.absorb_b128(&value, 1);
  t.absorb_b128(pr.partials.data(), 128);
  const std::vector<f162> batch = eq_expand_f162(t.sample_f162("switch-batch", 7));
  const b128 claimed = claim_of(pr.partials, lo);
  if (claimed.lo != value.lo || claimed.hi != value.hi) return reject("partial evaluation mismatch");
  f162 sum = slice_sum(pr.partials, batch);
  std::vector<f162> coords;
  for (int r = 0; r < sh.lp; ++r) {
    const f162 e0 = pr.rounds[2 * r], einf = pr.rounds[2 * r + 1];
    if (!canonical(e0) || !canonical(einf)) return reject("noncanonical F162 element");
    t.absorb_f162(&pr.rounds[2 * r], 2);
    const f162 ch = t.sample_f162("switch-round", 1)[0];
    const f162 e1 = f162_add(sum, e0);
    sum = f162_add(f162_add(e0, f162_mul(ch, f162_add(f162_add(e0, e1), einf))), f162_mul(f162_mul(ch, ch), einf));
    coords.push_back(ch);
  }
  if (!canonical(pr.opened)) return reject("noncanonical F162 element");
  const f162 d = transparent_coeff(hi, coords, batch);
  if (f162_eq(d, F_ZERO)) return reject("the switch left the opened value unbound");
  if (!f162_eq(sum, f162_mul(d, pr.opened))) return reject("sumcheck final check failed");
  t.absorb_f162(&pr.opened, 1);
  // ---- check_opening ----
  // The table passes, the fold's norm / range / parity scans, the commitment's coefficient range
  // and both ring products run on the device; the decisions are taken below in the reference's
  // order (main.rs:253-289, rq.rs:188-256), so a proof is rejected with the same message.
  const std::vector<f162> p0(coords.rbegin(), coords.rend() - COLUMN_LOG);  // main.rs:257-264
  const std::vector<f162> p1(coords.rend() - COLUMN_LOG, coords.rend());
  std::vector<f162> row;
  if (!unpack_row(pr.row, pr.row_len, row)) return reject("malformed row evaluation");
  const size_t nv = (size_t)RING_N * sh.ring_elements;
  if (pr.folded_len != 4 * nv) return reject("malformed folded witness");
  {  // RowEvaluation::absorb (scheme/commitment.rs:320-331)
    const char* label = "labinius/row-evaluation";
    t.absorb_bytes(label, strlen(label));
    t.absorb_bytes(row.data(), row.size() * 24);
  }
  const uint64_t E = sh.ring_elements;
  const size_t w = coefficient_bytes(q);
  const bool commit_shape = pr.commit_len == w * COLUMNS * RING_N;
  CK(ctx->hasher.ensure(sizeof(bk::Hasher)));
  CK(ctx->chal.ensure(COLUMNS * sizeof(Challenge)));
  CK(ctx->status.ensure(16));
  CK(ctx->p0.ensure(64 * 24));
  CK(ctx->eqt.ensure(sh.column_len * 24));
  CK(cudaMemcpyAsync(ctx->hasher.p, &t.h, sizeof(bk::Hasher), cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(ctx->status.p, 0, 16, st));
  CK(launch_challenges(ctx->hasher.p, t.counter, ctx->sign_key, ctx->phase.p, ctx->chal.as<Challenge>(), COLUMNS,
                       ctx->status.as<int>(), st));
  t.counter += COLUMNS;
  CK(cudaMemcpyAsync(ctx->p0.p, p0.data(), 24 * p0.size(), cudaMemcpyHostToDevice, st));
  launch_eq_table_f162(ctx->p0.as<f162>(), sh.rl, ctx->eqt.as<f162>(), st);
  StreamBuf vdev(st), vred(st), vhat(st), part(st), atv(st), chpart(st), checks(st);
  CK(vdev.alloc(4 * nv));
  CK(checks.alloc(64));
  CK(cudaMemcpyAsync(vdev.p, pr.folded, 4 * nv, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(checks.p, 0, 64, st));
  launch_fold_checks(vdev.as<int32_t>(), E, ctx->eqt.as<f162>(), checks.as<unsigned long long>(), st);
  const uint8_t* commit_dev = ctx->stream_buf.as<uint8_t>() + STREAM_PREFIX;  // copied there by absorb_commitment
  if (commit_shape) {
    int rc2 = ensure_key(ctx, q, sh, 15);  // |v| <= 2^15
    if (rc2) return rc2;
    const ModulusPlan& mp = ctx->key->mp;
    CK(vred.alloc((size_t)mp.nprimes * nv * 4));
    CK(vhat.alloc((size_t)mp.nprimes * E * 4 * LEAVES * 4));
    CK(part.alloc((size_t)mp.nprimes * COLUMNS * LEAVES * 16));
    CK(atv.alloc(RING_N * w + 64));
    CK(chpart.alloc((size_t)32 * (2 * RING_N - 1) * 16));
    launch_commit_range(commit_dev, (uint32_t)w, q, (uint64_t)COLUMNS * RING_N, checks.as<unsigned long long>() + 6, st);
    launch_a_times_v(mp, sh, vdev.as<int32_t>(), ctx->key->key.as<uint32_t>(), vred.as<uint32_t>(),
                     vhat.as<uint32_t>(), part.as<uint32_t>(), atv.as<uint8_t>(), st);
    launch_challenge_combination(commit_dev, (uint32_t)w, ctx->chal.as<Challenge>(), chpart.as<unsigned long long>(),
                                 st);
  }
  CKL("opening checks");
  std::vector<Challenge> ch(COLUMNS);
  int status[4];
  unsigned long long ck[8];
  std::vector<uint8_t> atv_host(RING_N * w);
  std::vector<unsigned long long> chp((size_t)32 * (2 * RING_N - 1) * 2);
  CK(cudaMemcpyAsync(ch.data(), ctx->chal.p, COLUMNS * sizeof(Challenge), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(status, ctx->status.p, 16, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(ck, checks.p, 64, cudaMemcpyDeviceToHost, st));
  if (commit_shape) {
    CK(cudaMemcpyAsync(atv_host.data(), atv.p, RING_N * w, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(chp.data(), chpart.p, chp.size() * 8, cudaMemcpyDeviceToHost, st));
  }
  CK(cudaStreamSynchronize(st));
  // ck: [0..2] parity sum (F162), [3] sum v^2, [4] max v + 2^31, [5] 2^31 - min v, [6] commitment out of range
  const int64_t vmax = (int64_t)ck[4] - (1ll << 31), vmin = (1ll << 31) - (int64_t)ck[5];
  if (vmin < -32768 || vmax > 32767) return reject("malformed folded witness");
  if (status[0] != 0) return fail(ctx, LF_E_INTERNAL, "challenge sampling exceeded its attempt bound");
  {
    const std::vector<f162> e1 = eq_table_host(p1);
    f162 acc = F_ZERO;
    for (int j = 0; j < COLUMNS; ++j) acc = f162_add(acc, f162_mul(e1[j], row[j]));
    if (!f162_eq(acc, pr.opened)) return reject("the row evaluation does not reduce to the opened value");
  }
  const uint64_t worst = (uint64_t)std::max(vmax, -vmin);
  if (ck[3] > fold_cap(sh)) return reject("the fold is longer than the cap");
  if ((u128)worst > (q - 1) / 2) return reject("the fold is not centered");
  if (!commit_shape || ck[6]) return reject("malformed commitment");
  {
    // sum the column runs (each below 32 x 28 x 2^96 in magnitude, so 32 of them fit an i128),
    // then X^648 = X^324 - 1 from the top (rq.rs fold into the ring)
    std::vector<__int128> raw(2 * RING_N - 1, 0);
    for (int run = 0; run < 32; ++run)
      for (int r = 0; r < 2 * RING_N - 1; ++r) {
        const size_t i = 2 * ((size_t)run * (2 * RING_N - 1) + r);
        raw[r] += (__int128)(((u128)chp[i + 1] << 64) | chp[i]);
      }
    for (int r = 0; r < 2 * RING_N - 1; ++r) raw[r] = (__int128)rem_euclid(raw[r], q);
    for (int k = 2 * RING_N - 2; k >= RING_N; --k) {
      const __int128 x = (__int128)rem_euclid(raw[k], q);
      raw[k] = 0;
      raw[k - RING_N / 2] += x;
      raw[k - RING_N] -= x;
    }
    for (int i = 0; i < RING_N; ++i) {
      const u128 want = rem_euclid(raw[i], q);
      u128 got = 0;
      for (size_t b = w; b-- > 0;) got = (got << 8) | atv_host[i * w + b];
      if (got != want) return reject("the fold does not open the folded commitment");
    }
  }
  {  // main.rs:266-289: the fold's parity against the challenges' combination of the row
    const f162 left = {ck[0], ck[1], ck[2]};
    f162 right = F_ZERO;
    for (int j = 0; j < COLUMNS; ++j) right = f162_add(right, f162_mul(challenge_f162(ch[j]), row[j]));
    if (!f162_eq(left, right)) return reject("the fold does not match the folded row evaluation");
  }
  return LF_OK;
}

// Table PRG (verifier/table_writer/src/main.rs:14-22): keyed BLAKE3 XOF of the context string.
__global__ void k_table_prg(bk::Pending root, uint64_t blocks, uint4* out) {
  uint64_t b = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (b >= blocks) return;
  uint32_t w[16];
  root.root_block(b, w);
  out[4 * b] = make_uint4(w[0], w[1], w[2], w[3]);
  out[4 * b + 1] = make_uint4(w[4], w[5], w[6], w[7]);
  out[4 * b + 2] = make_uint4(w[8], w[9], w[10], w[11]);
  out[4 * b + 3] = make_uint4(w[12], w[13], w[14], w[15]);
}

// ---------------------------------------------------------------------------------------------
// Challenge sampling that allocates no device memory.
//
// Some callers cannot let a library allocate device memory: a serving process that hands all of
// its HBM to its own pool before the first request (an allocation would fail, or take memory the
// pool has already promised), and a caller running next to latency-critical streams, where
// cudaMalloc / cudaFree can stall the whole device. For them the sampler's scratch lives in one
// file-scope device array of fixed size, located once per device with cudaGetSymbolAddress:
// the transcript state the kernel starts from, the status word (zeroed by every call before the
// launch) and the challenges until they are copied out, plus the phase tables, written once.
// All calls on a device share the array, so a process-wide lock serialises the calls and each
// returns only after its stream has drained; work on other streams never touches the array.
// ---------------------------------------------------------------------------------------------
constexpr uint32_t NOALLOC_MAX_CHALLENGES = 4096;
static_assert(NOALLOC_MAX_CHALLENGES == LF_NOALLOC_MAX_CHALLENGES, "the header's limit is the array's");
constexpr int NOALLOC_MAX_DEVICES = 64;

struct NoAllocScratch {
  bk::Hasher hasher;                      // Transcript::new(domain) after absorb_bytes(prefix)
  int status[4];                          // status[0] != 0: a challenge failed its norm bound
  Challenge chal[NOALLOC_MAX_CHALLENGES];
  uint8_t phase[PHASE_TABLE_BYTES];       // phase tables (f64 re, im; f32 re, im)
};

static __device__ __align__(256) uint8_t g_noalloc_scratch[sizeof(NoAllocScratch)];
static_assert(sizeof(NoAllocScratch) < 512 * 1024, "the header states the array as under 512 KB");

struct NoAllocDevice {
  bool ready = false;
  NoAllocScratch* scratch = nullptr;
  uint32_t sign_key[8];
};
std::mutex g_noalloc_mu;
NoAllocDevice g_noalloc_dev[NOALLOC_MAX_DEVICES];

// Once per device, with that device current: locate the array and upload the phase tables.
int noalloc_setup(NoAllocDevice& d) {
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return LF_E_CUDA;
  NoAllocScratch* sc = static_cast<NoAllocScratch*>(p);
  if (upload_phase_tables(sc->phase) != cudaSuccess) return LF_E_CUDA;
  bk::Hasher h;
  const char* c = "labinius 2026 challenge signs v1";
  h.init_derive(c, (uint32_t)strlen(c));
  memcpy(d.sign_key, h.key, 32);
  d.scratch = sc;
  d.ready = true;
  return LF_OK;
}

int noalloc_sample(NoAllocDevice& d, const char* domain, const uint8_t* prefix, size_t prefix_len, uint32_t n,
                   uint8_t* out, cudaStream_t st) {
  Transcript t;
  t.init(domain);
  t.absorb_bytes(prefix, prefix_len);
  NoAllocScratch* sc = d.scratch;
  int status[4] = {0, 0, 0, 0};
  // From the first enqueue on, every return waits for the stream: the array is shared, and the
  // next call (on any stream) must not overwrite it while this one's copies or kernel still run.
  bool ok = cudaMemcpyAsync(&sc->hasher, &t.h, sizeof(bk::Hasher), cudaMemcpyHostToDevice, st) == cudaSuccess &&
            cudaMemsetAsync(sc->status, 0, sizeof(sc->status), st) == cudaSuccess &&
            launch_challenges(&sc->hasher, t.counter, d.sign_key, sc->phase, sc->chal, (int)n, sc->status, st) ==
                cudaSuccess &&
            cudaMemcpyAsync(out, sc->chal, (size_t)n * sizeof(Challenge), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
            cudaMemcpyAsync(status, sc->status, sizeof(status), cudaMemcpyDeviceToHost, st) == cudaSuccess;
  ok = cudaStreamSynchronize(st) == cudaSuccess && ok;
  if (!ok) return LF_E_CUDA;
  return status[0] ? LF_E_INTERNAL : LF_OK;
}

}  // namespace

// =============================================================================================
// C ABI
// =============================================================================================
extern "C" {

int lf_ctx_create(const lf_config* cfg, lf_ctx** out) {
  if (!out) return LF_E_ARGS;
  *out = nullptr;
  lf_ctx* ctx = new lf_ctx();
  ctx->device = cfg ? cfg->device : 0;
  ctx->budget = cfg ? cfg->hbm_budget : 0;
  if (cfg && (cfg->lanes < 0 || cfg->lanes > 8)) {
    delete ctx;
    return LF_E_ARGS;
  }
  ctx->nlanes = cfg && cfg->lanes ? cfg->lanes : 8;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) {
    delete ctx;
    return LF_E_CUDA;
  }
  cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, ctx->device);
  cudaDeviceGetAttribute(&ctx->pageable_access, cudaDevAttrPageableMemoryAccess, ctx->device);
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return LF_E_CUDA;
  }
  for (auto& ev : ctx->ev) cudaEventCreate(&ev);
  {
    bk::Hasher h;
    const char* c = "labinius 2026 challenge signs v1";
    h.init_derive(c, (uint32_t)strlen(c));
    memcpy(ctx->sign_key, h.key, 32);
  }
  if (ctx->phase.ensure(PHASE_TABLE_BYTES) != cudaSuccess || upload_phase_tables(ctx->phase.p) != cudaSuccess ||
      ctx->msg.ensure(64) != cudaSuccess || cudaMemset(ctx->msg.p, 0, 64) != cudaSuccess ||
      cudaHostAlloc(reinterpret_cast<void**>(&ctx->msg_out), 64, cudaHostAllocMapped) != cudaSuccess ||
      cudaHostGetDevicePointer(reinterpret_cast<void**>(&ctx->msg_out_dev), ctx->msg_out, 0) != cudaSuccess) {
    lf_ctx_destroy(ctx);
    return LF_E_CUDA;
  }
  *out = ctx;
  return LF_OK;
}

void* lf_ctx_stream(lf_ctx* ctx) { return ctx ? static_cast<void*>(ctx->stream) : nullptr; }

void lf_ctx_destroy(lf_ctx* ctx) {
  if (!ctx) return;
  {
    std::lock_guard<std::mutex> lk(ctx->qmu);
    for (auto& item : ctx->queue) {
      lf_result r{};
      r.status = LF_E_INTERNAL;
      ctx->outcomes[item.ticket] = lf_ctx::Outcome{true, r};
    }
    ctx->queue.clear();
    ctx->stopping = true;
  }
  ctx->qcv.notify_all();
  for (auto& w : ctx->workers)
    if (w.joinable()) w.join();
  for (lf_ctx* l : ctx->lanes) lf_ctx_destroy(l);
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  DevBuf* bufs[] = {&ctx->table, &ctx->stream_buf, &ctx->partial, &ctx->sblk, &ctx->ehi, &ctx->elo,
                    &ctx->rhi, &ctx->vparts, &ctx->psi, &ctx->batch, &ctx->soa, &ctx->msg, &ctx->p0, &ctx->eqt,
                    &ctx->row, &ctx->hasher, &ctx->chal, &ctx->fold, &ctx->cvs, &ctx->cvs_scratch, &ctx->subtrees,
                    &ctx->status, &ctx->phase, &ctx->scratch_small, &ctx->wbuf, &ctx->rbuf};
  ctx->keys.clear();
  for (DevBuf* b : bufs) b->release();
  ctx->table2.release();
  if (ctx->msg_out) cudaFreeHost(ctx->msg_out);
  ctx->kb_ared.release();
  ctx->kb_leaf.release();
  ctx->kb_matrix.release();
  ctx->fold_strips.release();
  ctx->fold_part.release();
  for (auto& ev : ctx->ev) cudaEventDestroy(ev);
  for (auto& ev : ctx->uploaded)
    if (ev) cudaEventDestroy(ev);
  if (ctx->upload_stream) cudaStreamDestroy(ctx->upload_stream);
  if (ctx->touch_stream) cudaStreamDestroy(ctx->touch_stream);
  if (ctx->ready) cudaFree(ctx->ready);
  for (cudaEvent_t e : {ctx->touched, ctx->up_t0, ctx->up_t1})
    if (e) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

size_t lf_proof_size(const uint8_t q_le[16], uint32_t log_vars) {
  Shape s;
  if (!q_le || !s.set(log_vars) || s.lp < 12) return 0;
  u128 q = q_from_le(q_le);
  if (q < 2) return 0;
  return proof_size(q, s);
}

int lf_accept_modulus(const uint8_t q_le[16], uint32_t log_vars) {
  Shape s;
  if (!q_le) return LF_E_ARGS;
  if (!s.set(log_vars)) return LF_E_SHAPE;
  return accept_modulus(q_from_le(q_le), s) ? LF_OK : LF_E_MODULUS;
}

int lf_key_prepare(lf_ctx* ctx, const uint8_t q_le[16], uint32_t log_vars) {
  if (!ctx || !q_le) return LF_E_ARGS;
  std::lock_guard<std::mutex> g(ctx->mu);
  Shape s;
  if (!s.set(log_vars) || s.lp < 12) return fail(ctx, LF_E_SHAPE, "unsupported LOG_VARS");
  u128 q = q_from_le(q_le);
  if (!accept_modulus(q, s)) return fail(ctx, LF_E_MODULUS, "invalid commitment modulus");
  cudaSetDevice(ctx->device);
  int rc = ensure_key(ctx, q, s);
  if (rc == LF_OK) rc = reserve_buffers(ctx, q, s, ctx->key->mp.nprimes, true);
  for (lf_ctx* l : lanes_of(ctx)) {  // each lane keeps its own copy of the key and its own buffers
    if (rc != LF_OK) break;
    std::lock_guard<std::mutex> gl(l->mu);
    rc = ensure_key(l, q, s);
    if (rc == LF_OK) rc = reserve_buffers(l, q, s, l->key->mp.nprimes, true);
    if (rc) fail(ctx, rc, lf_last_error(l));
  }
  if (rc == LF_OK) CK(cudaDeviceSynchronize());  // the reservations are complete before any proof
  return rc;
}

int lf_prove_device(lf_ctx* ctx, const uint8_t seed[32], const uint8_t q_le[16], uint32_t log_vars,
                    const void* table_dev, uint8_t* proof, size_t proof_cap, size_t* proof_len) {
  if (!ctx || !seed || !table_dev) return fail(ctx, LF_E_ARGS, "null argument");
  std::lock_guard<std::mutex> g(ctx->mu);
  u128 q;
  Shape sh;
  int rc = check_request(ctx, q_le, log_vars, proof, proof_cap, proof_len, q, sh);
  if (rc) return rc;
  if ((rc = admit(ctx, q, sh, false))) return rc;
  cudaSetDevice(ctx->device);
  auto t0 = std::chrono::steady_clock::now();
  ctx->prof = lf_profile{};
  cudaEventRecord(ctx->ev[0], ctx->stream);
  rc = prove_device(ctx, seed, q, sh, reinterpret_cast<const uint4*>(table_dev), proof, proof_len, nullptr, true);
  if (ctx->touch_stream) cudaStreamSynchronize(ctx->touch_stream);  // (a proof that failed early)
  ctx->prof.total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}

int lf_prove(lf_ctx* ctx, const uint8_t seed[32], const uint8_t q_le[16], uint32_t log_vars, const void* table,
             size_t table_bytes, uint8_t* proof, size_t proof_cap, size_t* proof_len) {
  if (!ctx || !seed || !table) return fail(ctx, LF_E_ARGS, "null argument");
  std::lock_guard<std::mutex> g(ctx->mu);
  u128 q;
  Shape sh;
  int rc = check_request(ctx, q_le, log_vars, proof, proof_cap, proof_len, q, sh);
  if (rc) return rc;
  if (table_bytes != sh.words * 16) return fail(ctx, LF_E_TABLE_LEN, "witness table has the wrong length");
  if ((rc = admit(ctx, q, sh, true))) return rc;
  cudaSetDevice(ctx->device);
  auto t0 = std::chrono::steady_clock::now();
  ctx->prof = lf_profile{};
  // The table goes up on the copy stream while the prover's stream builds (or finds) the key; the
  // commitment reads it as it arrives (page-locked) or waits for it. A pageable proof buffer is
  // touched by the device meanwhile, so the first-access cost of its pages is not paid by the
  // proof's own copies.
  cudaEventRecord(ctx->ev[0], ctx->stream);
  TableStream tstream{};
  bool streamed = false;
  if ((rc = start_table_upload(ctx, table, table_bytes, sh, &tstream, &streamed))) return rc;
  ctx->test_withhold = -1;  // the test hooks apply to one proof
  ctx->test_ready_wait = 0;
  rc = prove_device(ctx, seed, q, sh, ctx->table.as<uint4>(), proof, proof_len, ctx->uploaded[0], true,
                    streamed ? &tstream : nullptr);
  if (streamed && tstream.next < tstream.nparts) enqueue_table_parts(ctx, &tstream, tstream.nparts);  // (an early failure)
  // (a proof that failed early may not have waited for the side streams)
  cudaStreamSynchronize(ctx->upload_stream);
  cudaStreamSynchronize(ctx->touch_stream);
  float upload_ms_f = 0;
  cudaEventElapsedTime(&upload_ms_f, ctx->up_t0, ctx->up_t1);
  ctx->prof.upload_ms = upload_ms_f;
  ctx->prof.total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}

int lf_write_table_device(lf_ctx* ctx, const uint8_t seed[32], uint32_t log_vars, void* out_dev) {
  if (!ctx || !seed || !out_dev) return LF_E_ARGS;
  std::lock_guard<std::mutex> g(ctx->mu);
  Shape s;
  if (!s.set(log_vars)) return fail(ctx, LF_E_SHAPE, "unsupported LOG_VARS");
  cudaSetDevice(ctx->device);
  bk::Hasher h;
  h.init_keyed(seed);
  const char* c = "labinius-fast/binary-table/v1";
  h.absorb((const uint8_t*)c, strlen(c));
  bk::Pending root = h.finish();
  uint64_t blocks = (s.words * 16) / 64;
  k_table_prg<<<(unsigned)((blocks + 255) / 256), 256, 0, ctx->stream>>>(root, blocks, reinterpret_cast<uint4*>(out_dev));
  CKL("table PRG");
  CK(cudaStreamSynchronize(ctx->stream));
  return LF_OK;
}

int lf_device_alloc(lf_ctx* ctx, size_t bytes, void** out_dev) {
  if (!ctx || !out_dev) return LF_E_ARGS;
  cudaSetDevice(ctx->device);
  CK(cudaMalloc(out_dev, bytes));
  return LF_OK;
}
int lf_device_free(lf_ctx* ctx, void* dev) {
  if (!ctx) return LF_E_ARGS;
  cudaSetDevice(ctx->device);
  CK(cudaFree(dev));
  return LF_OK;
}
int lf_memcpy_h2d(lf_ctx* ctx, void* dst_dev, const void* src, size_t bytes) {
  if (!ctx || !dst_dev || !src) return LF_E_ARGS;
  cudaSetDevice(ctx->device);
  CK(cudaMemcpy(dst_dev, src, bytes, cudaMemcpyHostToDevice));
  return LF_OK;
}

int lf_last_challenges(lf_ctx* ctx, uint8_t* out, size_t cap) {
  if (!ctx || !out) return LF_E_ARGS;
  if (cap < COLUMNS * sizeof(Challenge) || ctx->chal.cap < COLUMNS * sizeof(Challenge)) return LF_E_CAP;
  cudaSetDevice(ctx->device);
  CK(cudaMemcpy(out, ctx->chal.p, COLUMNS * sizeof(Challenge), cudaMemcpyDeviceToHost));
  return LF_OK;
}

int lf_sample_challenges(lf_ctx* ctx, const char* domain, const uint8_t* prefix, size_t prefix_len, uint32_t n,
                         uint8_t* out) {
  return lf_sample_challenges_traced(ctx, domain, prefix, prefix_len, n, out, nullptr);
}

int lf_sample_challenges_traced(lf_ctx* ctx, const char* domain, const uint8_t* prefix, size_t prefix_len, uint32_t n,
                                uint8_t* out, uint32_t* trace64) {
  if (!ctx || !domain || (!prefix && prefix_len) || !out) return LF_E_ARGS;
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  Transcript t;
  t.init(domain);
  t.absorb_bytes(prefix, prefix_len);
  CK(ctx->hasher.ensure(sizeof(bk::Hasher)));
  CK(ctx->chal.ensure(std::max<size_t>(n, COLUMNS) * sizeof(Challenge)));
  CK(ctx->status.ensure(16));
  CK(ctx->scratch_small.ensure(64 * 4));
  CK(cudaMemsetAsync(ctx->scratch_small.p, 0, 64 * 4, ctx->stream));
  CK(cudaMemcpyAsync(ctx->hasher.p, &t.h, sizeof(bk::Hasher), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemsetAsync(ctx->status.p, 0, 16, ctx->stream));
  CK(launch_challenges(ctx->hasher.p, t.counter, ctx->sign_key, ctx->phase.p, ctx->chal.as<Challenge>(), (int)n,
                       ctx->status.as<int>(), ctx->stream, trace64 ? ctx->scratch_small.as<uint32_t>() : nullptr));
  int status[4] = {0, 0, 0, 0};
  CK(cudaMemcpyAsync(out, ctx->chal.p, n * sizeof(Challenge), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(status, ctx->status.p, sizeof(status), cudaMemcpyDeviceToHost, ctx->stream));
  if (trace64) CK(cudaMemcpyAsync(trace64, ctx->scratch_small.p, 64 * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (status[0]) return fail(ctx, LF_E_INTERNAL, "challenge sampling exceeded its attempt bound");
  return LF_OK;
}

// One lane of a batch: takes the next job index until none is left, copies a host table on its
// own stream and proves it.
void batch_lane(lf_ctx* c, bool lock, const lf_job* jobs, lf_result* results, const std::vector<int>& pre,
                std::atomic<size_t>& next, size_t n, clk::time_point t_batch) {
  // The batch's own context is locked by the caller; a lane is locked here (a serving worker may
  // share it).
  std::unique_lock<std::mutex> g(c->mu, std::defer_lock);
  if (lock) g.lock();
  cudaSetDevice(c->device);
  for (size_t i = next++; i < n; i = next++) {
    lf_result& r = results[i];
    r = lf_result{};
    const auto start = clk::now();
    r.queue_ms = ms_between(t_batch, start);
    r.status = pre[i];
    if (r.status == LF_OK) r.status = run_job(c, jobs[i], &r.proof_len);
    r.run_ms = ms_between(start, clk::now());
    if (r.status == LF_OK) result_times(c, jobs[i], r);
  }
}

int lf_prove_batch(lf_ctx* ctx, size_t n, const lf_job* jobs, lf_result* results) {
  if (!ctx || (n && (!jobs || !results))) return LF_E_ARGS;
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  int src = side_streams(ctx);
  if (src) return src;
  const auto t_batch = clk::now();
  std::vector<int> pre(n, LF_OK);  // per-job check before any device work
  for (size_t i = 0; i < n; ++i) {
    u128 q;
    Shape sh;
    pre[i] = check_job(ctx, jobs[i], q, sh);
  }
  int first = LF_OK;
  if (n >= 2) {
    // Lanes: a proof waits on the host between switch rounds and for its downloads, so other
    // contexts on their own streams fill those gaps with the next jobs.
    const std::vector<lf_ctx*> lanes = lanes_of(ctx);
    if (!lanes.empty()) {
      std::atomic<size_t> next{0};
      std::vector<std::thread> others;
      for (size_t k = 0; k < lanes.size() && k + 1 < n; ++k)
        others.emplace_back(batch_lane, lanes[k], true, jobs, results, std::cref(pre), std::ref(next), n, t_batch);
      batch_lane(ctx, false, jobs, results, pre, next, n, t_batch);
      for (auto& t : others) t.join();
      for (size_t i = 0; i < n; ++i)
        if (results[i].status != LF_OK && first == LF_OK) first = results[i].status;
      return first;
    }
  }
  DevBuf* tb[2] = {&ctx->table, &ctx->table2};
  // Copy a host table into buffer b on the copy stream (job i), marking its completion.
  auto upload = [&](size_t i, int b) -> int {
    const lf_job& j = jobs[i];
    if (pre[i] != LF_OK || j.table_on_device) return LF_OK;
    CK(tb[b]->ensure(j.table_bytes));
    CK(cudaMemcpyAsync(tb[b]->p, j.table, j.table_bytes, cudaMemcpyHostToDevice, ctx->upload_stream));
    CK(cudaEventRecord(ctx->uploaded[b], ctx->upload_stream));
    return LF_OK;
  };
  int up = n ? upload(0, 0) : LF_OK;
  for (size_t i = 0; i < n; ++i) {
    lf_result& r = results[i];
    r = lf_result{};
    const auto start = clk::now();
    r.queue_ms = ms_between(t_batch, start);
    const lf_job& j = jobs[i];
    const int b = (int)(i & 1);
    r.status = pre[i] != LF_OK ? pre[i] : up;
    const uint4* table = reinterpret_cast<const uint4*>(j.table);
    if (r.status == LF_OK && !j.table_on_device) {
      table = tb[b]->as<uint4>();
      if (cudaStreamWaitEvent(ctx->stream, ctx->uploaded[b], 0) != cudaSuccess)
        r.status = fail(ctx, LF_E_CUDA, "stream wait failed");
    }
    // The other buffer's job finished (prove_device ends in a stream synchronisation): fill it.
    up = i + 1 < n ? upload(i + 1, b ^ 1) : LF_OK;
    if (r.status == LF_OK) {
      u128 q;
      Shape sh;
      check_job(ctx, j, q, sh);  // passed in pre[i]
      ctx->prof = lf_profile{};
      cudaEventRecord(ctx->ev[0], ctx->stream);
      r.status = prove_device(ctx, j.seed, q, sh, table, j.proof, &r.proof_len, nullptr, true);
    }
    r.run_ms = ms_between(start, clk::now());
    if (r.status != LF_OK && first == LF_OK) first = r.status;
  }
  cudaStreamSynchronize(ctx->upload_stream);
  return first;
}

int lf_submit(lf_ctx* ctx, const lf_job* job, uint64_t* ticket) {
  if (!ctx || !job || !ticket) return LF_E_ARGS;
  // Checked without the context's lock, which a worker holds while it proves: the checks read
  // only what is fixed at creation (budget, SM count).
  u128 q;
  Shape sh;
  int rc = check_job(ctx, *job, q, sh);
  if (rc) return rc;
  const size_t need = proof_footprint(sh, !job->table_on_device, ctx->sms, primes_for(q, sh));
  const std::vector<lf_ctx*> lanes = lanes_of(ctx);
  std::lock_guard<std::mutex> lk(ctx->qmu);
  if (ctx->stopping) return LF_E_ARGS;
  *ticket = ctx->next_ticket++;
  ctx->outcomes[*ticket] = lf_ctx::Outcome{};
  ctx->queue.push_back(lf_ctx::Queued{*ticket, *job, clk::now(), need});
  if (ctx->workers.empty()) {
    ctx->workers.emplace_back(serve_loop, ctx, ctx);
    for (lf_ctx* l : lanes) ctx->workers.emplace_back(serve_loop, ctx, l);
  }
  ctx->qcv.notify_all();
  return LF_OK;
}

int lf_tune(lf_ctx* ctx, const uint8_t q_le[16], uint32_t log_vars, const void* table_dev, lf_tune_result* out) {
  if (!ctx || !q_le || !table_dev) return fail(ctx, LF_E_ARGS, "null argument");
  Shape sh;
  if (!sh.set(log_vars) || sh.lp < 12) return fail(ctx, LF_E_SHAPE, "unsupported LOG_VARS");
  const u128 q = q_from_le(q_le);
  if (!accept_modulus(q, sh)) return fail(ctx, LF_E_MODULUS, "invalid commitment modulus");
  std::vector<lf_ctx*> lanes = lanes_of(ctx);
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  int rc = ensure_key(ctx, q, sh);
  if (rc) return rc;
  const ModulusPlan& mp = ctx->key->mp;
  const uint4* table = static_cast<const uint4*>(table_dev);
  cudaStream_t st = ctx->stream;
  const long blocks1 = (long)(COLUMNS / 128) * mp.nprimes * 3;  // blocks per split
  int best = commit_splits(sh.ring_elements, mp.nprimes, ctx->sms), tried = 0;
  float best_ms = 1e30f;
  CK(ctx->status.ensure(16));
  for (int sp = 1; sp <= 48; ++sp) {
    if ((uint64_t)sp > sh.ring_elements) break;
    const long blocks = blocks1 * sp, waves = (blocks + ctx->sms - 1) / ctx->sms;
    if (blocks < ctx->sms / 2 && sp != 1) continue;
    if ((double)blocks / (double)(waves * ctx->sms) < 0.75 && sp != best) continue;  // poor last wave
    CK(ctx->partial.ensure((size_t)sp * mp.nprimes * COLUMNS * LEAVES * 4 * 4));
    CK(cudaMemsetAsync(ctx->status.p, 0, 16, st));
    float ms = 0;
    for (int rep = 0; rep < 2; ++rep) {  // the second run is timed
      cudaEventRecord(ctx->ev[12], st);
      launch_commit(mp, sh, table, ctx->key->key.as<uint32_t>(), ctx->key->btiles.as<uint16_t>(),
                    ctx->partial.as<uint32_t>(), sp, ctx->status.as<int>(), st);
      cudaEventRecord(ctx->ev[13], st);
      CKL("tuning the commitment");
      CK(cudaEventSynchronize(ctx->ev[13]));
      cudaEventElapsedTime(&ms, ctx->ev[12], ctx->ev[13]);
    }
    ++tried;
    if (ms < best_ms) best_ms = ms, best = sp;
  }
  int status = 0;
  CK(cudaMemcpy(&status, ctx->status.p, 4, cudaMemcpyDeviceToHost));
  if (status) return fail(ctx, LF_E_INTERNAL, "the commitment kernel failed while tuning");
  ctx->tuned_splits[{sh.log_vars, mp.nprimes}] = best;

  // The fold's column-run count: the persistent kernel walks nbx x runs work units over the SMs,
  // so counts whose units fill the SMs' last round at least 3/4 are timed (the whole fold: strips,
  // the product and the runs' sum). Challenges of all-zero positions stand in for the proof's own
  // (the time does not depend on the values).
  const size_t fold_bytes = 4 * RING_N * sh.ring_elements;
  const long nbx = (long)((4 * sh.ring_elements + 127) / 128);
  int fbest = fold_splits(sh.ring_elements, ctx->sms), ftried = 0;
  float fbest_ms = 1e30f;
  CK(ctx->chal.ensure(COLUMNS * sizeof(Challenge)));
  CK(cudaMemsetAsync(ctx->chal.p, 0, COLUMNS * sizeof(Challenge), st));
  CK(ctx->fold.ensure(fold_bytes));
  CK(ctx->fold_strips.ensure(COLUMNS * FOLD_STRIP_BYTES));
  CK(cudaMemsetAsync(ctx->status.p, 0, 16, st));
  for (int sp = 1; sp <= 32; ++sp) {
    const long units = nbx * sp, rounds = (units + ctx->sms - 1) / ctx->sms;
    if ((double)units / (double)(rounds * ctx->sms) < 0.75 && sp != fbest) continue;
    CK(ctx->fold_part.ensure((size_t)sp * fold_bytes));
    float ms = 0;
    for (int rep = 0; rep < 2; ++rep) {  // the second run is timed
      cudaEventRecord(ctx->ev[12], st);
      launch_fold(table, sh.rl, sh.ring_elements, ctx->chal.as<Challenge>(), ctx->fold_strips.as<uint8_t>(),
                  ctx->fold_part.as<int32_t>(), sp, ctx->fold.as<int32_t>(), ctx->status.as<int>(), st);
      cudaEventRecord(ctx->ev[13], st);
      CKL("tuning the fold");
      CK(cudaEventSynchronize(ctx->ev[13]));
      cudaEventElapsedTime(&ms, ctx->ev[12], ctx->ev[13]);
    }
    ++ftried;
    if (ms < fbest_ms) fbest_ms = ms, fbest = sp;
  }
  CK(cudaMemcpy(&status, ctx->status.p, 4, cudaMemcpyDeviceToHost));
  if (status) return fail(ctx, LF_E_INTERNAL, "the fold kernel failed while tuning");
  ctx->tuned_fold[sh.log_vars] = fbest;
  for (lf_ctx* l : lanes) {
    std::lock_guard<std::mutex> gl(l->mu);
    l->tuned_splits[{sh.log_vars, mp.nprimes}] = best;
    l->tuned_fold[sh.log_vars] = fbest;
    cudaSetDevice(l->device);
    if (l->fold_part.ensure((size_t)fbest * fold_bytes) != cudaSuccess)  // no lane grows it inside a proof
      return fail(ctx, LF_E_OOM, "fold run buffer of a lane");
  }
  if (out) {
    out->commit_splits = best;
    out->commit_ms = best_ms;
    out->candidates = tried;
    out->fold_splits = fbest;
    out->fold_ms = fbest_ms;
    out->fold_candidates = ftried;
  }
  return LF_OK;
}

size_t lf_request_footprint(lf_ctx* ctx, const uint8_t q_le[16], uint32_t log_vars, int host_table) {
  if (!ctx || !q_le) return 0;
  Shape sh;
  if (!sh.set(log_vars) || sh.lp < 12) return 0;
  const u128 q = q_from_le(q_le);
  if (!accept_modulus(q, sh)) return 0;
  return proof_footprint(sh, host_table != 0, ctx->sms, primes_for(q, sh));
}

int lf_poll(lf_ctx* ctx, uint64_t ticket, uint32_t wait_ms, lf_result* out) {
  if (!ctx || !out) return LF_E_ARGS;
  std::unique_lock<std::mutex> lk(ctx->qmu);
  auto it = ctx->outcomes.find(ticket);
  if (it == ctx->outcomes.end()) return LF_E_TICKET;
  if (!it->second.done && wait_ms)
    ctx->qcv.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] {
      auto f = ctx->outcomes.find(ticket);
      return f == ctx->outcomes.end() || f->second.done;
    });
  it = ctx->outcomes.find(ticket);
  if (it == ctx->outcomes.end()) return LF_E_TICKET;
  if (!it->second.done) return LF_E_TIMEOUT;
  *out = it->second.result;
  ctx->outcomes.erase(it);
  return LF_OK;
}

int lf_sample_challenges_noalloc(int device, const char* domain, const uint8_t* prefix, size_t prefix_len, uint32_t n,
                                 uint8_t* out, void* stream) {
  if (!domain || (!prefix && prefix_len) || !out || n == 0 || device < 0 || device >= NOALLOC_MAX_DEVICES)
    return LF_E_ARGS;
  if (n > NOALLOC_MAX_CHALLENGES) return LF_E_LIMIT;
  std::lock_guard<std::mutex> g(g_noalloc_mu);
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess || cudaSetDevice(device) != cudaSuccess) return LF_E_CUDA;
  NoAllocDevice& d = g_noalloc_dev[device];
  int rc = d.ready ? LF_OK : noalloc_setup(d);
  if (rc == LF_OK)
    rc = noalloc_sample(d, domain, prefix, prefix_len, n, out, static_cast<cudaStream_t>(stream));
  cudaSetDevice(prev);
  return rc;
}

int lf_ring_mul(lf_ctx* ctx, const uint8_t q_le[16], size_t n, const void* a_dev, const void* b_dev, void* c_dev) {
  if (!ctx || !q_le || (n && (!a_dev || !b_dev || !c_dev))) return fail(ctx, LF_E_ARGS, "null argument");
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  const u128 q = q_from_le(q_le);
  RingCache* rc = nullptr;
  for (auto& r : ctx->rings)
    if (r->q == q) rc = r.get();
  if (!rc) {
    std::unique_ptr<RingCache> r(new RingCache());
    std::string e;
    if (!make_ring_plan(q, r->plan, e)) return fail(ctx, LF_E_MODULUS, e);
    CK(r->rps.ensure(sizeof(RingPrimeDev) * r->plan.dev.size()));
    CK(cudaMemcpyAsync(r->rps.p, r->plan.dev.data(), sizeof(RingPrimeDev) * r->plan.dev.size(),
                       cudaMemcpyHostToDevice, ctx->stream));
    r->q = q;
    if (ctx->rings.size() >= MAX_RINGS) ctx->rings.erase(ctx->rings.begin());
    ctx->rings.push_back(std::move(r));
    rc = ctx->rings.back().get();
  }
  if (!n) return LF_OK;
  CK(ctx->status.ensure(16));
  CK(cudaMemsetAsync(ctx->status.p, 0, 16, ctx->stream));
  launch_ring_mul(rc->plan, rc->rps.as<RingPrimeDev>(), a_dev, b_dev, c_dev, n, ctx->status.as<int>(), ctx->stream);
  CKL("ring products");
  int st = 0;
  CK(cudaMemcpyAsync(&st, ctx->status.p, 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (st & 1) return fail(ctx, LF_E_ARGS, "an operand coefficient is not below q");
  return LF_OK;
}

int lf_ghash_mul(lf_ctx* ctx, size_t n, const void* a_dev, const void* b_dev, void* c_dev) {
  if (!ctx || (n && (!a_dev || !b_dev || !c_dev))) return fail(ctx, LF_E_ARGS, "null argument");
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  launch_ghash_mul(a_dev, b_dev, c_dev, n, ctx->sms, ctx->stream);
  CKL("GHASH products");
  CK(cudaStreamSynchronize(ctx->stream));
  return LF_OK;
}

int lf_ajtai_matrix_device(lf_ctx* ctx, const uint8_t q_le[16], uint64_t elements, void* out_dev) {
  if (!ctx || !q_le || (elements && !out_dev)) return fail(ctx, LF_E_ARGS, "null argument");
  const u128 q = q_from_le(q_le);
  if (q < 2) return fail(ctx, LF_E_MODULUS, "a modulus is at least 2");
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  if (!elements) return LF_OK;
  StreamBuf mscratch(ctx->stream);
  CK(mscratch.alloc(matrix_scratch_bytes(elements, q)));
  launch_matrix_raw(q, elements, out_dev, mscratch.p, ctx->stream);
  CKL("matrix expansion");
  CK(cudaStreamSynchronize(ctx->stream));
  return LF_OK;
}

int lf_a_times_v(lf_ctx* ctx, const uint8_t q_le[16], uint64_t elements, const int16_t* v_dev, uint8_t* out) {
  if (!ctx || !q_le || !v_dev || !out) return fail(ctx, LF_E_ARGS, "null argument");
  int lg = 0;
  while (lg < 16 && ((uint64_t)1 << lg) < elements) ++lg;
  if (elements == 0 || ((uint64_t)1 << lg) != elements || lg > 15)
    return fail(ctx, LF_E_SHAPE, "elements must be a power of two up to 2^15");
  Shape sh;
  sh.set((uint32_t)(19 + lg));  // the proof shape whose columns have `elements` ring elements
  const u128 q = q_from_le(q_le);
  if (q < 2 || q >> 96) return fail(ctx, LF_E_MODULUS, "a_times_v covers moduli in [2, 2^96)");
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  int rc = ensure_key(ctx, q, sh, 15);  // |v| <= 2^15
  if (rc) return rc;
  const ModulusPlan& mp = ctx->key->mp;
  const size_t nv = (size_t)elements * RING_N, w = mp.width;
  StreamBuf v32(ctx->stream), vred(ctx->stream), vhat(ctx->stream), part(ctx->stream), atv(ctx->stream);
  CK(v32.alloc(4 * nv));
  CK(vred.alloc((size_t)mp.nprimes * nv * 4));
  CK(vhat.alloc((size_t)mp.nprimes * elements * 4 * LEAVES * 4));
  CK(part.alloc((size_t)mp.nprimes * COLUMNS * LEAVES * 16));
  CK(atv.alloc(RING_N * w + 64));
  launch_widen_i16(v_dev, v32.as<int32_t>(), nv, ctx->stream);
  launch_a_times_v(mp, sh, v32.as<int32_t>(), ctx->key->key.as<uint32_t>(), vred.as<uint32_t>(), vhat.as<uint32_t>(),
                   part.as<uint32_t>(), atv.as<uint8_t>(), ctx->stream);
  CKL("a_times_v");
  std::vector<uint8_t> packed(RING_N * w);
  CK(cudaMemcpyAsync(packed.data(), atv.p, RING_N * w, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  memset(out, 0, RING_N * 16);
  for (int i = 0; i < RING_N; ++i) memcpy(out + 16 * i, packed.data() + w * i, w);
  return LF_OK;
}

int lf_verify_device(lf_ctx* ctx, const uint8_t seed[32], uint32_t log_vars, const void* table_dev, const uint8_t* proof,
                     size_t proof_len) {
  if (!ctx || !seed || !table_dev || !proof) return fail(ctx, LF_E_ARGS, "null argument");
  std::lock_guard<std::mutex> g(ctx->mu);
  Shape sh;
  if (!sh.set(log_vars) || sh.lp < 12) return fail(ctx, LF_E_SHAPE, "unsupported LOG_VARS");
  cudaSetDevice(ctx->device);
  return verify_device(ctx, seed, sh, reinterpret_cast<const uint4*>(table_dev), proof, proof_len);
}

int lf_verify(lf_ctx* ctx, const uint8_t seed[32], uint32_t log_vars, const void* table, size_t table_bytes,
              const uint8_t* proof, size_t proof_len) {
  if (!ctx || !seed || !proof) return fail(ctx, LF_E_ARGS, "null argument");
  std::lock_guard<std::mutex> g(ctx->mu);
  Shape sh;
  if (!sh.set(log_vars) || sh.lp < 12) return fail(ctx, LF_E_SHAPE, "unsupported LOG_VARS");
  cudaSetDevice(ctx->device);
  CK(ctx->table.ensure(sh.words * 16));
  if (table) {
    if (table_bytes != sh.words * 16) return fail(ctx, LF_E_TABLE_LEN, "witness table has the wrong length");
    CK(cudaMemcpyAsync(ctx->table.p, table, table_bytes, cudaMemcpyHostToDevice, ctx->stream));
  } else {  // the table of the seed, as the checker regenerates it (main.rs:143-153)
    bk::Hasher h;
    h.init_keyed(seed);
    const char* c = "labinius-fast/binary-table/v1";
    h.absorb((const uint8_t*)c, strlen(c));
    const bk::Pending root = h.finish();
    const uint64_t blocks = (sh.words * 16) / 64;
    k_table_prg<<<(unsigned)((blocks + 255) / 256), 256, 0, ctx->stream>>>(root, blocks, ctx->table.as<uint4>());
    CKL("table PRG");
  }
  return verify_device(ctx, seed, sh, ctx->table.as<uint4>(), proof, proof_len);
}

int lf_last_profile(lf_ctx* ctx, lf_profile* out) {
  if (!ctx || !out) return LF_E_ARGS;
  *out = ctx->prof;
  return LF_OK;
}

int lf_test_set_point(lf_ctx* ctx, const uint8_t* r_hi, uint32_t n) {
  if (!ctx || (!r_hi && n)) return LF_E_ARGS;
  std::lock_guard<std::mutex> g(ctx->mu);
  ctx->test_hi.assign(n, b128{0, 0});
  if (n) memcpy(ctx->test_hi.data(), r_hi, 16 * (size_t)n);
  return LF_OK;
}

int lf_test_withhold_table_part(lf_ctx* ctx, int part, uint64_t wait_cycles) {
  if (!ctx || part < 0 || part >= TABLE_PARTS) return LF_E_ARGS;
  std::lock_guard<std::mutex> g(ctx->mu);
  ctx->test_withhold = part;
  ctx->test_ready_wait = (long long)std::min<uint64_t>(wait_cycles, (uint64_t)1 << 40);
  return LF_OK;
}

int lf_test_table_part_order(uint64_t ring_elements, int splits, int blocks_per_split, int sms, uint8_t* order,
                             int* nparts) {
  if (!order || !nparts || ring_elements < 1 || splits < 1 || blocks_per_split < 1 || sms < 1) return LF_E_ARGS;
  TableStream ts{};
  ts.elements = ring_elements;
  table_parts(ring_elements, &ts.part_elems, &ts.nparts);
  for (int i = 0; i < ts.nparts; ++i) ts.order[i] = (uint8_t)i;
  ts.next = 1;  // part 0 goes up first, before the commitment's layout is known
  order_table_parts(&ts, splits, blocks_per_split, sms);
  for (int i = 0; i < ts.nparts; ++i) order[i] = ts.order[i];
  *nparts = ts.nparts;
  return LF_OK;
}

const char* lf_strerror(int code) {
  switch (code) {
    case LF_OK: return "ok";
    case LF_E_ARGS: return "invalid argument";
    case LF_E_SHAPE: return "unsupported shape";
    case LF_E_MODULUS: return "invalid commitment modulus";
    case LF_E_TABLE_LEN: return "witness table has the wrong length";
    case LF_E_CAP: return "proof buffer too small";
    case LF_E_OOM: return "device memory exhausted";
    case LF_E_CUDA: return "CUDA error";
    case LF_E_INTERNAL: return "internal check failed";
    case LF_E_ADMISSION: return "request exceeds the HBM budget";
    case LF_E_TIMEOUT: return "the job has not finished yet";
    case LF_E_TICKET: return "no such ticket";
    case LF_E_REJECT: return "the proof does not verify";
    case LF_E_LIMIT: return "request exceeds the fixed scratch of lf_sample_challenges_noalloc (4096 challenges)";
    default: return "unknown error";
  }
}

const char* lf_last_error(lf_ctx* ctx) {
  if (!ctx) return "no context";
  thread_local std::string copy;  // valid until this thread's next call
  std::lock_guard<std::mutex> g(ctx->errmu);
  copy = ctx->err;
  return copy.c_str();
}

}  // extern "C"
