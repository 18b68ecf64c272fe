// The Ajtai commitment C_j = sum_m A_m W_{j,m} in R_Q = Z_Q[X]/(X^648 - X^324 + 1)
// (verifier/proof_verify/src/rq.rs:264-287, reference.rs:32-48), GB300 kernels.
//
// Transform. With Y = X^4 the ring modulus is Phi_486(Y) = Y^162 - Y^81 + 1, and a witness ring
// element W = sum_k X^k W_k(Y) has as W_k the 128 bits of table word 4m + k (coefficient 4p + k
// is bit p of that word). Modulo a prime p = 1 (mod 486) Phi_486 splits into the 162 linear
// factors Y - eta^e; the transform is a tree: the trinomial split into Y^81 - eta^81 and
// Y^81 - eta^405, then four radix-3 levels. A node Y^n - c splits into Y^(n/3) - c^(1/3) w^i.
// So W mod (X^4 - c) = sum_k W_k(c) X^k: each table word is transformed on its own, and the
// ring product at a leaf is a 4x4 product modulo X^4 - c (a "base multiplication") with the
// key's leaf polynomial. The first two levels of a binary word depend on 5 of its bits per output
// (positions q, q+27, q+54, q+81, q+108), so they are one lookup in a 32-entry table.
//
// Results modulo each prime are recombined by Garner's CRT. For Q = 3889*9721*17497 (the three
// primes of solution-arm/proof_generate/src/ntt.rs:37-40) the recombination is already modulo Q.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "lf_blake3.cuh"
#include "lf_internal.h"
#include "lf_tc.cuh"

namespace lf {


// Shape of K1 on the tensor cores (the kernel is described where it is defined).
constexpr int TC_COLS = 128;                         // table columns per block (MMA M)
constexpr int TC_LEAVES = 54;                        // leaves per block (a third of a prime)
constexpr int TC_N = 64;                             // MMA N: 6 groups of 10 rows (9 leaves + 1 zero), padded
constexpr int TC_K = 256;                            // MMA K: 128 bits x 2 limbs (A read twice)
constexpr int TC_THREADS = 32 * 32;                  // 24 epilogue, 4 producer and 4 issuer warps
constexpr int TC_B_BYTES = TC_N * TC_K * 2;          // 32 KB
constexpr int TC_KEY_INTS = TC_LEAVES * 16;          // one element's key rows for the block's leaves
constexpr int TC_SMEM0 =
    TC_B_BYTES + 4 * TC_KEY_INTS * 4 + 3 * TC_COLS * 64 + 3 * TC_KEY_INTS * 4 + 4 * TC_LEAVES * 16 + 16 * 8 + 16;
constexpr int TC_CONST_AT = (TC_SMEM0 + 127) / 128 * 128;  // A (128 x 16) and B (64 x 16) of the init MMA
constexpr int TC_SMEM = TC_CONST_AT + 4096 + 2048;
constexpr long long TC_WAIT_CYCLES = 2000000000LL;   // ~1 s at 2 GHz

static void fill_btiles(const PrimePlan& pl, const PrimeConst& c, uint16_t* out);

// ------------------------------------------------------------------------------------------------
// Host: plans
// ------------------------------------------------------------------------------------------------
static uint64_t powmod(uint64_t b, uint64_t e, uint64_t p) {
  uint64_t r = 1 % p;
  b %= p;
  while (e) {
    if (e & 1) r = r * b % p;
    b = b * b % p;
    e >>= 1;
  }
  return r;
}
static uint32_t inv_mod(uint64_t x, uint64_t p) { return (uint32_t)powmod(x % p, p - 2, p); }

bool make_plan(uint32_t p, PrimePlan& out) {
  if (p < 487 || (p - 1) % 486 != 0) return false;
  for (uint64_t d = 2; d * d <= p; ++d)
    if (p % d == 0) return false;
  uint64_t eta = 0;
  for (uint64_t g = 2; g < p; ++g) {
    uint64_t z = powmod(g, (p - 1) / 486, p);
    if (powmod(z, 243, p) != 1 && powmod(z, 162, p) != 1) {
      eta = z;
      break;
    }
  }
  if (!eta) return false;
  out.p = p;
  out.eta = (uint32_t)eta;
  out.pw.resize(486);
  for (int i = 0; i < 486; ++i) out.pw[i] = (uint32_t)powmod(eta, i, p);
  out.node_e[1] = {81, 405};
  for (int l = 1; l < 4; ++l) {
    out.node_e[l + 1].clear();
    for (uint32_t e : out.node_e[l])
      for (int i = 0; i < 3; ++i) out.node_e[l + 1].push_back((e / 3 + 162 * i) % 486);
  }
  int s = 0;
  for (uint32_t e : out.node_e[4])
    for (int i = 0; i < 3; ++i) out.leaf_e[s++] = (e / 3 + 162 * i) % 486;
  return true;
}

// Offsets of each level's nodes in the 80-node twiddle arrays.
__host__ __device__ constexpr int node_off(int level) { return level == 1 ? 0 : level == 2 ? 2 : level == 3 ? 8 : 26; }

static void fill_consts(const PrimePlan& pl, PrimeConst& c) {
  memset(&c, 0, sizeof c);
  const uint64_t p = pl.p;
  auto pw = [&](int64_t e) { return (uint64_t)pl.pw[((e % 486) + 486) % 486]; };
  c.p = pl.p;
  c.bar = (uint32_t)((1ull << 32) / p);
  c.om = (uint32_t)pw(162);
  for (int l = 1; l <= 4; ++l)
    for (size_t n = 0; n < pl.node_e[l].size(); ++n) {
      uint32_t e = pl.node_e[l][n];
      int k = node_off(l) + (int)n;
      c.fw[k][0] = (uint32_t)pw(e / 3);
      c.fw[k][1] = (uint32_t)pw(2 * (e / 3));
      c.itw[k][0] = (uint32_t)pw(-(int64_t)(e / 3));
      c.itw[k][1] = (uint32_t)pw(-2 * (int64_t)(e / 3));
    }
  c.inv3 = inv_mod(3, p);
  c.iom = (uint32_t)pw(-162);
  c.iom2 = (uint32_t)pw(-324);
  c.w = (uint32_t)pw(81);
  c.w5 = (uint32_t)pw(405);
  c.inv_split = inv_mod((c.w + p - c.w5) % p, p);
  {
    // |r| <= (p - 1) / 2 + 3, |key| <= (p - 1) / 2, 4 products per element; stay inside int32
    const uint64_t h = (p - 1) / 2, per = 4 * (h + 4) * h;
    uint64_t r = (0x7fffffffull - p) / per;
    c.reduce_every = (uint32_t)(r < 1 ? 1 : r);
  }
  for (int s = 0; s < LEAVES; ++s) c.leaf_root[s] = (uint32_t)pw(pl.leaf_e[s]);
}

static uint32_t bits_of(u128 x) {
  uint32_t n = 0;
  while (x) ++n, x >>= 1;
  return n;
}

static bool is_prime32(uint32_t n) {
  if (n < 2) return false;
  for (uint32_t d = 2; d * d <= n; ++d)
    if (n % d == 0) return false;
  return true;
}

bool make_modulus_plan(u128 q, uint64_t elements, int extra_bits, ModulusPlan& mp, std::string& err) {
  mp = ModulusPlan();
  mp.q = q;
  mp.bits = bits_of(q - 1);
  mp.width = (mp.bits + 7) / 8;
  const u128 baseline = (u128)3889 * 9721 * 17497;
  if (q == baseline) {
    mp.nprimes = 3;
    mp.primes[0] = 3889, mp.primes[1] = 9721, mp.primes[2] = 17497;
    mp.exact_lift = false;
  } else {
    // |c| <= elements * 2 * 648 * (q - 1): per element each reduced coefficient takes at most
    // 2 x 648 products a_i w_k (X^648 = X^324 - 1, X^972 = -1). Need prod(p) > 2 |c| + 1.
    // Compare in log2 with a margin (the product itself may exceed 128 bits).
    const double need =
        std::log2((double)elements) + std::log2(1296.0) + std::log2((double)(q - 1)) + 1.0 + extra_bits + 0.01;
    double have = 0;
    mp.exact_lift = true;
    for (uint32_t p = 32767; p > 486 && have <= need; --p) {
      if (p % 486 != 1 || !is_prime32(p)) continue;
      if (mp.nprimes == MAX_PRIMES) break;
      mp.primes[mp.nprimes++] = p;
      have += std::log2((double)p);
    }
    if (have <= need) {
      err = "no set of transform primes covers this modulus";
      return false;
    }
    // product mod q, and floor(product / 2) in the mixed radix of the primes (digit k in [0, p_k))
    u128 pm = 1 % q;
    for (int i = 0; i < mp.nprimes; ++i) pm = pm * mp.primes[i] % q;  // pm < 2^96, p < 2^15
    mp.p_mod_q = pm;
    // halving a mixed-radix number: digits from the most significant down, carrying remainders
    uint64_t rem = 0;
    std::vector<uint32_t> d(mp.nprimes, 0);
    // the product itself has digits (0, ..., 0, 1) one place above the top; halve that
    rem = 1;
    for (int k = mp.nprimes - 1; k >= 0; --k) {
      const uint64_t cur = rem * mp.primes[k];  // value of the remainder in units of the next digit
      d[k] = (uint32_t)(cur / 2);
      rem = cur % 2;
    }
    for (int k = 0; k < mp.nprimes; ++k) mp.half_digits[k] = d[k];
  }
  mp.consts.resize(mp.nprimes);
  mp.btiles.assign((size_t)mp.nprimes * 3 * (TC_B_BYTES / 2), 0);
  for (int i = 0; i < mp.nprimes; ++i) {
    PrimePlan pl;
    if (!make_plan(mp.primes[i], pl)) {
      err = "transform prime rejected";
      return false;
    }
    fill_consts(pl, mp.consts[i]);
    fill_btiles(pl, mp.consts[i], mp.btiles.data() + (size_t)i * 3 * (TC_B_BYTES / 2));
    for (int j = 0; j < i; ++j) mp.garner_inv[i][j] = inv_mod(mp.primes[j], mp.primes[i]);
  }
  return true;
}


// ------------------------------------------------------------------------------------------------
// Device arithmetic modulo a prime below 2^15
// ------------------------------------------------------------------------------------------------
// x * w mod p in [0, 2p) for any x < 2^32, w < p, ws = floor(w 2^32 / p) (Shoup).
__device__ __forceinline__ uint32_t shoup(uint32_t x, uint32_t w, uint32_t ws, uint32_t p) {
  return x * w - __umulhi(x, ws) * p;
}
// x mod p for x < 2^32 (Barrett with bar = floor(2^32 / p)).
__device__ __forceinline__ uint32_t reduce32(uint32_t x, uint32_t bar, uint32_t p) {
  uint32_t r = x - __umulhi(x, bar) * p;
  return r >= p ? r - p : r;
}

// ------------------------------------------------------------------------------------------------
// The public matrix (rq.rs:53-144): element i is the keyed BLAKE3 XOF (key [0x5a; 32]) of
// "labinius-fast/ajtai-matrix/v1" || q (16 LE) || elements (8 LE) || i (8 LE); each coefficient
// reads `width` bytes little-endian, keeps `bits` bits, and is redrawn while >= q.
// ------------------------------------------------------------------------------------------------
struct MatrixArgs {
  uint64_t q_lo, q_hi;
  uint32_t width, bits;
  int nprimes;
  uint32_t primes[MAX_PRIMES];
  uint32_t two64[MAX_PRIMES];  // 2^64 mod p
};

// With `raw` set, the coefficients themselves are written (u128 little-endian), else their residues.
// With `only_if` set, the kernel does nothing unless *only_if is nonzero (the fallback of the
// parallel expansion below, launched behind it on the same stream).
__global__ void k_matrix_expand(MatrixArgs a, uint64_t elements, uint32_t* ared, uint4* raw, const int* only_if) {
  if (only_if && *only_if == 0) return;
  uint64_t m = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (m >= elements) return;
  bk::Hasher h;
  uint8_t key[32];
  for (int i = 0; i < 32; ++i) key[i] = 0x5a;
  h.init_keyed(key);
  const char dom[] = "labinius-fast/ajtai-matrix/v1";
  h.absorb((const uint8_t*)dom, sizeof(dom) - 1);
  uint8_t b[16];
  for (int i = 0; i < 8; ++i) b[i] = (uint8_t)(a.q_lo >> (8 * i)), b[8 + i] = (uint8_t)(a.q_hi >> (8 * i));
  h.absorb(b, 16);
  h.absorb_u64(elements);
  h.absorb_u64(m);
  bk::Pending root = h.finish();
  u128 q = ((u128)a.q_hi << 64) | a.q_lo;
  u128 mask = a.bits >= 128 ? ~(u128)0 : (((u128)1 << a.bits) - 1);
  uint8_t buf[64];
  uint64_t blk = 0;
  int pos = 64;
  for (int t = 0; t < RING_N; ++t) {
    u128 v;
    for (;;) {
      v = 0;
      for (uint32_t i = 0; i < a.width; ++i) {
        if (pos == 64) {
          uint32_t w[16];
          root.root_block(blk++, w);
          bk::store_words(w, buf, 16);
          pos = 0;
        }
        v |= (u128)buf[pos++] << (8 * i);
      }
      v &= mask;
      if (v < q) break;
    }
    uint64_t lo = (uint64_t)v, hi = (uint64_t)(v >> 64);
    if (raw) {
      raw[m * RING_N + t] = make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi, (uint32_t)(hi >> 32));
      continue;
    }
    for (int i = 0; i < a.nprimes; ++i) {
      uint64_t p = a.primes[i];
      uint64_t r = ((hi % p) * a.two64[i] + lo % p) % p;
      ared[((size_t)i * elements + m) * RING_N + t] = (uint32_t)r;
    }
  }
}

// The same expansion in parallel. Draw i of an element always sits at bytes [i w, (i + 1) w) of its
// XOF stream (a rejected draw still consumes its bytes), so: one thread per element derives the
// stream's root node; one thread per (element, 64-byte block) produces the first MX_DRAWS draws'
// blocks; one warp per element then tests 32 draws at a time and gives each accepted draw its
// coefficient index by a ballot prefix count. Every modulus accepts a draw with probability
// q / 2^bits > 1/2, so 1600 draws fall short of 648 acceptances with probability below 1e-13 per
// element; if one does, a flag releases the sequential kernel for the whole matrix.
constexpr int MX_DRAWS = 1600;

__global__ void k_matrix_roots(MatrixArgs a, uint64_t elements, uint64_t m0, uint64_t count, bk::Pending* roots) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= count) return;
  const uint64_t m = m0 + i;
  bk::Hasher h;
  uint8_t key[32];
  for (int k = 0; k < 32; ++k) key[k] = 0x5a;
  h.init_keyed(key);
  const char dom[] = "labinius-fast/ajtai-matrix/v1";
  h.absorb((const uint8_t*)dom, sizeof(dom) - 1);
  uint8_t b[16];
  for (int k = 0; k < 8; ++k) b[k] = (uint8_t)(a.q_lo >> (8 * k)), b[8 + k] = (uint8_t)(a.q_hi >> (8 * k));
  h.absorb(b, 16);
  h.absorb_u64(elements);
  h.absorb_u64(m);
  roots[i] = h.finish();
}

__global__ void k_matrix_xof(const bk::Pending* __restrict__ roots, uint64_t count, int nblk, uint4* __restrict__ buf) {
  const uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (g >= count * (uint64_t)nblk) return;
  const uint64_t i = g / nblk, blk = g % nblk;
  uint32_t w[16];
  roots[i].root_block(blk, w);
  uint4* o = buf + g * 4;
  o[0] = make_uint4(w[0], w[1], w[2], w[3]);
  o[1] = make_uint4(w[4], w[5], w[6], w[7]);
  o[2] = make_uint4(w[8], w[9], w[10], w[11]);
  o[3] = make_uint4(w[12], w[13], w[14], w[15]);
}

__global__ void __launch_bounds__(256) k_matrix_draw(MatrixArgs a, uint64_t elements, uint64_t m0, uint64_t count,
                                                     int nblk, const uint8_t* __restrict__ buf,
                                                     uint32_t* __restrict__ ared, uint4* __restrict__ raw,
                                                     int* short_flag) {
  const uint64_t i = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= count) return;
  const uint64_t m = m0 + i;
  const uint8_t* src = buf + i * (uint64_t)nblk * 64;
  const u128 q = ((u128)a.q_hi << 64) | a.q_lo;
  const u128 mask = a.bits >= 128 ? ~(u128)0 : (((u128)1 << a.bits) - 1);
  int accepted = 0;
  for (int base = 0; base < MX_DRAWS && accepted < RING_N; base += 32) {
    const int d = base + lane;
    u128 v = 0;
    bool ok = false;
    if (d < MX_DRAWS) {
      const uint8_t* p = src + (size_t)d * a.width;
      for (int k = (int)a.width - 1; k >= 0; --k) v = (v << 8) | p[k];
      v &= mask;
      ok = v < q;
    }
    const uint32_t bal = __ballot_sync(0xffffffffu, ok);
    const int t = accepted + __popc(bal & ((1u << lane) - 1u));
    if (ok && t < RING_N) {
      if (raw) {
        const uint64_t lo = (uint64_t)v, hi = (uint64_t)(v >> 64);
        raw[m * RING_N + t] = make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi, (uint32_t)(hi >> 32));
      } else {
        const uint64_t lo = (uint64_t)v, hi = (uint64_t)(v >> 64);
        for (int k = 0; k < a.nprimes; ++k) {
          const uint64_t pk = a.primes[k];
          ared[((size_t)k * elements + m) * RING_N + t] = (uint32_t)(((hi % pk) * a.two64[k] + lo % pk) % pk);
        }
      }
    }
    accepted += __popc(bal);
  }
  if (lane == 0 && accepted < RING_N) atomicExch(short_flag, 1);
}

// Scratch bytes of the parallel expansion per element (the XOF blocks of MX_DRAWS draws).
static size_t matrix_blocks(uint32_t width) { return ((size_t)MX_DRAWS * width + 63) / 64; }
size_t matrix_scratch_bytes(uint64_t elements, u128 q) {
  const uint32_t bits = bits_of(q - 1), width = (bits + 7) / 8;
  const uint64_t chunk = std::min<uint64_t>(elements, 8192);
  return chunk * (matrix_blocks(width) * 64 + sizeof(bk::Pending)) + 64;
}

static void matrix_parallel(const MatrixArgs& a, uint64_t elements, uint32_t* ared, uint4* raw, void* scratch,
                            cudaStream_t s) {
  const int nblk = (int)matrix_blocks(a.width);
  const uint64_t chunk = std::min<uint64_t>(elements, 8192);
  int* flag = reinterpret_cast<int*>(scratch);
  bk::Pending* roots = reinterpret_cast<bk::Pending*>(static_cast<uint8_t*>(scratch) + 64);
  uint8_t* buf = reinterpret_cast<uint8_t*>(roots + chunk);
  cudaMemsetAsync(flag, 0, 4, s);
  for (uint64_t m0 = 0; m0 < elements; m0 += chunk) {
    const uint64_t count = std::min(chunk, elements - m0);
    k_matrix_roots<<<(unsigned)((count + 127) / 128), 128, 0, s>>>(a, elements, m0, count, roots);
    const uint64_t nb = count * (uint64_t)nblk;
    k_matrix_xof<<<(unsigned)((nb + 255) / 256), 256, 0, s>>>(roots, count, nblk, reinterpret_cast<uint4*>(buf));
    k_matrix_draw<<<(unsigned)((count * 32 + 255) / 256), 256, 0, s>>>(a, elements, m0, count, nblk, buf, ared, raw,
                                                                        flag);
  }
  // the sequential expansion, which returns at once unless an element fell short
  k_matrix_expand<<<(unsigned)((elements + 63) / 64), 64, 0, s>>>(a, elements, ared, raw, flag);
}

void launch_matrix_expand(const ModulusPlan& mp, uint64_t elements, uint32_t* ared, void* scratch, cudaStream_t s) {
  MatrixArgs a;
  memset(&a, 0, sizeof a);
  a.q_lo = (uint64_t)mp.q;
  a.q_hi = (uint64_t)(mp.q >> 64);
  a.width = mp.width;
  a.bits = mp.bits;
  a.nprimes = mp.nprimes;
  for (int i = 0; i < mp.nprimes; ++i) {
    a.primes[i] = mp.primes[i];
    a.two64[i] = (uint32_t)powmod(powmod(2, 32, mp.primes[i]), 2, mp.primes[i]);
  }
  matrix_parallel(a, elements, ared, nullptr, scratch, s);
}

void launch_matrix_raw(u128 q, uint64_t elements, void* out, void* scratch, cudaStream_t s) {
  MatrixArgs a;
  memset(&a, 0, sizeof a);
  a.q_lo = (uint64_t)q;
  a.q_hi = (uint64_t)(q >> 64);
  a.bits = bits_of(q - 1);
  a.width = (a.bits + 7) / 8;
  matrix_parallel(a, elements, nullptr, reinterpret_cast<uint4*>(out), scratch, s);
}

// ------------------------------------------------------------------------------------------------
// Key transform: A_m = sum_k X^k A_{m,k}(Y); the 162-point transform of each A_{m,k}, then the
// base-multiplication matrix of every leaf: M[k][l] = A_{l-k}(c) for l >= k, c A_{l-k+4}(c) else.
// ------------------------------------------------------------------------------------------------
__device__ void forward162(uint32_t* x, const PrimeConst& P) {
  // residues below p < 2^15: every sum of products below stays under 2^32 before its reduction
  const uint32_t p = P.p, bar = P.bar, w = P.w, w5 = P.w5;
  const uint32_t om = P.om, om2 = reduce32(P.om * P.om, bar, p);
  for (int j = 0; j < 81; ++j) {
    const uint32_t a = x[j], b = x[j + 81];
    x[j] = reduce32(a + w * b, bar, p);
    x[j + 81] = reduce32(a + w5 * b, bar, p);
  }
  int len = 81;
  for (int l = 1; l <= 4; ++l) {
    int sub = len / 3, nodes = 162 / len;
    for (int n = 0; n < nodes; ++n) {
      const uint32_t* tw = P.fw[node_off(l) + n];
      const uint32_t t0 = tw[0], t1 = tw[1];
      for (int q = 0; q < sub; ++q) {
        int o = n * len + q;
        const uint32_t a0 = x[o], a1 = reduce32(x[o + sub] * t0, bar, p), a2 = reduce32(x[o + 2 * sub] * t1, bar, p);
        x[o] = reduce32(a0 + a1 + a2, bar, p);
        x[o + sub] = reduce32(a0 + a1 * om + a2 * om2, bar, p);
        x[o + 2 * sub] = reduce32(a0 + a1 * om2 + a2 * om, bar, p);
      }
    }
    len = sub;
  }
}

__global__ void k_key_forward(const PrimeConst* __restrict__ pcs, int nprimes, uint64_t elements, const uint32_t* ared,
                              uint32_t* leafvals) {
  uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  uint64_t total = (uint64_t)nprimes * elements * 4;
  if (tid >= total) return;
  int k = (int)(tid & 3);
  uint64_t m = (tid >> 2) % elements;
  int pi = (int)((tid >> 2) / elements);
  const uint32_t* a = ared + ((size_t)pi * elements + m) * RING_N;
  uint32_t x[LEAVES];
  for (int p = 0; p < LEAVES; ++p) x[p] = a[4 * p + k];
  forward162(x, pcs[pi]);
  uint32_t* o = leafvals + (((size_t)pi * elements + m) * 4 + k) * LEAVES;
  for (int s = 0; s < LEAVES; ++s) o[s] = x[s];
}

__global__ void k_key_leafform(const PrimeConst* __restrict__ pcs, int nprimes, uint64_t elements,
                               const uint32_t* leafvals, uint32_t* key) {
  uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  uint64_t total = (uint64_t)nprimes * elements * LEAVES;
  if (tid >= total) return;
  int s = (int)(tid % LEAVES);
  uint64_t m = (tid / LEAVES) % elements;
  int pi = (int)(tid / LEAVES / elements);
  const PrimeConst& P = pcs[pi];
  const uint64_t p = P.p, c = P.leaf_root[s];
  const uint32_t* lv = leafvals + ((size_t)pi * elements + m) * 4 * LEAVES;
  uint64_t A[4];
  for (int k = 0; k < 4; ++k) A[k] = lv[k * LEAVES + s];
  uint32_t* o = key + (((size_t)pi * elements + m) * LEAVES + s) * 16;
  for (int k = 0; k < 4; ++k)
    for (int l = 0; l < 4; ++l) o[4 * k + l] = (uint32_t)(l >= k ? A[l - k] : c * A[l - k + 4] % p);
}

void launch_key_transform(const ModulusPlan& mp, uint64_t elements, const uint32_t* ared, uint32_t* leafvals,
                          uint32_t* key, cudaStream_t s) {
  uint64_t t1 = (uint64_t)mp.nprimes * elements * 4;
  k_key_forward<<<(unsigned)((t1 + 127) / 128), 128, 0, s>>>(mp.dconsts, mp.nprimes, elements, ared, leafvals);
  uint64_t t2 = (uint64_t)mp.nprimes * elements * LEAVES;
  k_key_leafform<<<(unsigned)((t2 + 127) / 128), 128, 0, s>>>(mp.dconsts, mp.nprimes, elements, leafvals, key);
}

// ------------------------------------------------------------------------------------------------
// K1 on the tensor cores.
//
// The transform of a table word (128 bits = the Y-coefficients 0..127 of one residue class of X
// mod 4) at leaf s is the evaluation sum_j bit_j zeta_s^j (mod p), zeta_s the leaf's root: a
// product with the Vandermonde matrix V[s][j] = zeta_s^j. On the tensor core it is exact:
//   A (M = 128 table columns x 128 bits) holds each set bit as a power of two a_kappa (bf16 with
//   one exponent bit, see commit_expand_word) and is read twice;
//   B (N = 64 x K = 256) holds per leaf (V mod 256) / a against the first reading and
//   (V >> 8) * 256 / a against the second (both exact in bf16), so the product adds
//   L = sum_j bit_j V[s][j] < 2^22, an exact integer.
// One more MMA per word (A and B constant tiles in shared memory) first sets every accumulator
// to k p, the least multiple of p at or above 2^23, so D = k p + L is an integer in [2^23, 2^24)
// (exact in f32 throughout: every partial sum is a nonnegative integer below 2^24) and its bit
// pattern is 0x4A800000 + D. The epilogue then reduces with one FFMA and one IMAD:
// bits(D * (1/p) + 1.5 * 2^23 - k) = 0x4B400000 + rint(L / p), and bits(D) - p * that = r + OFF
// (mod 2^32) with |r| <= p/2 + 3 and OFF a per-prime constant, and does the 4x4 base
// multiplication with the key on the integer pipe.
//
// Block = one prime x one third of its 162 leaves (54) x 128 table columns x an element range.
// Tensor memory (512 columns) holds four word stages k = 0..3 (the four words of an element):
// stage k = A (the expanded bits of word k of the current element, columns 128 k .. +63) and D
// (its 64 leaf sums, columns 128 k + 64 .. +63). Roles, all meeting on per-stage mbarriers:
//   warps 24-27 (producers; thread t = table column t = TMEM lane t): fetch words and key rows by
//     cp.async two elements ahead; per element centre the key rows into a 4-element ring
//     (arrive kfull), then per word k wait until the MMAs of the previous element's word k are
//     done (done[k]), expand the word into stage k's A columns with tcgen05.st and arrive full[k];
//   warp 28 + k (stage k's issuer): per element waits full[k] and dfree[k] (the epilogue has read
//     the previous D of stage k), issues the word's 16 MMAs (A from TMEM, B = the leaf tile in
//     shared memory) from lane 0 and commits them to done[k]. A thread issues a small MMA only
//     every 50-70 cycles, so each stage has its own issuer and no issuer does other work;
//   warps 0-23 (epilogue; warp w reads TMEM lanes 32 (w % 4) .. +31, leaves 9 (w / 4) + i, whose
//     D columns are 8 (w / 4) .. + 7 and 48 + w / 4, so two tcgen05.ld per word):
//     per word wait done[k], load the 9 sums, arrive dfree[k], reduce and accumulate 9 x 4 values.
// Registers: the block launches with 64 a thread; the issuers give theirs down to 32 and the
// producers to 48 (setmaxnreg), so each epilogue thread holds its 36 accumulators in 72.
// So the expansion, the MMAs and the epilogue of different words run at the same time, and no
// table bits pass through shared memory. Every wait is bounded (about a second); a timeout sets
// *status = 3 and the abort flag, on which every role leaves its loop; TMEM is released after the
// issuers' last commits drained.
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
// One table word -> the 64 TMEM columns of its A row (K positions 2o and 2o + 1 in column o): u32 o
// holds bits o % 16 and o % 16 + 16 of word o / 16, and a set bit at K position kappa is the bf16
// with the single exponent bit 11 + (kappa / 2 & 3): 2^-111, 2^-95, 2^-63 or 2. One shift of the
// source serves four columns through four masks; the B tiles carry the inverse powers of two, so
// every product is the integer bit * V.
__device__ __forceinline__ void commit_expand_word(uint32_t tA, uint4 v) {
  const uint32_t xs[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const uint32_t x = xs[m];
    uint32_t u[16];
#pragma unroll
    for (int qq = 0; qq < 4; ++qq) {
      const uint32_t y = qq < 3 ? x << (11 - 4 * qq) : x >> 1;
      u[4 * qq + 0] = y & 0x08000800u;
      u[4 * qq + 1] = y & 0x10001000u;
      u[4 * qq + 2] = y & 0x20002000u;
      u[4 * qq + 3] = y & 0x40004000u;
    }
    tc::tmem_st_x16(tA + 16 * m, u);
  }
}
// Value of a set bit at K position kappa (0..127) of an expanded word.
static double commit_bit_value(int kappa) {
  const int b = (kappa >> 1) & 3;
  return b == 3 ? 2.0 : b == 2 ? ldexp(1.0, -63) : b == 1 ? ldexp(1.0, -95) : ldexp(1.0, -111);
}

__global__ void __launch_bounds__(TC_THREADS, 1)
    k_commit_tc(const uint4* __restrict__ table, const uint32_t* __restrict__ key, const uint4* __restrict__ btiles,
                const PrimeConst* __restrict__ pcs, uint32_t* __restrict__ partial, int rl, int elements,
                int per_split, int nprimes, int split_base, int* status, const uint32_t* ready, uint32_t epoch,
                int part_elems, long long ready_wait) {
  extern __shared__ __align__(1024) uint8_t tsm[];
  uint8_t* sB = tsm;
  int* sKey = reinterpret_cast<int*>(tsm + TC_B_BYTES);                            // [4][TC_KEY_INTS]
  uint4* wring = reinterpret_cast<uint4*>(sKey + 4 * TC_KEY_INTS);                  // [3][128 columns][4 words]
  uint4* kraw = wring + 3 * TC_COLS * 4;                                            // [3][TC_KEY_INTS / 4]
  uint4* csum = kraw + 3 * (TC_KEY_INTS / 4);                                       // [4][TC_LEAVES]
  uint64_t* bars = reinterpret_cast<uint64_t*>(csum + 4 * TC_LEAVES);
  uint64_t* full = bars;        // [4] producers wrote stage k's A (128 arrivals)
  uint64_t* done = bars + 4;    // [4] the MMAs of stage k completed (tensor-core commit)
  uint64_t* dfree = bars + 8;   // [4] the epilogue loaded stage k's D (24 arrivals)
  uint64_t* kfull = bars + 12;  // [4] key ring slot ready (128 arrivals)
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 16);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);

  const int pi = blockIdx.x / 3, third = blockIdx.x % 3;
  const int col0 = blockIdx.y * TC_COLS;
  const int split = split_base + (int)blockIdx.z;
  const int m_begin = split * per_split;
  const int nelem = max(0, min(elements, m_begin + per_split) - m_begin);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    *abort_flag = 0;
    for (int k = 0; k < 4; ++k) {
      tc::mbar_init(&full[k], 4 * 32);
      tc::mbar_init(&done[k], 1);
      tc::mbar_init(&dfree[k], 24);
      tc::mbar_init(&kfull[k], 4 * 32);
    }
    tc::mbar_init_fence();
  }
  if (warp == 0) tc::tmem_alloc(tslot, 512);
  {
    const uint4* src = btiles + (size_t)blockIdx.x * (TC_B_BYTES / 16);
    for (int i = tid; i < TC_B_BYTES / 16; i += TC_THREADS) reinterpret_cast<uint4*>(sB)[i] = src[i];
    // the init MMA: A row = (1, 1, 1, 0, ...), B row = the three 8-bit pieces of k p (bf16-exact), so
    // every D entry starts at k p = the least multiple of p at or above 2^23
    const uint32_t pp = pcs[pi].p, kp = ((0x800000u + pp - 1) / pp) * pp;
    const uint16_t one = 0x3F80;
    const uint16_t pc[3] = {(uint16_t)(__float_as_uint((float)(kp & 0xFF0000u)) >> 16),
                            (uint16_t)(__float_as_uint((float)(kp & 0xFF00u)) >> 16),
                            (uint16_t)(__float_as_uint((float)(kp & 0xFFu)) >> 16)};
    uint16_t* ca = reinterpret_cast<uint16_t*>(tsm + TC_CONST_AT);
    for (int i = tid; i < (4096 + 2048) / 2; i += TC_THREADS) {
      uint16_t val = 0;
      // both tiles: core (row group, k core) at group * 256 + kcore * 128, row r at r * 16, k % 8 at 2 (k % 8)
      const int off = (i < 2048 ? i : i - 2048) * 2;
      const int kcore = (off >> 7) & 1, within = off & 127, k = kcore * 8 + ((within & 15) >> 1);
      if (k < 3) val = i < 2048 ? one : pc[k];
      ca[i] = val;
    }
  }
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *tslot;
  const uint32_t p = pcs[pi].p;
  int last_e = -1;  // an issuer's last commit

  // Registers: the launch gives 64 a thread (65,536); issuers keep 32, producers 48 and the
  // 24 epilogue warps take the rest, 72 each (768 x 72 + 128 x 48 + 128 x 32 = 65,536).
  if (warp >= 28) {
    // ---------------- issuer of stage k ----------------
    tc::regs_dec<32>();
    const int k = warp - 28;
    const uint32_t idesc = tc::idesc_bf16_f32(TC_COLS, TC_N);
    const uint64_t bdesc0 = tc::sdesc(tc::smem_u32(sB), 128, 4096);
    const uint64_t adesc_c = tc::sdesc(tc::smem_u32(tsm + TC_CONST_AT), 128, 256);
    const uint64_t bdesc_c = tc::sdesc(tc::smem_u32(tsm + TC_CONST_AT + 4096), 128, 256);
    const uint32_t st = tbase + 128 * k;
    for (int e = 0; e < nelem; ++e) {
      int iok = 1;
      if (lane == 0) {
        iok = tc::mbar_wait_fast(&full[k], e & 1, abort_flag, TC_WAIT_CYCLES) &&
              (e == 0 || tc::mbar_wait_fast(&dfree[k], (e - 1) & 1, abort_flag, TC_WAIT_CYCLES));
        if (iok) {
          tc::fence_after_sync();
          tc::mma_bf16(st + 64, adesc_c, bdesc_c, idesc, 0u);
#pragma unroll
          for (int kk = 0; kk < TC_K / 16; ++kk)
            tc::mma_bf16_ta(st + 64, st + 8 * (kk & 7), bdesc0 + (uint64_t)(kk * 16), idesc, 1u);
          tc::mma_commit(&done[k]);
          last_e = e;
        } else if (!*abort_flag) {
          *abort_flag = 1;
          atomicExch(status, 3);
        }
      }
      if (!__shfl_sync(0xffffffffu, iok, 0)) break;
    }
  } else if (warp >= 24) {
    // ---------------- producers ----------------
    tc::regs_dec<48>();
    const int t = tid - 24 * 32;  // table column, TMEM lane
    const uint4* wsrc = table + ((size_t)(col0 + t) << rl);
    const uint4* ksrc = reinterpret_cast<const uint4*>(key) +
                        ((size_t)pi * elements * LEAVES + TC_LEAVES * third) * 4;
    const int half = (int)(p - 1) / 2;
    const int reduce_every = (int)pcs[pi].reduce_every;
    uint4 cum[2] = {make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0)};
    const uint32_t tl = tbase + ((uint32_t)(32 * (warp - 24)) << 16);
    // The table is known to be in device memory below element next_wait (the end of the last
    // part waited for): one compare per element, the division only when a new part begins (an
    // integer division per element slowed every block of a streamed proof by 5 %).
    int next_wait = 0;
    auto fetch = [&](int e) {  // element e's words (this column) and key rows t, t + 128 into ring slot e % 3
      if (e < nelem && ready && m_begin + e >= next_wait) {
        // The table is still arriving: part (m_begin + e) / part_elems is there once the copy
        // stream has written the proof's epoch into its flag (after the part's copy).
        const int part = (m_begin + e) / part_elems;
        const long long t0 = clock64();
        while ((int)(ld_acquire_u32(ready + part) - epoch) < 0) {
          if (*abort_flag || *reinterpret_cast<volatile int*>(status) || clock64() - t0 > ready_wait) {
            if (!*abort_flag) {
              *abort_flag = 1;
              atomicExch(status, 3);
            }
            break;
          }
          __nanosleep(256);
        }
        next_wait = (part + 1) * part_elems;
      }
      if (e < nelem && !*abort_flag) {
        const size_t m = (size_t)(m_begin + e);
        uint4* w = wring + ((e % 3) * TC_COLS + t) * 4;
#pragma unroll
        for (int k = 0; k < 4; ++k) tc::cp_async16(w + k, wsrc + 4 * m + k);
        uint4* kr = kraw + (e % 3) * (TC_KEY_INTS / 4);
        tc::cp_async16(kr + t, ksrc + m * LEAVES * 4 + t);
        if (t + 128 < TC_KEY_INTS / 4) tc::cp_async16(kr + t + 128, ksrc + m * LEAVES * 4 + t + 128);
      }
      tc::cp_async_commit();
    };
    fetch(0);
    fetch(1);
    for (int e = 0; e < nelem; ++e) {
      if (__any_sync(0xffffffffu, *abort_flag)) break;
      fetch(e + 2);
      tc::cp_async_wait<2>();
      {
        const uint4* kr = kraw + (e % 3) * (TC_KEY_INTS / 4);
        int4* kd = reinterpret_cast<int4*>(sKey + (e & 3) * TC_KEY_INTS);
        const bool restart = e % reduce_every == 0;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const int i = t + 128 * j;  // key row: leaf i / 4, word i % 4
          uint4 v = make_uint4(0, 0, 0, 0);
          if (i < TC_KEY_INTS / 4) {
            const uint4 u = kr[i];  // centred into (-p/2, p/2]
            v.x = (int)u.x > half ? u.x - p : u.x;
            v.y = (int)u.y > half ? u.y - p : u.y;
            v.z = (int)u.z > half ? u.z - p : u.z;
            v.w = (int)u.w > half ? u.w - p : u.w;
            reinterpret_cast<uint4*>(kd)[i] = v;
          }
          // the leaf's four rows sit in lanes 4 (i / 4) .. + 3: their sum, and its running total
          // over the epilogue's reduction window, kept by the first of them (mod 2^32)
#pragma unroll
          for (int o = 1; o <= 2; o <<= 1) {
            v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
            v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
            v.z += __shfl_xor_sync(0xffffffffu, v.z, o);
            v.w += __shfl_xor_sync(0xffffffffu, v.w, o);
          }
          if (restart) cum[j] = make_uint4(0, 0, 0, 0);
          cum[j].x += v.x, cum[j].y += v.y, cum[j].z += v.z, cum[j].w += v.w;
          if ((t & 3) == 0 && i < TC_KEY_INTS / 4) csum[(e & 3) * TC_LEAVES + (i >> 2)] = cum[j];
        }
        tc::mbar_arrive(&kfull[e & 3]);
      }
      bool ok = true;
      for (int k = 0; k < 4 && ok; ++k) {
        if (e > 0) ok = __all_sync(0xffffffffu, tc::mbar_wait_fast(&done[k], (e - 1) & 1, abort_flag, TC_WAIT_CYCLES));
        if (!ok) break;
        tc::fence_after_sync();
        commit_expand_word(tl + 128 * k, wring[((e % 3) * TC_COLS + t) * 4 + k]);
        tc::tmem_wait_st();
        tc::fence_before_sync();
        tc::mbar_arrive(&full[k]);
      }
      if (!ok) {
        if (lane == 0 && !*abort_flag) {
          *abort_flag = 1;
          atomicExch(status, 3);
        }
        break;
      }
    }
    tc::cp_async_wait<0>();
  } else {
    // ---------------- epilogue ----------------
    tc::regs_inc<72>();
    const uint32_t bar = pcs[pi].bar;
    const int reduce_every = (int)pcs[pi].reduce_every;
    const int g = warp >> 2, qd = warp & 3;
    const int c = 32 * qd + lane;
    const float invp = 1.0f / (float)p;
    const uint32_t bias = (0x80000000u / p) * p;
    // D = k p + L (an integer in [2^23, 2^24): bits(D) = 0x4A800000 + D); rint(D / p) - k + 1.5 * 2^23
    // by one FFMA (Cq = 1.5 * 2^23 - k, exact); then bits(D) - p * bits(that) = r + OFF (mod 2^32)
    const uint32_t kk_ = (0x800000u + p - 1) / p, kp = kk_ * p;
    const float Cq = (float)(12582912u - kk_);
    const uint32_t OFF = 0x4A800000u + kp - p * 0x4B400000u;
    // acc accumulates key * (r + OFF) mod 2^32; settling a reduction window subtracts OFF times
    // the window's key sums (kept by the producers), which leaves the exact sum of key * r (it
    // fits in 32 bits over reduce_every elements), and reduces it mod p.
    uint32_t acc[9][4];
#pragma unroll
    for (int i = 0; i < 9; ++i)
#pragma unroll
      for (int l = 0; l < 4; ++l) acc[i][l] = 0;
    auto settle = [&](int e) {
      const uint4* cs = csum + (e & 3) * TC_LEAVES + 9 * g;
#pragma unroll
      for (int i = 0; i < 9; ++i) {
        const uint4 w = cs[i];
        acc[i][0] = reduce32(acc[i][0] - OFF * w.x + bias, bar, p);
        acc[i][1] = reduce32(acc[i][1] - OFF * w.y + bias, bar, p);
        acc[i][2] = reduce32(acc[i][2] - OFF * w.z + bias, bar, p);
        acc[i][3] = reduce32(acc[i][3] - OFF * w.w + bias, bar, p);
      }
    };
    const uint32_t tb = tbase + ((uint32_t)(32 * qd) << 16) + 64 + 8 * g;  // leaves 9 g .. + 7; 9 g + 8 at 48 + g
    int since = 0;
    bool ok = true;
    for (int e = 0; e < nelem && ok; ++e) {
      ok = __all_sync(0xffffffffu, tc::mbar_wait_fast(&kfull[e & 3], (e >> 2) & 1, abort_flag, TC_WAIT_CYCLES));
      const int4* kp = reinterpret_cast<const int4*>(sKey + (e & 3) * TC_KEY_INTS) + 9 * g * 4;
      for (int k = 0; k < 4 && ok; ++k) {
        ok = __all_sync(0xffffffffu, tc::mbar_wait_fast(&done[k], e & 1, abort_flag, TC_WAIT_CYCLES));
        if (!ok) break;
        tc::fence_after_sync();
        const uint32_t ta = tb + 128 * k;
        uint32_t v[9];
        tc::tmem_ld_x8(ta, v);
        tc::tmem_ld_x1(ta - 8 * g + 48 + g, v[8]);
        tc::tmem_wait_ld(v);
        tc::fence_before_sync();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&dfree[k]);
#pragma unroll
        for (int i = 0; i < 9; ++i) {
          const uint32_t qb = __float_as_uint(fmaf(__uint_as_float(v[i]), invp, Cq));  // 0x4B400000 + q
          const uint32_t ri = v[i] - p * qb;                                             // r + OFF
          const uint4 kv = reinterpret_cast<const uint4*>(kp)[i * 4 + k];
          acc[i][0] += kv.x * ri;
          acc[i][1] += kv.y * ri;
          acc[i][2] += kv.z * ri;
          acc[i][3] += kv.w * ri;
        }
      }
      if (ok && ++since == reduce_every) {
        since = 0;
        settle(e);
      }
    }
    if (!ok && lane == 0 && !*abort_flag) {
      *abort_flag = 1;
      atomicExch(status, 3);
    }
    if (!*abort_flag) {
      if (since > 0) settle(nelem - 1);
      uint32_t* out = partial + ((((size_t)split * nprimes + pi) * COLUMNS + col0 + c) * LEAVES + TC_LEAVES * third +
                                 9 * g) * 4;
#pragma unroll
      for (int i = 0; i < 9; ++i)
        reinterpret_cast<uint4*>(out)[i] = make_uint4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
    }
  }
  // Drain: an issuer's last commit covers every MMA it issued; TMEM is released only after them.
  if (warp >= 28 && lane == 0 && last_e >= 0) {
    const long long t0 = clock64();
    while (!tc::mbar_try_wait(&done[warp - 28], last_e & 1) && clock64() - t0 < TC_WAIT_CYCLES) {
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tbase, 512);
}

// B tiles of K1 on the tensor cores, per (prime, third): row 8 g + i = leaf 9 g + i of the third
// for i < 8, row 48 + g = leaf 9 g + 8 (rows 54..63 zero); K position kappa < 128 carries the low limb of bit j(kappa),
// kappa >= 128 the high limb of bit j(kappa - 128), j = tc::row_bit (the expansion's order); bf16 in
// the no-swizzle K-major core-matrix layout (8 x 16 B cores, K-adjacent 128 B apart, 8-row
// groups 4096 B apart).
static void fill_btiles(const PrimePlan& pl, const PrimeConst& c, uint16_t* out /* 3 x TC_B_BYTES/2 */) {
  const uint64_t p = pl.p;
  for (int third = 0; third < 3; ++third) {
    uint16_t* tile = out + (size_t)third * (TC_B_BYTES / 2);
    memset(tile, 0, TC_B_BYTES);
    for (int g = 0; g < 6; ++g)
      for (int i = 0; i < 9; ++i) {
        const int n = i < 8 ? 8 * g + i : 48 + g, s = TC_LEAVES * third + 9 * g + i;
        uint64_t pw[128];  // V[s][j] = zeta_s^j
        pw[0] = 1;
        for (int j = 1; j < 128; ++j) pw[j] = pw[j - 1] * c.leaf_root[s] % p;
        for (int kappa = 0; kappa < TC_K; ++kappa) {
          const int limb = kappa >> 7;
          const uint64_t V = pw[tc::row_bit(kappa & 127)];
          const double scale = 1.0 / commit_bit_value(kappa & 127);  // exact power of two
          const float f = (float)(limb == 0 ? (double)(V & 255) * scale : (double)(V >> 8) * 256.0 * scale);
          uint32_t u;
          memcpy(&u, &f, 4);
          const size_t off = (size_t)(n >> 3) * 4096 + (kappa >> 3) * 128 + (n & 7) * 16 + (kappa & 7) * 2;
          tile[off / 2] = (uint16_t)(u >> 16);
        }
      }
  }
}

// Element splits of K1: the grid (8 column tiles x primes x 3 leaf thirds x splits), one block
// per SM, should fill whole waves; among 8..40 splits take the one with the least idle SM time,
// then the fewest.
int commit_splits(uint64_t elements, int nprimes, int sms) {
  if (sms < 1) sms = 1;
  int best = 1;
  double best_eff = -1;
  for (int s = 8; s <= 40; ++s) {
    if ((uint64_t)s * 8 > elements) break;
    const long blocks = (long)(COLUMNS / TC_COLS) * nprimes * 3 * s;
    const long waves = (blocks + sms - 1) / sms;
    const double eff = (double)blocks / (double)(waves * sms);
    if (eff > best_eff + 1e-9) best_eff = eff, best = s;
  }
  if (best_eff < 0) {
    best = 1;
    while ((uint64_t)best * 2 <= elements && best < 8) best *= 2;
  }
  return best;
}

void launch_commit(const ModulusPlan& mp, const Shape& sh, const uint4* table, const uint32_t* key,
                   const uint16_t* btiles, uint32_t* partial, int splits, int* status, cudaStream_t s, int split_begin,
                   int split_end, const uint32_t* ready, uint32_t epoch, int part_elems, long long ready_wait) {
  const int elements = (int)sh.ring_elements;
  const int per = (elements + splits - 1) / splits;
  if (split_end < 0) split_end = splits;
  if (split_end <= split_begin) return;
  static std::atomic<unsigned long long> attr{0};
  smem_limit(k_commit_tc, TC_SMEM, attr);
  dim3 grid(mp.nprimes * 3, COLUMNS / TC_COLS, split_end - split_begin);
  k_commit_tc<<<grid, TC_THREADS, TC_SMEM, s>>>(table, key, reinterpret_cast<const uint4*>(btiles), mp.dconsts, partial,
                                                 sh.rl, elements, per, mp.nprimes, split_begin, status, ready, epoch,
                                                 part_elems > 0 ? part_elems : elements,
                                                 ready_wait > 0 ? ready_wait : TC_WAIT_CYCLES);
}

int commit_blocks_per_split(const ModulusPlan& mp) { return mp.nprimes * 3 * (COLUMNS / TC_COLS); }

// Element range [m0, m1) of split range [s0, s1): the part of every column those splits read.
void commit_split_elements(uint64_t elements, int splits, int s0, int s1, uint64_t& m0, uint64_t& m1) {
  const uint64_t per = (elements + splits - 1) / splits;
  m0 = std::min<uint64_t>(elements, (uint64_t)s0 * per);
  m1 = std::min<uint64_t>(elements, (uint64_t)s1 * per);
}

// ------------------------------------------------------------------------------------------------
// K2: sum the element splits, inverse transform per prime and coefficient of X, CRT, pack.
// One block per column.
// ------------------------------------------------------------------------------------------------
struct FinishArgs {
  int nprimes, splits;
  uint32_t width;
  int exact;                     // 1: lift to the signed integer, then mod q
  uint64_t q_lo, q_hi, pq_lo, pq_hi;  // q and (product of the primes) mod q
  uint32_t primes[MAX_PRIMES];
  uint32_t half[MAX_PRIMES];     // floor(product / 2), mixed radix
  uint32_t ginv[MAX_PRIMES][MAX_PRIMES];
  uint32_t bar[MAX_PRIMES];      // floor(2^32 / p): every reduction below is of a value under 2^32
};

__global__ void __launch_bounds__(256) k_commit_finish(FinishArgs a, const PrimeConst* __restrict__ pcs,
                                                       const uint32_t* __restrict__ partial, uint8_t* __restrict__ out) {
  __shared__ uint32_t v[MAX_PRIMES][4][LEAVES];
  const int col = blockIdx.x;
  for (int e = threadIdx.x; e < a.nprimes * 4 * LEAVES; e += blockDim.x) {
    int pi = e / (4 * LEAVES), rem = e % (4 * LEAVES), s = rem / 4, l = rem % 4;
    uint32_t sum = 0;  // at most 40 splits of residues below 2^15
    for (int sp = 0; sp < a.splits; ++sp)
      sum += partial[(((size_t)sp * a.nprimes + pi) * COLUMNS + col) * LEAVES * 4 + rem];
    v[pi][l][s] = reduce32(sum, a.bar[pi], a.primes[pi]);
  }
  __syncthreads();
  // Inverse radix-3 levels 4..1: nodes of length 3, 9, 27, 81.
  int len = 3;
  for (int lvl = 4; lvl >= 1; --lvl) {
    const int sub = len / 3, nodes = LEAVES / len, per_t = nodes * sub;
    for (int e = threadIdx.x; e < a.nprimes * 4 * per_t; e += blockDim.x) {
      int pi = e / (4 * per_t), rem = e % (4 * per_t), l = rem / per_t, r2 = rem % per_t;
      int n = r2 / sub, q = r2 % sub;
      const PrimeConst& P = pcs[pi];
      const uint32_t p = P.p, bar = P.bar;  // residues below 2^15: sums of two products stay under 2^32
      uint32_t* x = v[pi][l];
      int o = n * len + q;
      const uint32_t y0 = x[o], y1 = x[o + sub], y2 = x[o + 2 * sub];
      const uint32_t a0 = reduce32(y0 + y1 + y2, bar, p);
      const uint32_t a1 = reduce32(y0 + y1 * P.iom + y2 * P.iom2, bar, p);
      const uint32_t a2 = reduce32(y0 + y1 * P.iom2 + y2 * P.iom, bar, p);
      const uint32_t* it = P.itw[node_off(lvl) + n];
      x[o] = reduce32(a0 * P.inv3, bar, p);
      x[o + sub] = reduce32(reduce32(a1 * P.inv3, bar, p) * it[0], bar, p);
      x[o + 2 * sub] = reduce32(reduce32(a2 * P.inv3, bar, p) * it[1], bar, p);
    }
    __syncthreads();
    len *= 3;
  }
  for (int e = threadIdx.x; e < a.nprimes * 4 * 81; e += blockDim.x) {
    int pi = e / (4 * 81), rem = e % (4 * 81), l = rem / 81, j = rem % 81;
    const PrimeConst& P = pcs[pi];
    const uint32_t p = P.p, bar = P.bar;
    uint32_t* x = v[pi][l];
    const uint32_t u = x[j], w = x[j + 81];
    const uint32_t b = reduce32(reduce32(u + p - w, bar, p) * P.inv_split, bar, p);
    x[j] = reduce32(u + p * p - P.w * b, bar, p);
    x[j + 81] = b;
  }
  __syncthreads();
  // Coefficient 4p + l of the column is coefficient p of C_l. Garner's CRT into [0, Q).
  for (int i = threadIdx.x; i < RING_N; i += blockDim.x) {
    int pp = i >> 2, l = i & 3;
    uint32_t digit[MAX_PRIMES];
    for (int k = 0; k < a.nprimes; ++k) {
      const uint32_t pk = a.primes[k], bk = a.bar[k];
      uint32_t t = v[k][l][pp];
      // t <- (r_k - (d_0 + p_0 d_1 + ...)) / (p_0 ... p_{k-1}) mod p_k, digit by digit
      for (int j = 0; j < k; ++j) t = reduce32(reduce32(t + pk - reduce32(digit[j], bk, pk), bk, pk) * a.ginv[k][j], bk, pk);
      digit[k] = t;
    }
    u128 val = 0;
    if (!a.exact) {
      // the primes' product is q itself: the mixed-radix value is the coefficient in [0, q)
      for (int k = a.nprimes - 1; k >= 0; --k) val = val * a.primes[k] + digit[k];
    } else {
      // signed integer in (-P/2, P/2]: negative when the digits exceed floor(P/2)'s
      bool neg = false;
      for (int k = a.nprimes - 1; k >= 0; --k)
        if (digit[k] != a.half[k]) {
          neg = digit[k] > a.half[k];
          break;
        }
      const u128 q = ((u128)a.q_hi << 64) | a.q_lo;
      for (int k = a.nprimes - 1; k >= 0; --k) val = (val * a.primes[k] + digit[k]) % q;  // < 2^111 before %
      if (neg) {
        const u128 pq = ((u128)a.pq_hi << 64) | a.pq_lo;
        val = (val + q - pq) % q;
      }
    }
    uint8_t* o = out + ((size_t)col * RING_N + i) * a.width;
    for (uint32_t b = 0; b < a.width; ++b) o[b] = (uint8_t)(val >> (8 * b));
  }
}

void launch_commit_finish(const ModulusPlan& mp, const Shape& sh, const uint32_t* partial, int splits, uint8_t* out,
                          cudaStream_t s, int ncols) {
  (void)sh;
  FinishArgs a;
  memset(&a, 0, sizeof a);
  a.nprimes = mp.nprimes;
  a.splits = splits;
  a.width = mp.width;
  a.exact = mp.exact_lift ? 1 : 0;
  a.q_lo = (uint64_t)mp.q, a.q_hi = (uint64_t)(mp.q >> 64);
  a.pq_lo = (uint64_t)mp.p_mod_q, a.pq_hi = (uint64_t)(mp.p_mod_q >> 64);
  for (int i = 0; i < mp.nprimes; ++i) {
    a.primes[i] = mp.primes[i];
    a.half[i] = mp.half_digits[i];
    a.bar[i] = (uint32_t)((1ull << 32) / mp.primes[i]);
    for (int j = 0; j < i; ++j) a.ginv[i][j] = mp.garner_inv[i][j];
  }
  k_commit_finish<<<ncols, 256, 0, s>>>(a, mp.dconsts, partial, out);
}

// ------------------------------------------------------------------------------------------------
// Verifier: a_times_v (rq.rs:188-217) = sum_m A_m v_m in R_Q for the folded witness v (|v| <= 2^15):
// v mod p -> the same forward transform as the key (k_key_forward), base multiplication with the
// key's 4x4 matrices summed over the elements (one thread per prime, leaf and coefficient l),
// then K2 on that single column.
// ------------------------------------------------------------------------------------------------
__global__ void k_atv_reduce(const PrimeConst* __restrict__ pcs, int nprimes, uint64_t elements,
                             const int32_t* __restrict__ v, uint32_t* __restrict__ vred) {
  const uint64_t n = (uint64_t)nprimes * elements * RING_N;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const int pi = (int)(i / (elements * RING_N));
    const int64_t p = pcs[pi].p;
    const int64_t x = v[i % (elements * RING_N)];
    vred[i] = (uint32_t)(((x % p) + p) % p);
  }
}

// One block per (prime, leaf): thread t takes output l = t % 4 over the elements m = t / 4 (mod 64);
// the 64 partial sums (each below 64 x 4 x p^2 < 2^38) meet in shared memory.
__global__ void __launch_bounds__(256) k_atv_mac(const PrimeConst* __restrict__ pcs, int nprimes, uint64_t elements,
                                                 const uint32_t* __restrict__ key, const uint32_t* __restrict__ vhat,
                                                 uint32_t* __restrict__ out) {
  const int pi = blockIdx.x / LEAVES, s = blockIdx.x % LEAVES;
  const int l = threadIdx.x & 3, lane4 = threadIdx.x >> 2;
  const uint64_t p = pcs[pi].p;
  uint64_t acc = 0;
  for (uint64_t m = lane4; m < elements; m += 64) {
    const uint32_t* M = key + (((size_t)pi * elements + m) * LEAVES + s) * 16;
    const uint32_t* x = vhat + (((size_t)pi * elements + m) * 4) * LEAVES + s;
#pragma unroll
    for (int k = 0; k < 4; ++k) acc += (uint64_t)M[4 * k + l] * x[k * LEAVES];
  }
  __shared__ uint64_t part[256];
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w >= 4; w >>= 1) {
    if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  // K2's input layout with one element split: [split 0][prime][column 0][leaf][l]
  if (threadIdx.x < 4) out[((size_t)pi * COLUMNS) * LEAVES * 4 + s * 4 + threadIdx.x] = (uint32_t)(part[threadIdx.x] % p);
}

void launch_a_times_v(const ModulusPlan& mp, const Shape& sh, const int32_t* v, const uint32_t* key, uint32_t* vred,
                      uint32_t* vhat, uint32_t* partial, uint8_t* out, cudaStream_t s) {
  const uint64_t E = sh.ring_elements;
  k_atv_reduce<<<1024, 256, 0, s>>>(mp.dconsts, mp.nprimes, E, v, vred);
  const uint64_t total = (uint64_t)mp.nprimes * E * 4;
  k_key_forward<<<(unsigned)((total + 127) / 128), 128, 0, s>>>(mp.dconsts, mp.nprimes, E, vred, vhat);
  k_atv_mac<<<mp.nprimes * LEAVES, 256, 0, s>>>(mp.dconsts, mp.nprimes, E, key, vhat, partial);
  launch_commit_finish(mp, sh, partial, 1, out, s, 1);
}

// The checker's scans of the folded witness v (main.rs:266-289 and the norm / range tests): one
// thread per (element m, residue k): bit 0 of v[m][4 pp + k] for pp < 162 packed into an F162 (the
// fold mod 2, components_mod_2), times e0[4 m + k], XOR-summed; sum of v^2; max and min of v.
// out: [0..2] the F162 sum, [3] sum v^2, [4] max v + 2^31, [5] 2^31 - min v (zeroed by the caller).
__global__ void __launch_bounds__(256) k_fold_checks(const int32_t* __restrict__ v, uint64_t elements,
                                                     const f162* __restrict__ e0, unsigned long long* __restrict__ out) {
  const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  f162 acc = {0, 0, 0};
  unsigned long long sq = 0, hi = 0, lo = 0;
  if (t < 4 * elements) {
    const uint64_t m = t >> 2;
    const int k = (int)(t & 3);
    const int32_t* src = v + m * RING_N + k;
    f162 x = {0, 0, 0};
    int32_t mx = INT32_MIN, mn = INT32_MAX;
    for (int pp = 0; pp < RING_N / 4; ++pp) {
      const int32_t c = src[4 * pp];
      sq += (unsigned long long)((int64_t)c * c);
      mx = max(mx, c), mn = min(mn, c);
      const uint64_t bit = (uint64_t)(c & 1) << (pp & 63);
      if (pp < 64) x.w0 |= bit;
      else if (pp < 128) x.w1 |= bit;
      else x.w2 |= bit;
    }
    acc = f162_mul(e0[t], x);
    hi = (unsigned long long)((int64_t)mx + (1ll << 31));
    lo = (unsigned long long)((1ll << 31) - (int64_t)mn);
  }
  for (int o = 16; o; o >>= 1) {
    acc.w0 ^= __shfl_xor_sync(0xffffffffu, acc.w0, o);
    acc.w1 ^= __shfl_xor_sync(0xffffffffu, acc.w1, o);
    acc.w2 ^= __shfl_xor_sync(0xffffffffu, acc.w2, o);
    sq += __shfl_xor_sync(0xffffffffu, sq, o);
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    lo = max(lo, __shfl_xor_sync(0xffffffffu, lo, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicXor(out, (unsigned long long)acc.w0);
    atomicXor(out + 1, (unsigned long long)acc.w1);
    atomicXor(out + 2, (unsigned long long)acc.w2);
    atomicAdd(out + 3, sq);
    atomicMax(out + 4, hi);
    atomicMax(out + 5, lo);
  }
}

void launch_fold_checks(const int32_t* v, uint64_t elements, const f162* e0, unsigned long long* out, cudaStream_t s) {
  const uint64_t n = 4 * elements;
  k_fold_checks<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(v, elements, e0, out);
}

// *flag becomes nonzero when a commitment coefficient (w bytes little-endian) is not below q.
__global__ void k_commit_range(const uint8_t* __restrict__ c, uint32_t w, uint64_t q_lo, uint64_t q_hi, uint64_t n,
                               unsigned long long* __restrict__ flag) {
  const u128 q = ((u128)q_hi << 64) | q_lo;
  bool bad = false;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    u128 x = 0;
    for (int b = (int)w - 1; b >= 0; --b) x = (x << 8) | c[i * w + b];
    bad |= x >= q;
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1ull);
}

void launch_commit_range(const uint8_t* commit, uint32_t w, u128 q, uint64_t n, unsigned long long* flag,
                         cudaStream_t s) {
  k_commit_range<<<512, 256, 0, s>>>(commit, w, (uint64_t)q, (uint64_t)(q >> 64), n, flag);
}

// challenge_combination (rq.rs:226-256): raw[r] = sum_j sum_t sign_{j,t} C_j[r - 4 pos_{j,t}],
// the challenge sitting in R_Q as c(-X^4), sign = (-1)^(sign bit + pos). One thread per raw index
// and run of 32 columns; partial sums as signed 128-bit integers (|.| < 32 x 28 x 2^96),
// [run][raw index] -> (lo, hi), added and folded into the ring by the host.
__global__ void k_chcomb(const uint8_t* __restrict__ commit, uint32_t width, const Challenge* __restrict__ ch,
                         unsigned long long* __restrict__ part) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int run = blockIdx.y;
  if (r >= 2 * RING_N - 1) return;
  __int128 acc = 0;
  for (int j = 32 * run; j < 32 * run + 32; ++j) {
    const Challenge c = ch[j];
    for (uint32_t t = 0; t < c.weight; ++t) {
      const int m = c.positions[t];
      const int i = r - 4 * m;
      if (i < 0 || i >= RING_N) continue;
      const uint8_t* b = commit + ((size_t)j * RING_N + i) * width;
      unsigned __int128 x = 0;
      for (int k = (int)width - 1; k >= 0; --k) x = (x << 8) | b[k];
      const bool neg = (((c.signs >> t) & 1) ^ (m & 1)) != 0;
      acc += neg ? -(__int128)x : (__int128)x;
    }
  }
  part[2 * ((size_t)run * (2 * RING_N - 1) + r)] = (unsigned long long)(unsigned __int128)acc;
  part[2 * ((size_t)run * (2 * RING_N - 1) + r) + 1] = (unsigned long long)((unsigned __int128)acc >> 64);
}

void launch_challenge_combination(const uint8_t* commit, uint32_t width, const Challenge* ch,
                                  unsigned long long* part, cudaStream_t s) {
  k_chcomb<<<dim3((2 * RING_N - 1 + 127) / 128, COLUMNS / 32), 128, 0, s>>>(commit, width, ch, part);
}

}  // namespace lf
