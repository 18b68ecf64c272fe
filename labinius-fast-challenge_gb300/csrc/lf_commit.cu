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
#include <cstdio>
#include <cstring>

#include "lf_blake3.cuh"
#include "lf_internal.h"

namespace lf {

__constant__ PrimeConst c_prime[MAX_PRIMES];

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
  auto shoup = [&](uint64_t w) { return (uint32_t)((w << 32) / p); };
  c.p = pl.p;
  c.bar = (uint32_t)((1ull << 32) / p);
  c.om = (uint32_t)pw(162);
  c.om_s = shoup(c.om);
  for (int sb = 0; sb < 6; ++sb) {
    auto put = [&](int slot, uint32_t e) {
      uint64_t t1 = pw(e / 3), t2 = pw(2 * (e / 3));
      c.tw[sb][slot][0] = (uint32_t)t1, c.tw[sb][slot][1] = (uint32_t)t2;
      c.tws[sb][slot][0] = shoup(t1), c.tws[sb][slot][1] = shoup(t2);
    };
    put(0, pl.node_e[2][sb]);
    for (int a = 0; a < 3; ++a) put(1 + a, pl.node_e[3][3 * sb + a]);
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) put(4 + 3 * a + b, pl.node_e[4][9 * sb + 3 * a + b]);
    // Fused trinomial split + level-1 split for sub-block sb = (node n, child i).
    int n = sb / 3, i = sb % 3;
    uint64_t e = pl.node_e[1][n];
    uint64_t tau = pw(e / 3), om_i = pw(162 * i), c_n = pw(e);
    uint64_t coef[5];
    coef[0] = 1;
    coef[1] = tau * om_i % p;
    coef[2] = tau * tau % p * om_i % p * om_i % p;
    coef[3] = c_n;
    coef[4] = coef[1] * c_n % p;
    for (int idx = 0; idx < 32; ++idx) {
      uint64_t v = 0;
      for (int t = 0; t < 5; ++t)
        if ((idx >> t) & 1) v += coef[t];
      c.T[sb][idx] = (uint32_t)(v % p);
    }
  }
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
  for (int s = 0; s < LEAVES; ++s) c.leaf_root[s] = (uint32_t)pw(pl.leaf_e[s]);
}

// The level-2 split fused into the lookups: output (child a, position q < 9) of level-2 node sb
// is sum_t omega^(a t) tau^t T[sb][idx(q + 9 t)], tau = eta^(e/3) of node sb; entry
// [sb][a][t][idx] holds omega^(a t) tau^t T[sb][idx].
static void fill_t2(const PrimePlan& pl, const PrimeConst& c, uint32_t* t2) {
  const uint64_t p = pl.p;
  auto pw = [&](int64_t e) { return (uint64_t)pl.pw[((e % 486) + 486) % 486]; };
  for (int sb = 0; sb < 6; ++sb) {
    const uint64_t tau = pw(pl.node_e[2][sb] / 3);
    for (int a = 0; a < 3; ++a)
      for (int t = 0; t < 3; ++t) {
        uint64_t f = pw(162 * ((a * t) % 3));
        for (int i = 0; i < t; ++i) f = f * tau % p;
        for (int idx = 0; idx < 32; ++idx) t2[((sb * 3 + a) * 3 + t) * 32 + idx] = (uint32_t)(f * c.T[sb][idx] % p);
      }
  }
}

static uint32_t bits_of(u128 x) {
  uint32_t n = 0;
  while (x) ++n, x >>= 1;
  return n;
}

bool make_modulus_plan(u128 q, ModulusPlan& mp, std::string& err) {
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
    err = "this build commits only under Q = 661473542593 (3889*9721*17497)";
    return false;
  }
  mp.consts.resize(mp.nprimes);
  mp.t2.assign((size_t)mp.nprimes * T2_WORDS, 0);
  for (int i = 0; i < mp.nprimes; ++i) {
    PrimePlan pl;
    if (!make_plan(mp.primes[i], pl)) {
      err = "transform prime rejected";
      return false;
    }
    fill_consts(pl, mp.consts[i]);
    fill_t2(pl, mp.consts[i], mp.t2.data() + (size_t)i * T2_WORDS);
    for (int j = 0; j < i; ++j) mp.garner_inv[i][j] = inv_mod(mp.primes[j], mp.primes[i]);
  }
  return true;
}

void upload_prime_consts(const ModulusPlan& mp, cudaStream_t s) {
  cudaMemcpyToSymbolAsync(c_prime, mp.consts.data(), sizeof(PrimeConst) * mp.nprimes, 0, cudaMemcpyHostToDevice, s);
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

__global__ void k_matrix_expand(MatrixArgs a, uint64_t elements, uint32_t* ared) {
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
    for (int i = 0; i < a.nprimes; ++i) {
      uint64_t p = a.primes[i];
      uint64_t r = ((hi % p) * a.two64[i] + lo % p) % p;
      ared[((size_t)i * elements + m) * RING_N + t] = (uint32_t)r;
    }
  }
}

void launch_matrix_expand(const ModulusPlan& mp, uint64_t elements, uint32_t* ared, cudaStream_t s) {
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
  int threads = 64;
  k_matrix_expand<<<(unsigned)((elements + threads - 1) / threads), threads, 0, s>>>(a, elements, ared);
}

// ------------------------------------------------------------------------------------------------
// Key transform: A_m = sum_k X^k A_{m,k}(Y); the 162-point transform of each A_{m,k}, then the
// base-multiplication matrix of every leaf: M[k][l] = A_{l-k}(c) for l >= k, c A_{l-k+4}(c) else.
// ------------------------------------------------------------------------------------------------
__device__ void forward162(uint32_t* x, const PrimeConst& P) {
  const uint64_t p = P.p;
  for (int j = 0; j < 81; ++j) {
    uint64_t a = x[j], b = x[j + 81];
    x[j] = (uint32_t)((a + (uint64_t)P.w * b) % p);
    x[j + 81] = (uint32_t)((a + (uint64_t)P.w5 * b) % p);
  }
  int len = 81;
  for (int l = 1; l <= 4; ++l) {
    int sub = len / 3, nodes = 162 / len;
    for (int n = 0; n < nodes; ++n) {
      const uint32_t* tw = P.fw[node_off(l) + n];
      for (int q = 0; q < sub; ++q) {
        int o = n * len + q;
        uint64_t a0 = x[o], a1 = (uint64_t)x[o + sub] * tw[0] % p, a2 = (uint64_t)x[o + 2 * sub] * tw[1] % p;
        uint64_t om = P.om, om2 = (uint64_t)P.om * P.om % p;
        x[o] = (uint32_t)((a0 + a1 + a2) % p);
        x[o + sub] = (uint32_t)((a0 + a1 * om + a2 * om2) % p);
        x[o + 2 * sub] = (uint32_t)((a0 + a1 * om2 + a2 * om) % p);
      }
    }
    len = sub;
  }
}

__global__ void k_key_forward(int nprimes, uint64_t elements, const uint32_t* ared, uint32_t* leafvals) {
  uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  uint64_t total = (uint64_t)nprimes * elements * 4;
  if (tid >= total) return;
  int k = (int)(tid & 3);
  uint64_t m = (tid >> 2) % elements;
  int pi = (int)((tid >> 2) / elements);
  const uint32_t* a = ared + ((size_t)pi * elements + m) * RING_N;
  uint32_t x[LEAVES];
  for (int p = 0; p < LEAVES; ++p) x[p] = a[4 * p + k];
  forward162(x, c_prime[pi]);
  uint32_t* o = leafvals + (((size_t)pi * elements + m) * 4 + k) * LEAVES;
  for (int s = 0; s < LEAVES; ++s) o[s] = x[s];
}

__global__ void k_key_leafform(int nprimes, uint64_t elements, const uint32_t* leafvals, uint32_t* key) {
  uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  uint64_t total = (uint64_t)nprimes * elements * LEAVES;
  if (tid >= total) return;
  int s = (int)(tid % LEAVES);
  uint64_t m = (tid / LEAVES) % elements;
  int pi = (int)(tid / LEAVES / elements);
  const PrimeConst& P = c_prime[pi];
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
  k_key_forward<<<(unsigned)((t1 + 127) / 128), 128, 0, s>>>(mp.nprimes, elements, ared, leafvals);
  uint64_t t2 = (uint64_t)mp.nprimes * elements * LEAVES;
  k_key_leafform<<<(unsigned)((t2 + 127) / 128), 128, 0, s>>>(mp.nprimes, elements, leafvals, key);
}

// ------------------------------------------------------------------------------------------------
// K1: the commitment in the transform domain.
//   grid  (COLUMNS / 32 column tiles, primes, element splits); block 576 = 18 warps.
//   warp w = (level-2 node sb = w / 3, level-3 node a = w % 3) of every word; lane = column.
// A thread produces, per table word, the 9 leaves of its level-3 node: the first three levels
// (trinomial split, level-1 split, the level-2 split into node a) are three lookups in
// twiddled 32-entry tables, then two radix-3 levels; at each leaf it multiplies with the key's
// 4x4 base-multiplication matrix and accumulates 9 x 4 u32 over its split of the elements.
// ------------------------------------------------------------------------------------------------
constexpr int CT = 32;
constexpr int MB = 8;
constexpr int KWARPS = 18;
constexpr int KTHREADS = 32 * KWARPS;

// One radix-3 split of a node: inputs a (untwiddled), b, c; outputs in place.
__device__ __forceinline__ void split3(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t t1, uint32_t t1s, uint32_t t2,
                                       uint32_t t2s, uint32_t om, uint32_t oms, uint32_t p) {
  uint32_t b1 = shoup(b, t1, t1s, p);
  uint32_t c1 = shoup(c, t2, t2s, p);
  uint32_t m = shoup(b1 + 2 * p - c1, om, oms, p);
  uint32_t y0 = a + b1 + c1;
  uint32_t y1 = a + m + 2 * p - c1;
  uint32_t y2 = a + 4 * p - b1 - m;
  a = y0, b = y1, c = y2;
}

__device__ __forceinline__ uint32_t word_index_byte(uint32_t r0, uint32_t r1, uint32_t r2, uint32_t r3, uint32_t r4,
                                                    int q) {
  return ((r0 >> q) & 1) | (((r1 >> q) & 1) << 1) | (((r2 >> q) & 1) << 2) | (((r3 >> q) & 1) << 3) |
         (((r4 >> q) & 1) << 4);
}

size_t commit_smem_bytes() { return (size_t)(T2_WORDS + MB * LEAVES * 16) * 4 + (size_t)MB * CT * 27 * 4; }

__global__ void __launch_bounds__(KTHREADS, 1)
    k_commit_ntt(const uint4* __restrict__ table, const uint32_t* __restrict__ key, const uint32_t* __restrict__ t2g,
                 uint32_t* __restrict__ partial, int rl, int elements, int per_split, int nprimes, int reduce_every) {
  extern __shared__ __align__(16) uint32_t csm[];
  uint32_t* sT2 = csm;                                  // [sb][a][t][32]
  uint32_t* sKey = csm + T2_WORDS;                      // [MB][162][k][l]
  uint8_t* sIdx = reinterpret_cast<uint8_t*>(sKey + MB * LEAVES * 16);  // [MB][CT][27][k]
  const int pi = blockIdx.y;
  const int col0 = blockIdx.x * CT;
  const int split = blockIdx.z;
  const int m_begin = split * per_split;
  const int m_end = min(elements, m_begin + per_split);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int sb = warp / 3, na = warp % 3;
  const PrimeConst& P = c_prime[pi];
  const uint32_t p = P.p;
  for (int i = tid; i < T2_WORDS; i += KTHREADS) sT2[i] = t2g[pi * T2_WORDS + i];
  const uint32_t* t20 = sT2 + ((sb * 3 + na) * 3 + 0) * 32;
  const uint32_t* t21 = t20 + 32;
  const uint32_t* t22 = t20 + 64;
  // warp-uniform twiddles of the level-3 node (3 sb + na) and its three level-4 children
  const uint32_t w3a = P.tw[sb][1 + na][0], w3as = P.tws[sb][1 + na][0];
  const uint32_t w3b = P.tw[sb][1 + na][1], w3bs = P.tws[sb][1 + na][1];

  uint32_t acc[9][4];
#pragma unroll
  for (int q = 0; q < 9; ++q)
#pragma unroll
    for (int l = 0; l < 4; ++l) acc[q][l] = 0;

  int since = 0;
  for (int mc = m_begin; mc < m_end; mc += MB) {
    const int nm = min(MB, m_end - mc);
    __syncthreads();
    {
      const uint4* src = reinterpret_cast<const uint4*>(key + ((size_t)pi * elements + mc) * LEAVES * 16);
      uint4* dst = reinterpret_cast<uint4*>(sKey);
      for (int i = tid; i < nm * LEAVES * 4; i += KTHREADS) dst[i] = src[i];
    }
    // 27 five-bit indices per table word, one word per task: bits q, q+27, q+54, q+81, q+108.
    for (int task = tid; task < nm * CT * 4; task += KTHREADS) {
      const int k = task & 3, c = (task >> 2) % CT, ml = (task >> 2) / CT;
      const uint4 v = table[((size_t)(col0 + c) << rl) + 4 * (size_t)(mc + ml) + k];
      const uint32_t M27 = (1u << 27) - 1;
      const uint32_t r0 = v.x & M27;
      const uint32_t r1 = ((v.x >> 27) | (v.y << 5)) & M27;
      const uint32_t r2 = ((v.y >> 22) | (v.z << 10)) & M27;
      const uint32_t r3 = ((v.z >> 17) | (v.w << 15)) & M27;
      const uint32_t r4 = (v.w >> 12) & M27;
      uint8_t* dst = sIdx + ((size_t)(ml * CT + c) * 27) * 4 + k;
#pragma unroll
      for (int q = 0; q < 27; ++q) dst[4 * q] = (uint8_t)word_index_byte(r0, r1, r2, r3, r4, q);
    }
    __syncthreads();

    for (int ml = 0; ml < nm; ++ml) {
      const uint8_t* ib = sIdx + ((size_t)(ml * CT + lane) * 27) * 4;
      const uint32_t* kb = sKey + ((size_t)ml * LEAVES + 27 * sb + 9 * na) * 16;
#pragma unroll 1
      for (int k = 0; k < 4; ++k) {
        uint32_t x[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) x[q] = t20[ib[4 * q + k]] + t21[ib[4 * (q + 9) + k]] + t22[ib[4 * (q + 18) + k]];
        // level-3 node (9 -> 3 x 3)
#pragma unroll
        for (int q = 0; q < 3; ++q) split3(x[q], x[q + 3], x[q + 6], w3a, w3as, w3b, w3bs, P.om, P.om_s, p);
        // level-4 nodes (3 -> leaves)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
          const int t = 4 + 3 * na + b;
          split3(x[3 * b], x[3 * b + 1], x[3 * b + 2], P.tw[sb][t][0], P.tws[sb][t][0], P.tw[sb][t][1],
                 P.tws[sb][t][1], P.om, P.om_s, p);
        }
        // Base multiplication with the key's leaves: acc[q][l] += M[k][l] x[q].
#pragma unroll
        for (int q = 0; q < 9; ++q) {
          uint32_t v = x[q] - __umulhi(x[q], P.bar) * p;
          v = v >= p ? v - p : v;
          const uint4 kv = *reinterpret_cast<const uint4*>(kb + q * 16 + 4 * k);
          acc[q][0] += kv.x * v;
          acc[q][1] += kv.y * v;
          acc[q][2] += kv.z * v;
          acc[q][3] += kv.w * v;
        }
      }
      if (++since == reduce_every) {
        since = 0;
#pragma unroll
        for (int q = 0; q < 9; ++q)
#pragma unroll
          for (int l = 0; l < 4; ++l) acc[q][l] = reduce32(acc[q][l], P.bar, p);
      }
    }
  }
  uint32_t* out =
      partial + ((((size_t)split * nprimes + pi) * COLUMNS + col0 + lane) * LEAVES + 27 * sb + 9 * na) * 4;
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    uint4 v;
    v.x = reduce32(acc[q][0], P.bar, p);
    v.y = reduce32(acc[q][1], P.bar, p);
    v.z = reduce32(acc[q][2], P.bar, p);
    v.w = reduce32(acc[q][3], P.bar, p);
    reinterpret_cast<uint4*>(out)[q] = v;
  }
}

// Element splits of K1: the grid (32 column tiles x primes x splits) at one block per SM should
// fill whole waves; among 8..24 splits take the one with the least idle SM time, then the fewest.
int commit_splits(uint64_t elements, int nprimes, int sms) {
  if (sms < 1) sms = 1;
  int best = 1;
  double best_eff = -1;
  for (int s = 8; s <= 24; ++s) {
    if ((uint64_t)s * MB > elements) break;
    const long blocks = (long)(COLUMNS / CT) * nprimes * s;
    const long waves = (blocks + sms - 1) / sms;
    const double eff = (double)blocks / (double)(waves * sms);
    if (eff > best_eff + 1e-9) best_eff = eff, best = s;
  }
  if (best_eff < 0) {
    best = 1;
    while ((uint64_t)best * 2 * MB <= elements && best < 8) best *= 2;
  }
  return best;
}

void launch_commit(const ModulusPlan& mp, const Shape& sh, const uint4* table, const uint32_t* key, const uint32_t* t2,
                   uint32_t* partial, int splits, cudaStream_t s) {
  int elements = (int)sh.ring_elements;
  int per = (elements + splits - 1) / splits;
  // Accumulators take 4 products below p^2 per element; reduce before 2^32 can be reached.
  uint64_t pmax = 0;
  for (int i = 0; i < mp.nprimes; ++i) pmax = mp.primes[i] > pmax ? mp.primes[i] : pmax;
  uint64_t per_elem = 4 * (pmax - 1) * (pmax - 1);
  int reduce_every = (int)((0xffffffffull - pmax) / per_elem);
  if (reduce_every < 1) reduce_every = 1;
  dim3 grid(COLUMNS / CT, mp.nprimes, splits);
  const size_t smem = commit_smem_bytes();
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_commit_ntt, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  k_commit_ntt<<<grid, KTHREADS, smem, s>>>(table, key, t2, partial, sh.rl, elements, per, mp.nprimes, reduce_every);
}

// ------------------------------------------------------------------------------------------------
// K2: sum the element splits, inverse transform per prime and coefficient of X, CRT, pack.
// One block per column.
// ------------------------------------------------------------------------------------------------
struct FinishArgs {
  int nprimes, splits;
  uint32_t width;
  uint32_t primes[MAX_PRIMES];
  uint32_t ginv[MAX_PRIMES][MAX_PRIMES];
};

__global__ void __launch_bounds__(256) k_commit_finish(FinishArgs a, const uint32_t* __restrict__ partial,
                                                       uint8_t* __restrict__ out) {
  __shared__ uint32_t v[MAX_PRIMES][4][LEAVES];
  const int col = blockIdx.x;
  for (int e = threadIdx.x; e < a.nprimes * 4 * LEAVES; e += blockDim.x) {
    int pi = e / (4 * LEAVES), rem = e % (4 * LEAVES), s = rem / 4, l = rem % 4;
    uint64_t p = a.primes[pi], sum = 0;
    for (int sp = 0; sp < a.splits; ++sp)
      sum += partial[(((size_t)sp * a.nprimes + pi) * COLUMNS + col) * LEAVES * 4 + rem];
    v[pi][l][s] = (uint32_t)(sum % p);
  }
  __syncthreads();
  // Inverse radix-3 levels 4..1: nodes of length 3, 9, 27, 81.
  int len = 3;
  for (int lvl = 4; lvl >= 1; --lvl) {
    const int sub = len / 3, nodes = LEAVES / len, per_t = nodes * sub;
    for (int e = threadIdx.x; e < a.nprimes * 4 * per_t; e += blockDim.x) {
      int pi = e / (4 * per_t), rem = e % (4 * per_t), l = rem / per_t, r2 = rem % per_t;
      int n = r2 / sub, q = r2 % sub;
      const PrimeConst& P = c_prime[pi];
      const uint64_t p = P.p;
      uint32_t* x = v[pi][l];
      int o = n * len + q;
      uint64_t y0 = x[o], y1 = x[o + sub], y2 = x[o + 2 * sub];
      uint64_t a0 = (y0 + y1 + y2) % p;
      uint64_t a1 = (y0 + y1 * P.iom + y2 * P.iom2) % p;
      uint64_t a2 = (y0 + y1 * P.iom2 + y2 * P.iom) % p;
      const uint32_t* it = P.itw[node_off(lvl) + n];
      x[o] = (uint32_t)(a0 * P.inv3 % p);
      x[o + sub] = (uint32_t)(a1 * P.inv3 % p * it[0] % p);
      x[o + 2 * sub] = (uint32_t)(a2 * P.inv3 % p * it[1] % p);
    }
    __syncthreads();
    len *= 3;
  }
  for (int e = threadIdx.x; e < a.nprimes * 4 * 81; e += blockDim.x) {
    int pi = e / (4 * 81), rem = e % (4 * 81), l = rem / 81, j = rem % 81;
    const PrimeConst& P = c_prime[pi];
    const uint64_t p = P.p;
    uint32_t* x = v[pi][l];
    uint64_t u = x[j], w = x[j + 81];
    uint64_t b = (u + p - w) % p * P.inv_split % p;
    x[j] = (uint32_t)((u + p * p - (uint64_t)P.w * b) % p);
    x[j + 81] = (uint32_t)b;
  }
  __syncthreads();
  // Coefficient 4p + l of the column is coefficient p of C_l. Garner's CRT into [0, Q).
  for (int i = threadIdx.x; i < RING_N; i += blockDim.x) {
    int pp = i >> 2, l = i & 3;
    uint64_t digit[MAX_PRIMES];
    for (int k = 0; k < a.nprimes; ++k) {
      uint64_t pk = a.primes[k];
      uint64_t t = v[k][l][pp];
      // t <- (r_k - (d_0 + p_0 d_1 + ...)) / (p_0 ... p_{k-1}) mod p_k, digit by digit
      for (int j = 0; j < k; ++j) t = (t + pk - digit[j] % pk) % pk * a.ginv[k][j] % pk;
      digit[k] = t;
    }
    u128 val = 0;
    for (int k = a.nprimes - 1; k >= 0; --k) val = val * a.primes[k] + digit[k];
    uint8_t* o = out + ((size_t)col * RING_N + i) * a.width;
    for (uint32_t b = 0; b < a.width; ++b) o[b] = (uint8_t)(val >> (8 * b));
  }
}

void launch_commit_finish(const ModulusPlan& mp, const Shape& sh, const uint32_t* partial, int splits, uint8_t* out,
                          cudaStream_t s) {
  (void)sh;
  FinishArgs a;
  memset(&a, 0, sizeof a);
  a.nprimes = mp.nprimes;
  a.splits = splits;
  a.width = mp.width;
  for (int i = 0; i < mp.nprimes; ++i) {
    a.primes[i] = mp.primes[i];
    for (int j = 0; j < i; ++j) a.ginv[i][j] = mp.garner_inv[i][j];
  }
  k_commit_finish<<<COLUMNS, 256, 0, s>>>(a, partial, out);
}

}  // namespace lf
