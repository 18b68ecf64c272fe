// Batched arithmetic of R_Q = Z_Q[X]/(X^648 - X^324 + 1) and of the GHASH field, for many
// independent operand pairs at once: the ring product of rq.rs:171-186 (schoolbook, then
// fold_into_ring rq.rs:146-164) for any modulus 2 <= Q < 2^96, and the B128 product of
// fields/scalar.rs:61-72.
//
// Ring product. X^648 - X^324 + 1 is the 1944th cyclotomic polynomial, so modulo a prime
// p = 1 (mod 1944) it splits into 648 linear factors X - zeta^j (j a unit mod 1944, zeta a
// primitive 1944th root). The transform follows that factor tree: one split into the two factors
// X^324 - omega^{1,5} (omega = zeta^324), then radix 2, 2, 3, 3, 3, 3 splits of
// X^{rm} - zeta^s into X^m - zeta^{s/r + t 1944/r}; 1836 butterflies per transform. The product is
// pointwise on the 648 evaluations, and the inverse runs the tree back.
// The residues then give the product mod Q in one of two ways:
//  * Q is a product of distinct primes p = 1 (mod 1944) below 2^31 (the baseline
//    3889 * 9721 * 17497, or three 31-bit primes near 2^93): one transform per factor, and
//    Garner's mixed radix is the coefficient in [0, Q) directly;
//  * any other Q (2^64 among them): the transform runs modulo the largest primes p = 1 (mod 1944)
//    below 2^31 until their product P exceeds twice the largest |coefficient| of the integer
//    product reduced mod X^648 - X^324 + 1 (at most 972 (Q-1)^2); the centred mixed-radix value
//    is that integer, reduced mod Q by Horner with Barrett steps (a mask when Q is a power of 2).
//
// One CTA per product and one warp per prime: each warp reads the operands (the block's other
// warps hit L1), reduces them modulo its prime, transforms both in shared memory, multiplies
// pointwise (Montgomery) and transforms back; the CTA then recombines the residues of each
// coefficient.
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "lf_internal.h"
#include "lf_ring.h"

namespace lf {

// ------------------------------------------------------------------------------------------------
// Host: primes and plans
// ------------------------------------------------------------------------------------------------
namespace {

uint64_t pw64(uint64_t b, uint64_t e, uint64_t p) {
  uint64_t r = 1 % p;
  b %= p;
  while (e) {
    if (e & 1) r = r * b % p;
    b = b * b % p;
    e >>= 1;
  }
  return r;
}
uint32_t inv64(uint64_t x, uint64_t p) { return (uint32_t)pw64(x % p, p - 2, p); }

bool prime32(uint64_t n) {  // deterministic Miller-Rabin for n < 2^32 (bases 2, 7, 61)
  if (n < 2) return false;
  for (uint64_t sp : {2ull, 3ull, 5ull, 7ull, 11ull, 13ull, 61ull})
    if (n % sp == 0) return n == sp;
  uint64_t d = n - 1;
  int r = 0;
  while (!(d & 1)) d >>= 1, ++r;
  for (uint64_t a : {2ull, 7ull, 61ull}) {
    uint64_t x = pw64(a, d, n);
    if (x == 1 || x == n - 1) continue;
    bool comp = true;
    for (int i = 1; i < r && comp; ++i) {
      x = x * x % n;
      if (x == n - 1) comp = false;
    }
    if (comp) return false;
  }
  return true;
}

uint32_t shoup(uint32_t w, uint32_t p) { return (uint32_t)(((uint64_t)w << 32) / p); }
uint32_t bitlen(u128 x) {
  uint32_t b = 0;
  while (x) ++b, x >>= 1;
  return b;
}
uint32_t mod128(u128 x, uint32_t p) {
  const uint64_t hi = (uint64_t)(x >> 64), lo = (uint64_t)x;
  const uint64_t two64 = (~0ull % p + 1) % p;
  return (uint32_t)(((hi % p) * two64 % p + lo % p) % p);
}

// Per-prime device constants and the node twiddles of the factor tree.
void fill_prime(uint32_t p, RingPrimeDev& d) {
  memset(&d, 0, sizeof d);
  d.p = p;
  uint32_t inv = 1;  // p^-1 mod 2^32 by Newton
  for (int i = 0; i < 5; ++i) inv *= 2u - p * inv;
  d.pinv = 0u - inv;
  d.bar = shoup(1, p);
  uint64_t zeta = 0;
  for (uint64_t g = 2; g < p; ++g) {
    const uint64_t z = pw64(g, (p - 1) / 1944, p);
    if (pw64(z, 972, p) != 1 && pw64(z, 648, p) != 1) {
      zeta = z;
      break;
    }
  }
  std::vector<uint32_t> zp(1944);
  for (int i = 0; i < 1944; ++i) zp[i] = (uint32_t)pw64(zeta, i, p);
  auto set = [&](uint32_t& v, uint32_t& vs, uint64_t x) {
    v = (uint32_t)(x % p);
    vs = shoup(v, p);
  };
  set(d.om, d.om_s, zp[324]);
  set(d.w3, d.w3_s, zp[648]);
  set(d.isplit, d.isplit_s, inv64((2ull * zp[324] + p - 1) % p, p));
  // R / 324 mod p, R = 2^32: the pointwise Montgomery product leaves R^-1, the inverse levels 324
  set(d.scale, d.scale_s, pw64(2, 32, p) * inv64(324, p) % p);
  for (int k = 0; k < 3; ++k) set(d.in[k], d.in_s[k], pw64(2, 32 * (k + 1), p));
  // Node exponents level by level; level 0 = the two factors X^324 - zeta^{324, 1620}.
  std::vector<uint32_t> nodes = {324, 1620};
  const int radix[6] = {2, 2, 3, 3, 3, 3};
  int off = 0;
  for (int l = 0; l < 6; ++l) {
    const int r = radix[l];
    std::vector<uint32_t> next;
    for (size_t i = 0; i < nodes.size(); ++i) {
      const uint32_t s = nodes[i] / r;  // every node exponent here is divisible by its radix
      for (int t = 0; t < r; ++t) next.push_back((s + (uint32_t)t * (1944 / r)) % 1944);
      if (r == 2) {
        set(d.fw[off], d.fws[off], zp[s]);
        set(d.iw[off], d.iws[off], zp[(1944 - s) % 1944]);
        off += 1;
      } else {
        set(d.fw[off], d.fws[off], zp[s]);
        set(d.fw[off + 1], d.fws[off + 1], zp[(2 * s) % 1944]);
        set(d.iw[off], d.iws[off], zp[(1944 - s) % 1944]);
        set(d.iw[off + 1], d.iws[off + 1], zp[(1944 * 2 - 2 * s) % 1944]);
        off += 2;
      }
    }
    nodes.swap(next);
  }
}

// Largest |coefficient| of a product of two elements with coefficients in [0, q), reduced mod
// X^648 - X^324 + 1 over the integers, divided by (q - 1)^2: raw index r holds min(r, 1294 - r) + 1
// terms; X^r folds onto X^{r-324} - X^{r-648} (648 <= r < 972) or -X^{r-972} (r >= 972).
uint64_t product_weight() {
  auto cnt = [](int r) -> uint64_t { return (r < 0 || r > 1294) ? 0 : (uint64_t)(r < 648 ? r + 1 : 1295 - r); };
  uint64_t best = 0;
  for (int i = 0; i < RING_N; ++i) {
    uint64_t w = cnt(i);
    if (i >= 324) w += cnt(i + 324);
    if (i < 324) w += cnt(i + 648);
    w += cnt(i + 972);
    best = std::max(best, w);
  }
  return best;
}

}  // namespace

bool make_ring_plan(u128 q, RingPlan& rp, std::string& err) {
  rp = RingPlan();
  if (q < 2 || bitlen(q) > 96) {
    err = "ring modulus outside [2, 2^96)";
    return false;
  }
  rp.q = q;
  // Direct: q a product of distinct primes p = 1 (mod 1944) below 2^31 (then q = 1 mod 1944).
  std::vector<uint32_t> f;
  if (q % 1944 == 1) {
    u128 r = q;
    bool square = false;
    // trial division by the candidates p = 1 (mod 1944) up to sqrt(r)
    for (uint64_t p = 1945; r > 1 && p < (1ull << 31) && (u128)p * p <= r; p += 1944) {
      if (mod128(r, (uint32_t)p) != 0 || !prime32(p)) continue;
      f.push_back((uint32_t)p);
      r /= p;
      if (mod128(r, (uint32_t)p) == 0) {
        square = true;
        break;
      }
    }
    // what is left has no candidate factor up to its square root: usable only as one more prime
    if (!square && r > 1 && r < ((u128)1 << 31) && r % 1944 == 1 && prime32((uint64_t)r)) {
      f.push_back((uint32_t)r);
      r = 1;
    }
    if (square || r != 1 || f.size() > (size_t)MAX_RING_PRIMES) f.clear();
  }
  if (!f.empty()) {
    rp.mode = 0;
    rp.primes = f;
  } else {
    // Exact lift: P > 2 (product_weight (q-1)^2) + 1.
    rp.mode = (q & (q - 1)) == 0 ? 2 : 1;
    const double need = 2.0 * std::log2((double)(q - 1) + 1.0) + std::log2((double)product_weight()) + 2.0;
    double have = 0;
    for (uint64_t p = ((1ull << 31) - 1) / 1944 * 1944 + 1; have < need && p > 1944; p -= 1944) {
      if (!prime32(p)) continue;
      rp.primes.push_back((uint32_t)p);
      have += std::log2((double)p);
    }
    if (have < need || rp.primes.size() > (size_t)MAX_RING_PRIMES) {
      err = "no prime set covers this ring modulus";
      return false;
    }
  }
  const int k = (int)rp.primes.size();
  rp.dev.resize(k);
  for (int i = 0; i < k; ++i) fill_prime(rp.primes[i], rp.dev[i]);
  RingArgs& a = rp.args;
  memset(&a, 0, sizeof a);
  a.nprimes = k;
  a.mode = rp.mode;
  for (int i = 0; i < k; ++i) {
    a.primes[i] = rp.primes[i];
    for (int j = 0; j < i; ++j) {
      a.ginv[i][j] = inv64(rp.primes[j], rp.primes[i]);
      a.ginv_s[i][j] = shoup(a.ginv[i][j], rp.primes[i]);
    }
  }
  // floor(P / 2) in the primes' mixed radix (digit 0 least significant), and P mod q
  // (P mod 2^128 for a power-of-two q: the wrap is the reduction).
  {
    std::vector<uint32_t> big = {1};  // P as base-2^32 limbs
    for (int i = 0; i < k; ++i) {
      uint64_t carry = 0;
      for (auto& w : big) {
        const uint64_t t = (uint64_t)w * rp.primes[i] + carry;
        w = (uint32_t)t;
        carry = t >> 32;
      }
      if (carry) big.push_back((uint32_t)carry);
    }
    uint32_t c = 0;  // halve
    for (int i = (int)big.size() - 1; i >= 0; --i) {
      const uint32_t nc = big[i] & 1;
      big[i] = (big[i] >> 1) | (c << 31);
      c = nc;
    }
    for (int i = 0; i < k; ++i) {  // digits of floor(P/2): repeated division
      uint64_t rem = 0;
      for (int j = (int)big.size() - 1; j >= 0; --j) {
        const uint64_t t = (rem << 32) | big[j];
        big[j] = (uint32_t)(t / rp.primes[i]);
        rem = t % rp.primes[i];
      }
      a.half[i] = (uint32_t)rem;
    }
    u128 pq = rp.mode == 2 ? 1 : 1 % q;
    for (int i = 0; i < k; ++i) pq = rp.mode == 2 ? pq * rp.primes[i] : pq * rp.primes[i] % q;
    a.pq_lo = (uint64_t)pq;
    a.pq_hi = (uint64_t)(pq >> 64);
  }
  a.q_lo = (uint64_t)q;
  a.q_hi = (uint64_t)(q >> 64);
  a.qbits = bitlen(q);
  a.mu = rp.mode == 1 ? (uint64_t)((((u128)1) << (a.qbits + 31)) / q) : 0;
  return true;
}

// ------------------------------------------------------------------------------------------------
// Device arithmetic modulo p < 2^31
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t csub(uint32_t x, uint32_t p) { return x >= p ? x - p : x; }
__device__ __forceinline__ uint32_t addm(uint32_t a, uint32_t b, uint32_t p) { return csub(a + b, p); }
__device__ __forceinline__ uint32_t subm(uint32_t a, uint32_t b, uint32_t p) { return a >= b ? a - b : a + p - b; }
// x w mod p for any x < 2^32 and a constant w < p with ws = floor(w 2^32 / p) (Shoup).
__device__ __forceinline__ uint32_t mulw(uint32_t x, uint32_t w, uint32_t ws, uint32_t p) {
  const uint32_t q = __umulhi(x, ws);
  return csub(x * w - q * p, p);
}
// a b R^-1 mod p (Montgomery, R = 2^32) for a, b < p.
__device__ __forceinline__ uint32_t redc(uint32_t a, uint32_t b, uint32_t p, uint32_t pinv) {
  const uint64_t t = (uint64_t)a * b;
  const uint32_t lo = (uint32_t)t, hi = (uint32_t)(t >> 32);
  const uint32_t m = lo * pinv;
  return csub(hi + __umulhi(m, p) + (lo != 0), p);
}

// ---- transform levels on a warp's two operands (shared memory, 648 values each) ----
template <int N>  // node size; radix-2 split into N/2
__device__ __forceinline__ void fwd_r2(uint32_t* xa, uint32_t* xb, const uint32_t* tw, const uint32_t* tws,
                                       uint32_t p, int lane) {
  constexpr int M = N / 2;
  for (int bf = lane; bf < RING_N / 2; bf += 32) {
    const int node = bf / M, o = node * N + (bf - node * M);
    const uint32_t z = __ldg(tw + node), zs = __ldg(tws + node);
    const uint32_t ta = mulw(xa[o + M], z, zs, p), tb = mulw(xb[o + M], z, zs, p);
    const uint32_t a0 = xa[o], b0 = xb[o];
    xa[o] = addm(a0, ta, p), xa[o + M] = subm(a0, ta, p);
    xb[o] = addm(b0, tb, p), xb[o + M] = subm(b0, tb, p);
  }
  __syncwarp();
}

__device__ __forceinline__ void r3_out(uint32_t f0, uint32_t A, uint32_t B, uint32_t w, uint32_t ws, uint32_t p,
                                       uint32_t& o0, uint32_t& o1, uint32_t& o2) {
  const uint32_t T = mulw(subm(A, B, p), w, ws, p);
  o0 = addm(addm(f0, A, p), B, p);
  o1 = addm(subm(f0, B, p), T, p);
  o2 = subm(subm(f0, A, p), T, p);
}

template <int N>  // node size; radix-3 split into N/3
__device__ __forceinline__ void fwd_r3(uint32_t* xa, uint32_t* xb, const uint32_t* tw, const uint32_t* tws,
                                       uint32_t w, uint32_t ws, uint32_t p, int lane) {
  constexpr int M = N / 3;
  for (int bf = lane; bf < RING_N / 3; bf += 32) {
    const int node = bf / M, o = node * N + (bf - node * M);
    const uint32_t z1 = __ldg(tw + 2 * node), z1s = __ldg(tws + 2 * node);
    const uint32_t z2 = __ldg(tw + 2 * node + 1), z2s = __ldg(tws + 2 * node + 1);
    {
      const uint32_t A = mulw(xa[o + M], z1, z1s, p), B = mulw(xa[o + 2 * M], z2, z2s, p);
      r3_out(xa[o], A, B, w, ws, p, xa[o], xa[o + M], xa[o + 2 * M]);
    }
    {
      const uint32_t A = mulw(xb[o + M], z1, z1s, p), B = mulw(xb[o + 2 * M], z2, z2s, p);
      r3_out(xb[o], A, B, w, ws, p, xb[o], xb[o + M], xb[o + 2 * M]);
    }
  }
  __syncwarp();
}

template <int N>  // node size after merging N/3-sized children; result scaled by 3
__device__ __forceinline__ void inv_r3(uint32_t* x, const uint32_t* tw, const uint32_t* tws, uint32_t w, uint32_t ws,
                                       uint32_t p, int lane) {
  constexpr int M = N / 3;
  for (int bf = lane; bf < RING_N / 3; bf += 32) {
    const int node = bf / M, o = node * N + (bf - node * M);
    const uint32_t o0 = x[o], o1 = x[o + M], o2 = x[o + 2 * M];
    const uint32_t T = mulw(subm(o1, o2, p), w, ws, p);
    const uint32_t S1 = subm(subm(o0, o1, p), T, p), S2 = addm(subm(o0, o2, p), T, p);
    x[o] = addm(addm(o0, o1, p), o2, p);
    x[o + M] = mulw(S1, __ldg(tw + 2 * node), __ldg(tws + 2 * node), p);
    x[o + 2 * M] = mulw(S2, __ldg(tw + 2 * node + 1), __ldg(tws + 2 * node + 1), p);
  }
  __syncwarp();
}

template <int N>  // radix-2 merge; result scaled by 2
__device__ __forceinline__ void inv_r2(uint32_t* x, const uint32_t* tw, const uint32_t* tws, uint32_t p, int lane) {
  constexpr int M = N / 2;
  for (int bf = lane; bf < RING_N / 2; bf += 32) {
    const int node = bf / M, o = node * N + (bf - node * M);
    const uint32_t u = x[o], v = x[o + M];
    x[o] = addm(u, v, p);
    x[o + M] = mulw(subm(u, v, p), __ldg(tw + node), __ldg(tws + node), p);
  }
  __syncwarp();
}

// Offsets of each level's twiddles: 2 + 4 radix-2 nodes, then 8, 24, 72, 216 radix-3 nodes (2 each).
constexpr int TW_L1 = 0, TW_L2 = 2, TW_L3 = 6, TW_L4 = 22, TW_L5 = 70, TW_L6 = 214;

__global__ void __launch_bounds__(32 * MAX_RING_PRIMES)
    k_ring_mul(RingArgs A, const RingPrimeDev* __restrict__ rps, const uint4* __restrict__ a,
               const uint4* __restrict__ b, uint4* __restrict__ c, int* status) {
  extern __shared__ __align__(16) uint8_t rsm[];
  uint32_t* res = reinterpret_cast<uint32_t*>(rsm);  // [prime][2][648]
  const size_t prod = blockIdx.x;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, nt = blockDim.x;
  const u128 q = ((u128)A.q_hi << 64) | A.q_lo;
  // Every warp reads the operands itself (the other warps of the block find them in L1); warp 0
  // also checks that they are below q.
  const uint4* ia = a + prod * RING_N;
  const uint4* ib = b + prod * RING_N;
  if (warp == 0) {
    bool bad = false;
    for (int i = lane; i < RING_N; i += 32) {
      const uint4 x = ia[i], y = ib[i];
      const u128 xv = ((u128)(((uint64_t)x.w << 32) | x.z) << 64) | (((uint64_t)x.y << 32) | x.x);
      const u128 yv = ((u128)(((uint64_t)y.w << 32) | y.z) << 64) | (((uint64_t)y.y << 32) | y.x);
      bad |= xv >= q || yv >= q;
    }
    if (bad) atomicOr(status, 1);
  }
  {
    const RingPrimeDev& P = rps[warp];
    const uint32_t p = P.p;
    uint32_t* xa = res + warp * 2 * RING_N;
    uint32_t* xb = xa + RING_N;
    const uint32_t c1 = P.in[0], c1s = P.in_s[0], c2 = P.in[1], c2s = P.in_s[1], c3 = P.in[2], c3s = P.in_s[2];
    const uint32_t bar = P.bar;
    auto red = [&](uint4 v) {
      uint32_t r = mulw(v.x, 1, bar, p);
      r = addm(r, mulw(v.y, c1, c1s, p), p);
      r = addm(r, mulw(v.z, c2, c2s, p), p);
      return addm(r, mulw(v.w, c3, c3s, p), p);
    };
    for (int i = lane; i < RING_N; i += 32) xa[i] = red(ia[i]), xb[i] = red(ib[i]);
    __syncwarp();
    // the two factors X^324 - omega, X^324 - omega^5: u = lo + omega hi, v = lo + hi - omega hi
    const uint32_t om = P.om, oms = P.om_s;
    for (int i = lane; i < RING_N / 2; i += 32) {
      uint32_t lo = xa[i], hi = xa[i + 324], t = mulw(hi, om, oms, p);
      xa[i] = addm(lo, t, p), xa[i + 324] = subm(addm(lo, hi, p), t, p);
      lo = xb[i], hi = xb[i + 324], t = mulw(hi, om, oms, p);
      xb[i] = addm(lo, t, p), xb[i + 324] = subm(addm(lo, hi, p), t, p);
    }
    __syncwarp();
    const uint32_t w = P.w3, ws = P.w3_s;
    fwd_r2<324>(xa, xb, P.fw + TW_L1, P.fws + TW_L1, p, lane);
    fwd_r2<162>(xa, xb, P.fw + TW_L2, P.fws + TW_L2, p, lane);
    fwd_r3<81>(xa, xb, P.fw + TW_L3, P.fws + TW_L3, w, ws, p, lane);
    fwd_r3<27>(xa, xb, P.fw + TW_L4, P.fws + TW_L4, w, ws, p, lane);
    fwd_r3<9>(xa, xb, P.fw + TW_L5, P.fws + TW_L5, w, ws, p, lane);
    fwd_r3<3>(xa, xb, P.fw + TW_L6, P.fws + TW_L6, w, ws, p, lane);
    for (int i = lane; i < RING_N; i += 32) xa[i] = redc(xa[i], xb[i], p, P.pinv);
    __syncwarp();
    inv_r3<3>(xa, P.iw + TW_L6, P.iws + TW_L6, w, ws, p, lane);
    inv_r3<9>(xa, P.iw + TW_L5, P.iws + TW_L5, w, ws, p, lane);
    inv_r3<27>(xa, P.iw + TW_L4, P.iws + TW_L4, w, ws, p, lane);
    inv_r3<81>(xa, P.iw + TW_L3, P.iws + TW_L3, w, ws, p, lane);
    inv_r2<162>(xa, P.iw + TW_L2, P.iws + TW_L2, p, lane);
    inv_r2<324>(xa, P.iw + TW_L1, P.iws + TW_L1, p, lane);
    // h = (u - v) / (2 omega - 1), lo = u - omega h; then the scale R / 324
    const uint32_t is = P.isplit, iss = P.isplit_s, sc = P.scale, scs = P.scale_s;
    for (int i = lane; i < RING_N / 2; i += 32) {
      const uint32_t u = xa[i], v = xa[i + 324];
      const uint32_t h = mulw(subm(u, v, p), is, iss, p);
      const uint32_t lo = subm(u, mulw(h, om, oms, p), p);
      xa[i] = mulw(lo, sc, scs, p);
      xa[i + 324] = mulw(h, sc, scs, p);
    }
  }
  __syncthreads();
  // Garner: digit k = (r_k - d_0 - p_0 d_1 - ...) / (p_0 ... p_{k-1}) mod p_k.
  const int k = A.nprimes;
  for (int i = tid; i < RING_N; i += nt) {
    uint32_t d[MAX_RING_PRIMES];
    for (int j = 0; j < k; ++j) {
      const uint32_t pj = A.primes[j];
      const uint32_t barj = rps[j].bar;
      uint32_t t = res[j * 2 * RING_N + i];
      for (int m = 0; m < j; ++m) t = mulw(subm(t, mulw(d[m], 1, barj, pj), pj), A.ginv[j][m], A.ginv_s[j][m], pj);
      d[j] = t;
    }
    u128 v = 0;
    if (A.mode == 0) {
      for (int j = k - 1; j >= 0; --j) v = v * A.primes[j] + d[j];  // < q < 2^96
    } else {
      bool neg = false;  // the centred value is negative when the digits exceed floor(P/2)'s
      for (int j = k - 1; j >= 0; --j)
        if (d[j] != A.half[j]) {
          neg = d[j] > A.half[j];
          break;
        }
      const u128 pq = ((u128)A.pq_hi << 64) | A.pq_lo;
      if (A.mode == 2) {  // q = 2^s: arithmetic mod 2^128, then the mask
        for (int j = k - 1; j >= 0; --j) v = v * A.primes[j] + d[j];
        if (neg) v -= pq;
        v &= q - 1;
      } else {
        const int s = (int)A.qbits;
        for (int j = k - 1; j >= 0; --j) {
          const u128 t = v * A.primes[j] + d[j];  // < q 2^31
          const uint64_t x = (uint64_t)(t >> (s - 1));
          const uint64_t qh = (x * A.mu) >> 32;  // Barrett: q - 2 <= qh <= floor(t / q)
          u128 r = t - (u128)qh * q;
          if (r >= q) r -= q;
          if (r >= q) r -= q;
          v = r;
        }
        if (neg) v = v >= pq ? v - pq : v + q - pq;
      }
    }
    c[prod * RING_N + i] = make_uint4((uint32_t)v, (uint32_t)(v >> 32), (uint32_t)(v >> 64), (uint32_t)(v >> 96));
  }
}

size_t ring_mul_smem(int nprimes) { return (size_t)nprimes * 2 * RING_N * 4; }

void launch_ring_mul(const RingPlan& rp, const RingPrimeDev* rps_dev, const void* a, const void* b, void* c, size_t n,
                     int* status, cudaStream_t s) {
  const int k = (int)rp.primes.size();
  const size_t smem = ring_mul_smem(k);
  static std::atomic<unsigned long long> attr{0};
  smem_limit(k_ring_mul, (int)ring_mul_smem(MAX_RING_PRIMES), attr);
  for (size_t done = 0; done < n;) {  // grids of at most 2^31 - 1 products
    const size_t m = std::min(n - done, (size_t)0x7fffffff);
    k_ring_mul<<<(unsigned)m, 32 * k, smem, s>>>(rp.args, rps_dev, reinterpret_cast<const uint4*>(a) + done * RING_N,
                                                 reinterpret_cast<const uint4*>(b) + done * RING_N,
                                                 reinterpret_cast<uint4*>(c) + done * RING_N, status);
    done += m;
  }
}

// ------------------------------------------------------------------------------------------------
// GHASH products: c_i = a_i b_i in B128, 16-byte little-endian elements.
// ------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_ghash_mul(const uint4* __restrict__ a, const uint4* __restrict__ b,
                                                   uint4* __restrict__ c, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const uint4 x = a[i], y = b[i];
    const b128 r = b128_mul({((uint64_t)x.y << 32) | x.x, ((uint64_t)x.w << 32) | x.z},
                            {((uint64_t)y.y << 32) | y.x, ((uint64_t)y.w << 32) | y.z});
    c[i] = make_uint4((uint32_t)r.lo, (uint32_t)(r.lo >> 32), (uint32_t)r.hi, (uint32_t)(r.hi >> 32));
  }
}

void launch_ghash_mul(const void* a, const void* b, void* c, size_t n, int sms, cudaStream_t s) {
  if (!n) return;
  const size_t blocks = std::min((n + 255) / 256, (size_t)sms * 16);
  k_ghash_mul<<<(unsigned)blocks, 256, 0, s>>>(reinterpret_cast<const uint4*>(a), reinterpret_cast<const uint4*>(b),
                                               reinterpret_cast<uint4*>(c), n);
}

__global__ void k_touch_pages(uint8_t* __restrict__ p, size_t n) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t pages = (n + 4095) / 4096;
  if (i < pages) p[i * 4096] = 0;
  if (i == 0 && n) p[n - 1] = 0;
}

void launch_touch_pages(uint8_t* host, size_t n, cudaStream_t s) {
  const size_t pages = (n + 4095) / 4096;
  if (pages) k_touch_pages<<<(unsigned)((pages + 255) / 256), 256, 0, s>>>(host, n);
}

__global__ void k_widen_i16(const int16_t* __restrict__ v, int32_t* __restrict__ out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = v[i];
}

void launch_widen_i16(const int16_t* v, int32_t* out, size_t n, cudaStream_t s) {
  if (n) k_widen_i16<<<(unsigned)std::min((n + 255) / 256, (size_t)4096), 256, 0, s>>>(v, out, n);
}

}  // namespace lf
