// Batched ring and GHASH products (lf_ring.cu): plans and launch wrappers.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "lf_internal.h"

namespace lf {

constexpr int MAX_RING_PRIMES = 8;  // 8 distinct factors p = 1 (mod 1944) stay below 2^96
constexpr int RING_TW = 646;        // node twiddles of one transform: 2 + 4 + 2 (8 + 24 + 72 + 216)

// One transform prime p = 1 (mod 1944), p < 2^31: Shoup pairs (w, floor(w 2^32 / p)) for every
// constant the kernel multiplies by.
struct RingPrimeDev {
  uint32_t p, pinv, bar;            // pinv = -p^-1 mod 2^32; bar = floor(2^32 / p)
  uint32_t om, om_s;                // omega = zeta^324 (primitive 6th root)
  uint32_t w3, w3_s;                // zeta^648 (primitive cube root)
  uint32_t isplit, isplit_s;        // (2 omega - 1)^-1
  uint32_t scale, scale_s;          // 2^32 / 324
  uint32_t in[3], in_s[3];          // 2^32, 2^64, 2^96 mod p (operand reduction)
  uint32_t fw[RING_TW], fws[RING_TW];  // forward node twiddles zeta^s (and zeta^2s for radix 3)
  uint32_t iw[RING_TW], iws[RING_TW];  // their inverses
};

struct RingArgs {
  int nprimes, mode;  // mode 0: q = product of the primes; 1: exact lift, Barrett mod q; 2: lift, q = 2^s
  uint32_t primes[MAX_RING_PRIMES];
  uint32_t ginv[MAX_RING_PRIMES][MAX_RING_PRIMES], ginv_s[MAX_RING_PRIMES][MAX_RING_PRIMES];
  uint32_t half[MAX_RING_PRIMES];  // floor(P / 2) in mixed radix
  uint32_t qbits;
  uint64_t mu;                     // floor(2^(qbits + 31) / q)
  uint64_t q_lo, q_hi, pq_lo, pq_hi;
};

struct RingPlan {
  u128 q = 0;
  int mode = 0;
  std::vector<uint32_t> primes;
  std::vector<RingPrimeDev> dev;
  RingArgs args;
};

bool make_ring_plan(u128 q, RingPlan& rp, std::string& err);
// c[i] = a[i] * b[i] in R_q for i < n; 648 little-endian u128 coefficients per element, device
// pointers. status bit 0 is set when an operand coefficient is not below q.
void launch_ring_mul(const RingPlan& rp, const RingPrimeDev* rps_dev, const void* a, const void* b, void* c, size_t n,
                     int* status, cudaStream_t s);
// c[i] = a[i] * b[i] in B128 for i < n (16-byte little-endian elements), device pointers.
void launch_ghash_mul(const void* a, const void* b, void* c, size_t n, int sms, cudaStream_t s);
void launch_widen_i16(const int16_t* v, int32_t* out, size_t n, cudaStream_t s);

}  // namespace lf
