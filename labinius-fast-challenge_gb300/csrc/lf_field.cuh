// Binary-field arithmetic shared by host and device code of the prover.
//
//   B128 = GF(2)[x] / (x^128 + x^7 + x^2 + x + 1), plain little-endian bit order (bit i is the
//          coefficient of x^i) -- the GHASH field of solution-arm/labinius/crates/pcs/src/fields/
//          scalar.rs:4-72.
//   F162 = GF(2)[x] / (x^162 + x^81 + 1), three u64 limbs, the top limb 34 bits wide
//          (scalar.rs:104-155). B128 lifts into F162 bit for bit (scalar.rs:111-113).
//
// GPUs have no carry-less multiply instruction. The 32x32 -> 64 carry-less product below uses
// integer multiplication on operands masked to every fourth bit, so that the at most eight
// partial products landing on one bit position never carry into the next position of the same
// residue class (T. Pornin's constant-time GHASH technique, BearSSL ghash_ctmul). Wider products
// are Karatsuba over that primitive.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define LF_HD __host__ __device__ __forceinline__
#else
#define LF_HD inline
#endif

namespace lf {

struct b128 {
  uint64_t lo, hi;
};
struct f162 {
  uint64_t w0, w1, w2;
};

constexpr uint64_t F162_TOP_MASK = (1ull << 34) - 1;

LF_HD b128 b128_add(b128 a, b128 b) { return {a.lo ^ b.lo, a.hi ^ b.hi}; }
LF_HD f162 f162_add(f162 a, f162 b) { return {a.w0 ^ b.w0, a.w1 ^ b.w1, a.w2 ^ b.w2}; }
LF_HD f162 f162_lift(b128 a) { return {a.lo, a.hi, 0}; }
LF_HD bool f162_eq(f162 a, f162 b) { return a.w0 == b.w0 && a.w1 == b.w1 && a.w2 == b.w2; }

LF_HD uint64_t clmul32(uint32_t x, uint32_t y) {
  const uint32_t m0 = 0x11111111u, m1 = 0x22222222u, m2 = 0x44444444u, m3 = 0x88888888u;
  uint64_t x0 = x & m0, x1 = x & m1, x2 = x & m2, x3 = x & m3;
  uint64_t y0 = y & m0, y1 = y & m1, y2 = y & m2, y3 = y & m3;
  uint64_t z0 = (x0 * y0) ^ (x1 * y3) ^ (x2 * y2) ^ (x3 * y1);
  uint64_t z1 = (x0 * y1) ^ (x1 * y0) ^ (x2 * y3) ^ (x3 * y2);
  uint64_t z2 = (x0 * y2) ^ (x1 * y1) ^ (x2 * y0) ^ (x3 * y3);
  uint64_t z3 = (x0 * y3) ^ (x1 * y2) ^ (x2 * y1) ^ (x3 * y0);
  return (z0 & 0x1111111111111111ull) | (z1 & 0x2222222222222222ull) | (z2 & 0x4444444444444444ull) |
         (z3 & 0x8888888888888888ull);
}

// 64x64 -> 128 carry-less, Karatsuba over 32-bit halves.
LF_HD void clmul64(uint64_t a, uint64_t b, uint64_t& lo, uint64_t& hi) {
  uint32_t a0 = (uint32_t)a, a1 = (uint32_t)(a >> 32), b0 = (uint32_t)b, b1 = (uint32_t)(b >> 32);
  uint64_t l = clmul32(a0, b0), h = clmul32(a1, b1);
  uint64_t m = clmul32(a0 ^ a1, b0 ^ b1) ^ l ^ h;
  lo = l ^ (m << 32);
  hi = h ^ (m >> 32);
}

// Multiplication by x^128 mod the GHASH polynomial is multiplication by x^7 + x^2 + x + 1.
LF_HD b128 b128_reduce(uint64_t p0, uint64_t p1, uint64_t p2, uint64_t p3) {
  // H = (p2, p3); H * (1 + x + x^2 + x^7) as 135 bits, then the 7 overflow bits once more.
  uint64_t l0 = p2 ^ (p2 << 1) ^ (p2 << 2) ^ (p2 << 7);
  uint64_t l1 = p3 ^ (p3 << 1) ^ (p3 << 2) ^ (p3 << 7) ^ (p2 >> 63) ^ (p2 >> 62) ^ (p2 >> 57);
  uint64_t o = (p3 >> 63) ^ (p3 >> 62) ^ (p3 >> 57);
  l0 ^= o ^ (o << 1) ^ (o << 2) ^ (o << 7);
  return {p0 ^ l0, p1 ^ l1};
}

// a X^b for b < 128, reduced (a shift, then the GHASH reduction).
LF_HD b128 b128_shl(b128 a, int b) {
  const int r = b & 63;
  const uint64_t s0 = a.lo << r, s1 = (a.hi << r) | (r ? a.lo >> (64 - r) : 0), s2 = r ? a.hi >> (64 - r) : 0;
  return b < 64 ? b128_reduce(s0, s1, s2, 0) : b128_reduce(0, s0, s1, s2);
}

LF_HD b128 b128_mul(b128 a, b128 b) {
  uint64_t l0, h0, l1, h1, lm, hm;
  clmul64(a.lo, b.lo, l0, h0);
  clmul64(a.hi, b.hi, l1, h1);
  clmul64(a.lo ^ a.hi, b.lo ^ b.hi, lm, hm);
  lm ^= l0 ^ l1;
  hm ^= h0 ^ h1;
  return b128_reduce(l0, h0 ^ lm, l1 ^ hm, h1);
}

// Reduce a product of two F162 (at most 323 bits in p0..p5) modulo x^162 + x^81 + 1.
LF_HD f162 f162_reduce(uint64_t p0, uint64_t p1, uint64_t p2, uint64_t p3, uint64_t p4, uint64_t p5) {
  // H = p >> 162 (at most 161 bits).
  uint64_t h0 = (p2 >> 34) | (p3 << 30);
  uint64_t h1 = (p3 >> 34) | (p4 << 30);
  uint64_t h2 = (p4 >> 34) | (p5 << 30);
  uint64_t r0 = p0 ^ h0, r1 = p1 ^ h1, r2 = (p2 & F162_TOP_MASK) ^ h2;
  // + H * x^81
  r1 ^= h0 << 17;
  r2 ^= (h0 >> 47) | (h1 << 17);
  uint64_t r3 = (h1 >> 47) | (h2 << 17);
  // bits 162.. of r once more (at most 80 bits): G = r >> 162.
  uint64_t g0 = (r2 >> 34) | (r3 << 30), g1 = r3 >> 34;
  r2 &= F162_TOP_MASK;
  r0 ^= g0;
  r1 ^= g1 ^ (g0 << 17);
  r2 ^= (g0 >> 47) | (g1 << 17);
  return {r0, r1, r2};
}

// Three-way Karatsuba over the 64-bit limbs.
LF_HD f162 f162_mul(f162 a, f162 b) {
  uint64_t p0l, p0h, p1l, p1h, p2l, p2h, q01l, q01h, q02l, q02h, q12l, q12h;
  clmul64(a.w0, b.w0, p0l, p0h);
  clmul64(a.w1, b.w1, p1l, p1h);
  clmul64(a.w2, b.w2, p2l, p2h);
  clmul64(a.w0 ^ a.w1, b.w0 ^ b.w1, q01l, q01h);
  clmul64(a.w0 ^ a.w2, b.w0 ^ b.w2, q02l, q02h);
  clmul64(a.w1 ^ a.w2, b.w1 ^ b.w2, q12l, q12h);
  // c1 = q01 + p0 + p1 ; c2 = q02 + p0 + p2 + p1 ; c3 = q12 + p1 + p2
  uint64_t c1l = q01l ^ p0l ^ p1l, c1h = q01h ^ p0h ^ p1h;
  uint64_t c2l = q02l ^ p0l ^ p2l ^ p1l, c2h = q02h ^ p0h ^ p2h ^ p1h;
  uint64_t c3l = q12l ^ p1l ^ p2l, c3h = q12h ^ p1h ^ p2h;
  uint64_t r0 = p0l;
  uint64_t r1 = p0h ^ c1l;
  uint64_t r2 = c1h ^ c2l;
  uint64_t r3 = c2h ^ c3l;
  uint64_t r4 = c3h ^ p2l;
  uint64_t r5 = p2h;
  return f162_reduce(r0, r1, r2, r3, r4, r5);
}

// a * lift(x): the second operand has no third limb.
LF_HD f162 f162_mul_lifted(f162 a, b128 x) {
  uint64_t p0l, p0h, p1l, p1h, q01l, q01h, q2l, q2h, q3l, q3h;
  clmul64(a.w0, x.lo, p0l, p0h);
  clmul64(a.w1, x.hi, p1l, p1h);
  clmul64(a.w0 ^ a.w1, x.lo ^ x.hi, q01l, q01h);
  clmul64(a.w2, x.lo, q2l, q2h);
  clmul64(a.w2, x.hi, q3l, q3h);
  uint64_t m_l = q01l ^ p0l ^ p1l, m_h = q01h ^ p0h ^ p1h;
  uint64_t r0 = p0l;
  uint64_t r1 = p0h ^ m_l;
  uint64_t r2 = m_h ^ p1l ^ q2l;
  uint64_t r3 = p1h ^ q2h ^ q3l;
  uint64_t r4 = q3h;
  return f162_reduce(r0, r1, r2, r3, r4, 0);
}

// x * X: one shift with the GHASH reduction (used to build multiplication matrices).
LF_HD b128 b128_mulx(b128 a) {
  uint64_t top = a.hi >> 63;
  b128 r = {a.lo << 1, (a.hi << 1) | (a.lo >> 63)};
  r.lo ^= top * 0x87ull;
  return r;
}

LF_HD bool b128_bit(b128 a, int k) { return k < 64 ? (a.lo >> k) & 1 : (a.hi >> (k - 64)) & 1; }

}  // namespace lf
