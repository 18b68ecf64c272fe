// F162 x lift(B128) products where a whole block multiplies by the same F162 value e (the
// materialisation of the switch and the row evaluation: one multiplier per table row, many
// table words). The product is GF(2)-linear in the B128 operand, so with the 4-bit window table
//   T[g][v] = e * (v X^(4g)),  g < 32, v < 16   (512 F162 = 12 KB of shared memory)
// e * lift(x) = XOR_g T[g][nibble g of x]: 32 table reads and XORs instead of five 64 x 64
// carry-less products. The table is built from the 128 values e X^b (shifts reduced modulo
// x^162 + x^81 + 1), each entry the XOR of at most four of them.
#pragma once
#include "lf_field.cuh"

namespace lf {

// e X^b for b < 128, reduced.
__device__ __forceinline__ f162 f162_shl(f162 e, int b) {
  const int r = b & 63;
  uint64_t s0 = e.w0 << r, s1 = (e.w1 << r) | (r ? e.w0 >> (64 - r) : 0),
           s2 = (e.w2 << r) | (r ? e.w1 >> (64 - r) : 0), s3 = r ? e.w2 >> (64 - r) : 0;
  if (b < 64) return f162_reduce(s0, s1, s2, s3, 0, 0);
  return f162_reduce(0, s0, s1, s2, s3, 0);
}

struct WinTable {
  uint64_t w0[512], w1[512], w2[512];  // entry 16 g + v, limbs apart (conflict-free lookups)
  f162 base[128];                      // e X^b
};

// Every thread of the block takes part; the table is ready after the call (two barriers).
__device__ __forceinline__ void win_build(WinTable& T, f162 e, int tid, int nt) {
  for (int b = tid; b < 128; b += nt) T.base[b] = f162_shl(e, b);
  __syncthreads();
  for (int idx = tid; idx < 512; idx += nt) {
    const int g = idx >> 4, v = idx & 15;
    f162 acc = {0, 0, 0};
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if ((v >> k) & 1) acc = f162_add(acc, T.base[4 * g + k]);
    T.w0[idx] = acc.w0, T.w1[idx] = acc.w1, T.w2[idx] = acc.w2;
  }
  __syncthreads();
}

__device__ __forceinline__ void win_mul_add(const WinTable& T, uint4 x, f162& acc) {
  const uint32_t xs[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
  for (int g = 0; g < 32; ++g) {
    const int idx = 16 * g + ((xs[g >> 3] >> (4 * (g & 7))) & 15);
    acc.w0 ^= T.w0[idx], acc.w1 ^= T.w1[idx], acc.w2 ^= T.w2[idx];
  }
}

}  // namespace lf
