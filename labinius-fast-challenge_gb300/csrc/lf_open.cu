// The opening on the GPU: row evaluation, folding challenges, the fold, and the BLAKE3 tree
// hashing of the transcript's large absorb.
#include <cstdio>

#include "lf_blake3.cuh"
#include "lf_internal.h"

namespace lf {

// ---------------------------------------------------------------------------------------------
// Row evaluation (verifier/proof_verify/src/reference.rs:50-70; eval.rs:173-185):
// u_j = sum_i eq_table(p0)[i] * lift(W[i + COLUMN_LEN j]). One block per column.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ f162 shfl_xor_f162(f162 v, int m) {
  v.w0 ^= __shfl_xor_sync(0xffffffffu, v.w0, m);
  v.w1 ^= __shfl_xor_sync(0xffffffffu, v.w1, m);
  v.w2 ^= __shfl_xor_sync(0xffffffffu, v.w2, m);
  return v;
}

__global__ void __launch_bounds__(256) k_row_eval(const uint4* __restrict__ table, int rl, const f162* __restrict__ eqt,
                                                  f162* __restrict__ row) {
  const int col = blockIdx.x;
  const uint64_t n = 1ull << rl;
  const uint4* w = table + ((uint64_t)col << rl);
  f162 acc = {0, 0, 0};
  for (uint64_t i = threadIdx.x; i < n; i += blockDim.x) {
    uint4 x = w[i];
    b128 b = {(uint64_t)x.x | ((uint64_t)x.y << 32), (uint64_t)x.z | ((uint64_t)x.w << 32)};
    acc = f162_add(acc, f162_mul_lifted(eqt[i], b));
  }
  for (int m = 16; m; m >>= 1) acc = shfl_xor_f162(acc, m);
  __shared__ f162 part[8];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    f162 s = {0, 0, 0};
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s = f162_add(s, part[i]);
    row[col] = s;
  }
}

void launch_row_eval(const uint4* table, int rl, const f162* eqt, f162* row, cudaStream_t s) {
  k_row_eval<<<COLUMNS, 256, 0, s>>>(table, rl, eqt, row);
}

// ---------------------------------------------------------------------------------------------
// Folding challenges (challenge.rs:343-755). One warp per challenge. The XOF of derivation
// base + i of the transcript is read as a byte stream; an attempt is a partial Fisher-Yates over
// the 162 positions driven by little-endian u16 draws, the positions sorted, signed by a keyed
// hash of the position set, and accepted when every one of the 81 phase lanes keeps
// re^2 + im^2 <= bound_sq (f64, round-to-nearest, no fused multiply-add).
// ---------------------------------------------------------------------------------------------
constexpr int CH_WARPS = 4;
constexpr int XOF_BUF = 32 * 64;
constexpr int N162 = 162;
constexpr int WEIGHT = 28;
constexpr int PHASE_LANES = 88;
constexpr uint64_t MAX_ATTEMPTS = 1ull << 22;

struct ChWarp {
  uint8_t buf[XOF_BUF];
  uint8_t perm[176];
  uint32_t root[27];
};

__device__ __forceinline__ void xof_refill(ChWarp& s, const bk::Pending& root, uint64_t& next_block, int lane) {
  __syncwarp();  // every lane has read the previous buffer before any lane overwrites it
  uint32_t w[16];
  root.root_block(next_block + lane, w);
  uint32_t* dst = reinterpret_cast<uint32_t*>(s.buf + 64 * lane);
#pragma unroll
  for (int i = 0; i < 16; ++i) dst[i] = w[i];
  next_block += 32;
  __syncwarp();
}

__global__ void __launch_bounds__(32 * CH_WARPS) k_challenges(const bk::Hasher* __restrict__ state, uint64_t base,
                                                              bk::Pending sign_key_node, const double* __restrict__ re,
                                                              const double* __restrict__ im, double bound_sq,
                                                              Challenge* __restrict__ out, int n, int* status,
                                                              uint32_t* __restrict__ dbg) {
  __shared__ ChWarp sw[CH_WARPS];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int ci = blockIdx.x * CH_WARPS + wid;
  if (ci >= n) return;
  ChWarp& s = sw[wid];
  if (lane == 0) {
    if (dbg != nullptr && ci == 0) {
      dbg[48] = state->key[0], dbg[49] = state->mode, dbg[50] = state->depth, dbg[51] = state->chunk.buf_len;
      dbg[52] = state->chunk.blocks, dbg[53] = (uint32_t)state->chunk.index, dbg[54] = state->chunk.h[0];
      dbg[56] = (uint32_t)sizeof(bk::Hasher);
    }
    bk::Pending r = bk::derive_root(*state, base + (uint64_t)ci, "short-challenge", 15);
    for (int i = 0; i < 8; ++i) s.root[i] = r.h[i];
    for (int i = 0; i < 16; ++i) s.root[8 + i] = r.m[i];
    s.root[24] = (uint32_t)r.t;
    s.root[25] = r.len;
    s.root[26] = r.flags;
  }
  __syncwarp();
  bk::Pending root;
  for (int i = 0; i < 8; ++i) root.h[i] = s.root[i];
  for (int i = 0; i < 16; ++i) root.m[i] = s.root[8 + i];
  root.t = s.root[24];
  root.len = s.root[25];
  root.flags = s.root[26];
  uint64_t next_block = 0;
  int pos = XOF_BUF;
  const bool trace = dbg != nullptr && ci == 0;
  if (trace && lane == 0)
    for (int i = 0; i < 27; ++i) dbg[i] = s.root[i];
  auto byte = [&]() -> uint32_t {
    if (pos == XOF_BUF) {
      xof_refill(s, root, next_block, lane);
      pos = 0;
    }
    return s.buf[pos++];
  };
  for (uint64_t attempt = 0; attempt < MAX_ATTEMPTS; ++attempt) {
    for (int i = lane; i < N162; i += 32) s.perm[i] = (uint8_t)i;
    __syncwarp();
    for (int i = 0; i < WEIGHT; ++i) {
      const uint32_t nn = (uint32_t)(N162 - i);
      const uint32_t limit = (65536u / nn) * nn;
      const uint64_t magic = (1ull << 32) / nn + 1;
      uint32_t r;
      do {
        uint32_t lo = byte();
        uint32_t hi = byte();
        r = lo | (hi << 8);
      } while (r >= limit);
      uint32_t q = (uint32_t)(((uint64_t)r * magic) >> 32);
      int j = i + (int)(r - q * nn);
      if (lane == 0) {
        uint8_t t = s.perm[i];
        s.perm[i] = s.perm[j];
        s.perm[j] = t;
      }
      __syncwarp();
    }
    // Sorted positions: lane l < 28 places perm[l] by its rank.
    uint32_t mine = lane < WEIGHT ? s.perm[lane] : 255;
    int rank = 0;
    for (int t = 0; t < WEIGHT; ++t) rank += (int)(s.perm[t] < mine);
    __syncwarp();
    __shared__ uint8_t sorted[CH_WARPS][32];
    if (lane < WEIGHT) sorted[wid][rank] = (uint8_t)mine;
    __syncwarp();
    // Signs: derive-key hash of (weight as u64 LE || positions), first four bytes LE.
    uint32_t signs = 0;
    if (lane == 0) {
      uint8_t blk[64];
      for (int i = 0; i < 64; ++i) blk[i] = 0;
      blk[0] = (uint8_t)WEIGHT;
      for (int i = 0; i < WEIGHT; ++i) blk[8 + i] = sorted[wid][i];
      uint32_t m[16], o[16];
      bk::load_words(blk, m, 16);
      bk::compress16(sign_key_node.h, m, 0, 8 + WEIGHT, sign_key_node.flags | bk::F_ROOT, o);
      signs = o[0] & ((1u << WEIGHT) - 1);
    }
    signs = __shfl_sync(0xffffffffu, signs, 0);
    if (trace && attempt == 0 && lane == 0) {
      for (int i = 0; i < 32; ++i) reinterpret_cast<uint8_t*>(dbg + 27)[i] = s.buf[i];
      for (int i = 0; i < 28; ++i) reinterpret_cast<uint8_t*>(dbg + 35)[i] = sorted[wid][i];
      dbg[42] = signs;
    }
    bool over = false;
    for (int k = lane; k < 81; k += 32) {
      double vr = 0.0, vi = 0.0;
      for (int t = 0; t < WEIGHT; ++t) {
        int b = sorted[wid][t] * PHASE_LANES + k;
        double pr = re[b], pi = im[b];
        if ((signs >> t) & 1) pr = -pr, pi = -pi;
        vr = __dadd_rn(vr, pr);
        vi = __dadd_rn(vi, pi);
      }
      double m2 = __dadd_rn(__dmul_rn(vr, vr), __dmul_rn(vi, vi));
      over |= m2 > bound_sq;
      if (trace && attempt == 0 && k == 0) {
        double* d = reinterpret_cast<double*>(dbg + 44);
        d[0] = m2;
        d[1] = vr;
      }
    }
    const bool any_over = __any_sync(0xffffffffu, over);
    if (trace && attempt == 0 && lane == 0) dbg[43] = any_over;
    if (!any_over) {
      if (lane < WEIGHT) out[ci].positions[lane] = sorted[wid][lane];
      else out[ci].positions[lane] = 0;
      if (lane == 0) {
        out[ci].signs = signs;
        out[ci].weight = WEIGHT;
      }
      return;
    }
    __syncwarp();
  }
  if (lane == 0) atomicExch(status, 1);
}

void launch_challenges(const void* hasher_dev, uint64_t base_counter, const uint32_t sign_key[8], const double* phase_re,
                       const double* phase_im, Challenge* out, int n, int* status, cudaStream_t s, uint32_t* dbg) {
  bk::Pending sk;
  for (int i = 0; i < 8; ++i) sk.h[i] = sign_key[i];
  for (int i = 0; i < 16; ++i) sk.m[i] = 0;
  sk.t = 0;
  sk.len = 0;
  sk.flags = bk::F_DERIVE_MAT | bk::F_CHUNK_START | bk::F_CHUNK_END;
  const double bound_sq = 12.0 * 12.0 + 1e-12;
  k_challenges<<<(n + CH_WARPS - 1) / CH_WARPS, 32 * CH_WARPS, 0, s>>>(
      reinterpret_cast<const bk::Hasher*>(hasher_dev), base_counter, sk, phase_re, phase_im, bound_sq, out, n, status, dbg);
}

// ---------------------------------------------------------------------------------------------
// Fold (reference.rs:72-133): v_m = sum_j c_j W_{j,m} over the integers. A challenge sits in R_648
// as c(-X^4), so with Y = X^4 each table word k of element m is folded on its own:
// V_{m,k}(Y) = sum_j sum_t s_{j,t} Y^{pos_{j,t}} W_{j,m,k}(Y), s = sign bit XOR (pos odd), then
// Y^162 = Y^81 - 1. Bit-sliced: a block handles 8 elements (32 words, one per bit of a u32),
// thread y owns raw position y (0..288) as a 16-plane two's-complement counter.
// ---------------------------------------------------------------------------------------------
constexpr int FOLD_ELEMS = 8;
constexpr int FOLD_THREADS = 320;
constexpr int FOLD_BATCH = FOLD_THREADS / 32;  // columns transposed per step, one per warp
constexpr int RAW_Y = 128 + 161;               // 289 raw positions

__global__ void __launch_bounds__(FOLD_THREADS) k_fold(const uint4* __restrict__ table, int rl,
                                                      uint64_t ring_elements, const Challenge* __restrict__ ch,
                                                      int32_t* __restrict__ out, int* status) {
  __shared__ uint32_t vec[FOLD_BATCH][128];
  __shared__ uint8_t cpos[FOLD_BATCH][32];
  __shared__ uint32_t csign[FOLD_BATCH];
  __shared__ int32_t raw[32][RAW_Y + 1];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t m0 = (uint64_t)blockIdx.x * FOLD_ELEMS;
  // Columns with fewer than 8 ring elements: lanes past the last element fold zero words.
  const int live_words = (int)min((uint64_t)FOLD_ELEMS, ring_elements - m0) * 4;
  uint32_t P[16];
#pragma unroll
  for (int b = 0; b < 16; ++b) P[b] = 0;
  for (int j0 = 0; j0 < COLUMNS; j0 += FOLD_BATCH) {
    const int j = j0 + warp;
    if (j < COLUMNS) {
      uint4 v = lane < live_words ? table[((uint64_t)j << rl) + 4 * m0 + lane] : make_uint4(0, 0, 0, 0);
      uint32_t keep[4] = {0, 0, 0, 0};
#pragma unroll
      for (int b = 0; b < 128; ++b) {
        uint32_t word = b < 32 ? v.x : b < 64 ? v.y : b < 96 ? v.z : v.w;
        uint32_t m = __ballot_sync(0xffffffffu, (word >> (b & 31)) & 1);
        if (lane == (b & 31)) keep[b >> 5] = m;
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) vec[warp][32 * i + lane] = keep[i];
      cpos[warp][lane] = ch[j].positions[lane];
      if (lane == 0) csign[warp] = ch[j].signs;
    }
    __syncthreads();
    if (tid < RAW_Y) {
      const int nb = min(FOLD_BATCH, COLUMNS - j0);
      for (int c = 0; c < nb; ++c) {
        const uint32_t sg = csign[c];
        for (int t = 0; t < WEIGHT; ++t) {
          const int pos = cpos[c][t];
          const int p = tid - pos;
          if ((unsigned)p >= 128u) continue;
          uint32_t x = vec[c][p];
          if (!x) continue;
          const bool neg = (((sg >> t) & 1) ^ (pos & 1)) != 0;
          if (neg) {
#pragma unroll
            for (int b = 0; b < 16; ++b) {
              uint32_t t2 = ~P[b] & x;
              P[b] ^= x;
              x = t2;
              if (!x) break;
            }
          } else {
#pragma unroll
            for (int b = 0; b < 16; ++b) {
              uint32_t t2 = P[b] & x;
              P[b] ^= x;
              x = t2;
              if (!x) break;
            }
          }
        }
      }
    }
    __syncthreads();
  }
  if (tid < RAW_Y) {
    for (int l = 0; l < 32; ++l) {
      int32_t v = 0;
#pragma unroll
      for (int b = 0; b < 16; ++b) v |= (int32_t)((P[b] >> l) & 1) << b;
      v = (v ^ 0x8000) - 0x8000;
      raw[l][tid] = v;
    }
  }
  __syncthreads();
  if (tid < 32) {
    int32_t* r = raw[tid];
    for (int y = RAW_Y - 1; y >= N162; --y) {
      int32_t v = r[y];
      r[y - 81] += v;
      r[y - N162] -= v;
    }
  }
  __syncthreads();
  for (int idx = tid; idx < (live_words / 4) * 648; idx += FOLD_THREADS) {
    const int m = idx / 648, c = idx % 648, y = c >> 2, k = c & 3;
    const int32_t v = raw[4 * m + k][y];
    if (v < -32768 || v > 32767) atomicExch(status, 2);
    out[(m0 + m) * 648 + c] = v;
  }
}

// Fold, carry-save version. A block folds 16 elements (64 table words: two 32-bit bit-slices per
// thread) over a share of the columns; thread y owns raw position y. Per column the 128 bit
// vectors of the 64 words sit in shared memory zero-padded to positions -161..288, so term t of
// a challenge contributes vec[y - pos_t] with no range test. A negative term contributes the
// complemented vector: sum_t s_t x_t = sum_{t+} x_t + sum_{t-} ~x_t - (number of negative terms),
// and that count does not depend on y or on the lane, so it is subtracted once at the end.
// The inputs (28 per column, 8 columns per step = 14 groups of 16) go through Harley-Seal
// carry-save adders into a 16-plane counter. Shares of columns are summed with atomicAdd.
constexpr int F2_BATCH = 8;                 // columns per step, one transposing warp each
constexpr int F2_THREADS = 320;
constexpr int F2_PAD = 161;                 // vec index = p + 161, p in [-161, 288]
constexpr int F2_VEC = 450;
constexpr int F2_INPUTS = F2_BATCH * WEIGHT;  // 224 = 14 x 16

__device__ __forceinline__ void csa(uint32_t& h, uint32_t& l, uint32_t a, uint32_t b, uint32_t c) {
  uint32_t u = a ^ b;
  h = (a & b) | (u & c);
  l = u ^ c;
}

__global__ void __launch_bounds__(F2_THREADS) k_fold2(const uint4* __restrict__ table, int rl, uint64_t ring_elements,
                                                     const Challenge* __restrict__ ch, int col_share,
                                                     int32_t* __restrict__ out) {
  extern __shared__ __align__(16) uint8_t f2smem[];
  uint2* vec = reinterpret_cast<uint2*>(f2smem);                                      // [F2_BATCH][F2_VEC]
  int* toff = reinterpret_cast<int*>(f2smem + F2_BATCH * F2_VEC * 8);                  // [F2_INPUTS]
  uint32_t* tmask = reinterpret_cast<uint32_t*>(toff + F2_INPUTS);                     // [F2_INPUTS]
  __shared__ int neg_total;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t m0 = (uint64_t)blockIdx.x * 16;
  const int live = (int)min((uint64_t)16, ring_elements - m0) * 4;  // live words of the 64
  const int c_begin = blockIdx.y * col_share, c_end = min(COLUMNS, c_begin + col_share);
  for (int i = tid; i < F2_BATCH * F2_VEC; i += F2_THREADS) vec[i] = make_uint2(0, 0);
  if (tid == 0) neg_total = 0;
  uint32_t ones[2] = {0, 0}, twos[2] = {0, 0}, fours[2] = {0, 0}, eights[2] = {0, 0};
  uint32_t P[2][12];
#pragma unroll
  for (int h = 0; h < 2; ++h)
#pragma unroll
    for (int b = 0; b < 12; ++b) P[h][b] = 0;
  __syncthreads();
  for (int j0 = c_begin; j0 < c_end; j0 += F2_BATCH) {
    const int nb = min(F2_BATCH, c_end - j0);
    if (warp < nb) {
      const int j = j0 + warp;
      const uint4* w = table + ((uint64_t)j << rl) + 4 * m0;
      uint4 v0 = lane < live ? w[lane] : make_uint4(0, 0, 0, 0);
      uint4 v1 = lane + 32 < live ? w[lane + 32] : make_uint4(0, 0, 0, 0);
      uint32_t keep0[4] = {0, 0, 0, 0}, keep1[4] = {0, 0, 0, 0};
#pragma unroll
      for (int b = 0; b < 128; ++b) {
        const uint32_t a0 = b < 32 ? v0.x : b < 64 ? v0.y : b < 96 ? v0.z : v0.w;
        const uint32_t a1 = b < 32 ? v1.x : b < 64 ? v1.y : b < 96 ? v1.z : v1.w;
        const uint32_t m0b = __ballot_sync(0xffffffffu, (a0 >> (b & 31)) & 1);
        const uint32_t m1b = __ballot_sync(0xffffffffu, (a1 >> (b & 31)) & 1);
        if (lane == (b & 31)) keep0[b >> 5] = m0b, keep1[b >> 5] = m1b;
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) vec[warp * F2_VEC + F2_PAD + 32 * i + lane] = make_uint2(keep0[i], keep1[i]);
      if (lane < WEIGHT) {
        const int pos = ch[j].positions[lane];
        const bool neg = (((ch[j].signs >> lane) & 1) ^ (pos & 1)) != 0;
        toff[warp * WEIGHT + lane] = warp * F2_VEC + F2_PAD - pos;
        tmask[warp * WEIGHT + lane] = neg ? 0xffffffffu : 0u;
        const unsigned nn = __ballot_sync(0x0fffffffu, neg);
        if (lane == 0) atomicAdd(&neg_total, __popc(nn));
      }
    } else if (warp < F2_BATCH) {
      // columns past the end of the share: zero vectors, no negative terms
#pragma unroll
      for (int i = 0; i < 4; ++i) vec[warp * F2_VEC + F2_PAD + 32 * i + lane] = make_uint2(0, 0);
      if (lane < WEIGHT) {
        toff[warp * WEIGHT + lane] = warp * F2_VEC + F2_PAD;
        tmask[warp * WEIGHT + lane] = 0u;
      }
    }
    __syncthreads();
    if (tid < RAW_Y) {
#pragma unroll 1
      for (int g = 0; g < F2_INPUTS / 16; ++g) {
        uint32_t x[2][16];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int k = 16 * g + i;
          const uint2 v = vec[toff[k] + tid];
          const uint32_t m = tmask[k];
          x[0][i] = v.x ^ m, x[1][i] = v.y ^ m;
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          uint32_t twosA, twosB, foursA, foursB, eightsA, eightsB, sixteens;
          csa(twosA, ones[h], ones[h], x[h][0], x[h][1]);
          csa(twosB, ones[h], ones[h], x[h][2], x[h][3]);
          csa(foursA, twos[h], twos[h], twosA, twosB);
          csa(twosA, ones[h], ones[h], x[h][4], x[h][5]);
          csa(twosB, ones[h], ones[h], x[h][6], x[h][7]);
          csa(foursB, twos[h], twos[h], twosA, twosB);
          csa(eightsA, fours[h], fours[h], foursA, foursB);
          csa(twosA, ones[h], ones[h], x[h][8], x[h][9]);
          csa(twosB, ones[h], ones[h], x[h][10], x[h][11]);
          csa(foursA, twos[h], twos[h], twosA, twosB);
          csa(twosA, ones[h], ones[h], x[h][12], x[h][13]);
          csa(twosB, ones[h], ones[h], x[h][14], x[h][15]);
          csa(foursB, twos[h], twos[h], twosA, twosB);
          csa(eightsB, fours[h], fours[h], foursA, foursB);
          csa(sixteens, eights[h], eights[h], eightsA, eightsB);
          uint32_t c = sixteens;
#pragma unroll
          for (int b = 0; b < 12; ++b) {
            const uint32_t t = P[h][b] & c;
            P[h][b] ^= c;
            c = t;
          }
        }
      }
    }
    __syncthreads();
  }
  // Un-slice: raw[lane][y] for the 64 words, then the ring reduction Y^162 = Y^81 - 1 per word.
  int32_t* raw = reinterpret_cast<int32_t*>(f2smem);  // [64][RAW_Y + 1], reuses the vectors' space
  const int ntot = neg_total;
  if (tid < RAW_Y) {
#pragma unroll
    for (int h = 0; h < 2; ++h)
      for (int l = 0; l < 32; ++l) {
        int32_t v = (int32_t)((ones[h] >> l) & 1) | ((int32_t)((twos[h] >> l) & 1) << 1) |
                    ((int32_t)((fours[h] >> l) & 1) << 2) | ((int32_t)((eights[h] >> l) & 1) << 3);
#pragma unroll
        for (int b = 0; b < 12; ++b) v |= (int32_t)((P[h][b] >> l) & 1) << (b + 4);
        raw[(32 * h + l) * (RAW_Y + 1) + tid] = v - ntot;
      }
  }
  __syncthreads();
  if (tid < 64) {
    int32_t* r = raw + tid * (RAW_Y + 1);
    for (int y = RAW_Y - 1; y >= N162; --y) {
      const int32_t v = r[y];
      r[y - 81] += v;
      r[y - N162] -= v;
    }
  }
  __syncthreads();
  for (int idx = tid; idx < (live / 4) * 648; idx += F2_THREADS) {
    const int m = idx / 648, c = idx % 648, y = c >> 2, k = c & 3;
    atomicAdd(&out[(m0 + m) * 648 + c], raw[(4 * m + k) * (RAW_Y + 1) + y]);
  }
}

__global__ void k_fold_range(const int32_t* __restrict__ out, uint64_t n, int* status) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    if (out[i] < -32768 || out[i] > 32767) atomicExch(status, 2);
}

void launch_fold(const uint4* table, int rl, uint64_t ring_elements, const Challenge* ch, int32_t* out, int* status,
                 cudaStream_t s) {
  const int smem_vec = F2_BATCH * F2_VEC * 8 + 2 * F2_INPUTS * 4;
  const int smem_raw = 64 * (RAW_Y + 1) * 4;
  const int smem = smem_vec > smem_raw ? smem_vec : smem_raw;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_fold2, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    attr = true;
  }
  const unsigned blocks = (unsigned)((ring_elements + 15) / 16);
  // Enough blocks to cover the SMs: split the columns when there are few element blocks.
  int shares = 1;
  while (blocks * shares < 2 * 152 && shares < 64) shares *= 2;
  const int col_share = COLUMNS / shares;
  cudaMemsetAsync(out, 0, ring_elements * 648 * 4, s);
  k_fold2<<<dim3(blocks, shares), F2_THREADS, smem, s>>>(table, rl, ring_elements, ch, col_share, out);
  k_fold_range<<<256, 256, 0, s>>>(out, ring_elements * 648, status);
}

// ---------------------------------------------------------------------------------------------
// BLAKE3 tree hashing of a stream (the transcript's commitment absorb, challenge.rs:152-223).
// ---------------------------------------------------------------------------------------------
struct KeyArg {
  uint32_t k[8];
};

__global__ void k_chunk_cvs(const uint8_t* __restrict__ stream, uint64_t nchunks, KeyArg key, uint32_t mode,
                            uint32_t* __restrict__ cvs) {
  uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (c >= nchunks) return;
  const uint4* src = reinterpret_cast<const uint4*>(stream + c * 1024);
  uint32_t h[8];
  for (int i = 0; i < 8; ++i) h[i] = key.k[i];
  for (int b = 0; b < 16; ++b) {
    uint32_t m[16];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      uint4 v = src[4 * b + i];
      m[4 * i] = v.x, m[4 * i + 1] = v.y, m[4 * i + 2] = v.z, m[4 * i + 3] = v.w;
    }
    uint32_t f = mode | (b == 0 ? bk::F_CHUNK_START : 0) | (b == 15 ? bk::F_CHUNK_END : 0);
    uint32_t o[16];
    bk::compress16(h, m, c, 64, f, o);
    for (int i = 0; i < 8; ++i) h[i] = o[i];
  }
  for (int i = 0; i < 8; ++i) cvs[c * 8 + i] = h[i];
}

__global__ void __launch_bounds__(1024) k_subtrees(const uint32_t* __restrict__ cvs, uint32_t* scratch, uint64_t nchunks,
                                                   KeyArg key, uint32_t mode, uint32_t* __restrict__ out) {
  uint32_t* bufA = scratch;
  uint32_t* bufB = scratch + nchunks * 8;
  uint64_t off = 0;
  int d = 0;
  for (int bit = 63; bit >= 0; --bit) {
    uint64_t size = 1ull << bit;
    if (!(nchunks & size)) continue;
    const uint32_t* src = cvs + off * 8;
    uint32_t* dst = bufA;
    uint64_t cnt = size;
    while (cnt > 1) {
      for (uint64_t i = threadIdx.x; i < cnt / 2; i += blockDim.x) {
        uint32_t l[8], r[8], o[8];
        for (int k = 0; k < 8; ++k) l[k] = src[(2 * i) * 8 + k], r[k] = src[(2 * i + 1) * 8 + k];
        bk::parent(l, r, key.k, mode, o);
        for (int k = 0; k < 8; ++k) dst[i * 8 + k] = o[k];
      }
      __syncthreads();
      cnt /= 2;
      src = dst;
      dst = (dst == bufA) ? bufB : bufA;
    }
    if (threadIdx.x < 8) out[d * 8 + threadIdx.x] = src[threadIdx.x];
    __syncthreads();
    ++d;
    off += size;
  }
}

void launch_chunk_cvs(const uint8_t* stream, uint64_t nchunks, const uint32_t key[8], uint32_t mode, uint32_t* cvs,
                      cudaStream_t s) {
  KeyArg k;
  for (int i = 0; i < 8; ++i) k.k[i] = key[i];
  if (nchunks) k_chunk_cvs<<<(unsigned)((nchunks + 127) / 128), 128, 0, s>>>(stream, nchunks, k, mode, cvs);
}

void launch_subtrees(uint32_t* cvs, uint32_t* scratch, uint64_t nchunks, const uint32_t key[8], uint32_t mode,
                     uint32_t* out, cudaStream_t s) {
  KeyArg k;
  for (int i = 0; i < 8; ++i) k.k[i] = key[i];
  if (nchunks) k_subtrees<<<1, 1024, 0, s>>>(cvs, scratch, nchunks, k, mode, out);
}

}  // namespace lf
