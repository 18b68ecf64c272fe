// The opening on the GPU: row evaluation, folding challenges, the fold, and the BLAKE3 tree
// hashing of the transcript's large absorb.
#include <algorithm>
#include <cstdio>

#include "lf_blake3.cuh"
#include "lf_internal.h"
#include "lf_tc.cuh"
#include "lf_window.cuh"

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

// One block per run of `share` rows i, all columns (RW_COLS per thread): the window table of
// eq[i] serves the 1024 products of row i; each thread reads its columns' words in order of i.
// row (1024 F162) is zeroed by the caller and receives the blocks' shares by XOR.
constexpr int RW_COLS = COLUMNS / 256;
__global__ void __launch_bounds__(256) k_row_eval(const uint4* __restrict__ table, int rl, uint64_t share,
                                                  const f162* __restrict__ eqt, f162* __restrict__ row) {
  __shared__ WinTable T;
  const uint64_t n = 1ull << rl;
  const uint64_t i0 = blockIdx.x * share, i1 = min(n, i0 + share);
  f162 acc[RW_COLS];
#pragma unroll
  for (int k = 0; k < RW_COLS; ++k) acc[k] = {0, 0, 0};
  for (uint64_t i = i0; i < i1; ++i) {
    uint4 v[RW_COLS];
#pragma unroll
    for (int k = 0; k < RW_COLS; ++k) v[k] = table[((uint64_t)(threadIdx.x + 256 * k) << rl) + i];
    win_build(T, eqt[i], threadIdx.x, 256);
#pragma unroll
    for (int k = 0; k < RW_COLS; ++k) win_mul_add(T, v[k], acc[k]);
    __syncthreads();
  }
#pragma unroll
  for (int k = 0; k < RW_COLS; ++k) {
    unsigned long long* o = reinterpret_cast<unsigned long long*>(row + threadIdx.x + 256 * k);
    atomicXor(o, (unsigned long long)acc[k].w0);
    atomicXor(o + 1, (unsigned long long)acc[k].w1);
    atomicXor(o + 2, (unsigned long long)acc[k].w2);
  }
}

void launch_row_eval(const uint4* table, int rl, const f162* eqt, f162* row, int sms, cudaStream_t s) {
  // one wave: the runs of rows split over the blocks resident at once (three per SM)
  const uint64_t n = 1ull << rl;
  const uint64_t share = std::max<uint64_t>(1, (n + 3ull * sms - 1) / (3ull * sms));
  cudaMemsetAsync(row, 0, COLUMNS * sizeof(f162), s);
  k_row_eval<<<(unsigned)((n + share - 1) / share), 256, 0, s>>>(table, rl, share, eqt, row);
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

// Per draw i of an attempt (n = 162 - i candidates): the rejection limit (65536 / n) * n and the
// multiplier (2^32 / n) + 1 whose high product word is r / n for every r < 2^16, tabulated so that
// no draw divides.
struct DrawConsts {
  uint32_t limit[WEIGHT], magic[WEIGHT];
};
constexpr DrawConsts make_draw_consts() {
  DrawConsts d{};
  for (int i = 0; i < WEIGHT; ++i) {
    const uint32_t n = (uint32_t)(N162 - i);
    d.limit[i] = (65536u / n) * n;
    d.magic[i] = (uint32_t)((1ull << 32) / n + 1);
  }
  return d;
}
__constant__ DrawConsts kDraw = make_draw_consts();

struct __align__(16) ChWarp {
  uint8_t buf[XOF_BUF];
  uint8_t perm[176];
  uint32_t root[27];
};

// The XOF output as a ring of 32 blocks of 64 bytes: blocks [lo, lo + 32) of the stream sit in
// slots block % 32. xof_blocks(first, count): lanes < count produce blocks first + lane.
__device__ __forceinline__ void xof_blocks(ChWarp& s, const bk::Pending& root, uint64_t first, int count, int lane) {
  __syncwarp();  // every lane has read the slots before any lane overwrites them
  if (lane < count) {
    uint32_t w[16];
    root.root_block(first + lane, w);
    uint32_t* dst = reinterpret_cast<uint32_t*>(s.buf + 64 * ((first + lane) % 32));
#pragma unroll
    for (int i = 0; i < 16; ++i) dst[i] = w[i];
  }
  __syncwarp();
}

__global__ void __launch_bounds__(32 * CH_WARPS) k_challenges(const bk::Hasher* __restrict__ state, uint64_t base,
                                                              bk::Pending sign_key_node, const double* __restrict__ re,
                                                              const double* __restrict__ im, const float* __restrict__ re32,
                                                              const float* __restrict__ im32, double bound_sq,
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
  // The byte stream: the next byte is at A (even: every draw reads two), the ring holds blocks
  // [lo, lo + 32). An attempt starts with at least 160 bytes ahead (56 without rejected draws).
  uint64_t lo = 0, A = 0;
  xof_blocks(s, root, 0, 32, lane);
  const bool trace = dbg != nullptr && ci == 0;
  if (trace && lane == 0)
    for (int i = 0; i < 27; ++i) dbg[i] = s.root[i];
  auto advance = [&]() {  // the oldest 16 blocks (read) make room for the next 16
    xof_blocks(s, root, lo + 32, 16, lane);
    lo += 16;
  };
  for (uint64_t attempt = 0; attempt < MAX_ATTEMPTS; ++attempt) {
    if (A + 160 > (lo + 32) * 64) advance();
    for (int i = lane; i < N162; i += 32) s.perm[i] = (uint8_t)i;
    __syncwarp();
    // Lane 0 alone runs the partial Fisher-Yates (no warp barrier per draw): draw i reads a
    // little-endian u16, rejects it above the largest multiple of n = 162 - i, and swaps slot i
    // with slot i + r mod n.
    for (int i = 0;;) {
      if (lane == 0) {
        while (i < WEIGHT && A + 2 <= (lo + 32) * 64) {
          const uint32_t r = *reinterpret_cast<const uint16_t*>(s.buf + (A % XOF_BUF));
          A += 2;
          if (r >= kDraw.limit[i]) continue;
          const uint32_t nn = (uint32_t)(N162 - i);
          const uint32_t q = (uint32_t)(((uint64_t)r * kDraw.magic[i]) >> 32);
          const int j = i + (int)(r - q * nn);
          const uint8_t t = s.perm[i];
          s.perm[i] = s.perm[j];
          s.perm[j] = t;
          ++i;
        }
      }
      i = __shfl_sync(0xffffffffu, i, 0);
      A = ((uint64_t)__shfl_sync(0xffffffffu, (uint32_t)(A >> 32), 0) << 32) | __shfl_sync(0xffffffffu, (uint32_t)A, 0);
      if (i == WEIGHT) break;
      advance();  // (more than 52 rejected draws in one attempt)
    }
    __syncwarp();
    // Sorted positions: lane l < 28 places perm[l] by its rank.
    uint32_t mine = lane < WEIGHT ? s.perm[lane] : 255;
    int rank = 0;
    for (int t = 0; t < WEIGHT; ++t) rank += (int)(s.perm[t] < mine);
    __syncwarp();
    __shared__ __align__(4) uint8_t sorted[CH_WARPS][32];
    static_assert(WEIGHT % 4 == 0, "positions fill whole message words");
    if (lane < WEIGHT) sorted[wid][rank] = (uint8_t)mine;
    __syncwarp();
    // Signs: derive-key hash of (weight as u64 LE || positions), first four bytes LE.
    uint32_t signs = 0;
    if (lane == 0) {
      // the block (weight as u64 LE || the 28 positions) as message words, straight from the
      // sorted positions (4 per word, little-endian) without a byte array in local memory
      uint32_t m[16], o[16];
      const uint32_t* sp = reinterpret_cast<const uint32_t*>(sorted[wid]);
      m[0] = (uint32_t)WEIGHT, m[1] = 0;
#pragma unroll
      for (int q = 0; q < WEIGHT / 4; ++q) m[2 + q] = sp[q];
#pragma unroll
      for (int q = 2 + WEIGHT / 4; q < 16; ++q) m[q] = 0;
      bk::compress16(sign_key_node.h, m, 0, 8 + WEIGHT, sign_key_node.flags | bk::F_ROOT, o);
      signs = o[0] & ((1u << WEIGHT) - 1);
    }
    signs = __shfl_sync(0xffffffffu, signs, 0);
    if (trace && attempt == 0 && lane == 0) {
      for (int i = 0; i < 32; ++i) reinterpret_cast<uint8_t*>(dbg + 27)[i] = s.buf[i];
      for (int i = 0; i < 28; ++i) reinterpret_cast<uint8_t*>(dbg + 35)[i] = sorted[wid][i];
      dbg[42] = signs;
    }
    // The norm test first in f32: 28 terms of magnitude <= 1 put the f32 |c|^2 within 0.01 of the
    // f64 value (the table's f32 rounding and 28 additions each contribute < 2^-24 per term, and
    // |c| < 29), so outside [bound - 0.05, bound + 0.05] the f32 decision is the f64 decision.
    // Inside that window (rare) the lane repeats the reference's f64 sequence exactly.
    const float bound_f = (float)bound_sq;
    bool over = false;
    // The attempt's 28 table rows, then all 56 loads of a lane's phase at once (one load latency
    // per phase lane instead of 28 dependent ones: the loop ran 26 us per attempt rolled).
    int rowoff[WEIGHT];
#pragma unroll
    for (int t = 0; t < WEIGHT; ++t) rowoff[t] = sorted[wid][t] * PHASE_LANES;
    for (int k = lane; k < 81; k += 32) {
      float pr[WEIGHT], pi[WEIGHT];
#pragma unroll
      for (int t = 0; t < WEIGHT; ++t) pr[t] = __ldg(re32 + rowoff[t] + k), pi[t] = __ldg(im32 + rowoff[t] + k);
      float fr = 0.0f, fi = 0.0f;
#pragma unroll
      for (int t = 0; t < WEIGHT; ++t) {
        const bool neg = (signs >> t) & 1;
        fr += neg ? -pr[t] : pr[t];
        fi += neg ? -pi[t] : pi[t];
      }
      const float m2f = fr * fr + fi * fi;
      const bool traced = trace && attempt == 0 && k == 0;  // the diagnostic records the f64 values
      if (!traced && m2f > bound_f + 0.05f) {
        over = true;
        continue;
      }
      if (!traced && m2f < bound_f - 0.05f) continue;
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

cudaError_t launch_challenges(const void* hasher_dev, uint64_t base_counter, const uint32_t sign_key[8],
                              const void* phase, Challenge* out, int n, int* status, cudaStream_t s, uint32_t* dbg) {
  const size_t np = 162 * PHASE_LANES;
  const double* phase_re = static_cast<const double*>(phase);
  const double* phase_im = phase_re + np;
  const float* re32 = reinterpret_cast<const float*>(phase_im + np);
  const float* im32 = re32 + np;
  bk::Pending sk;
  for (int i = 0; i < 8; ++i) sk.h[i] = sign_key[i];
  for (int i = 0; i < 16; ++i) sk.m[i] = 0;
  sk.t = 0;
  sk.len = 0;
  sk.flags = bk::F_DERIVE_MAT | bk::F_CHUNK_START | bk::F_CHUNK_END;
  double bound_sq = 12.0 * 12.0 + 1e-12;
  // cudaLaunchKernel reports this launch's own outcome (a triple-chevron launch leaves it in the
  // thread's last-error state, where an earlier error of the caller's may also wait).
  const bk::Hasher* h = reinterpret_cast<const bk::Hasher*>(hasher_dev);
  void* args[] = {&h, &base_counter, &sk, &phase_re, &phase_im, &re32, &im32, &bound_sq, &out, &n, &status, &dbg};
  return cudaLaunchKernel(reinterpret_cast<const void*>(k_challenges), dim3((n + CH_WARPS - 1) / CH_WARPS),
                          dim3(32 * CH_WARPS), args, 0, s);
}

// ---------------------------------------------------------------------------------------------
// Fold (reference.rs:72-133): v_m = sum_j c_j W_{j,m} over the integers. A challenge sits in R_648
// as c(-X^4), so with Y = X^4 each table word k of element m is folded on its own:
//   V_{m,k}(Y) = sum_j sum_t s_{j,t} Y^{pos_{j,t}} W_{j,m,k}(Y),  s = sign bit XOR (pos odd),
// raw positions y = x + pos in [0, 289), then Y^162 = Y^81 - 1 (so Y^y = Y^(y-81) - Y^(y-162)
// for 162 <= y < 243 and Y^y = -Y^(y-243) above).
//
// On the tensor cores this is one product per block of 128 table words (rows) and run of columns,
// with the reduction already in the second operand. Output coefficient i receives the raw
// positions y = i (+), y = i + 81 (+, when 81 <= i), y = i + 162 (-, when i < 81) and y = i + 243
// (-, when i < 46), and a raw position is x + pos, so with d = i - x and C_j the signed challenge
// (+-1 at its 28 positions, 0 outside [0, 162)):
//   i <  81:  coefficient += bit_x * (C_j[d] - C_j[d + 162] - C_j[d + 243])   (for 46 <= i < 81
//             the last index is at least 162, so one formula serves the whole range)
//   i >= 81:  coefficient += bit_x * (C_j[d] + C_j[d + 81])
// Each range is a function of d alone. With n = 80 - i (low range) or n = 161 - i (high range),
// B[x][n] = f(const - n - x) depends on x + n only. The operands are 8-bit floats (e4m3, the
// tensor cores' kind::f8f6f4 at twice the bf16 rate): every B value is a sum of up to three
// +-0.5 (0, +-0.5, +-1, +-1.5 are exact in e4m3) and every A value 2.0 or 0, so each product is an
// exact integer and D sums them exactly in f32. A K-major core matrix of B is 8 rows (n) x 16
// bytes (x): core (n group g, k group h) holds f(const - (8 g + 16 h + r + c)), a function of
// e = g + 2 h, so one strip of 26 cores per range and column (k_fold_cores) serves every MMA through
// a descriptor whose 8-row-group stride is one core and whose K stride is two. A = the words
// expanded to e4m3 (bits in natural order) in tensor memory. D = 128 x 192 (two MMAs of N = 96 per
// K = 32, 81 columns used in each), exact in f32 (integers well inside 2^24).
// ---------------------------------------------------------------------------------------------
constexpr int FT_RCORES = 26;                   // cores per range strip: e = g + 2 h <= 11 + 2 * 7
constexpr int FT_STRIP = 2 * FT_RCORES * 128;   // both ranges' strips of a column: 6656 bytes
constexpr int FT_N = 96;                        // MMA N per range (81 coefficients used)
constexpr int FT_WORDS = 128 * 16;              // a column's 128 table words of the block: 2048 bytes
constexpr int FT_SLOT = FT_STRIP + FT_WORDS;    // one column's bulk copies
constexpr int FT_STAGES = 4;                    // A stages in tensor memory, 32 columns each
constexpr int FT_RING = 12;                     // column slots: the loader runs up to 12 columns ahead
constexpr int FT_PRODUCERS = 512;               // four groups of 128 (a word each): warps 5-20
constexpr int FT_ISSUERS = 4;                   // lane 0 of warps 0-3 issue the MMAs
constexpr int FT_THREADS = FT_PRODUCERS + 288;  // + the issuers' warps, the loader's (lane 0 of warp 4), read-out
// More than half of an SM's shared memory, so one block holds the SM's 512 tensor-memory columns.
constexpr int FT_SMEM = 120 * 1024;
static_assert(FT_RING * FT_SLOT + (FT_STAGES + 2 * FT_RING + 4) * 8 + 16 <= FT_SMEM, "fold shared memory");
constexpr long long FT_WAIT_CYCLES = 2000000000LL;

// e4m3 code of a sum of up to three +-0.5: 0, +-0.5 (0x30), +-1 (0x38) or +-1.5 (0x3C).
__device__ __forceinline__ uint32_t e4m3_halves(float f) {
  const float a = fabsf(f);
  const uint32_t m = a == 0.5f ? 0x30u : a == 1.0f ? 0x38u : a == 1.5f ? 0x3Cu : 0u;
  return m | (f < 0.0f && m ? 0x80u : 0u);
}

// Strips of column j, low range then high range: byte (r, c) of core e of a range (row r, byte c)
// holds f(const - (8 e + r + c)) in e4m3, with f and const of the range (80 and the three-term
// difference below i = 81, 161 and the two-term sum above) and the challenge's values +-0.5.
__global__ void __launch_bounds__(128) k_fold_cores(const Challenge* __restrict__ ch, uint8_t* __restrict__ strips) {
  __shared__ float dense[N162];
  const int j = blockIdx.x, tid = threadIdx.x;
  for (int i = tid; i < N162; i += 128) dense[i] = 0.0f;
  __syncthreads();
  if (tid < WEIGHT) {
    const int pos = ch[j].positions[tid];
    const bool neg = (((ch[j].signs >> tid) & 1) ^ (pos & 1)) != 0;
    dense[pos] = neg ? -0.5f : 0.5f;
  }
  __syncthreads();
  auto C = [&](int z) { return (z >= 0 && z < N162) ? dense[z] : 0.0f; };
  uint32_t* out = reinterpret_cast<uint32_t*>(strips + (size_t)j * FT_STRIP);
  for (int u = tid; u < FT_STRIP / 4; u += 128) {  // four elements per u32
    const int high = u >= FT_RCORES * 32, uu = high ? u - FT_RCORES * 32 : u;
    const int e = uu >> 5, r = (uu >> 2) & 7, c0 = 4 * (uu & 3);
    uint32_t w = 0;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int d = (high ? 161 : 80) - (8 * e + r + c0 + t);
      const float f = high ? C(d) + C(d + 81) : C(d) - C(d + 162) - C(d + 243);
      w |= e4m3_halves(f) << (8 * t);
    }
    out[u] = w;
  }
}

// A table word -> its 32 tensor-memory A columns: column o holds K positions 4 o .. 4 o + 3 (bits
// 4 o .. 4 o + 3 of the word, natural order, the Hankel operand's order), byte i = e4m3 2.0 (0x40)
// when bit 4 o + i is set. The nibble times 0x08102040 puts its bits at 6, 14, 22 and 30 (the four
// shifted copies do not overlap, so nothing carries).
__device__ __forceinline__ void fold_expand_word(uint4 v, uint32_t (&u)[32]) {
  const uint32_t xs[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int t = 0; t < 8; ++t) u[8 * q + t] = (((xs[q] >> (4 * t)) & 0xFu) * 0x08102040u) & 0x40404040u;
}

// Work unit = 128 table words (32 ring elements) x a run of columns; out: part[split][m][4 y + k]
// for the unit's elements, the column run's share of the fold. Persistent: one CTA per SM takes the
// units u = blockIdx.x + i gridDim.x (row block u % nbx, column run u / nbx) and runs their columns
// as one stream T through the ring and the stages, with D double-buffered in tensor memory, so the
// read-out of a unit overlaps the next unit's copies and MMAs.
//
// Tensor memory (512 columns): D buffers b = 0, 1 at 192 b (two ranges of N = 96 each), A stages
// s = 0..3 at 384 + 32 s (a column's 128 words, K = 128 bits as e4m3, read by the MMAs from tensor
// memory, so the shared-memory port carries only the strips). Roles, meeting on mbarriers:
//   lane 0 of warp 4 (loader): per column T, once the MMAs of the column that used its ring slot
//     FT_RING columns earlier are done (done[slot]), two bulk copies into slot T % FT_RING (the
//     column's strips, 6656 bytes, and the unit's 128 words, 2048 bytes) completing on wfull[slot];
//   warps 5-20 (producers; warp w holds tensor-memory lanes 32 (w % 4) .. +31 = words, and group
//     g = (w - 5) / 4 takes the columns T = g mod 4, so stage g): per column wait until the stage is
//     free (done of the group's previous column) and the words landed, expand the words with
//     tcgen05.st, arrive full[g]. Four groups keep four columns' expansions in flight;
//   lane 0 of warp i < 4 (issuer of range i % 2, K half i / 2): before a unit's first column wait
//     until its D buffer was read out and cleared (dfree), then per column wait full[s], issue its
//     2 MMAs (A from tensor memory, B = the range's strip through the Hankel descriptor) and commit
//     to done[slot]; after the unit's last column commit to dfull. One thread issues a tcgen05
//     operation only about every 100 cycles, so the column's 8 MMAs come from four threads;
//   warps 21-24 (read-out; lane quarter w % 4 = the unit's rows): per unit wait dfull, read D and
//     store each row's 162 coefficients, clear D (tcgen05.st) and arrive dfree.
// Every wait is bounded; a timeout sets *status = 5 and the abort flag, on which every role leaves
// its loop. The loader waits for its own copies in flight before the block ends, and tensor memory
// is freed only after the issuers' last commits drained.
constexpr int FT_EPI_WARP = 5 + FT_PRODUCERS / 32;  // warps 21-24 read D out
static_assert(FT_THREADS == 32 * FT_EPI_WARP + 128, "fold roles");

struct FoldUnits {  // the CTA's units and their column runs
  int nbx, cols_per_split;
  uint64_t ring_elements;
  __device__ int unit(int i) const { return blockIdx.x + i * gridDim.x; }
  __device__ int c_begin(int u) const { return (u / nbx) * cols_per_split; }
  __device__ int ncols(int u) const { return max(0, min(COLUMNS, c_begin(u) + cols_per_split) - c_begin(u)); }
  __device__ uint64_t w0(int u) const { return (uint64_t)(u % nbx) * 128; }
  __device__ int nw(int u) const { return (int)min((uint64_t)128, 4 * ring_elements - w0(u)); }
};

__global__ void __launch_bounds__(FT_THREADS, 1)
    k_fold_tc(const uint4* __restrict__ table, int rl, uint64_t ring_elements, const uint8_t* __restrict__ strips,
              int cols_per_split, int nunits, int32_t* __restrict__ part, int* status) {
  extern __shared__ __align__(1024) uint8_t fsm[];
  uint8_t* ring = fsm;                                                  // [FT_RING][FT_SLOT]: strips, words
  uint64_t* done = reinterpret_cast<uint64_t*>(fsm + FT_RING * FT_SLOT);  // [FT_RING] a slot's column's MMAs done
  uint64_t* full = done + FT_RING;                                      // [FT_STAGES] a stage written
  uint64_t* wfull = full + FT_STAGES;                                   // [FT_RING] a slot's copies landed
  uint64_t* dfull = wfull + FT_RING;                                    // [2] a D buffer's unit complete
  uint64_t* dfree = dfull + 2;                                          // [2] a D buffer read out and cleared
  uint32_t* tslot = reinterpret_cast<uint32_t*>(dfree + 2);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const FoldUnits U{(int)((4 * ring_elements + 127) / 128), cols_per_split, ring_elements};
  const int nu = blockIdx.x < nunits ? (nunits - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  if (tid == 0) {
    *abort_flag = 0;
    for (int i = 0; i < FT_RING; ++i) {
      tc::mbar_init(&done[i], FT_ISSUERS);
      tc::mbar_init(&wfull[i], 1);
    }
    for (int i = 0; i < FT_STAGES; ++i) tc::mbar_init(&full[i], FT_PRODUCERS / FT_STAGES);
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&dfull[i], FT_ISSUERS);
      tc::mbar_init(&dfree[i], 128);
    }
    tc::mbar_init_fence();
  }
  if (warp == 0) tc::tmem_alloc(tslot, 512);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *tslot;
  uint32_t zero16[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) zero16[i] = 0;
  if (warp >= FT_EPI_WARP) {  // both D buffers = 0: every MMA accumulates, in any order of the issuers
    for (int n0 = 0; n0 < 4 * FT_N; n0 += 16)
      tc::tmem_st_x16(tbase + ((uint32_t)(32 * (warp & 3)) << 16) + n0, zero16);
    tc::tmem_wait_st();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t id96 = tc::idesc_e4m3_f32(128, FT_N);  // both K-major
  auto give_up = [&]() {
    if (!*abort_flag) {
      *abort_flag = 1;
      atomicExch(status, 5);
    }
  };

  if (warp >= 5 && warp < FT_EPI_WARP) {  // producers
    const int group = (warp - 5) >> 2, s = group, row = 32 * (warp & 3) + lane;
    const uint32_t tA = tbase + ((uint32_t)(32 * (warp & 3)) << 16) + 384 + 32 * s;
    int i = 0, it = group, T = group;  // unit, column within it, column of the stream
    while (i < nu && it >= U.ncols(U.unit(i))) it -= U.ncols(U.unit(i)), ++i;
    for (; i < nu; T += FT_STAGES) {
      const int u = U.unit(i), slot = T % FT_RING;
      bool ok = T < FT_STAGES || tc::mbar_wait_fast(&done[(T - FT_STAGES) % FT_RING],
                                                    ((T - FT_STAGES) / FT_RING) & 1, abort_flag, FT_WAIT_CYCLES);
      ok = ok && tc::mbar_wait_fast(&wfull[slot], (T / FT_RING) & 1, abort_flag, FT_WAIT_CYCLES);
      if (!__all_sync(0xffffffffu, ok)) give_up();
      if (!*abort_flag) {
        tc::fence_after_sync();
        const uint4 v = row < U.nw(u) ? reinterpret_cast<const uint4*>(ring + slot * FT_SLOT + FT_STRIP)[row]
                                      : make_uint4(0, 0, 0, 0);
        uint32_t w[32];
        fold_expand_word(v, w);
        tc::tmem_st_x16(tA, *reinterpret_cast<const uint32_t(*)[16]>(w));
        tc::tmem_st_x16(tA + 16, *reinterpret_cast<const uint32_t(*)[16]>(w + 16));
        tc::tmem_wait_st();
      }
      tc::fence_before_sync();
      tc::mbar_arrive(&full[s]);
      for (it += FT_STAGES; i < nu && it >= U.ncols(U.unit(i));) it -= U.ncols(U.unit(i)), ++i;
    }
  } else if (tid == 128) {  // loader
    int issued = 0;
    for (int i = 0; i < nu && !*abort_flag; ++i) {
      const int u = U.unit(i), nc = U.ncols(u), nw = U.nw(u), cb = U.c_begin(u);
      const uint64_t w0 = U.w0(u);
      for (int it = 0; it < nc && !*abort_flag; ++it, ++issued) {
        const int T = issued, slot = T % FT_RING;
        if (T >= FT_RING && !tc::mbar_wait(&done[slot], ((T / FT_RING) - 1) & 1, abort_flag, FT_WAIT_CYCLES)) {
          give_up();
          break;
        }
        uint8_t* dst = ring + slot * FT_SLOT;
        tc::mbar_expect_tx(&wfull[slot], FT_STRIP + 16 * nw);
        tc::bulk_load(dst, strips + (size_t)(cb + it) * FT_STRIP, FT_STRIP, &wfull[slot]);
        tc::bulk_load(dst + FT_STRIP, table + ((uint64_t)(cb + it) << rl) + w0, 16 * nw, &wfull[slot]);
      }
    }
    // the copies in flight land before the block leaves
    for (int T = issued > FT_RING ? issued - FT_RING : 0; T < issued; ++T) {
      const long long t0 = clock64();
      while (!tc::mbar_try_wait(&wfull[T % FT_RING], (T / FT_RING) & 1) && clock64() - t0 < FT_WAIT_CYCLES) {
      }
    }
  } else if (warp < FT_ISSUERS && lane == 0) {  // issuer: range warp % 2, MMAs kk = 2 (warp / 2) + 0, 1
    const int range = warp & 1, kh = warp >> 1;
    const uint32_t boff = FT_RCORES * 128 * range;
    int T = 0, last = -1;
    for (int i = 0; i < nu && !*abort_flag; ++i) {
      const int buf = i & 1, nc = U.ncols(U.unit(i));
      const uint32_t d = tbase + 2 * FT_N * buf + FT_N * range;
      if (i >= 2 && !tc::mbar_wait(&dfree[buf], ((i >> 1) - 1) & 1, abort_flag, FT_WAIT_CYCLES)) give_up();
      for (int it = 0; it < nc; ++it, ++T) {
        const int s = T % FT_STAGES, slot = T % FT_RING;
        if (!tc::mbar_wait_fast(&full[s], (T / FT_STAGES) & 1, abort_flag, FT_WAIT_CYCLES) ||
            !tc::mbar_wait_fast(&wfull[slot], (T / FT_RING) & 1, abort_flag, FT_WAIT_CYCLES))
          give_up();
        if (*abort_flag) break;
        tc::fence_after_sync();
        const uint32_t a0 = tbase + 384 + 32 * s, b0 = tc::smem_u32(ring + slot * FT_SLOT) + boff;
#pragma unroll
        for (int k2 = 0; k2 < 2; ++k2) {  // K = 32 kk: k groups 2 kk, 2 kk + 1, so core e starts at 4 kk
          const int kk = 2 * kh + k2;
          tc::mma_e4m3_ta(d, a0 + 8 * kk, tc::sdesc(b0 + 4 * kk * 128, 256, 128), id96, 1u);
        }
        tc::mma_commit(&done[slot]);
        last = T;
      }
      if (!*abort_flag) tc::mma_commit(&dfull[buf]);
    }
    if (last >= 0) {  // drain: the last commits cover every MMA
      const long long t0 = clock64();
      while (!tc::mbar_try_wait(&done[last % FT_RING], (last / FT_RING) & 1) && clock64() - t0 < FT_WAIT_CYCLES) {
      }
    }
  } else if (warp >= FT_EPI_WARP) {  // read-out: row r = 4 m + k of the unit = TMEM lane r
    const int qd = warp & 3, r = 32 * qd + lane;
    for (int i = 0; i < nu; ++i) {
      const int u = U.unit(i), buf = i & 1;
      if (!__all_sync(0xffffffffu, tc::mbar_wait(&dfull[buf], (i >> 1) & 1, abort_flag, FT_WAIT_CYCLES))) {
        give_up();
        break;
      }
      tc::fence_after_sync();
      const uint64_t m0 = U.w0(u) / 4;
      const int nel = (int)min((uint64_t)32, ring_elements - m0), m = r >> 2, k = r & 3;
      // part[split][(m0 + m) * 648 + 4 i + k]: four rows of an element fill 16 consecutive bytes
      int32_t* dst = part + ((uint64_t)(u / U.nbx) * ring_elements + m0 + m) * 648 + k;
      const uint32_t tb = tbase + ((uint32_t)(32 * qd) << 16) + 2 * FT_N * buf;
#pragma unroll 1
      for (int n0 = 0; n0 < 2 * FT_N; n0 += 16) {
        uint32_t v[16];
        tc::tmem_ld_x16(tb + n0, v);
        tc::tmem_wait_ld(v);
#pragma unroll
        for (int t = 0; t < 16; ++t) {
          const int n = n0 + t, high = n >= FT_N, nn = high ? n - FT_N : n;
          if (nn < 81 && m < nel) dst[4 * (high ? 161 - nn : 80 - nn)] = (int32_t)__float2int_rn(__uint_as_float(v[t]));
        }
        tc::tmem_st_x16(tb + n0, zero16);  // cleared for the unit after next
      }
      tc::tmem_wait_st();
      tc::fence_before_sync();
      tc::mbar_arrive(&dfree[buf]);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tbase, 512);
}

// out = sum over the column runs; every coefficient must fit the wire's i16 range (status 2).
__global__ void k_fold_sum(const int32_t* __restrict__ part, int splits, uint64_t n, int32_t* __restrict__ out,
                           int* status) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    int32_t v = 0;
    for (int s = 0; s < splits; ++s) v += part[(uint64_t)s * n + i];
    out[i] = v;
    if (v < -32768 || v > 32767) atomicExch(status, 2);
  }
}

// Column runs of the fold: blocks = ceil(words / 128) x splits should fill whole waves of the SMs.
int fold_splits(uint64_t ring_elements, int sms) {
  const uint64_t blocks = (4 * ring_elements + 127) / 128;
  int best = 1;
  double best_eff = -1;
  for (int s = 1; s <= 32; ++s) {
    const uint64_t total = blocks * s, waves = (total + sms - 1) / sms;
    const double eff = (double)total / (double)(waves * sms) - 0.004 * s;  // small cost per extra run
    if (eff > best_eff) best_eff = eff, best = s;
  }
  return best;
}

void launch_fold(const uint4* table, int rl, uint64_t ring_elements, const Challenge* ch, uint8_t* strips,
                 int32_t* part, int splits, int32_t* out, int* status, cudaStream_t s) {
  static std::atomic<unsigned long long> attr{0};
  smem_limit(k_fold_tc, FT_SMEM, attr);
  k_fold_cores<<<COLUMNS, 128, 0, s>>>(ch, strips);
  static int sms = 0;  // one CTA per SM (the kernel walks its units)
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  const int units = (int)((4 * ring_elements + 127) / 128) * splits;
  const int per = (COLUMNS + splits - 1) / splits;
  k_fold_tc<<<(unsigned)std::min(units, sms), FT_THREADS, FT_SMEM, s>>>(table, rl, ring_elements, strips, per, units,
                                                                        part, status);
  k_fold_sum<<<1024, 256, 0, s>>>(part, splits, ring_elements * 648, out, status);
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

// The chaining values of the complete subtrees of the stream's finished chunks (sizes = the set
// bits of nchunks, largest first). All subtrees are reduced together, one tree level per pass:
// level L halves every subtree still larger than 2^L, so the block runs max(log2 size) dependent
// parent compressions instead of their sum. Subtree s keeps its chunk offset in the ping-pong
// buffers A and B (level 0 reads the chunk values themselves).
__global__ void __launch_bounds__(1024) k_subtrees(const uint32_t* __restrict__ cvs, uint32_t* scratch, uint64_t nchunks,
                                                   KeyArg key, uint32_t mode, uint32_t* __restrict__ out) {
  uint32_t* buf[2] = {scratch, scratch + nchunks * 8};
  int nsub = 0, top = 0;
  uint64_t offs[64];
  int bits[64];
  {
    uint64_t off = 0;
    for (int bit = 63; bit >= 0; --bit)
      if (nchunks >> bit & 1) {
        offs[nsub] = off, bits[nsub] = bit, ++nsub;
        off += 1ull << bit;
        top = max(top, bit);
      }
  }
  for (int L = 0; L < top; ++L) {
    const uint32_t* src = L == 0 ? cvs : buf[(L - 1) & 1];
    uint32_t* dst = buf[L & 1];
    uint64_t total = 0;  // the level's pairs of all subtrees, spread over the block as one range
    for (int sidx = 0; sidx < nsub; ++sidx)
      if (bits[sidx] > L) total += 1ull << (bits[sidx] - L - 1);
    for (uint64_t g = threadIdx.x; g < total; g += blockDim.x) {
      uint64_t i = g;
      int sidx = 0;
      for (; sidx < nsub; ++sidx) {
        if (bits[sidx] <= L) continue;
        const uint64_t pairs = 1ull << (bits[sidx] - L - 1);
        if (i < pairs) break;
        i -= pairs;
      }
      const uint32_t* a = src + (offs[sidx] + 2 * i) * 8;
      uint32_t l[8], r[8], o[8];
      for (int k = 0; k < 8; ++k) l[k] = a[k], r[k] = a[8 + k];
      bk::parent(l, r, key.k, mode, o);
      for (int k = 0; k < 8; ++k) dst[(offs[sidx] + i) * 8 + k] = o[k];
    }
    __syncthreads();
  }
  // subtree s's value: its single chunk value (size 1) or the last level that halved it
  for (int sidx = 0; sidx < nsub; ++sidx) {
    const uint32_t* src = bits[sidx] == 0 ? cvs : buf[(bits[sidx] - 1) & 1];
    if (threadIdx.x < 8) out[sidx * 8 + threadIdx.x] = src[offs[sidx] * 8 + threadIdx.x];
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
