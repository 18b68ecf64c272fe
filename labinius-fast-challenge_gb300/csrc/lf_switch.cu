// The GHASH -> F162 field switch on the GPU: eq tables, the 128 partial evaluations, and the
// sumcheck rounds (solution-arm/labinius/crates/pcs/src/fields/crossfield.rs:66-170, 548-701;
// fields/sumcheck.rs:128-251).
//
// Partials. v[k] = sum_j bit_k(pi0[j]) eq[j] with eq[j] = E_hi[j >> 12] * E_lo[j & 4095]
// (eq over the leading and the trailing 12 coordinates of r_hi; r_hi[0] is the most significant
// index bit, crossfield.rs:126-137). Writing T_h[b'] = sum_jl bit_b'(E_lo[jl]) pi0[h, jl] (a
// GF(2) product of bit planes, no field multiplication) gives
// v[k] = sum_h E_hi[h] * S_h[k] with S_h[k] = sum_jl bit_k(pi0[h, jl]) E_lo[jl] = column k of T_h.
// So the table pass is a 128 x 4096 by 4096 x 128 bit-matrix product per block of 4096 words,
// done with AND/XOR on 32-bit planes and a final parity, and only 128 * 2^(LP-12) GHASH products
// remain.
#include <algorithm>
#include <cstdio>

#include "lf_internal.h"
#include "lf_tc.cuh"
#include "lf_window.cuh"

namespace lf {

// ---------------------------------------------------------------------------------------------
// eq tables
// ---------------------------------------------------------------------------------------------
// eq_expand_b128 (crossfield.rs:81-137): r[0] is the most significant bit of the index.
__global__ void k_eq_b128(const b128* __restrict__ r, int n, b128* __restrict__ out) {
  uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (j >= (1ull << n)) return;
  b128 v = {1, 0};
  for (int i = 0; i < n; ++i) {
    b128 f = r[i];
    if (!((j >> (n - 1 - i)) & 1)) f.lo ^= 1;
    v = b128_mul(v, f);
  }
  out[j] = v;
}

// eq_table (eval.rs:50-85): variable k is bit k of the index.
__global__ void k_eq_table_f162(const f162* __restrict__ ps, int n, f162* __restrict__ out) {
  uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (j >= (1ull << n)) return;
  f162 v = {1, 0, 0};
  for (int k = 0; k < n; ++k) {
    f162 f = ps[k];
    if (!((j >> k) & 1)) f.w0 ^= 1;
    v = f162_mul(v, f);
  }
  out[j] = v;
}

// ---------------------------------------------------------------------------------------------
// S blocks on the tensor cores: sblk[h][c] (16 bytes, bit b) = parity of
//   count_h[c][b] = sum_{j < 4096} bit_c(pi0[4096 h + j]) bit_b(E_lo[j]),
// an exact integer in f32. Operands are 8-bit floats (e4m3, kind::f8f6f4): every word is expanded
// to a row of 128 bytes, byte i = 2.0 (0x40) when bit i is set, read MN-major (row = entry j = K).
// A = E_lo's rows (M = b), B = the rows of a pair of blocks h side by side (N = 256: 128 h + c), so
// one MMA of K = 32 covers both blocks and D = 128 lanes (b) x 256 columns, 4 x count (<= 16384,
// exact); the count's parity is bit 2 of the f32 mantissa after adding 2^23.
//
// Persistent: one CTA per SM walks the pairs p = blockIdx.x + q gridDim.x, each pair 32 k-tiles of
// 128 entries, as one continuous stream of k-tiles T = 32 q + t through four shared-memory stages,
// with D double-buffered in tensor memory (pair q in columns 256 (q % 2) ..), so the next pair's
// copies, expansion and MMAs overlap the previous pair's read-out. Roles, on mbarriers:
//   lane 0 of warp 1 (loader): per k-tile three bulk copies of 2048 bytes (E_lo's entries and the
//     pair's entries 128 t .. +127) into ring slot T % SBT_RING, completing on wfull[slot], once the
//     producers have read the slot's previous k-tile (cfree);
//   warps 2-25 (producers, two groups of 384 threads, one row each: E_lo, block 0, block 1; group g
//     takes the k-tiles T = g mod 2): wait until stage T % 4 is free (done, the MMAs of k-tile T - 4)
//     and the words landed, read their word, expand it, fence, arrive cfree and full;
//   lane 0 of warp 0 (issuer): per k-tile wait full, issue 4 MMAs, commit to done; before a pair's
//     first k-tile wait until its D buffer was read out (dfree), after its last commit to dfull;
//   warps 26-29 (epilogue; lane quarter w % 4): per pair wait dfull, read D (bits b of the quarter,
//     256 columns), assemble each c's parity word from one ballot per 32 b, arrive dfree.
// Every wait is bounded; a timeout sets *status = 4 and the abort flag, on which every role leaves
// its loop; tensor memory is freed after the issuer's last commit drained.
// ---------------------------------------------------------------------------------------------
constexpr int SBT_GROUPS = 2;
constexpr int SBT_ROWS = 3 * 128;                             // a k-tile's rows: E_lo, block 0, block 1
constexpr int SBT_PRODUCERS = SBT_GROUPS * SBT_ROWS;          // warps 2-25
constexpr int SBT_EPI_WARP = 2 + SBT_PRODUCERS / 32;          // warps 26-29 read D out
constexpr int SBT_THREADS = SBT_PRODUCERS + 64 + 128;
constexpr int SBT_OPA = 128 * 128;                            // E_lo rows: 128 entries x 128 bytes
constexpr int SBT_STAGE = 3 * SBT_OPA;                        // [A][B: 128 entries x 256 bytes]
constexpr int SBT_STAGES = 4;
constexpr int SBT_RING = 4;
constexpr int SBT_SLOT = 3 * 2048;                            // a k-tile's words: E_lo, block 0, block 1
constexpr int SBT_BARS = SBT_STAGES * SBT_STAGE + SBT_RING * SBT_SLOT;
constexpr int SBT_SMEM = SBT_BARS + (2 * SBT_STAGES + 2 * SBT_RING + 4) * 8 + 16;
constexpr long long SBT_WAIT_CYCLES = 2000000000LL;

// A 128-bit word -> row r of an MN-major e4m3 tile (8-row x 16-byte core matrices, cores adjacent
// along the row 128 bytes apart, 8-row groups `kstride` apart): byte i = 0x40 when bit i is set.
__device__ __forceinline__ void sblock_write_row(uint8_t* tile, int r, int kstride, uint4 v) {
  const uint32_t xs[4] = {v.x, v.y, v.z, v.w};
  uint8_t* dst = tile + (r >> 3) * kstride + (r & 7) * 16;
#pragma unroll
  for (int q = 0; q < 8; ++q) {  // bits 16 q .. 16 q + 15 -> core q
    const uint32_t x = xs[q >> 1] >> (16 * (q & 1));
    uint32_t u[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) u[t] = (((x >> (4 * t)) & 0xFu) * 0x08102040u) & 0x40404040u;
    *reinterpret_cast<uint4*>(dst + q * 128) = make_uint4(u[0], u[1], u[2], u[3]);
  }
}

__global__ void __launch_bounds__(SBT_THREADS, 1)
    k_sblock_tc(const uint4* __restrict__ table, uint64_t nblocks, const uint4* __restrict__ elo,
                uint8_t* __restrict__ sblk, int* status) {
  extern __shared__ __align__(1024) uint8_t sbs[];
  uint8_t* ring = sbs + SBT_STAGES * SBT_STAGE;                       // [SBT_RING][SBT_SLOT]
  uint64_t* done = reinterpret_cast<uint64_t*>(sbs + SBT_BARS);      // [SBT_STAGES] MMAs of a stage done
  uint64_t* full = done + SBT_STAGES;                                 // [SBT_STAGES] a stage written
  uint64_t* wfull = full + SBT_STAGES;                                // [SBT_RING] a slot's copies landed
  uint64_t* cfree = wfull + SBT_RING;                                 // [SBT_RING] a slot's words read
  uint64_t* dfull = cfree + SBT_RING;                                 // [2] a D buffer's pair complete
  uint64_t* dfree = dfull + 2;                                        // [2] a D buffer read out
  uint32_t* tslot = reinterpret_cast<uint32_t*>(dfree + 2);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint64_t npairs = (nblocks + 1) / 2;
  const int nq = blockIdx.x < npairs ? (int)((npairs - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  const int ntiles = 32 * nq;
  auto pair_h0 = [&](int q) { return 2 * ((uint64_t)blockIdx.x + (uint64_t)q * gridDim.x); };
  if (tid == 0) {
    *abort_flag = 0;
    for (int i = 0; i < SBT_STAGES; ++i) {
      tc::mbar_init(&done[i], 1);
      tc::mbar_init(&full[i], SBT_ROWS);
    }
    for (int i = 0; i < SBT_RING; ++i) {
      tc::mbar_init(&wfull[i], 1);
      tc::mbar_init(&cfree[i], SBT_ROWS);
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&dfull[i], 1);
      tc::mbar_init(&dfree[i], 128);
    }
    tc::mbar_init_fence();
  }
  if (warp == 0) tc::tmem_alloc(tslot, 512);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *tslot;
  // A and B MN-major, M = 128, N = 256
  const uint32_t idesc = tc::idesc_e4m3_f32(128, 256) | (1u << 15) | (1u << 16);
  auto give_up = [&]() {
    if (!*abort_flag) {
      *abort_flag = 1;
      atomicExch(status, 4);
    }
  };

  if (warp >= 2 && warp < SBT_EPI_WARP) {
    const int p = tid - 64, group = p / SBT_ROWS, op = (p % SBT_ROWS) >> 7, j = p & 127;
    // E_lo: A tile, 8-row groups 1024 bytes apart; block op - 1: B tile cores 8 (op - 1) .. + 7,
    // 8-row groups 2048 bytes apart
    const int kstride = op == 0 ? 1024 : 2048;
    const int at = op == 0 ? 0 : SBT_OPA + (op - 1) * 8 * 128;
    for (int T = group; T < ntiles; T += SBT_GROUPS) {
      const int s = T % SBT_STAGES, slot = T % SBT_RING;
      const bool live = op < 2 || pair_h0(T / 32) + 1 < nblocks;
      bool ok = T < SBT_STAGES ||
                tc::mbar_wait_fast(&done[s], ((T / SBT_STAGES) - 1) & 1, abort_flag, SBT_WAIT_CYCLES);
      ok = ok && tc::mbar_wait_fast(&wfull[slot], (T / SBT_RING) & 1, abort_flag, SBT_WAIT_CYCLES);
      if (!__all_sync(0xffffffffu, ok)) give_up();
      const uint4 w = live && !*abort_flag ? reinterpret_cast<const uint4*>(ring + slot * SBT_SLOT)[128 * op + j]
                                           : make_uint4(0, 0, 0, 0);
      if (!*abort_flag) sblock_write_row(sbs + s * SBT_STAGE + at, j, kstride, w);
      // The proxy fence orders this thread's generic accesses before the async proxy's: the stage
      // writes before the MMAs read them, and the word's read from the ring before the next bulk
      // copy overwrites it (a release on the barrier alone does not order the copy engine's write;
      // without the fence a word was at times read after its slot was refilled).
      tc::fence_proxy_async();
      tc::mbar_arrive(&cfree[slot]);
      tc::mbar_arrive(&full[s]);
    }
  } else if (tid == 32) {  // loader
    int issued = 0;
    for (int T = 0; T < ntiles && !*abort_flag; ++T, ++issued) {
      const int slot = T % SBT_RING, t = T % 32;
      if (T >= SBT_RING && !tc::mbar_wait(&cfree[slot], ((T / SBT_RING) - 1) & 1, abort_flag, SBT_WAIT_CYCLES)) {
        give_up();
        break;
      }
      const uint64_t h0 = pair_h0(T / 32);
      const bool two = h0 + 1 < nblocks;
      uint8_t* dst = ring + slot * SBT_SLOT;
      tc::mbar_expect_tx(&wfull[slot], two ? 3 * 2048 : 2 * 2048);
      tc::bulk_load(dst, elo + 128 * t, 2048, &wfull[slot]);
      tc::bulk_load(dst + 2048, table + h0 * 4096 + 128 * t, 2048, &wfull[slot]);
      if (two) tc::bulk_load(dst + 4096, table + (h0 + 1) * 4096 + 128 * t, 2048, &wfull[slot]);
    }
    // the copies in flight land before the block leaves
    for (int T = issued > SBT_RING ? issued - SBT_RING : 0; T < issued; ++T) {
      const long long t0 = clock64();
      while (!tc::mbar_try_wait(&wfull[T % SBT_RING], (T / SBT_RING) & 1) && clock64() - t0 < SBT_WAIT_CYCLES) {
      }
    }
  } else if (tid == 0) {  // issuer
    int last = -1;  // k-tile of the last commit
    for (int T = 0; T < ntiles; ++T) {
      const int s = T % SBT_STAGES, t = T % 32, q = T / 32, buf = q & 1;
      if (t == 0 && q >= 2 && !tc::mbar_wait(&dfree[buf], ((q >> 1) - 1) & 1, abort_flag, SBT_WAIT_CYCLES))
        give_up();
      if (!tc::mbar_wait_fast(&full[s], (T / SBT_STAGES) & 1, abort_flag, SBT_WAIT_CYCLES)) give_up();
      if (*abort_flag) break;
      tc::fence_after_sync();
      const uint32_t a0 = tc::smem_u32(sbs + s * SBT_STAGE), b0 = a0 + SBT_OPA;
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)  // K = 32: four 8-row groups
        tc::mma_e4m3(tbase + 256 * buf, tc::sdesc(a0 + kk * 4096, 1024, 128), tc::sdesc(b0 + kk * 8192, 2048, 128),
                     idesc, (t | kk) ? 1u : 0u);
      tc::mma_commit(&done[s]);
      if (t == 31) tc::mma_commit(&dfull[buf]);
      last = T;
    }
    // Drain: the issuer's last commit covers every MMA it issued (also after an abort).
    if (last >= 0) {
      const long long t0 = clock64();
      while (!tc::mbar_try_wait(&done[last % SBT_STAGES], (last / SBT_STAGES) & 1) &&
             clock64() - t0 < SBT_WAIT_CYCLES) {
      }
    }
  } else if (warp >= SBT_EPI_WARP) {  // TMEM lanes 32 (w % 4) .. + 31 = bits b
    const int qd = warp & 3;
    for (int q = 0; q < nq; ++q) {
      const int buf = q & 1;
      if (!__all_sync(0xffffffffu, tc::mbar_wait(&dfull[buf], (q >> 1) & 1, abort_flag, SBT_WAIT_CYCLES))) {
        give_up();
        break;
      }
      tc::fence_after_sync();
      const uint64_t h0 = pair_h0(q);
      for (int hh = 0; hh < 2 && h0 + hh < nblocks; ++hh) {
        uint32_t* out = reinterpret_cast<uint32_t*>(sblk + (h0 + hh) * 128 * 16) + qd;
#pragma unroll 1
        for (int c0 = 0; c0 < 128; c0 += 32) {
          uint32_t mine = 0;
#pragma unroll
          for (int n0 = 0; n0 < 32; n0 += 16) {
            uint32_t v[16];
            tc::tmem_ld_x16(tbase + ((uint32_t)(32 * qd) << 16) + 256 * buf + 128 * hh + c0 + n0, v);
            tc::tmem_wait_ld(v);
#pragma unroll
            for (int i = 0; i < 16; ++i) {
              // both operands hold set bits as 2.0: D = 4 x count, so the count's parity is bit 2
              const uint32_t bal =
                  __ballot_sync(0xffffffffu, (__float_as_uint(__uint_as_float(v[i]) + 8388608.0f) >> 2) & 1u);
              if (lane == n0 + i) mine = bal;
            }
          }
          out[4 * (c0 + lane)] = mine;  // word qd of c = c0 + lane: bits b = 32 qd + lane'
        }
      }
      tc::fence_before_sync();
      tc::mbar_arrive(&dfree[buf]);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (*abort_flag && tid == 0) atomicExch(status, 4);
  if (warp == 0) tc::tmem_dealloc(tbase, 512);
}

// v[c] = sum_h E_hi[h] * S_h[c]: block of 128 threads (one per c) over a run of h.
__global__ void k_partials_combine(const b128* __restrict__ ehi, const uint8_t* __restrict__ sblk, int nblocks, int run,
                                   unsigned long long* __restrict__ v) {
  const int c = threadIdx.x;
  const int h0 = blockIdx.x * run;
  b128 acc = {0, 0};
  for (int h = h0; h < min(nblocks, h0 + run); ++h) {
    const uint64_t* s = reinterpret_cast<const uint64_t*>(sblk + ((size_t)h * 128 + c) * 16);
    b128 sv = {s[0], s[1]};
    acc = b128_add(acc, b128_mul(ehi[h], sv));
  }
  atomicXor(&v[2 * c], (unsigned long long)acc.lo);
  atomicXor(&v[2 * c + 1], (unsigned long long)acc.hi);
}

// ---------------------------------------------------------------------------------------------
// Switch rounds on materialised a and p (SoA limbs): the last 12 rounds, 4096 entries.
// ---------------------------------------------------------------------------------------------
// psi_table (crossfield.rs:150-161): tab[c][m] = sum_{b in m} batch[8c + b].
__global__ void k_psi_tables(const f162* __restrict__ batch, f162* __restrict__ tab) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 16 * 256) return;
  int c = e >> 8, m = e & 255;
  f162 v = {0, 0, 0};
  for (int b = 0; b < 8; ++b)
    if ((m >> b) & 1) v = f162_add(v, batch[8 * c + b]);
  tab[e] = v;
}

__device__ __forceinline__ f162 shfl_xor_f162(f162 v, int m) {
  v.w0 ^= __shfl_xor_sync(0xffffffffu, v.w0, m);
  v.w1 ^= __shfl_xor_sync(0xffffffffu, v.w1, m);
  v.w2 ^= __shfl_xor_sync(0xffffffffu, v.w2, m);
  return v;
}

// A round message's blocks XOR their shares into msg[0..5] (device) and count themselves in
// msg[6]; the last block to arrive forwards the message to `out` (host memory the device writes
// through) and clears msg for the next round, so a round needs no separate clear or copy. After
// the six words it sets out[7] to 1 with a system-scope release, so the host, which cleared
// out[7] before the launch, can read the message as soon as the flag lands instead of waiting
// for the kernel and the stream to complete. Called by every thread of the block after its
// shares were added; no block waits for another.
__device__ __forceinline__ void msg_forward(unsigned long long* msg, unsigned long long* out) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(msg + 6, 1ull) == (unsigned long long)gridDim.x - 1;
  __syncthreads();
  if (last && threadIdx.x < 32) {
    if (threadIdx.x < 6) {
      __threadfence();
      out[threadIdx.x] = atomicExch(msg + threadIdx.x, 0ull);
      __threadfence_system();
    }
    __syncwarp();
    if (threadIdx.x == 0) {
      msg[6] = 0;
      asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(out + 7), "l"(1ull) : "memory");
    }
  }
}

// msg = [sum_{j<half} a_j p_j, sum (a_j + a_{j+half})(p_j + p_{j+half})] (sumcheck.rs:128-189)
__global__ void __launch_bounds__(256) k_switch_msg(Soa a, Soa p, uint64_t half, unsigned long long* __restrict__ msg,
                                                    unsigned long long* __restrict__ out) {
  f162 e0 = {0, 0, 0}, ei = {0, 0, 0};
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < half; j += (uint64_t)gridDim.x * blockDim.x) {
    f162 a0 = a.get(j), a1 = a.get(j + half), p0 = p.get(j), p1 = p.get(j + half);
    e0 = f162_add(e0, f162_mul(a0, p0));
    ei = f162_add(ei, f162_mul(f162_add(a0, a1), f162_add(p0, p1)));
  }
  for (int m = 16; m; m >>= 1) e0 = shfl_xor_f162(e0, m), ei = shfl_xor_f162(ei, m);
  __shared__ f162 part[2][8];
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) part[0][warp] = e0, part[1][warp] = ei;
  __syncthreads();
  if (threadIdx.x < 2) {
    f162 s = {0, 0, 0};
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s = f162_add(s, part[threadIdx.x][w]);
    unsigned long long* o = msg + 3 * threadIdx.x;
    atomicXor(o, (unsigned long long)s.w0);
    atomicXor(o + 1, (unsigned long long)s.w1);
    atomicXor(o + 2, (unsigned long long)s.w2);
  }
  msg_forward(msg, out);
}

// x[j] <- x[j] + r (x[j] + x[j + half]) for j < half, both polynomials (sumcheck.rs:191-245)
__global__ void __launch_bounds__(256) k_switch_fold(Soa a, Soa p, uint64_t half, f162 r) {
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < half; j += (uint64_t)gridDim.x * blockDim.x) {
    f162 a0 = a.get(j), a1 = a.get(j + half), p0 = p.get(j), p1 = p.get(j + half);
    a.put(j, f162_add(a0, f162_mul(r, f162_add(a0, a1))));
    p.put(j, f162_add(p0, f162_mul(r, f162_add(p0, p1))));
  }
}

// The fold of a round and the message of the next in one pass. Four lanes per pair j < half / 2
// of the next round: lane q folds entry j (q = 0, 2) or j + half / 2 (q = 1, 3) of a (q < 2) or
// p (q >= 2), reading it and its partner half entries up, which no other lane touches, and writes
// it back; the four values then meet by shuffles and lanes 0 and 1 add the pair's terms of the
// next message (sumcheck.rs:128-245).
__global__ void __launch_bounds__(256) k_switch_fold_msg(Soa a, Soa p, uint64_t half, f162 r,
                                                         unsigned long long* __restrict__ msg,
                                                         unsigned long long* __restrict__ out) {
  const uint64_t h2 = half >> 1;
  const int q = threadIdx.x & 3, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const Soa& x = q < 2 ? a : p;
  f162 e0 = {0, 0, 0}, ei = {0, 0, 0};
  // every lane of a warp runs the same number of iterations (the shuffles below are warp-wide)
  const uint64_t stride = (uint64_t)gridDim.x * (blockDim.x >> 2);
  const uint64_t j0 = blockIdx.x * (uint64_t)(blockDim.x >> 2) + (threadIdx.x >> 2);
  for (uint64_t jb = j0 - (threadIdx.x >> 2) % 8; jb < h2; jb += stride) {
    const uint64_t j = jb + (threadIdx.x >> 2) % 8;
    const bool live = j < h2;
    f162 v = {0, 0, 0};
    if (live) {
      const uint64_t i = j + (q & 1) * h2;
      const f162 x0 = x.get(i);
      v = f162_add(x0, f162_mul(r, f162_add(x0, x.get(i + half))));
      x.put(i, v);
    }
    const int base = lane & ~3;
    f162 a0, a1, p0, p1;
    a0.w0 = __shfl_sync(0xffffffffu, v.w0, base), a0.w1 = __shfl_sync(0xffffffffu, v.w1, base),
    a0.w2 = __shfl_sync(0xffffffffu, v.w2, base);
    a1.w0 = __shfl_sync(0xffffffffu, v.w0, base + 1), a1.w1 = __shfl_sync(0xffffffffu, v.w1, base + 1),
    a1.w2 = __shfl_sync(0xffffffffu, v.w2, base + 1);
    p0.w0 = __shfl_sync(0xffffffffu, v.w0, base + 2), p0.w1 = __shfl_sync(0xffffffffu, v.w1, base + 2),
    p0.w2 = __shfl_sync(0xffffffffu, v.w2, base + 2);
    p1.w0 = __shfl_sync(0xffffffffu, v.w0, base + 3), p1.w1 = __shfl_sync(0xffffffffu, v.w1, base + 3),
    p1.w2 = __shfl_sync(0xffffffffu, v.w2, base + 3);
    if (live && q == 0) e0 = f162_add(e0, f162_mul(a0, p0));
    if (live && q == 1) ei = f162_add(ei, f162_mul(f162_add(a0, a1), f162_add(p0, p1)));
  }
  for (int m = 16; m; m >>= 1) e0 = shfl_xor_f162(e0, m), ei = shfl_xor_f162(ei, m);
  __shared__ f162 part[2][8];
  if (lane == 0) part[0][warp] = e0, part[1][warp] = ei;
  __syncthreads();
  if (threadIdx.x < 2) {
    f162 s = {0, 0, 0};
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s = f162_add(s, part[threadIdx.x][w]);
    unsigned long long* o = msg + 3 * threadIdx.x;
    atomicXor(o, (unsigned long long)s.w0);
    atomicXor(o + 1, (unsigned long long)s.w1);
    atomicXor(o + 2, (unsigned long long)s.w2);
  }
  msg_forward(msg, out);
}

// ---------------------------------------------------------------------------------------------
// Switch from the partials' blocks (rounds r < HB = LP - 12).
//
// After r folds with challenges r'_0..r'_{r-1}, a_r[j] = Phi_r(E_r(j)), E_r = eq over
// r_hi[r..LP], and Phi_r(y) = sum_b bit_b(y) G_r[b] is GF(2)-linear with G_0 = batch and
// G_{r+1}[b] = (1 + r'_r) Phi_r((1 + rho_r) X^b) + r'_r Phi_r(rho_r X^b), rho_r = r_hi[r]
// (the LeanSwitch algebra of crossfield.rs:1478-1509, without any division). The folded
// p_r[j] = sum_x w_x lift(pi0[x || j]) with w_x = eq over r'_0..r'_{r-1}.
// With the blocks S_h[c] = sum_jl bit_c(pi0[h, jl]) E_lo[jl] folded from the bottom,
// R_k[e][c] = sum_l eq(r_hi[HB-k..HB], l) S_{e 2^k + l}[c], the round message is
//   e0   = sum_x w_x sum_c X^c Phi_r((1 + rho_r) R[2x][c]),
//   einf = sum_x w_x sum_c X^c Phi_r(R[2x][c] + R[2x + 1][c]),   R = R_{HB - r - 1},
// so these rounds read no table word; one pass then materialises p_HB (4096 entries).
// ---------------------------------------------------------------------------------------------
// R_{k+1}[i][c] = (1 + rho) R_k[2i][c] + rho R_k[2i + 1][c]
__global__ void k_rblock_level(const b128* __restrict__ in, uint64_t nout, b128 rho, b128* __restrict__ out) {
  uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (t >= nout * 128) return;
  const uint64_t i = t >> 7, c = t & 127;
  const b128 v0 = in[(2 * i) * 128 + c], v1 = in[(2 * i + 1) * 128 + c];
  // (1 + rho) v0 + rho v1 = v0 + rho (v0 + v1)
  out[t] = b128_add(v0, b128_mul(rho, b128_add(v0, v1)));
}

// x * X^c modulo x^162 + x^81 + 1, c < 128
__device__ __forceinline__ f162 f162_shift(f162 f, int c) {
  uint64_t w[6] = {f.w0, f.w1, f.w2, 0, 0, 0};
  if (c >= 64) {
    w[3] = w[2], w[2] = w[1], w[1] = w[0], w[0] = 0;
    c -= 64;
  }
  if (c) {
    w[4] = w[3] >> (64 - c);
    w[3] = (w[3] << c) | (w[2] >> (64 - c));
    w[2] = (w[2] << c) | (w[1] >> (64 - c));
    w[1] = (w[1] << c) | (w[0] >> (64 - c));
    w[0] = w[0] << c;
  }
  return f162_reduce(w[0], w[1], w[2], w[3], w[4], 0);
}

__device__ __forceinline__ f162 phi_apply(const f162* tab, b128 e) {
  f162 v = {0, 0, 0};
#pragma unroll
  for (int c = 0; c < 16; ++c) {
    uint32_t byte = (uint32_t)((c < 8 ? e.lo >> (8 * c) : e.hi >> (8 * (c - 8))) & 0xff);
    v = f162_add(v, tab[c * 256 + byte]);
  }
  return v;
}

// One round's message from R (2X entries of 128 columns). Block of 128 threads: thread = column.
constexpr int RB_DEFER = 64;  // x per block whose weighting is deferred to one parallel pass
__global__ void __launch_bounds__(128) k_switch_round_blocks(const b128* __restrict__ R, uint64_t X, b128 rho,
                                                            const f162* __restrict__ phi, const f162* __restrict__ w,
                                                            unsigned long long* __restrict__ msg,
                                                            unsigned long long* __restrict__ out) {
  extern __shared__ __align__(16) uint64_t sm64[];
  f162* tab = reinterpret_cast<f162*>(sm64);
  for (int i = threadIdx.x; i < 16 * 256; i += blockDim.x) tab[i] = phi[i];
  __syncthreads();
  __shared__ f162 part[2][4];
  __shared__ f162 sums[2][RB_DEFER];  // the block's column sums per x, weighted after the loop
  const int c = threadIdx.x, lane = c & 31, warp = c >> 5;
  const b128 one_rho = {rho.lo ^ 1, rho.hi};
  f162 e0 = {0, 0, 0}, ei = {0, 0, 0};
  int nx = 0;
  for (uint64_t x = blockIdx.x; x < X; x += gridDim.x, ++nx) {
    const b128 v0 = R[(2 * x) * 128 + c], v1 = R[(2 * x + 1) * 128 + c];
    f162 s0 = f162_shift(phi_apply(tab, b128_mul(one_rho, v0)), c);
    f162 si = f162_shift(phi_apply(tab, b128_add(v0, v1)), c);
    for (int m = 16; m; m >>= 1) {
      s0.w0 ^= __shfl_xor_sync(0xffffffffu, s0.w0, m);
      s0.w1 ^= __shfl_xor_sync(0xffffffffu, s0.w1, m);
      s0.w2 ^= __shfl_xor_sync(0xffffffffu, s0.w2, m);
      si.w0 ^= __shfl_xor_sync(0xffffffffu, si.w0, m);
      si.w1 ^= __shfl_xor_sync(0xffffffffu, si.w1, m);
      si.w2 ^= __shfl_xor_sync(0xffffffffu, si.w2, m);
    }
    if (lane == 0) part[0][warp] = s0, part[1][warp] = si;
    __syncthreads();
    if (c == 0) {
      const f162 a0 = f162_add(f162_add(part[0][0], part[0][1]), f162_add(part[0][2], part[0][3]));
      const f162 ai = f162_add(f162_add(part[1][0], part[1][1]), f162_add(part[1][2], part[1][3]));
      if (nx < RB_DEFER) {
        sums[0][nx] = a0, sums[1][nx] = ai;
      } else {  // more x than the deferral buffer holds (only at very large shapes): weight now
        const f162 wx = w[x];
        e0 = f162_add(e0, f162_mul(wx, a0));
        ei = f162_add(ei, f162_mul(wx, ai));
      }
    }
    __syncthreads();
  }
  // the weights w_x times the deferred sums, one product per thread, then one reduction
  {
    f162 d0 = {0, 0, 0}, di = {0, 0, 0};
    const int nd = min(nx, RB_DEFER);
    for (int k = c; k < 2 * nd; k += blockDim.x) {
      const int which = k / nd, i = k % nd;
      const f162 prod = f162_mul(w[blockIdx.x + (uint64_t)i * gridDim.x], sums[which][i]);
      if (which == 0) d0 = f162_add(d0, prod); else di = f162_add(di, prod);
    }
    for (int m = 16; m; m >>= 1) d0 = shfl_xor_f162(d0, m), di = shfl_xor_f162(di, m);
    if (lane == 0) part[0][warp] = d0, part[1][warp] = di;
    __syncthreads();
    if (c == 0)
      for (int q = 0; q < 4; ++q) e0 = f162_add(e0, part[0][q]), ei = f162_add(ei, part[1][q]);
  }
  if (c == 0) {
    atomicXor(&msg[0], (unsigned long long)e0.w0);
    atomicXor(&msg[1], (unsigned long long)e0.w1);
    atomicXor(&msg[2], (unsigned long long)e0.w2);
    atomicXor(&msg[3], (unsigned long long)ei.w0);
    atomicXor(&msg[4], (unsigned long long)ei.w1);
    atomicXor(&msg[5], (unsigned long long)ei.w2);
  }
  msg_forward(msg, out);
}

// After a block round: the next round's byte tables and weights in one launch.
// Blocks c < 16: G_{r+1}[b] = Phi_r(y1) + r' (Phi_r(y1) + Phi_r(y2)), y1 = (1 + rho) X^b, y2 = rho X^b,
// for the block's b = 8c .. 8c + 7 (Phi_r through the round's byte tables psi, rho X^b a shift:
// no GHASH product), then table c of psi_next from them. Blocks c >= 16: the weights
// w_{r+1}[2x] = (1 + r') w_r[x], w_{r+1}[2x + 1] = r' w_r[x].
__global__ void __launch_bounds__(256) k_round_update(const f162* __restrict__ psi, b128 rho, f162 rp,
                                                      f162* __restrict__ psi_next, const f162* __restrict__ w,
                                                      uint64_t X, f162* __restrict__ wn) {
  if (blockIdx.x >= 16) {
    const uint64_t x = (blockIdx.x - 16) * (uint64_t)blockDim.x + threadIdx.x;
    if (x >= X) return;
    const f162 t = f162_mul(w[x], rp);
    wn[2 * x] = f162_add(w[x], t);
    wn[2 * x + 1] = t;
    return;
  }
  __shared__ f162 gb[8];
  const int c = blockIdx.x;
  if (threadIdx.x < 8) {
    const int b = 8 * c + threadIdx.x;
    const b128 xb = {b < 64 ? 1ull << b : 0, b >= 64 ? 1ull << (b - 64) : 0};
    const b128 y2 = b128_shl(rho, b);
    const b128 y1 = b128_add(xb, y2);
    const f162 p1 = phi_apply(psi, y1), p2 = phi_apply(psi, y2);
    gb[threadIdx.x] = f162_add(p1, f162_mul(rp, f162_add(p1, p2)));
  }
  __syncthreads();
  const int m = threadIdx.x;
  f162 v = {0, 0, 0};
#pragma unroll
  for (int b = 0; b < 8; ++b)
    if ((m >> b) & 1) v = f162_add(v, gb[b]);
  psi_next[256 * c + m] = v;
}

// a[j] = Phi(E_lo[j]) for the 4096 low entries.
__global__ void __launch_bounds__(256) k_phi_apply(const b128* __restrict__ e, uint64_t n, const f162* __restrict__ phi,
                                                   Soa a) {
  extern __shared__ __align__(16) uint64_t sm64[];
  f162* tab = reinterpret_cast<f162*>(sm64);
  for (int i = threadIdx.x; i < 16 * 256; i += blockDim.x) tab[i] = phi[i];
  __syncthreads();
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < n; j += (uint64_t)gridDim.x * blockDim.x)
    a.put(j, phi_apply(tab, e[j]));
}

// p[j] = sum_x w[x] lift(pi0[x 2^12 + j]) for j < 4096: block (j tile of 256, x share).
// p[j] += sum over the block's x of w[x] * lift(table[4096 x + j]): one window table per x (w[x] is
// the block's common multiplier), MW_J entries j per thread.
constexpr int MW_J = 2;
__global__ void __launch_bounds__(256) k_materialize(const uint4* __restrict__ table, const f162* __restrict__ w,
                                                     uint64_t X, uint64_t x_share, Soa p) {
  __shared__ WinTable T;
  const uint64_t j0 = blockIdx.x * (256ull * MW_J) + threadIdx.x;
  const uint64_t x0 = blockIdx.y * x_share, x1 = min(X, x0 + x_share);
  f162 acc[MW_J];
#pragma unroll
  for (int k = 0; k < MW_J; ++k) acc[k] = {0, 0, 0};
  for (uint64_t x = x0; x < x1; ++x) {
    uint4 v[MW_J];
#pragma unroll
    for (int k = 0; k < MW_J; ++k) v[k] = table[(x << 12) + j0 + 256 * k];
    win_build(T, w[x], threadIdx.x, 256);
#pragma unroll
    for (int k = 0; k < MW_J; ++k) win_mul_add(T, v[k], acc[k]);
    __syncthreads();  // the next x rebuilds the table
  }
#pragma unroll
  for (int k = 0; k < MW_J; ++k) {
    const uint64_t j = j0 + 256 * k;
    atomicXor(reinterpret_cast<unsigned long long*>(p.w0 + j), (unsigned long long)acc[k].w0);
    atomicXor(reinterpret_cast<unsigned long long*>(p.w1 + j), (unsigned long long)acc[k].w1);
    atomicXor(reinterpret_cast<unsigned long long*>(p.w2 + j), (unsigned long long)acc[k].w2);
  }
}

// ---------------------------------------------------------------------------------------------
// Launch wrappers
// ---------------------------------------------------------------------------------------------
void launch_rblock_level(const b128* in, uint64_t nout, b128 rho, b128* out, cudaStream_t s) {
  uint64_t n = nout * 128;
  k_rblock_level<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, nout, rho, out);
}
void launch_switch_round_blocks(const b128* R, uint64_t X, b128 rho, const f162* phi, const f162* w,
                                unsigned long long* msg, unsigned long long* out, int sms, cudaStream_t s) {
  const int smem = 16 * 256 * 24;
  static std::atomic<unsigned long long> attr{0};
  smem_limit(k_switch_round_blocks, smem, attr);
  unsigned g = (unsigned)(X < 2ull * sms ? X : 2ull * sms);  // two blocks per SM (98 KB tables each)
  k_switch_round_blocks<<<g, 128, smem, s>>>(R, X, rho, phi, w, msg, out);
}
void launch_round_update(const f162* psi, b128 rho, f162 rp, f162* psi_next, const f162* w, uint64_t X, f162* wn,
                         cudaStream_t s) {
  k_round_update<<<(unsigned)(16 + (X + 255) / 256), 256, 0, s>>>(psi, rho, rp, psi_next, w, X, wn);
}
void launch_phi_apply(const b128* e, uint64_t n, const f162* phi, Soa a, cudaStream_t s) {
  const int smem = 16 * 256 * 24;
  static std::atomic<unsigned long long> attr{0};
  smem_limit(k_phi_apply, smem, attr);
  k_phi_apply<<<16, 256, smem, s>>>(e, n, phi, a);
}
void launch_materialize(const uint4* table, const f162* w, uint64_t X, Soa p, int sms, cudaStream_t s) {
  // one wave: 8 j tiles x shares = the blocks resident at once (five per SM)
  const uint64_t tiles = 4096 / (256 * MW_J);
  uint64_t shares = std::max<uint64_t>(1, std::min<uint64_t>(X, 5ull * sms / tiles));
  const uint64_t x_share = (X + shares - 1) / shares;
  shares = (X + x_share - 1) / x_share;
  k_materialize<<<dim3((unsigned)tiles, (unsigned)shares), 256, 0, s>>>(table, w, X, x_share, p);
}
static unsigned grid_for(uint64_t n, int threads, unsigned cap) {
  uint64_t g = (n + threads - 1) / threads;
  if (g > cap) g = cap;
  return (unsigned)(g ? g : 1);
}

void launch_eq_b128(const b128* r, int n, b128* out, cudaStream_t s) {
  uint64_t N = 1ull << n;
  k_eq_b128<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(r, n, out);
}
void launch_eq_table_f162(const f162* ps, int n, f162* out, cudaStream_t s) {
  uint64_t N = 1ull << n;
  k_eq_table_f162<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(ps, n, out);
}
void launch_sblock(const uint4* table, uint64_t nblocks, const b128* elo, uint8_t* sblk, int* status,
                   cudaStream_t s) {
  static std::atomic<unsigned long long> attr{0};
  smem_limit(k_sblock_tc, SBT_SMEM, attr);
  static int sms = 0;  // one CTA per SM (the kernel walks its pairs)
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  const uint64_t npairs = (nblocks + 1) / 2;
  k_sblock_tc<<<(unsigned)std::min<uint64_t>(npairs, (uint64_t)sms), SBT_THREADS, SBT_SMEM, s>>>(
      table, nblocks, reinterpret_cast<const uint4*>(elo), sblk, status);
}
void launch_partials_combine(const b128* ehi, const uint8_t* sblk, int nblocks, unsigned long long* v, cudaStream_t s) {
  int run = 16;
  k_partials_combine<<<(nblocks + run - 1) / run, 128, 0, s>>>(ehi, sblk, nblocks, run, v);
}
void launch_psi_tables(const f162* batch, f162* tab, cudaStream_t s) { k_psi_tables<<<16, 256, 0, s>>>(batch, tab); }
void launch_switch_msg(Soa a, Soa p, uint64_t half, unsigned long long* msg, unsigned long long* out, int sms,
                       cudaStream_t s) {
  k_switch_msg<<<grid_for(half, 256, sms * 8), 256, 0, s>>>(a, p, half, msg, out);
}
void launch_switch_fold_msg(Soa a, Soa p, uint64_t half, f162 r, unsigned long long* msg, unsigned long long* out,
                            int sms, cudaStream_t s) {
  k_switch_fold_msg<<<grid_for(2 * half, 256, sms * 8), 256, 0, s>>>(a, p, half, r, msg, out);  // 4 lanes a pair
}
void launch_switch_fold(Soa a, Soa p, uint64_t half, f162 r, int sms, cudaStream_t s) {
  k_switch_fold<<<grid_for(half, 256, sms * 8), 256, 0, s>>>(a, p, half, r);
}

}  // namespace lf
