// Device builds of the prover's shared BLAKE3 and field code (csrc/lf_blake3.cuh, lf_field.cuh)
// against their host builds, case by case. Built with nvcc and run by tests/test_gpu_primitives.py.
// Prints one line per failing case and "OK <cases>".
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "../labinius-fast-challenge_gb300/csrc/lf_blake3.cuh"
#include "../labinius-fast-challenge_gb300/csrc/lf_field.cuh"

using namespace lf;

constexpr int NCASE = 64;

struct Case {
  uint8_t data[3000];
  uint32_t len;
  uint32_t split;  // absorb in two pieces at this offset
  uint32_t mode;   // 0 plain, 1 keyed, 2 derive
  uint8_t key[32];
};

__global__ void k_hash(const Case* cs, uint8_t* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NCASE) return;
  const Case& c = cs[i];
  bk::Hasher h;
  if (c.mode == 0) h.init();
  if (c.mode == 1) h.init_keyed(c.key);
  if (c.mode == 2) h.init_derive("lf device check", 15);
  h.absorb(c.data, c.split);
  h.absorb(c.data + c.split, c.len - c.split);
  h.finish().root_bytes(0, out + 64 * i, 64);
}

// A hasher copied from global memory, then absorbing more (the transcript derivation pattern).
__global__ void k_copy_absorb(const bk::Hasher* st, const uint8_t* more, uint32_t n, uint8_t* out) {
  if (threadIdx.x || blockIdx.x) return;
  bk::Hasher h = *st;
  h.absorb(more, n);
  h.finish().root_bytes(0, out, 64);
}

// The challenge derivation exactly as the prover's sampler writes it: lane 0 extends a copied
// transcript image by counter, label length and label, then shares the root with its warp.
struct RootShare {
  uint32_t root[27];
};
__global__ void __launch_bounds__(128) k_derive_pattern(const bk::Hasher* __restrict__ state, uint64_t base,
                                                        uint32_t* __restrict__ out, int n) {
  __shared__ RootShare sw[4];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int ci = blockIdx.x * 4 + wid;
  if (ci >= n) return;
  RootShare& s = sw[wid];
  if (lane == 0) {
    bk::Pending r = bk::derive_root(*state, base + (uint64_t)ci, "short-challenge", 15);
    for (int i = 0; i < 8; ++i) s.root[i] = r.h[i];
    for (int i = 0; i < 16; ++i) s.root[8 + i] = r.m[i];
    s.root[24] = (uint32_t)r.t;
    s.root[25] = r.len;
    s.root[26] = r.flags;
  }
  __syncwarp();
  if (lane < 27) out[ci * 27 + lane] = s.root[lane];
}

// Bisection variants of the derivation: the 31 suffix bytes from global memory in three
// pieces (v = 1), or from one local array in one piece (v = 2).
__global__ void k_derive_variant(const bk::Hasher* __restrict__ state, const uint8_t* __restrict__ suffix, int v,
                                 uint32_t* __restrict__ out) {
  if (threadIdx.x || blockIdx.x) return;
  bk::Hasher h = *state;
  if (v == 1) {
    h.absorb(suffix, 8);
    h.absorb(suffix + 8, 8);
    h.absorb(suffix + 16, 15);
  } else {
    uint8_t local[31];
    for (int i = 0; i < 31; ++i) local[i] = suffix[i];
    h.absorb(local, 31);
  }
  bk::Pending r = h.finish();
  for (int i = 0; i < 8; ++i) out[i] = r.h[i];
}

__global__ void k_fields(const b128* a, const b128* b, const f162* x, const f162* y, b128* o1, f162* o2, f162* o3,
                         int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  o1[i] = b128_mul(a[i], b[i]);
  o2[i] = f162_mul(x[i], y[i]);
  o3[i] = f162_mul_lifted(x[i], a[i]);
}

#define CK(x)                                                   \
  do {                                                          \
    cudaError_t e = (x);                                        \
    if (e != cudaSuccess) {                                     \
      printf("cuda error %s at %d\n", cudaGetErrorString(e), __LINE__); \
      return 2;                                                 \
    }                                                           \
  } while (0)

int main() {
  std::mt19937_64 rng(7);
  int fails = 0, cases = 0;
  std::vector<Case> cs(NCASE);
  const uint32_t lens[] = {0, 1, 40, 63, 64, 65, 71, 100, 127, 128, 129, 1023, 1024, 1025, 2048, 2999};
  for (int i = 0; i < NCASE; ++i) {
    for (auto& b : cs[i].data) b = (uint8_t)rng();
    cs[i].len = lens[i % 16];
    cs[i].split = cs[i].len ? (uint32_t)(rng() % (cs[i].len + 1)) : 0;
    cs[i].mode = (uint32_t)(i / 16) % 3;
    for (auto& k : cs[i].key) k = (uint8_t)rng();
  }
  Case* dcs;
  uint8_t* dout;
  CK(cudaMalloc(&dcs, sizeof(Case) * NCASE));
  CK(cudaMalloc(&dout, 64 * NCASE));
  CK(cudaMemcpy(dcs, cs.data(), sizeof(Case) * NCASE, cudaMemcpyHostToDevice));
  k_hash<<<1, NCASE>>>(dcs, dout);
  CK(cudaGetLastError());
  std::vector<uint8_t> got(64 * NCASE);
  CK(cudaMemcpy(got.data(), dout, got.size(), cudaMemcpyDeviceToHost));
  for (int i = 0; i < NCASE; ++i) {
    const Case& c = cs[i];
    bk::Hasher h;
    if (c.mode == 0) h.init();
    if (c.mode == 1) h.init_keyed(c.key);
    if (c.mode == 2) h.init_derive("lf device check", 15);
    h.absorb(c.data, c.split);
    h.absorb(c.data + c.split, c.len - c.split);
    uint8_t want[64];
    h.finish().root_bytes(0, want, 64);
    ++cases;
    if (memcmp(want, &got[64 * i], 64)) {
      if (fails++ < 8) printf("hash mismatch case %d len %u split %u mode %u\n", i, c.len, c.split, c.mode);
    }
  }
  // copy-then-absorb
  for (uint32_t pre : {0u, 40u, 63u, 64u, 1000u, 1024u, 2500u}) {
    bk::Hasher h;
    h.init();
    h.absorb(cs[0].data, pre);
    bk::Hasher* dst;
    uint8_t* dmore;
    CK(cudaMalloc(&dst, sizeof(bk::Hasher)));
    CK(cudaMalloc(&dmore, 64));
    CK(cudaMemcpy(dst, &h, sizeof h, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dmore, cs[1].data, 31, cudaMemcpyHostToDevice));
    k_copy_absorb<<<1, 32>>>(dst, dmore, 31, dout);
    CK(cudaGetLastError());
    uint8_t g[64], want[64];
    CK(cudaMemcpy(g, dout, 64, cudaMemcpyDeviceToHost));
    h.absorb(cs[1].data, 31);
    h.finish().root_bytes(0, want, 64);
    ++cases;
    if (memcmp(g, want, 64)) {
      if (fails++ < 16) printf("copy-absorb mismatch prefix %u\n", pre);
    }
    cudaFree(dst);
    cudaFree(dmore);
  }
  // the sampler's derivation pattern, several transcript sizes and counters
  for (uint32_t pre : {40u, 100u, 1000u, 3000u}) {
    bk::Hasher h;
    h.init();
    h.absorb(cs[2].data, pre > 3000 ? 3000 : pre);
    bk::Hasher* dst;
    uint32_t* dout2;
    const int nd = 8;
    CK(cudaMalloc(&dst, sizeof(bk::Hasher)));
    CK(cudaMalloc(&dout2, nd * 27 * 4));
    CK(cudaMemcpy(dst, &h, sizeof h, cudaMemcpyHostToDevice));
    k_derive_pattern<<<2, 128>>>(dst, 5, dout2, nd);
    CK(cudaGetLastError());
    uint32_t g[nd * 27];
    CK(cudaMemcpy(g, dout2, sizeof g, cudaMemcpyDeviceToHost));
    for (int ci = 0; ci < nd; ++ci) {
      bk::Hasher c = h;
      c.absorb_u64(5 + ci);
      c.absorb_u64(15);
      c.absorb((const uint8_t*)"short-challenge", 15);
      bk::Pending r = c.finish();
      uint32_t w[27];
      for (int i = 0; i < 8; ++i) w[i] = r.h[i];
      for (int i = 0; i < 16; ++i) w[8 + i] = r.m[i];
      w[24] = (uint32_t)r.t, w[25] = r.len, w[26] = r.flags;
      ++cases;
      if (memcmp(w, g + 27 * ci, sizeof w)) {
        if (fails++ < 24) printf("derive mismatch prefix %u ci %d\n", pre, ci);
      }
    }
    cudaFree(dst);
    cudaFree(dout2);
  }
  // bisection variants
  {
    bk::Hasher h;
    h.init();
    h.absorb(cs[2].data, 40);
    uint8_t suffix[31];
    for (int i = 0; i < 8; ++i) suffix[i] = (uint8_t)(5 >> (8 * i));
    suffix[8] = 15;
    for (int i = 9; i < 16; ++i) suffix[i] = 0;
    memcpy(suffix + 16, "short-challenge", 15);
    bk::Hasher c = h;
    c.absorb(suffix, 31);
    bk::Pending r = c.finish();
    bk::Hasher* dst;
    uint8_t* dsuf;
    uint32_t* dres;
    CK(cudaMalloc(&dst, sizeof(bk::Hasher)));
    CK(cudaMalloc(&dsuf, 32));
    CK(cudaMalloc(&dres, 32));
    CK(cudaMemcpy(dst, &h, sizeof h, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dsuf, suffix, 31, cudaMemcpyHostToDevice));
    for (int v = 1; v <= 2; ++v) {
      k_derive_variant<<<1, 32>>>(dst, dsuf, v, dres);
      CK(cudaGetLastError());
      uint32_t g[8];
      CK(cudaMemcpy(g, dres, 32, cudaMemcpyDeviceToHost));
      ++cases;
      if (memcmp(g, r.h, 32)) {
        if (fails++ < 40) printf("variant %d mismatch\n", v);
      }
    }
  }
  // field products
  const int n = 4096;
  std::vector<b128> a(n), b(n), o1(n);
  std::vector<f162> x(n), y(n), o2(n), o3(n);
  for (int i = 0; i < n; ++i) {
    a[i] = {rng(), rng()}, b[i] = {rng(), rng()};
    x[i] = {rng(), rng(), rng() & F162_TOP_MASK}, y[i] = {rng(), rng(), rng() & F162_TOP_MASK};
  }
  b128 *da, *db, *do1;
  f162 *dx, *dy, *do2, *do3;
  CK(cudaMalloc(&da, n * 16));
  CK(cudaMalloc(&db, n * 16));
  CK(cudaMalloc(&do1, n * 16));
  CK(cudaMalloc(&dx, n * 24));
  CK(cudaMalloc(&dy, n * 24));
  CK(cudaMalloc(&do2, n * 24));
  CK(cudaMalloc(&do3, n * 24));
  CK(cudaMemcpy(da, a.data(), n * 16, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(db, b.data(), n * 16, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dx, x.data(), n * 24, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dy, y.data(), n * 24, cudaMemcpyHostToDevice));
  k_fields<<<n / 128, 128>>>(da, db, dx, dy, do1, do2, do3, n);
  CK(cudaGetLastError());
  CK(cudaMemcpy(o1.data(), do1, n * 16, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(o2.data(), do2, n * 24, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(o3.data(), do3, n * 24, cudaMemcpyDeviceToHost));
  for (int i = 0; i < n; ++i) {
    b128 w1 = b128_mul(a[i], b[i]);
    f162 w2 = f162_mul(x[i], y[i]), w3 = f162_mul_lifted(x[i], a[i]);
    cases += 3;
    if (memcmp(&w1, &o1[i], 16) || memcmp(&w2, &o2[i], 24) || memcmp(&w3, &o3[i], 24)) {
      if (fails++ < 20) printf("field mismatch %d\n", i);
    }
  }
  if (fails) {
    printf("FAIL %d of %d\n", fails, cases);
    return 1;
  }
  printf("OK %d\n", cases);
  return 0;
}
