// Host emulation of the device challenge sampler (csrc/lf_open.cu, k_challenges) step by step,
// using the prover's own BLAKE3 (csrc/lf_blake3.cuh), against the oracle's sample_short_challenges.
// Built and run by tests/test_host_primitives.py.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../labinius-fast-challenge_gb300/csrc/lf_blake3.cuh"
#include "../oracle/oracle.h"

using namespace lf;

int main() {
  const char* domain = "labinius/test/batch";
  const uint8_t prefix[] = {'l', 'f', 'c', 'h', 'k'};
  const int n = 48;
  // Transcript::new(domain) + absorb_bytes(prefix)
  bk::Hasher t;
  t.init();
  t.absorb_u64(strlen(domain));
  t.absorb((const uint8_t*)domain, strlen(domain));
  t.absorb_u64(sizeof prefix);
  t.absorb(prefix, sizeof prefix);
  // phase tables as the prover builds them
  std::vector<double> re(162 * 88, 0.0), im(162 * 88, 0.0);
  int units[162], nu = 0;
  for (int x = 1; x < 243; ++x)
    if (x % 3) units[nu++] = x;
  for (int p = 0; p < 162; ++p)
    for (int k = 0; k < 81; ++k) {
      int m = (p * units[k]) % 243;
      volatile double two_pi = 2.0 * M_PI;
      double angle = two_pi * (double)m;
      angle = angle / 243.0;
      re[p * 88 + k] = cos(angle);
      im[p * 88 + k] = sin(angle);
    }
  bk::Hasher sk;
  sk.init_derive("labinius 2026 challenge signs v1", 32);
  std::vector<uint8_t> want(40 * n);
  lfo_short_challenges(domain, prefix, sizeof prefix, n, want.data());
  int bad = 0;
  for (int ci = 0; ci < n; ++ci) {
    bk::Hasher h = t;
    h.absorb_u64((uint64_t)ci);
    h.absorb_u64(15);
    h.absorb((const uint8_t*)"short-challenge", 15);
    bk::Pending root = h.finish();
    uint8_t buf[2048];
    uint64_t next_block = 0;
    int pos = 2048;
    auto byte = [&]() -> uint32_t {
      if (pos == 2048) {
        for (int l = 0; l < 32; ++l) {
          uint32_t w[16];
          root.root_block(next_block + l, w);
          memcpy(buf + 64 * l, w, 64);
        }
        next_block += 32;
        pos = 0;
      }
      return buf[pos++];
    };
    uint8_t got_pos[32];
    uint32_t got_signs = 0;
    for (;;) {
      uint8_t perm[162];
      for (int i = 0; i < 162; ++i) perm[i] = (uint8_t)i;
      for (int i = 0; i < 28; ++i) {
        uint32_t nn = 162 - i, limit = (65536u / nn) * nn;
        uint64_t magic = (1ull << 32) / nn + 1;
        uint32_t r;
        do {
          uint32_t lo = byte(), hi = byte();
          r = lo | (hi << 8);
        } while (r >= limit);
        uint32_t q = (uint32_t)(((uint64_t)r * magic) >> 32);
        int j = i + (int)(r - q * nn);
        uint8_t tt = perm[i];
        perm[i] = perm[j];
        perm[j] = tt;
      }
      uint8_t sorted[32] = {0};
      for (int l = 0; l < 28; ++l) {
        int rank = 0;
        for (int u = 0; u < 28; ++u) rank += perm[u] < perm[l];
        sorted[rank] = perm[l];
      }
      uint8_t blk[64] = {0};
      blk[0] = 28;
      memcpy(blk + 8, sorted, 28);
      uint32_t m[16], o[16];
      bk::load_words(blk, m, 16);
      bk::compress16(sk.key, m, 0, 36, bk::F_DERIVE_MAT | bk::F_CHUNK_START | bk::F_CHUNK_END | bk::F_ROOT, o);
      uint32_t signs = o[0] & ((1u << 28) - 1);
      bool over = false;
      for (int k = 0; k < 81; ++k) {
        double vr = 0.0, vi = 0.0;
        for (int u = 0; u < 28; ++u) {
          double pr = re[sorted[u] * 88 + k], pi = im[sorted[u] * 88 + k];
          if ((signs >> u) & 1) pr = -pr, pi = -pi;
          vr = vr + pr;
          vi = vi + pi;
        }
        double a = vr * vr, b = vi * vi;
        if (a + b > 144.0 + 1e-12) over = true;
      }
      if (!over) {
        memcpy(got_pos, sorted, 32);
        got_signs = signs;
        break;
      }
    }
    if (memcmp(got_pos, &want[40 * ci], 28) || memcmp(&got_signs, &want[40 * ci + 32], 4)) {
      if (bad++ < 3) printf("challenge %d differs\n", ci);
    }
  }
  if (bad) {
    printf("FAIL %d\n", bad);
    return 1;
  }
  printf("OK %d\n", n);
  return 0;
}
