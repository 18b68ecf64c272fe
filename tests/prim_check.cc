// Host build of the prover's shared host/device primitives (csrc/lf_field.cuh, csrc/lf_blake3.cuh)
// checked against the CPU oracle. Built and run by tests/test_host_primitives.py. Prints one line
// per failing case and "OK <cases>" at the end.
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "../labinius-fast-challenge_gb300/csrc/lf_blake3.cuh"
#include "../labinius-fast-challenge_gb300/csrc/lf_field.cuh"
#include "../oracle/oracle.h"

using namespace lf;

static std::mt19937_64 rng(12345);
static uint64_t r64() { return rng(); }

int main() {
  int fails = 0, cases = 0;
  // Field products.
  for (int i = 0; i < 20000; ++i) {
    b128 a = {r64(), r64()}, b = {r64(), r64()};
    if (i < 8) a = {i == 0 ? 0ull : 1ull << (i * 9), i == 1 ? ~0ull : 0}, b = {~0ull, 1ull << 63};
    b128 c = b128_mul(a, b);
    uint8_t ab[16], bb[16], ob[16];
    memcpy(ab, &a, 16), memcpy(bb, &b, 16);
    lfo_b128_mul(ab, bb, ob, 1);
    ++cases;
    if (memcmp(ob, &c, 16)) {
      if (fails++ < 5) printf("b128 mismatch %d\n", i);
    }
    // shifts by X^k (the window-table bases) against the product with the monomial
    {
      const int k = (int)(r64() % 128);
      const b128 xk = {k < 64 ? 1ull << k : 0, k >= 64 ? 1ull << (k - 64) : 0};
      const b128 s = b128_shl(a, k), m = b128_mul(a, xk);
      ++cases;
      if (s.lo != m.lo || s.hi != m.hi) {
        if (fails++ < 5) printf("b128 shift mismatch %d k=%d\n", i, k);
      }
    }
    f162 x = {r64(), r64(), r64() & F162_TOP_MASK}, y = {r64(), r64(), r64() & F162_TOP_MASK};
    if (i % 97 == 0) x.w2 = F162_TOP_MASK, y.w2 = F162_TOP_MASK;
    f162 z = f162_mul(x, y);
    uint8_t xb[24], yb[24], zb[24];
    memcpy(xb, &x, 24), memcpy(yb, &y, 24);
    lfo_f162_mul(xb, yb, zb, 1);
    ++cases;
    if (memcmp(zb, &z, 24)) {
      if (fails++ < 5) printf("f162 mismatch %d\n", i);
    }
    f162 zl = f162_mul_lifted(x, a);
    f162 la = f162_lift(a);
    memcpy(yb, &la, 24);
    lfo_f162_mul(xb, yb, zb, 1);
    ++cases;
    if (memcmp(zb, &zl, 24)) {
      if (fails++ < 5) printf("f162 lifted mismatch %d\n", i);
    }
  }
  // BLAKE3 modes, lengths across block and chunk boundaries, output seeks.
  std::vector<uint8_t> data(9000);
  for (auto& d : data) d = (uint8_t)r64();
  uint8_t key[32];
  for (auto& k : key) k = (uint8_t)r64();
  const size_t lens[] = {0, 1, 63, 64, 65, 127, 128, 1023, 1024, 1025, 2047, 2048, 2049, 3072, 4097, 8192, 9000};
  for (size_t n : lens)
    for (int mode = 0; mode < 3; ++mode) {
      bk::Hasher h;
      if (mode == 0) h.init();
      if (mode == 1) h.init_keyed(key);
      if (mode == 2) h.init_derive("lf test context", 15);
      // absorb in uneven pieces
      size_t at = 0, step = 1;
      while (at < n) {
        size_t t = std::min(step, n - at);
        h.absorb(data.data() + at, t);
        at += t;
        step = step * 3 + 1;
      }
      for (uint64_t seek : {0ull, 3ull, 64ull, 1000ull}) {
        uint8_t got[200], want[200];
        h.finish().root_bytes(seek, got, sizeof got);
        lfo_blake3(mode == 1 ? key : nullptr, mode == 2 ? "lf test context" : nullptr, data.data(), n, seek, want,
                   sizeof want);
        ++cases;
        if (memcmp(got, want, sizeof got)) {
          if (fails++ < 10) printf("blake3 mismatch mode %d len %zu seek %llu\n", mode, n, (unsigned long long)seek);
        }
      }
    }
  // The transcript's large absorb as the device does it: chunk chaining values of all complete
  // chunks but the last, merged into the complete subtrees (set bits of the count), then the tail.
  for (size_t total : {112ull, 1024ull, 1136ull, 2048ull, 5000ull, 8192ull, 9000ull}) {
    bk::Hasher ref;
    ref.init();
    ref.absorb(data.data(), total);
    uint64_t nchunks = (total - 1) / 1024;
    std::vector<std::vector<uint32_t>> cvs;
    for (uint64_t c = 0; c < nchunks; ++c) {
      bk::Chunk ch;
      ch.start(ref.key, c, 0);
      ch.absorb(data.data() + 1024 * c, 1024);
      std::vector<uint32_t> cv(8);
      ch.pending().cv(cv.data());
      cvs.push_back(cv);
    }
    bk::Hasher dev;
    dev.init();
    uint64_t off = 0;
    int d = 0;
    for (int bit = 63; bit >= 0; --bit) {
      uint64_t size = 1ull << bit;
      if (!(nchunks & size)) continue;
      std::vector<std::vector<uint32_t>> lvl(cvs.begin() + off, cvs.begin() + off + size);
      while (lvl.size() > 1) {
        std::vector<std::vector<uint32_t>> nx;
        for (size_t i = 0; i < lvl.size(); i += 2) {
          std::vector<uint32_t> o(8);
          bk::parent(lvl[i].data(), lvl[i + 1].data(), dev.key, 0, o.data());
          nx.push_back(o);
        }
        lvl.swap(nx);
      }
      memcpy(dev.stack[d++], lvl[0].data(), 32);
      off += size;
    }
    dev.depth = d;
    dev.chunk.start(dev.key, nchunks, 0);
    dev.chunk.absorb(data.data() + 1024 * nchunks, total - 1024 * nchunks);
    dev.absorb(data.data(), 77);
    ref.absorb(data.data(), 77);
    uint8_t a[64], b[64];
    dev.finish().root_bytes(0, a, 64);
    ref.finish().root_bytes(0, b, 64);
    ++cases;
    if (memcmp(a, b, 64)) {
      if (fails++ < 10) printf("subtree absorb mismatch total %zu\n", total);
    }
  }
  if (fails) {
    printf("FAIL %d of %d\n", fails, cases);
    return 1;
  }
  printf("OK %d\n", cases);
  return 0;
}
