// BLAKE3 for the prover, host and device, from the published specification (BLAKE3 paper,
// sections 2.1-2.6): the compression function, 1024-byte chunks, the binary tree of parent nodes,
// the keyed and derive-key modes and the extendable output.
//
// The reference reaches BLAKE3 through the un-vendored `blake3` crate 1.8.7; its uses are the
// transcript (solution-arm/labinius/crates/pcs/src/challenge.rs:60-341), the public matrix
// (verifier/proof_verify/src/rq.rs:53-91), the input table (verifier/table_writer/src/main.rs:17-20)
// and the challenge signs (challenge.rs:417-449).
#pragma once
#include <stdint.h>
#include <string.h>

#include "lf_field.cuh"

namespace lf {
namespace bk {

enum : uint32_t {
  F_CHUNK_START = 1,
  F_CHUNK_END = 2,
  F_PARENT = 4,
  F_ROOT = 8,
  F_KEYED = 16,
  F_DERIVE_CTX = 32,
  F_DERIVE_MAT = 64,
};

#ifdef __CUDACC__
#define LF_CONST_TABLE __host__ __device__
#endif

LF_HD uint32_t iv(int i) {
  const uint32_t v[8] = {0x6A09E667u, 0xBB67AE85u, 0x3C6EF372u, 0xA54FF53Au,
                         0x510E527Fu, 0x9B05688Cu, 0x1F83D9ABu, 0x5BE0CD19u};
  return v[i];
}

LF_HD uint32_t rot(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

#define LF_G(a, b, c, d, x, y)    \
  do {                            \
    s[a] = s[a] + s[b] + (x);     \
    s[d] = rot(s[d] ^ s[a], 16);  \
    s[c] = s[c] + s[d];           \
    s[b] = rot(s[b] ^ s[c], 12);  \
    s[a] = s[a] + s[b] + (y);     \
    s[d] = rot(s[d] ^ s[a], 8);   \
    s[c] = s[c] + s[d];           \
    s[b] = rot(s[b] ^ s[c], 7);   \
  } while (0)

// The 16 output words of one compression. The message words are re-indexed each round by the
// permutation of the specification, applied cumulatively.
LF_HD void compress16(const uint32_t h[8], const uint32_t m_in[16], uint64_t t, uint32_t len, uint32_t flags,
                      uint32_t out[16]) {
  uint32_t s[16];
#pragma unroll
  for (int i = 0; i < 8; ++i) s[i] = h[i];
  s[8] = iv(0), s[9] = iv(1), s[10] = iv(2), s[11] = iv(3);
  s[12] = (uint32_t)t, s[13] = (uint32_t)(t >> 32), s[14] = len, s[15] = flags;
  uint32_t m[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) m[i] = m_in[i];
#pragma unroll
  for (int r = 0; r < 7; ++r) {
    LF_G(0, 4, 8, 12, m[0], m[1]);
    LF_G(1, 5, 9, 13, m[2], m[3]);
    LF_G(2, 6, 10, 14, m[4], m[5]);
    LF_G(3, 7, 11, 15, m[6], m[7]);
    LF_G(0, 5, 10, 15, m[8], m[9]);
    LF_G(1, 6, 11, 12, m[10], m[11]);
    LF_G(2, 7, 8, 13, m[12], m[13]);
    LF_G(3, 4, 9, 14, m[14], m[15]);
    if (r < 6) {
      uint32_t p[16] = {m[2], m[6],  m[3],  m[10], m[7],  m[0],  m[4],  m[13],
                        m[1], m[11], m[12], m[5],  m[9],  m[14], m[15], m[8]};
#pragma unroll
      for (int i = 0; i < 16; ++i) m[i] = p[i];
    }
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    out[i] = s[i] ^ s[i + 8];
    out[i + 8] = s[i + 8] ^ h[i];
  }
}
#undef LF_G

LF_HD void load_words(const uint8_t* b, uint32_t* w, int n) {
  for (int i = 0; i < n; ++i)
    w[i] = (uint32_t)b[4 * i] | ((uint32_t)b[4 * i + 1] << 8) | ((uint32_t)b[4 * i + 2] << 16) |
           ((uint32_t)b[4 * i + 3] << 24);
}
LF_HD void store_words(const uint32_t* w, uint8_t* b, int n) {
  for (int i = 0; i < n; ++i) {
    b[4 * i] = (uint8_t)w[i];
    b[4 * i + 1] = (uint8_t)(w[i] >> 8);
    b[4 * i + 2] = (uint8_t)(w[i] >> 16);
    b[4 * i + 3] = (uint8_t)(w[i] >> 24);
  }
}

// A node waiting for its last compression: its chaining value, or the root output stream.
struct Pending {
  uint32_t h[8];
  uint32_t m[16];
  uint64_t t;
  uint32_t len;
  uint32_t flags;

  LF_HD void cv(uint32_t out[8]) const {
    uint32_t o[16];
    compress16(h, m, t, len, flags, o);
    for (int i = 0; i < 8; ++i) out[i] = o[i];
  }
  // 64-byte block `index` of the root output, as 16 words.
  LF_HD void root_block(uint64_t index, uint32_t out[16]) const { compress16(h, m, index, len, flags | F_ROOT, out); }
  LF_HD void root_bytes(uint64_t offset, uint8_t* out, uint64_t n) const {
    uint64_t blk = offset >> 6;
    uint32_t skip = (uint32_t)(offset & 63);
    while (n) {
      uint32_t w[16];
      uint8_t b[64];
      root_block(blk, w);
      store_words(w, b, 16);
      uint64_t take = 64 - skip;
      if (take > n) take = n;
      for (uint64_t i = 0; i < take; ++i) out[i] = b[skip + i];
      out += take;
      n -= take;
      skip = 0;
      ++blk;
    }
  }
};

LF_HD void parent(const uint32_t l[8], const uint32_t r[8], const uint32_t key[8], uint32_t mode, uint32_t out[8]) {
  uint32_t m[16];
  for (int i = 0; i < 8; ++i) m[i] = l[i], m[i + 8] = r[i];
  uint32_t o[16];
  compress16(key, m, 0, 64, F_PARENT | mode, o);
  for (int i = 0; i < 8; ++i) out[i] = o[i];
}

// A 1024-byte chunk in progress.
struct Chunk {
  uint32_t h[8];
  uint64_t index;
  uint8_t buf[64];
  uint32_t buf_len;
  uint32_t blocks;
  uint32_t mode;

  LF_HD void start(const uint32_t key[8], uint64_t idx, uint32_t md) {
    for (int i = 0; i < 8; ++i) h[i] = key[i];
    index = idx;
    for (int i = 0; i < 64; ++i) buf[i] = 0;
    buf_len = 0;
    blocks = 0;
    mode = md;
  }
  LF_HD uint32_t size() const { return 64 * blocks + buf_len; }
  LF_HD void absorb(const uint8_t* p, uint64_t n) {
    while (n) {
      if (buf_len == 64) {
        uint32_t m[16], o[16];
        load_words(buf, m, 16);
        compress16(h, m, index, 64, mode | (blocks == 0 ? F_CHUNK_START : 0), o);
        for (int i = 0; i < 8; ++i) h[i] = o[i];
        ++blocks;
        buf_len = 0;
        for (int i = 0; i < 64; ++i) buf[i] = 0;
      }
      uint64_t take = 64 - buf_len;
      if (take > n) take = n;
      for (uint64_t i = 0; i < take; ++i) buf[buf_len + i] = p[i];
      buf_len += (uint32_t)take;
      p += take;
      n -= take;
    }
  }
  LF_HD Pending pending() const {
    Pending o;
    for (int i = 0; i < 8; ++i) o.h[i] = h[i];
    load_words(buf, o.m, 16);
    o.t = index;
    o.len = buf_len;
    o.flags = mode | (blocks == 0 ? F_CHUNK_START : 0) | F_CHUNK_END;
    return o;
  }
};

constexpr int MAX_STACK = 54;

// The incremental hash of a byte stream: the chaining values of the complete subtrees to the
// left (sizes given by the set bits of the number of finished chunks) and the chunk in progress.
struct Hasher {
  uint32_t key[8];
  uint32_t mode;
  uint32_t depth;
  uint32_t stack[MAX_STACK][8];
  Chunk chunk;

  LF_HD void init_with(const uint32_t k[8], uint32_t md) {
    for (int i = 0; i < 8; ++i) key[i] = k[i];
    mode = md;
    depth = 0;
    chunk.start(key, 0, mode);
  }
  LF_HD void init() {
    uint32_t k[8];
    for (int i = 0; i < 8; ++i) k[i] = iv(i);
    init_with(k, 0);
  }
  LF_HD void init_keyed(const uint8_t k32[32]) {
    uint32_t k[8];
    load_words(k32, k, 8);
    init_with(k, F_KEYED);
  }
  // The key of the derive-key mode: the context string hashed under DERIVE_KEY_CONTEXT.
  LF_HD void init_derive(const char* ctx, uint32_t ctx_len) {
    Hasher c;
    uint32_t k[8];
    for (int i = 0; i < 8; ++i) k[i] = iv(i);
    c.init_with(k, F_DERIVE_CTX);
    c.absorb((const uint8_t*)ctx, ctx_len);
    uint8_t out[32];
    c.finish().root_bytes(0, out, 32);
    load_words(out, k, 8);
    init_with(k, F_DERIVE_MAT);
  }
  LF_HD void push_chunk_cv(const uint32_t cv_in[8], uint64_t finished) {
    uint32_t cv[8];
    for (int i = 0; i < 8; ++i) cv[i] = cv_in[i];
    while ((finished & 1) == 0) {
      --depth;
      parent(stack[depth], cv, key, mode, cv);
      finished >>= 1;
    }
    for (int i = 0; i < 8; ++i) stack[depth][i] = cv[i];
    ++depth;
  }
  LF_HD void absorb(const uint8_t* p, uint64_t n) {
    while (n) {
      if (chunk.size() == 1024) {
        uint32_t cv[8];
        chunk.pending().cv(cv);
        uint64_t finished = chunk.index + 1;
        push_chunk_cv(cv, finished);
        chunk.start(key, finished, mode);
      }
      uint64_t take = 1024 - chunk.size();
      if (take > n) take = n;
      chunk.absorb(p, take);
      p += take;
      n -= take;
    }
  }
  LF_HD void absorb_u64(uint64_t x) {
    uint8_t b[8];
    for (int i = 0; i < 8; ++i) b[i] = (uint8_t)(x >> (8 * i));
    absorb(b, 8);
  }
  LF_HD Pending finish() const { return merge_up(chunk.pending()); }
  // The root node over the stack with `out` as the rightmost node (the pending chunk).
  LF_HD Pending merge_up(Pending out) const {
    for (uint32_t i = depth; i-- > 0;) {
      uint32_t right[8];
      out.cv(right);
      Pending p;
      for (int j = 0; j < 8; ++j) p.h[j] = key[j], p.m[j] = stack[i][j], p.m[j + 8] = right[j];
      p.t = 0;
      p.len = 64;
      p.flags = F_PARENT | mode;
      out = p;
    }
    return out;
  }
  LF_HD uint64_t count() const { return chunk.index * 1024 + chunk.size(); }
};

// The root of one transcript derivation (challenge.rs:335-341): the stream so far, then the
// counter (u64 LE), the label length (u64 LE) and the label. The suffix is assembled in one local
// buffer and absorbed in a single call; on sm_103a a sequence of small absorbs from separate local
// arrays (two u64 helpers and a label literal) produced a wrong chaining value, while this form
// matches the host build (tests/dev_blake3_check.cu).
LF_HD Pending derive_root(const Hasher& state, uint64_t counter, const char* label, uint32_t label_len) {
  uint8_t suffix[16 + 64];
  for (int i = 0; i < 8; ++i) suffix[i] = (uint8_t)(counter >> (8 * i));
  for (int i = 0; i < 8; ++i) suffix[8 + i] = (uint8_t)((uint64_t)label_len >> (8 * i));
  for (uint32_t i = 0; i < label_len && i < 64; ++i) suffix[16 + i] = (uint8_t)label[i];
  const uint32_t n = 16 + (label_len < 64 ? label_len : 64);
  if (state.chunk.size() + n <= 1024) {
    // The suffix stays inside the pending chunk: copy only the chunk (not the whole stack) and
    // merge up through the state's own stack.
    Chunk c = state.chunk;
    c.absorb(suffix, n);
    return state.merge_up(c.pending());
  }
  Hasher h = state;
  h.absorb(suffix, n);
  return h.finish();
}

}  // namespace bk
}  // namespace lf
