// BLAKE3 restated from the published specification; see blake3_spec.h.
// TEST INFRASTRUCTURE (oracle only).
#include "blake3_spec.h"

namespace b3 {

const uint32_t IV[8] = {0x6A09E667u, 0xBB67AE85u, 0x3C6EF372u, 0xA54FF53Au,
                        0x510E527Fu, 0x9B05688Cu, 0x1F83D9ABu, 0x5BE0CD19u};

// The message word schedule applied between rounds (specification, section 2.2).
static const uint8_t SCHEDULE[16] = {2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8};

static inline uint32_t rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

static inline void quarter(uint32_t* v, int a, int b, int c, int d, uint32_t x, uint32_t y) {
  v[a] = v[a] + v[b] + x;
  v[d] = rotr(v[d] ^ v[a], 16);
  v[c] = v[c] + v[d];
  v[b] = rotr(v[b] ^ v[c], 12);
  v[a] = v[a] + v[b] + y;
  v[d] = rotr(v[d] ^ v[a], 8);
  v[c] = v[c] + v[d];
  v[b] = rotr(v[b] ^ v[c], 7);
}

void compress(const uint32_t cv[8], const uint32_t block[16], uint64_t counter, uint32_t block_len,
              uint32_t flags, uint32_t out[16]) {
  uint32_t v[16] = {cv[0], cv[1], cv[2], cv[3], cv[4], cv[5], cv[6], cv[7],
                    IV[0], IV[1], IV[2], IV[3], (uint32_t)counter, (uint32_t)(counter >> 32),
                    block_len, flags};
  uint32_t m[16];
  memcpy(m, block, sizeof m);
  for (int round = 0; round < 7; ++round) {
    quarter(v, 0, 4, 8, 12, m[0], m[1]);
    quarter(v, 1, 5, 9, 13, m[2], m[3]);
    quarter(v, 2, 6, 10, 14, m[4], m[5]);
    quarter(v, 3, 7, 11, 15, m[6], m[7]);
    quarter(v, 0, 5, 10, 15, m[8], m[9]);
    quarter(v, 1, 6, 11, 12, m[10], m[11]);
    quarter(v, 2, 7, 8, 13, m[12], m[13]);
    quarter(v, 3, 4, 9, 14, m[14], m[15]);
    if (round < 6) {
      uint32_t t[16];
      for (int i = 0; i < 16; ++i) t[i] = m[SCHEDULE[i]];
      memcpy(m, t, sizeof m);
    }
  }
  for (int i = 0; i < 8; ++i) {
    out[i] = v[i] ^ v[i + 8];
    out[i + 8] = v[i + 8] ^ cv[i];
  }
}

static void words_from_bytes(const uint8_t* in, uint32_t* out, int n) {
  for (int i = 0; i < n; ++i)
    out[i] = (uint32_t)in[4 * i] | ((uint32_t)in[4 * i + 1] << 8) | ((uint32_t)in[4 * i + 2] << 16) |
             ((uint32_t)in[4 * i + 3] << 24);
}

void Node::chaining_value(uint32_t out[8]) const {
  uint32_t w[16];
  compress(cv, block, counter, block_len, flags, w);
  memcpy(out, w, 32);
}

void Node::root_bytes(uint64_t offset, uint8_t* out, size_t n) const {
  uint64_t blk = offset / 64;
  size_t skip = (size_t)(offset % 64);
  while (n > 0) {
    uint32_t w[16];
    compress(cv, block, blk, block_len, flags | ROOT, w);
    uint8_t bytes[64];
    for (int i = 0; i < 16; ++i) {
      bytes[4 * i] = (uint8_t)w[i];
      bytes[4 * i + 1] = (uint8_t)(w[i] >> 8);
      bytes[4 * i + 2] = (uint8_t)(w[i] >> 16);
      bytes[4 * i + 3] = (uint8_t)(w[i] >> 24);
    }
    size_t take = 64 - skip;
    if (take > n) take = n;
    memcpy(out, bytes + skip, take);
    out += take;
    n -= take;
    skip = 0;
    ++blk;
  }
}

void ChunkState::init(const uint32_t key[8], uint64_t counter, uint32_t f) {
  memcpy(cv, key, 32);
  chunk_counter = counter;
  memset(buf, 0, sizeof buf);
  buf_len = 0;
  blocks_compressed = 0;
  flags = f;
}

void ChunkState::update(const uint8_t* in, size_t n) {
  while (n > 0) {
    if (buf_len == BLOCK_LEN) {
      uint32_t words[16], w[16];
      words_from_bytes(buf, words, 16);
      compress(cv, words, chunk_counter, BLOCK_LEN, flags | (blocks_compressed == 0 ? CHUNK_START : 0),
               w);
      memcpy(cv, w, 32);
      ++blocks_compressed;
      buf_len = 0;
      memset(buf, 0, sizeof buf);
    }
    size_t take = BLOCK_LEN - buf_len;
    if (take > n) take = n;
    memcpy(buf + buf_len, in, take);
    buf_len += (uint32_t)take;
    in += take;
    n -= take;
  }
}

Node ChunkState::output() const {
  Node o;
  memcpy(o.cv, cv, 32);
  uint8_t padded[64] = {0};
  memcpy(padded, buf, buf_len);
  words_from_bytes(padded, o.block, 16);
  o.counter = chunk_counter;
  o.block_len = buf_len;
  o.flags = flags | (blocks_compressed == 0 ? CHUNK_START : 0) | CHUNK_END;
  return o;
}

void parent_cv(const uint32_t left[8], const uint32_t right[8], const uint32_t key[8], uint32_t flags,
               uint32_t out[8]) {
  Node n;
  memcpy(n.cv, key, 32);
  memcpy(n.block, left, 32);
  memcpy(n.block + 8, right, 32);
  n.counter = 0;
  n.block_len = BLOCK_LEN;
  n.flags = PARENT | flags;
  n.chaining_value(out);
}

void Hasher::init_plain() {
  memcpy(key, IV, 32);
  flags = 0;
  chunk.init(key, 0, flags);
  stack_len = 0;
}

void Hasher::init_keyed(const uint8_t key32[32]) {
  words_from_bytes(key32, key, 8);
  flags = KEYED_HASH;
  chunk.init(key, 0, flags);
  stack_len = 0;
}

void Hasher::init_derive_key(const char* context) {
  Hasher ctx;
  memcpy(ctx.key, IV, 32);
  ctx.flags = DERIVE_KEY_CONTEXT;
  ctx.chunk.init(ctx.key, 0, ctx.flags);
  ctx.stack_len = 0;
  ctx.update(context, strlen(context));
  uint8_t ck[32];
  ctx.finalize(ck, 32);
  words_from_bytes(ck, key, 8);
  flags = DERIVE_KEY_MATERIAL;
  chunk.init(key, 0, flags);
  stack_len = 0;
}

void Hasher::add_chunk_cv(const uint32_t cv_in[8], uint64_t total_chunks) {
  uint32_t cv[8];
  memcpy(cv, cv_in, 32);
  while ((total_chunks & 1) == 0) {
    --stack_len;
    parent_cv(stack[stack_len], cv, key, flags, cv);
    total_chunks >>= 1;
  }
  memcpy(stack[stack_len], cv, 32);
  ++stack_len;
}

void Hasher::update(const void* in_v, size_t n) {
  const uint8_t* in = (const uint8_t*)in_v;
  while (n > 0) {
    if (chunk.len() == CHUNK_LEN) {
      uint32_t cv[8];
      chunk.output().chaining_value(cv);
      uint64_t total = chunk.chunk_counter + 1;
      add_chunk_cv(cv, total);
      chunk.init(key, total, flags);
    }
    size_t take = CHUNK_LEN - chunk.len();
    if (take > n) take = n;
    chunk.update(in, take);
    in += take;
    n -= take;
  }
}

Node Hasher::finalize_node() const {
  Node out = chunk.output();
  for (uint32_t i = stack_len; i-- > 0;) {
    uint32_t right[8];
    out.chaining_value(right);
    Node p;
    memcpy(p.cv, key, 32);
    memcpy(p.block, stack[i], 32);
    memcpy(p.block + 8, right, 32);
    p.counter = 0;
    p.block_len = BLOCK_LEN;
    p.flags = PARENT | flags;
    out = p;
  }
  return out;
}

}  // namespace b3
