// BLAKE3, restated from the published specification (O'Connor, Aumasson, Neves,
// Wilcox-O'Hearn, "BLAKE3: one function, fast everywhere", 2020), for the CPU oracle.
//
// TEST INFRASTRUCTURE: this file belongs to the oracle (the checker). Only tests, the smoke
// check and the CPU-baseline leg of bench.py may link it. The prover library has its own,
// independent implementation.
//
// The reference reaches BLAKE3 through the `blake3` crate 1.8.7 (verifier/proof_verify/Cargo.lock,
// solution/proof_generate/Cargo.lock), which is not vendored under the reference tree. Its call
// sites are: the table PRG (verifier/table_writer/src/main.rs:17-20), the matrix expansion
// (verifier/proof_verify/src/rq.rs:62-78), the transcript (solution-arm/labinius/crates/pcs/
// src/challenge.rs:226-341) and the challenge sign key (challenge.rs:417-449).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cstring>

namespace b3 {

enum : uint32_t {
  CHUNK_START = 1u << 0,
  CHUNK_END = 1u << 1,
  PARENT = 1u << 2,
  ROOT = 1u << 3,
  KEYED_HASH = 1u << 4,
  DERIVE_KEY_CONTEXT = 1u << 5,
  DERIVE_KEY_MATERIAL = 1u << 6,
};
constexpr size_t BLOCK_LEN = 64;
constexpr size_t CHUNK_LEN = 1024;

extern const uint32_t IV[8];

// One compression: the 16 output words.
void compress(const uint32_t cv[8], const uint32_t block[16], uint64_t counter, uint32_t block_len,
              uint32_t flags, uint32_t out[16]);

// The pending last node of a tree: enough state to produce a chaining value or root output.
struct Node {
  uint32_t cv[8];
  uint32_t block[16];
  uint64_t counter;
  uint32_t block_len;
  uint32_t flags;
  void chaining_value(uint32_t out[8]) const;
  // Root output bytes [offset, offset + n) of the extendable output.
  void root_bytes(uint64_t offset, uint8_t* out, size_t n) const;
};

struct ChunkState {
  uint32_t cv[8];
  uint64_t chunk_counter;
  uint8_t buf[BLOCK_LEN];
  uint32_t buf_len;
  uint32_t blocks_compressed;
  uint32_t flags;
  void init(const uint32_t key[8], uint64_t counter, uint32_t flags);
  size_t len() const { return BLOCK_LEN * blocks_compressed + buf_len; }
  void update(const uint8_t* in, size_t n);
  Node output() const;
};

// An incremental hasher over a byte stream.
struct Hasher {
  uint32_t key[8];
  ChunkState chunk;
  uint32_t stack[54][8];
  uint32_t stack_len;
  uint32_t flags;

  void init_plain();
  void init_keyed(const uint8_t key32[32]);
  void init_derive_key(const char* context);
  void update(const void* in, size_t n);
  Node finalize_node() const;
  void finalize(uint8_t* out, size_t n) const { finalize_node().root_bytes(0, out, n); }
  uint64_t count() const { return chunk.chunk_counter * CHUNK_LEN + chunk.len(); }

 private:
  void add_chunk_cv(const uint32_t cv[8], uint64_t total_chunks);
};

// A buffered reader over a root output (the XOF).
struct Reader {
  Node node;
  uint64_t pos;  // next byte offset of the output stream
  void fill(uint8_t* out, size_t n) {
    node.root_bytes(pos, out, n);
    pos += n;
  }
};

void parent_cv(const uint32_t left[8], const uint32_t right[8], const uint32_t key[8], uint32_t flags,
               uint32_t out[8]);

}  // namespace b3
