// CPU oracle for the Labinius opening prover: a plain restatement of the reference prover and
// verifier (verifier/proof_verify/src/{main,reference,rq}.rs and the `labinius` library pieces
// they call), parameterised in LOG_VARS so that small shapes run in seconds.
//
// TEST INFRASTRUCTURE. This is the checker, not the product: only tests/, the smoke check of
// __graft_entry__.py and the cpu_baseline / reference leg of bench.py load it. The prover library
// (liblabinius_gpu.so) never links or calls it.
#pragma once
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LFO_OK 0
#define LFO_E_ARGS -1
#define LFO_E_SHAPE -2
#define LFO_E_MODULUS -3
#define LFO_E_CAP -4
#define LFO_E_REJECT -5

// BLAKE3 of `in` (plain, keyed when key32 != NULL, derive-key when ctx != NULL), `n_out` bytes of
// extendable output starting at output byte `seek`.
int lfo_blake3(const uint8_t* key32, const char* ctx, const uint8_t* in, size_t n, uint64_t seek,
               uint8_t* out, size_t n_out);
// The input table: keyed BLAKE3 XOF (key = seed) of "labinius-fast/binary-table/v1", 2^log_vars/8 bytes.
int lfo_write_table(const uint8_t seed[32], uint32_t log_vars, uint8_t* out);
// Field products, n pairs: B128 as 16 LE bytes, F162 as three LE u64 (24 bytes).
int lfo_b128_mul(const uint8_t* a, const uint8_t* b, uint8_t* out, size_t n);
int lfo_f162_mul(const uint8_t* a, const uint8_t* b, uint8_t* out, size_t n);
// The public matrix (rq::ajtai_matrix): elements*648 u128 LE.
int lfo_ajtai_matrix(const uint8_t q_le[16], uint64_t elements, uint8_t* out);
// rq::a_times_v (rq.rs:188-217): A v with A = ajtai_matrix(q, elements) and v the elements*648
// signed coefficients; out = 648 u128 LE in [0, q).
int lfo_a_times_v(const uint8_t q_le[16], uint64_t elements, const int16_t* v, uint8_t* out);
// Bytes of one proof at this modulus and shape.
size_t lfo_proof_size(const uint8_t q_le[16], uint32_t log_vars);
// The commitment bytes of `table` (schoolbook when mode == 0, 3-prime transforms when mode == 1
// and the modulus is 3889*9721*17497).
int lfo_commit(const uint8_t q_le[16], uint32_t log_vars, const uint8_t* table, int mode, uint8_t* out);
// The reference prover. `trace`, when not NULL, receives the intermediate values (see oracle.cc).
int lfo_prove(const uint8_t seed[32], const uint8_t q_le[16], uint32_t log_vars, const uint8_t* table,
              int commit_mode, uint8_t* proof, size_t cap, size_t* len, uint8_t* trace, size_t trace_cap);
// The same proof with the packed point coordinates r_hi (LOG_VARS - 7 GHASH elements, 16 bytes LE
// each) in place of the sampled ones: the generic switch (crossfield.rs:600-634) at any point,
// including coordinates equal to one (solution/proof_generate/src/main.rs:1929-1962).
int lfo_prove_at_point(const uint8_t seed[32], const uint8_t q_le[16], uint32_t log_vars, const uint8_t* table,
                       const uint8_t* r_hi, uint8_t* proof, size_t cap, size_t* len);
// The checker, shape-parameterised. table == NULL regenerates the table from the seed.
// Returns LFO_OK or LFO_E_REJECT with a message in err.
int lfo_verify(const uint8_t seed[32], uint32_t log_vars, const uint8_t* table, const uint8_t* proof,
               size_t len, char* err, size_t err_cap);
// Modulus gate (main.rs:85-96) at this shape: 0 accept, LFO_E_MODULUS refuse.
int lfo_accept_modulus(const uint8_t q_le[16], uint32_t log_vars);
uint64_t lfo_fold_cap(uint32_t log_vars);
// Short challenges: n challenges sampled after absorbing `prefix` into Transcript::new(domain).
// Each challenge is 32 position bytes, u32 signs, u32 weight (40 bytes).
int lfo_short_challenges(const char* domain, const uint8_t* prefix, size_t prefix_len, uint32_t n,
                         uint8_t* out);
// max_u |c(zeta^u)|^2 by the blocked accumulation and by Horner over all 162 roots.
double lfo_norm_blocked(const uint8_t positions[32], uint32_t signs, uint32_t weight);
double lfo_norm_horner(const uint8_t positions[32], uint32_t signs, uint32_t weight);
void lfo_set_threads(int n);

#ifdef __cplusplus
}
#endif
