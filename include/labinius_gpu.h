/* liblabinius_gpu: the GB300 Labinius opening prover behind a C ABI.
 *
 * The boundary is the reference prover's own: `prove(seed, Q, table) -> proof bytes` of
 * solution/proof_generate/src/main.rs:1692-2009 (prove) and :1252-1416 (the bincode layout
 * written by encode_into), reached from the `labinius-fast --prove FILE --table FILE
 * [--modulus Q]` command (main.rs:2050-2090, LABINIUS_SEED in the environment). The proof bytes
 * are the layout of verifier/proof_verify/src/main.rs:98-124.
 *
 * All buffers are caller-owned. Return codes are 0 or one of the negative LF_E_* values.
 * A context is bound to one CUDA device; calls on one context are serialised. */
#ifndef LABINIUS_GPU_H
#define LABINIUS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LF_OK 0
#define LF_E_ARGS (-1)      /* a null or inconsistent argument */
#define LF_E_SHAPE (-2)     /* LOG_VARS outside what the prover supports */
#define LF_E_MODULUS (-3)   /* the modulus fails the checker's gate (main.rs:85-96) or the prover's support */
#define LF_E_TABLE_LEN (-4) /* table bytes != 2^LOG_VARS / 8 (main.rs:143-153) */
#define LF_E_CAP (-5)       /* proof buffer smaller than lf_proof_size() */
#define LF_E_OOM (-6)       /* device memory could not be reserved */
#define LF_E_CUDA (-7)      /* a CUDA call failed; see lf_last_error() */
#define LF_E_INTERNAL (-8)  /* a device-side check failed (challenge sampling bound, fold range) */
#define LF_E_ADMISSION (-9) /* the request does not fit the context's HBM budget */
#define LF_E_LIMIT (-10)    /* the request exceeds a fixed-size scratch (lf_sample_challenges_noalloc) */
#define LF_E_TIMEOUT (-11)  /* lf_poll: the job has not finished within the wait */
#define LF_E_TICKET (-12)   /* lf_poll: no such ticket (never issued, or its result was already taken) */
#define LF_E_REJECT (-13)   /* lf_verify: the proof does not verify; lf_last_error names the check */

typedef struct lf_ctx lf_ctx;

typedef struct lf_config {
  int device;             /* CUDA ordinal */
  size_t hbm_budget;      /* bytes the context may hold on the device; 0 = no limit */
  int lanes;              /* proofs a batch or the serving queue may run at once, each on its own
                             stream and host thread (1..8); 0 = the default, 8 */
} lf_config;

/* Per-phase device times of the last lf_prove* call on a context, in milliseconds
 * (the reference's labinius-profile line, solution/proof_generate/src/main.rs:1999-2007). */
typedef struct lf_profile {
  double upload_ms, key_ms, commit_ms, finish_ms, transcript_ms, partials_ms, switch_ms, row_ms, challenges_ms,
      fold_ms, download_ms, total_ms;
  int launches; /* kernels this library launched for the proof (key preparation excluded when cached) */
  /* switch_ms in three parts: the rounds on the partials' blocks, the materialisation pass, the last
   * 12 rounds (each round's host Fiat-Shamir step included) */
  double switch_blocks_ms, switch_materialize_ms, switch_tail_ms;
} lf_profile;

/* Context lifetime. Replaces the process-wide pool and allocator of the reference prover
 * (solution/labinius/crates/pcs/src/par.rs, solution/proof_generate/src/main.rs:1427-1569). */
int lf_ctx_create(const lf_config* cfg, lf_ctx** out);
void lf_ctx_destroy(lf_ctx* ctx);
/* The context's CUDA stream (a cudaStream_t), on which every kernel and copy of its calls runs, so
 * that a caller can order its own work or timing events with them. No counterpart in the
 * reference (its prover has no device). */
void* lf_ctx_stream(lf_ctx* ctx);

/* Size of the proof for modulus q (16 bytes little-endian) at 2^log_vars table bits; 0 if the
 * shape is unsupported. Replaces ProofLayout::instance (solution/proof_generate/src/main.rs:1252-1310). */
size_t lf_proof_size(const uint8_t q_le[16], uint32_t log_vars);

/* The checker's modulus gate at this shape (verifier/proof_verify/src/main.rs:85-96):
 * LF_OK or LF_E_MODULUS. */
int lf_accept_modulus(const uint8_t q_le[16], uint32_t log_vars);

/* Expand the public matrix A for (q, 2^log_vars) and transform it to the device key; cached on
 * the context and each of its lanes (solution/proof_generate/src/keygen.rs:139-266, build-time key
 * images main.rs:1712-1757). Also grows every device work buffer a proof of this shape uses (a
 * host-table copy included) on the context and its lanes, so that later proofs of the shape
 * allocate and free no device memory (a free waits for the whole device). */
int lf_key_prepare(lf_ctx* ctx, const uint8_t q_le[16], uint32_t log_vars);

/* One proof of the table (host memory, table_bytes = 2^log_vars / 8, little-endian u128 words as
 * the table file holds them) for seed and modulus q. Writes *proof_len bytes into proof.
 * A page-locked table is copied in element ranges that the commitment starts on as they arrive;
 * any other host memory (a mapped file included) is copied whole first. The table must stay
 * unchanged until the call returns.
 * Replaces prove() + Output::write (solution/proof_generate/src/main.rs:1692-2009, 1650-1689). */
int lf_prove(lf_ctx* ctx, const uint8_t seed[32], const uint8_t q_le[16], uint32_t log_vars, const void* table,
             size_t table_bytes, uint8_t* proof, size_t proof_cap, size_t* proof_len);

/* The same with the table already resident in device memory (a device pointer of this context's
 * device). */
int lf_prove_device(lf_ctx* ctx, const uint8_t seed[32], const uint8_t q_le[16], uint32_t log_vars,
                    const void* table_dev, uint8_t* proof, size_t proof_cap, size_t* proof_len);

/* The input table for a seed, written on the device by the table PRG (keyed BLAKE3 XOF,
 * verifier/table_writer/src/main.rs:14-22): 2^log_vars / 8 bytes into out_dev (device memory). */
int lf_write_table_device(lf_ctx* ctx, const uint8_t seed[32], uint32_t log_vars, void* out_dev);

/* Device buffers of the context (for hosts that keep tables resident). */
int lf_device_alloc(lf_ctx* ctx, size_t bytes, void** out_dev);
int lf_device_free(lf_ctx* ctx, void* dev);
int lf_memcpy_h2d(lf_ctx* ctx, void* dst_dev, const void* src, size_t bytes);

int lf_last_profile(lf_ctx* ctx, lf_profile* out);

/* Diagnostics: the 1024 folding challenges of the last proof, 40 bytes each (32 position bytes,
 * u32 sign bits, u32 weight), as sample_short_challenges returns them
 * (solution-arm/labinius/crates/pcs/src/challenge.rs:707-737). The proof itself carries only
 * their effect, the fold. */
int lf_last_challenges(lf_ctx* ctx, uint8_t* out, size_t cap);

/* One proof request. The table is 2^log_vars / 8 bytes, in host memory (copied by the library)
 * or, with table_on_device = 1, a device pointer on the context's GPU. All buffers stay owned by
 * the caller and must stay valid until the job's result is reported. */
typedef struct lf_job {
  const uint8_t* seed; /* 32 bytes */
  const uint8_t* q_le; /* 16 bytes, little-endian */
  uint32_t log_vars;
  int table_on_device;
  const void* table;
  size_t table_bytes;
  uint8_t* proof; /* at least lf_proof_size(q_le, log_vars) bytes */
  size_t proof_cap;
} lf_job;

typedef struct lf_result {
  int status;       /* LF_OK or the job's LF_E_* code */
  size_t proof_len; /* bytes written to the job's proof buffer */
  double queue_ms;  /* submission (or batch start) to the start of the proof */
  double run_ms;    /* start of the proof to its bytes in the proof buffer */
  /* where run_ms went: device time of the proof's own work on its stream (commitment through the
   * proof's download; lf_profile's phases summed), of its commitment kernel, and of the host
   * table's copy on the copy stream (0 for a device table) */
  double device_ms, commit_ms, upload_ms;
} lf_result;

/* Proves n independent jobs (any mix of shapes and moduli; each (Q, shape) key is built once and
 * cached) on the context's GPU. With two or more jobs they run on the lanes of the context
 * (lf_config.lanes, eight by default: one stream and host thread each, taking jobs in order from
 * one counter), so one proof's host work overlaps other proofs' kernels; with one lane the next
 * job's host table is copied on a second stream while the current job is proven. results[i] receives job i's outcome; the return value
 * is LF_OK if every job succeeded, else the first failing job's code.
 * The reference proves one table per process (solution/proof_generate/src/main.rs:2050-2090);
 * this is the batched form of that call. */
int lf_prove_batch(lf_ctx* ctx, size_t n, const lf_job* jobs, lf_result* results);

/* Serving: lf_submit queues a job (FIFO) and returns a ticket. One worker thread per lane of the
 * context (lf_config.lanes) takes requests from the queue: the front request starts when no
 * other request is in flight or when the device footprints (lf_request_footprint) of those in
 * flight and its own fit the context's HBM budget together, so requests that arrive while others
 * are on the GPU overlap them as lanes and memory allow. A job whose own footprint exceeds the budget is refused here with LF_E_ADMISSION.
 * lf_poll waits up to wait_ms (0 = just look) for the
 * ticket: LF_OK with *out filled (the ticket is then retired), LF_E_TIMEOUT while the job is
 * queued or running, LF_E_TICKET for an unknown ticket. lf_ctx_destroy completes the job in
 * progress and reports LF_E_INTERNAL for jobs still queued. No counterpart in the reference. */
int lf_submit(lf_ctx* ctx, const lf_job* job, uint64_t* ticket);
/* Tuning: the commitment kernel's element-split count (its grid depth, the analogue of the
 * reference's commit column-group choice, solution/labinius/crates/pcs/src/simd/commit.rs:98-107)
 * is measured on this device for the shape, using table_dev (a device table of the shape: the
 * result does not depend on its content), over the candidates whose last wave is at least 3/4
 * full; the fastest is kept for this shape and modulus on every lane of the context (the proof
 * bytes do not depend on it). The fold's column-run count (its persistent kernel walks row blocks
 * x runs work units over the SMs) is measured the same way, over the counts whose last round of
 * units fills at least 3/4 of the SMs, and kept for the shape. Without tuning wave-balance
 * heuristics choose both. */
typedef struct lf_tune_result {
  int commit_splits;   /* the count kept */
  float commit_ms;     /* its measured commitment time */
  int candidates;      /* counts measured */
  int fold_splits;     /* the fold's column-run count kept */
  float fold_ms;       /* its measured fold time (strips, product, sum of the runs) */
  int fold_candidates; /* run counts measured */
} lf_tune_result;
int lf_tune(lf_ctx* ctx, const uint8_t q_le[16], uint32_t log_vars, const void* table_dev, lf_tune_result* out);

/* Device bytes one request of this shape and modulus holds while it is proven on this context's
 * GPU (table copy when host_table, key, work buffers, transient key-build buffers): the figure
 * admission compares with the budget. 0 for an unsupported shape or modulus. */
size_t lf_request_footprint(lf_ctx* ctx, const uint8_t q_le[16], uint32_t log_vars, int host_table);
int lf_poll(lf_ctx* ctx, uint64_t ticket, uint32_t wait_ms, lf_result* out);

/* The checker (verifier/proof_verify/src/main.rs:293-409: check_proof_shape, check_field_switch,
 * check_opening) on the GPU: LF_OK if the proof verifies against the table (host memory, or
 * NULL to regenerate the seed's table with the table PRG as main.rs:143-153 does), LF_E_REJECT
 * with the failing check in lf_last_error otherwise. lf_verify_device takes a device table. */
int lf_verify(lf_ctx* ctx, const uint8_t seed[32], uint32_t log_vars, const void* table, size_t table_bytes,
              const uint8_t* proof, size_t proof_len);
int lf_verify_device(lf_ctx* ctx, const uint8_t seed[32], uint32_t log_vars, const void* table_dev, const uint8_t* proof,
                     size_t proof_len);

/* The arithmetic under the commitment, batched on the device (all pointers device memory; each
 * call returns when its work is done on the context's stream).
 *
 * lf_ring_mul: c[i] = a[i] * b[i] in R_Q = Z_Q[X]/(X^648 - X^324 + 1) for i < n, elements of 648
 * little-endian u128 coefficients in [0, Q), any 2 <= Q < 2^96: rq::mul and fold_into_ring
 * (verifier/proof_verify/src/rq.rs:146-186) over many independent pairs. LF_E_ARGS if an operand
 * coefficient is not below Q, LF_E_MODULUS outside the range.
 * lf_ghash_mul: c[i] = a[i] * b[i] in GF(2^128) (GHASH, 16-byte little-endian elements;
 * solution-arm/labinius/crates/pcs/src/fields/scalar.rs:61-72).
 * lf_ajtai_matrix_device: rq::ajtai_matrix(Q, elements) (rq.rs:114-148), elements * 648 u128
 * little-endian coefficients into out_dev.
 * lf_a_times_v: rq::a_times_v (rq.rs:188-217) of ajtai_matrix(Q, elements) and the signed
 * coefficients v_dev (elements * 648 int16), elements a power of two up to 2^15, 2 <= Q < 2^96;
 * `out` (host) receives 648 u128 little-endian coefficients in [0, Q). The key of (Q, elements)
 * is built on first use and cached with the proof keys. */
int lf_ring_mul(lf_ctx* ctx, const uint8_t q_le[16], size_t n, const void* a_dev, const void* b_dev, void* c_dev);
int lf_ghash_mul(lf_ctx* ctx, size_t n, const void* a_dev, const void* b_dev, void* c_dev);
int lf_ajtai_matrix_device(lf_ctx* ctx, const uint8_t q_le[16], uint64_t elements, void* out_dev);
int lf_a_times_v(lf_ctx* ctx, const uint8_t q_le[16], uint64_t elements, const int16_t* v_dev, uint8_t* out);

/* Diagnostics: n folding challenges sampled on the device from Transcript::new(domain) after
 * absorb_bytes(prefix) (challenge.rs:240-259, 707-737), 40 bytes each as above. */
int lf_sample_challenges(lf_ctx* ctx, const char* domain, const uint8_t* prefix, size_t prefix_len, uint32_t n,
                         uint8_t* out);
/* The same, also returning 64 words describing challenge 0's first attempt: the XOF root node
 * (27 words), its first 32 output bytes, the attempt's sorted positions, sign bits, rejection flag
 * and lane 0's squared norm. */
int lf_sample_challenges_traced(lf_ctx* ctx, const char* domain, const uint8_t* prefix, size_t prefix_len, uint32_t n,
                                uint8_t* out, uint32_t* trace64);
/* lf_sample_challenges without a context and without allocating device memory. No counterpart
 * in the reference (its sampler runs on the host, challenge.rs:707-737); it exists for callers
 * that must not allocate on the device. Output as lf_sample_challenges. Limits: 1 <= n <=
 * LF_NOALLOC_MAX_CHALLENGES, larger n returns LF_E_LIMIT before any device work; device < 64.
 * Scratch is one fixed device array per device (just under 512 KB: the 342,144 bytes of phase
 * tables, 40 bytes per challenge slot and the transcript state), shared by all calls: calls are
 * serialised by a process-wide lock and return after `stream` (a cudaStream_t; NULL = the
 * legacy default stream) has drained. The first call on a device locates that array and
 * uploads the phase tables with synchronous copies; make it before any stream of the device
 * begins a capture. The caller's current device is restored on return. */
#define LF_NOALLOC_MAX_CHALLENGES 4096
int lf_sample_challenges_noalloc(int device, const char* domain, const uint8_t* prefix, size_t prefix_len, uint32_t n,
                                 uint8_t* out, void* stream);
/* Test hooks. No counterpart in the reference: they let tests reach paths that seeded inputs
 * reach with negligible probability. Each changes the NEXT proof of this context (lf_prove,
 * lf_prove_device, or a job of lf_prove_batch / lf_submit run on the context itself), once.
 *
 * lf_test_set_point: that proof takes r_hi (n = LOG_VARS - 7 GHASH elements, 16 bytes little-endian
 * each) as the packed coordinates of its evaluation point instead of sampling them ("r-hi",
 * verifier/proof_verify/src/main.rs:177-182). Its transcript then no longer matches the checker's,
 * but every later field of the proof is a deterministic function of that point, so it can be
 * compared with another prover given the same point, e.g. one with a coordinate equal to one,
 * where solution/proof_generate/src/main.rs:1929-1962 switches to its generic prover. n = 0 clears
 * a pending point. LF_E_ARGS from the proof if n does not match its shape.
 *
 * lf_test_withhold_table_part: if that proof streams a page-locked table (lf_prove), the ready flag
 * of element range `part` (0..63; a table is streamed in min(64, ring elements per column / 16) ranges, at least one) is not written, and the commitment kernel gives up waiting for it
 * after wait_cycles SM cycles (0 = its default of about a second): the proof returns LF_E_INTERNAL
 * and the context stays usable. */
int lf_test_set_point(lf_ctx* ctx, const uint8_t* r_hi, uint32_t n);
/* lf_test_table_part_order (host only): the copy order of a streamed table's parts for a
 * commitment grid of `splits` element splits of blocks_per_split blocks each on `sms` SMs, as
 * lf_prove uses it; order receives *nparts part indices (at most 64). */
int lf_test_table_part_order(uint64_t ring_elements, int splits, int blocks_per_split, int sms, uint8_t* order,
                             int* nparts);
int lf_test_withhold_table_part(lf_ctx* ctx, int part, uint64_t wait_cycles);

const char* lf_strerror(int code);
const char* lf_last_error(lf_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif
