// Internal declarations shared by the prover's translation units (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <atomic>
#include <string>
#include <vector>

#include "lf_field.cuh"

namespace lf {

typedef unsigned __int128 u128;

// Raises a kernel's dynamic shared-memory limit once per device (idempotent; concurrent first
// calls from several lanes may both set it, which is harmless).
template <class K>
inline void smem_limit(K kernel, int bytes, std::atomic<unsigned long long>& done) {
  int dev = 0;
  cudaGetDevice(&dev);
  const unsigned long long bit = 1ull << (dev & 63);
  if (!(done.load(std::memory_order_acquire) & bit)) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    done.fetch_or(bit, std::memory_order_release);
  }
}

constexpr int RING_N = 648;      // degree of R_Q = Z_Q[X]/(X^648 - X^324 + 1)
constexpr int LEAVES = 162;      // slots of the transform over Y = X^4
constexpr int COLUMN_LOG = 10;   // verifier/proof_verify/src/main.rs:37
constexpr int COLUMNS = 1 << COLUMN_LOG;
constexpr int MAX_PRIMES = 12;
constexpr int STREAM_PREFIX = 112;  // transcript bytes before the commitment (see host code)

// The shape of one instance, derived from LOG_VARS (main.rs:32-46).
struct Shape {
  int log_vars = 0, lp = 0, rl = 0;
  size_t words = 0, column_len = 0, ring_elements = 0;
  bool set(uint32_t l) {
    if (l < 19 || l > 34) return false;
    log_vars = (int)l;
    lp = log_vars - 7;
    rl = lp - COLUMN_LOG;
    words = (size_t)1 << lp;
    column_len = (size_t)1 << rl;
    ring_elements = column_len / 4;
    return true;
  }
};

// One transform prime p = 1 (mod 486): the 162-point transform of Z_p[Y]/(Y^162 - Y^81 + 1).
struct PrimePlan {
  uint32_t p;
  uint32_t eta;                 // primitive 486th root of unity
  std::vector<uint32_t> pw;     // eta^i, i < 486
  // Node exponents (in powers of eta) of the 80 internal radix-3 nodes, level by level:
  // level 1: 2 nodes (length 81), level 2: 6 (27), level 3: 18 (9), level 4: 54 (3).
  std::vector<uint32_t> node_e[5];
  uint32_t leaf_e[LEAVES];      // slot s holds the evaluation at Y = eta^leaf_e[s]
};
bool make_plan(uint32_t p, PrimePlan& out);

// Device-side constants of one prime, uploaded once per modulus.
struct PrimeConst {
  uint32_t p, bar;                 // bar = floor(2^32 / p)
  uint32_t om;                     // cube root of unity eta^162
  uint32_t itw[80][2];             // inverse twiddles eta^-(e/3), eta^-(2e/3) per internal node
  uint32_t inv3, iom, iom2;        // 1/3, omega^-1, omega^-2
  uint32_t w, w5, inv_split;       // eta^81, eta^405, 1/(eta^81 - eta^405)
  uint32_t fw[80][2];              // forward twiddles per internal node (key transform)
  uint32_t leaf_root[LEAVES];      // eta^leaf_e[s]
  uint32_t reduce_every;           // elements the commitment epilogue may accumulate before reducing
};

struct ModulusPlan {
  u128 q = 0;
  uint32_t width = 0, bits = 0;    // coefficient bytes and bits (rq.rs:40-48)
  int nprimes = 0;
  uint32_t primes[MAX_PRIMES];
  bool exact_lift = false;         // true: CRT gives the integer product, reduced mod q after
  u128 p_mod_q = 0;                // product of the primes mod q (exact lift: negative values)
  uint32_t half_digits[MAX_PRIMES];  // floor(product / 2) in the primes' mixed radix (sign test)
  std::vector<PrimeConst> consts;
  const PrimeConst* dconsts = nullptr;  // device copy of consts, owned by the key that holds the plan
  // Per prime and third of its leaves, the Vandermonde limbs of the tensor-core commitment
  // (bf16 bits in the MMA's shared-memory layout).
  std::vector<uint16_t> btiles;
  // Garner constants: inv[i][j] = p_j^-1 mod p_i for j < i
  uint32_t garner_inv[MAX_PRIMES][MAX_PRIMES];
};
// The commitment's primes for modulus q at `elements` ring elements per column: for the baseline
// Q = 3889 * 9721 * 17497 its three factors (CRT gives the value mod q directly); for any other
// q, primes p = 1 (mod 486) below 2^15, largest first, until their product exceeds twice the
// largest |coefficient| of the integer product (elements * 1296 * (q - 1)).
// extra_bits widens the bound (the verifier's a_times_v multiplies by |v| <= 2^15).
bool make_modulus_plan(u128 q, uint64_t elements, int extra_bits, ModulusPlan& mp, std::string& err);

struct ProveProfile {
  double key_ms, commit_ms, finish_ms, transcript_ms, partials_ms, switch_ms, row_ms, challenges_ms,
      fold_ms, encode_ms, total_ms;
};

// Three limb arrays of F162 values (structure of arrays, coalesced per limb).
struct Soa {
  uint64_t *w0, *w1, *w2;
#ifdef __CUDACC__
  __device__ __forceinline__ f162 get(uint64_t i) const { return {w0[i], w1[i], w2[i]}; }
  __device__ __forceinline__ void put(uint64_t i, f162 v) const { w0[i] = v.w0, w1[i] = v.w1, w2[i] = v.w2; }
#endif
};

// A short challenge (challenge.rs:407-415): sorted positions, sign bits, weight.
struct Challenge {
  uint8_t positions[32];
  uint32_t signs;
  uint32_t weight;
};

// ---- launch wrappers (lf_switch.cu) ----
void launch_eq_b128(const b128* r, int n, b128* out, cudaStream_t s);
void launch_eq_table_f162(const f162* ps, int n, f162* out, cudaStream_t s);
// S blocks: E_lo (4096 GHASH entries) as 16-byte words; each block expands the k-tile's rows itself.
void launch_sblock(const uint4* table, uint64_t nblocks, const b128* elo, uint8_t* sblk, int* status,
                   cudaStream_t s);
void launch_partials_combine(const b128* ehi, const uint8_t* sblk, int nblocks, unsigned long long* v, cudaStream_t s);
void launch_psi_tables(const f162* batch, f162* tab, cudaStream_t s);
void launch_rblock_level(const b128* in, uint64_t nout, b128 rho, b128* out, cudaStream_t s);
// The round-message kernels: msg = 7 device words (6 accumulators + a block count, zero between
// rounds; the last block clears them), out = 6 words the message is forwarded to (mapped host
// memory).
void launch_switch_round_blocks(const b128* R, uint64_t X, b128 rho, const f162* phi, const f162* w,
                                unsigned long long* msg, unsigned long long* out, int sms, cudaStream_t s);
// After block round r: psi_next = the byte tables of Phi_{r+1} (from those of Phi_r, rho = r_hi[r],
// the challenge rp) and wn = the weights w_{r+1} of the 2X entries (from w_r).
void launch_round_update(const f162* psi, b128 rho, f162 rp, f162* psi_next, const f162* w, uint64_t X, f162* wn,
                         cudaStream_t s);
void launch_phi_apply(const b128* e, uint64_t n, const f162* phi, Soa a, cudaStream_t s);
void launch_materialize(const uint4* table, const f162* w, uint64_t X, Soa p, int sms, cudaStream_t s);
void launch_switch_msg(Soa a, Soa p, uint64_t half, unsigned long long* msg, unsigned long long* out, int sms,
                       cudaStream_t s);
void launch_switch_fold(Soa a, Soa p, uint64_t half, f162 r, int sms, cudaStream_t s);
// The fold of a round (half pairs) and the message of the next (half / 2 pairs) in one launch.
void launch_switch_fold_msg(Soa a, Soa p, uint64_t half, f162 r, unsigned long long* msg, unsigned long long* out,
                            int sms, cudaStream_t s);

// ---- launch wrappers (lf_open.cu) ----
void launch_row_eval(const uint4* table, int rl, const f162* eqt, f162* row, int sms, cudaStream_t s);
struct HasherImage;  // a bk::Hasher copied to the device
// PHASE[162][88] as f64 re, f64 im, f32 re, f32 im, one after the other.
constexpr size_t PHASE_TABLE_BYTES = 162 * 88 * (8 + 8 + 4 + 4);
// Returns the launch's own status (cudaLaunchKernel), not the thread's last error.
cudaError_t launch_challenges(const void* hasher_dev, uint64_t base_counter, const uint32_t sign_key[8],
                              const void* phase, Challenge* out, int n, int* status, cudaStream_t s,
                              uint32_t* dbg = nullptr);
int fold_splits(uint64_t ring_elements, int sms);
constexpr size_t FOLD_STRIP_BYTES = 2 * 26 * 128;  // per column: the low and the high range's strips
void launch_fold(const uint4* table, int rl, uint64_t ring_elements, const Challenge* ch, uint8_t* strips,
                 int32_t* part, int splits, int32_t* out, int* status, cudaStream_t s);
void launch_chunk_cvs(const uint8_t* stream, uint64_t nchunks, const uint32_t key[8], uint32_t mode, uint32_t* cvs,
                      cudaStream_t s);
// Reduce nchunks chunk values to the chaining values of the complete subtrees of the stream
// (largest first, sizes = set bits of nchunks); returns them in out (at most 64 x 8 words).
void launch_subtrees(uint32_t* cvs, uint32_t* scratch, uint64_t nchunks, const uint32_t key[8], uint32_t mode,
                     uint32_t* out, cudaStream_t s);

// One device write of zero per 4 KB of a host buffer the device reaches through the host's page
// tables (and its last byte), so later copies into it find the pages already mapped for the device.
void launch_touch_pages(uint8_t* host, size_t n, cudaStream_t s);

// ---- launch wrappers (lf_commit.cu) ----
// The public matrix reduced modulo each prime: ared[prime][m][648].
// scratch: matrix_scratch_bytes(elements, q) bytes of device memory.
void launch_matrix_expand(const ModulusPlan& mp, uint64_t elements, uint32_t* ared, void* scratch, cudaStream_t s);
// The public matrix itself: elements x 648 coefficients in [0, q) as u128 little-endian.
void launch_matrix_raw(u128 q, uint64_t elements, void* out, void* scratch, cudaStream_t s);
size_t matrix_scratch_bytes(uint64_t elements, u128 q);
// Leaf-form key: key[prime][m][162][16] u16.
void launch_key_transform(const ModulusPlan& mp, uint64_t elements, const uint32_t* ared, uint32_t* leafvals,
                          uint32_t* key, cudaStream_t s);
int commit_splits(uint64_t elements, int nprimes, int sms);
// Splits [split_begin, split_end) of the `splits` element splits (split_end < 0: all of them).
// ready (device, may be null): the table is still being copied in parts of part_elems ring
// elements (of every column); part i may be read once ready[i] - epoch >= 0 (as int32), and a
// block gives up waiting for it after ready_wait SM cycles (0: about a second), setting *status = 3.
void launch_commit(const ModulusPlan& mp, const Shape& sh, const uint4* table, const uint32_t* key,
                   const uint16_t* btiles, uint32_t* partial, int splits, int* status, cudaStream_t s,
                   int split_begin = 0, int split_end = -1, const uint32_t* ready = nullptr, uint32_t epoch = 0,
                   int part_elems = 0, long long ready_wait = 0);
void commit_split_elements(uint64_t elements, int splits, int s0, int s1, uint64_t& m0, uint64_t& m1);
// Blocks of the commitment's grid per element split (they run one split after another).
int commit_blocks_per_split(const ModulusPlan& mp);
void launch_commit_finish(const ModulusPlan& mp, const Shape& sh, const uint32_t* partial, int splits, uint8_t* out,
                          cudaStream_t s, int ncols = COLUMNS);
// Verifier pieces (lf_commit.cu): a_times_v into `out` (648 coefficients of `width` bytes) and
// challenge_combination's partial sums [32 column runs][1295] as signed 128-bit (lo, hi).
void launch_a_times_v(const ModulusPlan& mp, const Shape& sh, const int32_t* v, const uint32_t* key, uint32_t* vred,
                      uint32_t* vhat, uint32_t* partial, uint8_t* out, cudaStream_t s);
void launch_challenge_combination(const uint8_t* commit, uint32_t width, const Challenge* ch,
                                  unsigned long long* part, cudaStream_t s);
// The checker's scans of the folded witness (elements x 648 int32): out[0..2] = sum over (m, k) of
// e0[4 m + k] times the F162 of bit 0 of v[m][4 pp + k], out[3] = sum v^2, out[4] = max v + 2^31,
// out[5] = 2^31 - min v; out zeroed by the caller.
void launch_fold_checks(const int32_t* v, uint64_t elements, const f162* e0, unsigned long long* out, cudaStream_t s);
// *flag |= 1 when one of the n commitment coefficients (w bytes LE) is not below q.
void launch_commit_range(const uint8_t* commit, uint32_t w, u128 q, uint64_t n, unsigned long long* flag,
                         cudaStream_t s);

}  // namespace lf
