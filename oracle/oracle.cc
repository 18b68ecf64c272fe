// CPU oracle: restatement of the reference prover and checker. TEST INFRASTRUCTURE only; see
// oracle.h. Every function names the reference file:line it restates (paths relative to the
// reference project root).
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "blake3_spec.h"

typedef unsigned __int128 u128;
typedef __int128 i128;

namespace {

int g_threads = 0;
int threads() {
  if (g_threads > 0) return g_threads;
  unsigned h = std::thread::hardware_concurrency();
  return h ? (int)h : 1;
}

// Runs fn(begin, end) over [0, n) split into contiguous blocks, one per worker.
template <class F>
void parallel_for(size_t n, F fn, size_t min_per = 1) {
  size_t t = (size_t)threads();
  if (n / min_per < t) t = std::max<size_t>(1, n / min_per);
  if (t <= 1) {
    fn((size_t)0, n);
    return;
  }
  std::vector<std::thread> ws;
  size_t per = (n + t - 1) / t;
  for (size_t i = 0; i < t; ++i) {
    size_t b = i * per, e = std::min(n, b + per);
    if (b >= e) break;
    ws.emplace_back([=] { fn(b, e); });
  }
  for (auto& w : ws) w.join();
}

// ---------------------------------------------------------------------------------------------
// Shape (verifier/proof_verify/src/main.rs:32-46), with LOG_VARS a parameter.
// ---------------------------------------------------------------------------------------------
constexpr int N = 648;           // ring degree, rq.rs:13
constexpr int SPLIT = N / 2;     // rq.rs:15
constexpr int COLUMN_LOG = 10;   // main.rs:37
constexpr int COLUMNS = 1 << COLUMN_LOG;
constexpr int LOG_PACK = 7;      // crossfield.rs:7

struct Shape {
  int log_vars, lp, rl;
  size_t words, column_len, ring_elements;
  bool set(uint32_t l) {
    if (l < 19 || l > 40) return false;
    log_vars = (int)l;
    lp = log_vars - LOG_PACK;
    rl = lp - COLUMN_LOG;
    words = (size_t)1 << lp;
    column_len = (size_t)1 << rl;
    ring_elements = column_len / 4;
    return true;
  }
};

// ---------------------------------------------------------------------------------------------
// Binary fields (fields/scalar.rs:4-155): B128 = GF(2)[x]/(x^128 + x^7 + x^2 + x + 1) in plain
// little-endian bit order; F162 = GF(2)[x]/(x^162 + x^81 + 1), three u64 limbs, top limb 34 bits.
// ---------------------------------------------------------------------------------------------
struct B128 {
  uint64_t lo, hi;
  bool bit(int k) const { return k < 64 ? (lo >> k) & 1 : (hi >> (k - 64)) & 1; }
  bool operator==(const B128& o) const { return lo == o.lo && hi == o.hi; }
};
struct F162 {
  uint64_t w[3];
  bool operator==(const F162& o) const { return w[0] == o.w[0] && w[1] == o.w[1] && w[2] == o.w[2]; }
  bool operator!=(const F162& o) const { return !(*this == o); }
};
constexpr uint64_t M34 = (1ull << 34) - 1;
inline B128 badd(B128 a, B128 b) { return {a.lo ^ b.lo, a.hi ^ b.hi}; }
inline F162 fadd(F162 a, F162 b) { return {{a.w[0] ^ b.w[0], a.w[1] ^ b.w[1], a.w[2] ^ b.w[2]}}; }
const F162 F_ZERO = {{0, 0, 0}};
const F162 F_ONE = {{1, 0, 0}};
const B128 B_ONE = {1, 0};
inline F162 lift(B128 x) { return {{x.lo, x.hi, 0}}; }  // F162::from_b128, scalar.rs:111-113

// Carry-less 64x64 -> 128 by 4-bit windows.
inline void clmul64(uint64_t a, uint64_t b, uint64_t& lo, uint64_t& hi) {
  uint64_t tl[16], th[16];
  tl[0] = th[0] = 0;
  tl[1] = a;
  th[1] = 0;
  for (int i = 2; i < 16; i += 2) {
    tl[i] = tl[i / 2] << 1;
    th[i] = (th[i / 2] << 1) | (tl[i / 2] >> 63);
    tl[i + 1] = tl[i] ^ a;
    th[i + 1] = th[i];
  }
  lo = hi = 0;
  for (int s = 60; s >= 0; s -= 4) {
    hi = (hi << 4) | (lo >> 60);
    lo <<= 4;
    unsigned n = (unsigned)(b >> s) & 15;
    lo ^= tl[n];
    hi ^= th[n];
  }
}

B128 bmul(B128 a, B128 b) {
  uint64_t p[4] = {0, 0, 0, 0}, l, h;
  clmul64(a.lo, b.lo, l, h);
  p[0] ^= l, p[1] ^= h;
  clmul64(a.lo, b.hi, l, h);
  p[1] ^= l, p[2] ^= h;
  clmul64(a.hi, b.lo, l, h);
  p[1] ^= l, p[2] ^= h;
  clmul64(a.hi, b.hi, l, h);
  p[2] ^= l, p[3] ^= h;
  // x^128 = x^7 + x^2 + x + 1 (0x87): fold p[2..3] down twice.
  uint64_t l2, h2, l3, h3;
  clmul64(p[2], 0x87, l2, h2);
  clmul64(p[3], 0x87, l3, h3);
  uint64_t r0 = p[0] ^ l2, r1 = p[1] ^ h2 ^ l3;
  uint64_t l4, h4;
  clmul64(h3, 0x87, l4, h4);
  r0 ^= l4;
  r1 ^= h4;
  return {r0, r1};
}

// (x >> s) of a little-endian multiword value, into n words.
inline void shr_words(const uint64_t* x, int xn, int s, uint64_t* out, int n) {
  int q = s / 64, r = s % 64;
  for (int i = 0; i < n; ++i) {
    uint64_t a = (i + q < xn) ? x[i + q] : 0;
    uint64_t b = (i + q + 1 < xn) ? x[i + q + 1] : 0;
    out[i] = r ? (a >> r) | (b << (64 - r)) : a;
  }
}

// Reduce a polynomial of up to 6 words modulo x^162 + x^81 + 1.
F162 f162_reduce(uint64_t p[6]) {
  for (int pass = 0; pass < 3; ++pass) {
    uint64_t h[4];
    shr_words(p, 6, 162, h, 4);
    if (!(h[0] | h[1] | h[2] | h[3])) break;
    p[2] &= M34;
    p[3] = p[4] = p[5] = 0;
    // p += h + h * x^81
    for (int i = 0; i < 4; ++i) p[i] ^= h[i];
    uint64_t s[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < 4; ++i) {
      s[i + 1] ^= h[i] << 17;
      s[i + 2] ^= h[i] >> 47;
    }
    for (int i = 0; i < 6; ++i) p[i] ^= s[i];
  }
  return {{p[0], p[1], p[2]}};
}

F162 fmul(F162 a, F162 b) {
  uint64_t p[6] = {0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      uint64_t l, h;
      clmul64(a.w[i], b.w[j], l, h);
      p[i + j] ^= l;
      p[i + j + 1] ^= h;
    }
  return f162_reduce(p);
}

// ---------------------------------------------------------------------------------------------
// eq expansions
// ---------------------------------------------------------------------------------------------
// crossfield.rs:81-137 (eq_expand_b128, expand_from): r[0] ends at the most significant index bit.
std::vector<B128> eq_expand_b128(const B128* r, int n) {
  std::vector<B128> t((size_t)1 << n);
  t[0] = B_ONE;
  for (int round = 0; round < n; ++round)
    for (size_t i = ((size_t)1 << round); i-- > 0;) {
      B128 hi = bmul(t[i], r[round]);
      t[2 * i + 1] = hi;
      t[2 * i] = badd(t[i], hi);
    }
  return t;
}
// The same table, parallel over the low variables (same per-entry operations).
void eq_expand_b128_par(const B128* r, int n, B128* t) {
  int top = std::min(n, 8);
  std::vector<B128> prefix = eq_expand_b128(r, top);
  size_t sub = (size_t)1 << (n - top);
  parallel_for(prefix.size(), [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      B128* blk = t + i * sub;
      blk[0] = prefix[i];
      for (int round = top; round < n; ++round) {
        size_t cnt = (size_t)1 << (round - top);
        for (size_t x = cnt; x-- > 0;) {
          B128 hi = bmul(blk[x], r[round]);
          blk[2 * x + 1] = hi;
          blk[2 * x] = badd(blk[x], hi);
        }
      }
    }
  });
}
// crossfield.rs:67-79 (eq_expand_f162): the same index convention over F162.
std::vector<F162> eq_expand_f162(const F162* r, int n) {
  std::vector<F162> t(1, F_ONE);
  for (int i = 0; i < n; ++i) {
    std::vector<F162> nx;
    nx.reserve(t.size() * 2);
    for (auto& x : t) {
      F162 hi = fmul(x, r[i]);
      nx.push_back(fadd(x, hi));
      nx.push_back(hi);
    }
    t.swap(nx);
  }
  return t;
}
// eval.rs:50-85 (eq_table): variable k is bit k of the index.
std::vector<F162> eq_table(const F162* ps, int n) {
  std::vector<F162> t((size_t)1 << n, F_ZERO);
  t[0] = F_ONE;
  size_t m = 1;
  for (int k = 0; k < n; ++k) {
    for (size_t i = 0; i < m; ++i) {
      F162 xp = fmul(t[i], ps[k]);
      t[i + m] = xp;
      t[i] = fadd(t[i], xp);
    }
    m *= 2;
  }
  return t;
}

// ---------------------------------------------------------------------------------------------
// Transcript (solution-arm/labinius/crates/pcs/src/challenge.rs:226-341): a BLAKE3 stream;
// every derivation clones it and appends counter, label length and label.
// ---------------------------------------------------------------------------------------------
void put_u64(uint8_t* p, uint64_t x) {
  for (int i = 0; i < 8; ++i) p[i] = (uint8_t)(x >> (8 * i));
}
uint64_t get_u64(const uint8_t* p) {
  uint64_t x = 0;
  for (int i = 0; i < 8; ++i) x |= (uint64_t)p[i] << (8 * i);
  return x;
}

struct Transcript {
  b3::Hasher h;
  uint64_t counter = 0;
  explicit Transcript(const char* domain) {
    h.init_plain();
    absorb_len(strlen(domain));
    h.update(domain, strlen(domain));
  }
  void absorb_len(uint64_t n) {
    uint8_t b[8];
    put_u64(b, n);
    h.update(b, 8);
  }
  void absorb_bytes(const void* p, size_t n) {
    absorb_len(n);
    h.update(p, n);
  }
  void absorb_u64(uint64_t x) { absorb_len(x); }
  void absorb_b128(const B128* xs, size_t n) {
    absorb_len(n);
    for (size_t i = 0; i < n; ++i) {
      uint8_t b[16];
      put_u64(b, xs[i].lo);
      put_u64(b + 8, xs[i].hi);
      h.update(b, 16);
    }
  }
  void absorb_f162(const F162* xs, size_t n) {
    absorb_len(n);
    for (size_t i = 0; i < n; ++i) {
      uint8_t b[24];
      for (int k = 0; k < 3; ++k) put_u64(b + 8 * k, xs[i].w[k]);
      h.update(b, 24);
    }
  }
  b3::Reader derive(uint64_t ctr, const char* label) const {  // challenge.rs:335-341
    b3::Hasher c = h;
    uint8_t b[8];
    put_u64(b, ctr);
    c.update(b, 8);
    put_u64(b, strlen(label));
    c.update(b, 8);
    c.update(label, strlen(label));
    return b3::Reader{c.finalize_node(), 0};
  }
  b3::Reader reader(const char* label) { return derive(counter++, label); }
  void fill(const char* label, uint8_t* out, size_t n) { reader(label).fill(out, n); }
  std::vector<F162> sample_f162(const char* label, size_t n) {  // challenge.rs:304-315
    std::vector<uint8_t> b(24 * n);
    fill(label, b.data(), b.size());
    std::vector<F162> out(n);
    for (size_t i = 0; i < n; ++i)
      out[i] = {{get_u64(&b[24 * i]), get_u64(&b[24 * i + 8]), get_u64(&b[24 * i + 16]) & M34}};
    return out;
  }
  std::vector<B128> sample_b128(const char* label, size_t n) {  // challenge.rs:317-324
    std::vector<uint8_t> b(16 * n);
    fill(label, b.data(), b.size());
    std::vector<B128> out(n);
    for (size_t i = 0; i < n; ++i) out[i] = {get_u64(&b[16 * i]), get_u64(&b[16 * i + 8])};
    return out;
  }
};

// ---------------------------------------------------------------------------------------------
// Short challenges (challenge.rs:343-755).
// ---------------------------------------------------------------------------------------------
constexpr int N162 = 162;
constexpr int WEIGHT = 28;       // DEFAULT_WEIGHT, challenge.rs:51
constexpr double BOUND = 12.0;   // DEFAULT_BOUND, challenge.rs:54
constexpr int HALF_ROOTS = 81;   // challenge.rs:499
constexpr int LANES = 88;        // challenge.rs:503

struct Challenge {
  uint8_t positions[32];
  uint32_t signs;
  uint32_t weight;
};

// Buffered XOF bytes (challenge.rs:344-388).
struct Xof {
  b3::Reader r;
  uint8_t buf[256];
  int pos = 256;
  uint8_t byte() {
    if (pos == 256) {
      r.fill(buf, 256);
      pos = 0;
    }
    return buf[pos++];
  }
  uint16_t u16() {
    uint8_t a = byte();
    uint8_t b = byte();
    return (uint16_t)(a | (b << 8));
  }
  // DIVIDE table (challenge.rs:390-401) and `below` (challenge.rs:377-387).
  uint16_t below(uint16_t n) {
    uint32_t limit = ((65535u + 1) / n) * n;
    uint64_t magic = ((uint64_t)1 << 32) / n + 1;
    for (;;) {
      uint32_t r = u16();
      if (r < limit) {
        uint32_t q = (uint32_t)(((uint64_t)r * magic) >> 32);
        return (uint16_t)(r - q * n);
      }
    }
  }
};

struct Phase {
  std::vector<double> re, im;
  uint16_t units[N162];
  Phase() : re(N162 * LANES, 0.0), im(N162 * LANES, 0.0) {  // challenge.rs:512-540
    int n = 0;
    for (int x = 1; x < 243; ++x)
      if (x % 3) units[n++] = (uint16_t)x;
    for (int p = 0; p < N162; ++p)
      for (int k = 0; k < HALF_ROOTS; ++k) {
        int m = (p * units[k]) % 243;
        double angle = 2.0 * M_PI * (double)m / 243.0;
        re[p * LANES + k] = cos(angle);
        im[p * LANES + k] = sin(angle);
      }
  }
};
const Phase& phase() {
  static Phase ph;
  return ph;
}

// Sign key: Hasher::new_derive_key("labinius 2026 challenge signs v1") (challenge.rs:417-449).
const b3::Hasher& sign_key() {
  static b3::Hasher h = [] {
    b3::Hasher x;
    x.init_derive_key("labinius 2026 challenge signs v1");
    return x;
  }();
  return h;
}
void sign(Challenge& c) {
  b3::Hasher h = sign_key();
  uint8_t w[8];
  put_u64(w, c.weight);
  h.update(w, 8);
  h.update(c.positions, c.weight);
  uint8_t out[4];
  h.finalize(out, 4);
  uint32_t bits = (uint32_t)out[0] | ((uint32_t)out[1] << 8) | ((uint32_t)out[2] << 16) |
                  ((uint32_t)out[3] << 24);
  uint32_t mask = (uint32_t)(((uint64_t)1 << c.weight) - 1);
  c.signs = bits & mask;
}

// accumulate + block_sq over all lanes (challenge.rs:542-599): per lane, the signed phase rows
// summed in position order, then re*re + im*im.
double lane_norm(const Challenge& c, int k) {
  const Phase& ph = phase();
  double vr = 0.0, vi = 0.0;
  for (uint32_t i = 0; i < c.weight; ++i) {
    size_t b = (size_t)c.positions[i] * LANES + k;
    double pr = ph.re[b], pi = ph.im[b];
    if ((c.signs >> i) & 1) pr = -pr, pi = -pi;
    vr = vr + pr;
    vi = vi + pi;
  }
  double a = vr * vr;
  double b = vi * vi;
  return a + b;
}
bool within(const Challenge& c, double bound_sq) {  // challenge.rs:583-625
  for (int k = 0; k < HALF_ROOTS; ++k)
    if (lane_norm(c, k) > bound_sq) return false;
  return true;
}
double norm_blocked(const Challenge& c) {
  double m = 0.0;
  for (int k = 0; k < HALF_ROOTS; ++k) m = std::max(m, lane_norm(c, k));
  return m;
}
double norm_horner(const Challenge& c) {  // challenge.rs:629-647
  int coeffs[N162] = {0};
  for (uint32_t i = 0; i < c.weight; ++i) coeffs[c.positions[i]] = 1 - 2 * (int)((c.signs >> i) & 1);
  const Phase& ph = phase();
  double best = 0.0;
  for (int u = 0; u < N162; ++u) {
    double angle = 2.0 * M_PI * (double)ph.units[u] / 243.0;
    double zr = cos(angle), zi = sin(angle), ar = 0.0, ai = 0.0;
    for (int p = N162 - 1; p >= 0; --p) {
      double nr = ar * zr - ai * zi, ni = ar * zi + ai * zr;
      ar = nr + (double)coeffs[p];
      ai = ni;
    }
    double m = ar * ar + ai * ai;
    if (m > best) best = m;
  }
  return best;
}

Challenge attempt(Xof& x, int weight) {  // challenge.rs:664-692
  uint8_t perm[N162];
  for (int i = 0; i < N162; ++i) perm[i] = (uint8_t)i;
  for (int i = 0; i < weight; ++i) {
    int j = i + x.below((uint16_t)(N162 - i));
    std::swap(perm[i], perm[j]);
  }
  uint64_t seen[3] = {0, 0, 0};
  for (int i = 0; i < weight; ++i) seen[perm[i] >> 6] |= 1ull << (perm[i] & 63);
  Challenge c;
  memset(&c, 0, sizeof c);
  c.weight = (uint32_t)weight;
  int n = 0;
  for (int w = 0; w < 3; ++w)
    for (uint64_t b = seen[w]; b; b &= b - 1) c.positions[n++] = (uint8_t)(64 * w + __builtin_ctzll(b));
  return c;
}

// sample_short_challenges (challenge.rs:707-737): challenge i reads derivation counter base + i.
std::vector<Challenge> short_challenges(Transcript& t, uint32_t n) {
  uint64_t base = t.counter;
  double bound_sq = BOUND * BOUND + 1e-12;
  std::vector<Challenge> out(n);
  phase();
  sign_key();
  parallel_for(n, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      Xof x{t.derive(base + i, "short-challenge")};
      for (;;) {
        Challenge c = attempt(x, WEIGHT);
        sign(c);
        if (within(c, bound_sq)) {
          out[i] = c;
          break;
        }
      }
    }
  });
  t.counter += n;
  return out;
}

F162 challenge_to_f162(const Challenge& c) {  // challenge.rs:454-461
  F162 x = F_ZERO;
  for (uint32_t i = 0; i < c.weight; ++i) x.w[c.positions[i] >> 6] |= 1ull << (c.positions[i] & 63);
  return x;
}

// ---------------------------------------------------------------------------------------------
// R_Q (verifier/proof_verify/src/rq.rs)
// ---------------------------------------------------------------------------------------------
const u128 MAX_MODULUS = (u128)1 << 96;               // rq.rs:25
const u128 MIN_MODULUS = 34816965049ull;              // main.rs:54
const u128 BASELINE_Q = (u128)3889 * 9721 * 17497;   // solution-arm/proof_generate/src/ntt.rs:37-40

u128 q_from_le(const uint8_t* b) {
  u128 q = 0;
  for (int i = 15; i >= 0; --i) q = (q << 8) | b[i];
  return q;
}
uint32_t modulus_bits(u128 q) {  // rq.rs:40-43
  u128 x = q - 1;
  uint32_t n = 0;
  while (x) ++n, x >>= 1;
  return n;
}
size_t coefficient_bytes(u128 q) { return (modulus_bits(q) + 7) / 8; }  // rq.rs:46-48

// rq.rs:53-91 (Expansion) and :114-144 (ajtai_matrix).
void expand_element(u128 q, uint64_t elements, uint64_t index, u128* out) {
  b3::Hasher h;
  uint8_t key[32];
  memset(key, 0x5a, 32);
  h.init_keyed(key);
  const char* dom = "labinius-fast/ajtai-matrix/v1";
  h.update(dom, strlen(dom));
  uint8_t b[16];
  for (int i = 0; i < 16; ++i) b[i] = (uint8_t)(q >> (8 * i));
  h.update(b, 16);
  put_u64(b, elements);
  h.update(b, 8);
  put_u64(b, index);
  h.update(b, 8);
  b3::Reader r{h.finalize_node(), 0};
  size_t width = coefficient_bytes(q);
  uint32_t bits = modulus_bits(q);
  u128 mask = bits == 128 ? ~(u128)0 : (((u128)1 << bits) - 1);
  std::vector<uint8_t> buf(8192);
  size_t pos = buf.size();
  for (int t = 0; t < N; ++t) {
    for (;;) {
      if (pos + width > buf.size()) {
        size_t rest = buf.size() - pos;
        memmove(buf.data(), buf.data() + pos, rest);
        r.fill(buf.data() + rest, buf.size() - rest);
        pos = 0;
      }
      u128 v = 0;
      for (size_t i = width; i-- > 0;) v = (v << 8) | buf[pos + i];
      pos += width;
      v &= mask;
      if (v < q) {
        out[t] = v;
        break;
      }
    }
  }
}
std::vector<u128> ajtai_matrix(u128 q, uint64_t elements) {
  std::vector<u128> m(elements * N);
  parallel_for(elements, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) expand_element(q, elements, i, &m[i * N]);
  });
  return m;
}

inline i128 rem_euclid(i128 x, i128 m) {
  i128 r = x % m;
  return r < 0 ? r + m : r;
}
// rq.rs:152-165
void fold_into_ring(i128* raw, u128 q, u128* out) {
  i128 m = (i128)q;
  for (int k = 2 * N - 2; k >= N; --k) {
    i128 v = rem_euclid(raw[k], m);
    raw[k] = 0;
    raw[k - SPLIT] += v;
    raw[k - N] -= v;
  }
  for (int i = 0; i < N; ++i) out[i] = (u128)rem_euclid(raw[i], m);
}

// rq.rs:264-287 (commit_binary_column): ring element m of a column has coefficient 4p + k equal
// to bit p of word 4m + k.
void commit_binary_column(const u128* matrix, const B128* column, size_t elements, u128 q, u128* out) {
  std::vector<i128> raw(2 * N - 1, 0);
  for (size_t m = 0; m < elements; ++m) {
    const u128* a = matrix + m * N;
    for (int k = 0; k < 4; ++k) {
      B128 x = column[4 * m + k];
      for (int p = 0; p < 128; ++p) {
        if (!x.bit(p)) continue;
        i128* w = &raw[4 * p + k];
        for (int t = 0; t < N; ++t) w[t] += (i128)a[t];
      }
    }
  }
  fold_into_ring(raw.data(), q, out);
}

void pack_ring_elements(const u128* c, size_t n, u128 q, uint8_t* out) {  // rq.rs:291-299
  size_t w = coefficient_bytes(q);
  for (size_t i = 0; i < n; ++i)
    for (size_t b = 0; b < w; ++b) out[i * w + b] = (uint8_t)(c[i] >> (8 * b));
}

// rq.rs:188-217 (a_times_v), reduced per worker and summed.
std::vector<u128> a_times_v(const std::vector<u128>& a, const std::vector<int16_t>& v, u128 q) {
  size_t elements = a.size() / N;
  std::vector<std::vector<u128>> parts(threads());
  std::atomic<int> slot{0};
  parallel_for(elements, [&](size_t b, size_t e) {
    int me = slot++;
    std::vector<i128> raw(2 * N - 1, 0);
    for (size_t el = b; el < e; ++el) {
      const u128* ae = &a[el * N];
      const int16_t* ve = &v[el * N];
      for (int j = 0; j < N; ++j) {
        int c = ve[j];
        if (!c) continue;
        i128* w = &raw[j];
        i128 wt = c;
        for (int t = 0; t < N; ++t) w[t] += (i128)ae[t] * wt;
      }
      if ((el - b + 1) % 64 == 0)
        for (auto& s : raw) s = rem_euclid(s, (i128)q);
    }
    std::vector<u128> out(N);
    fold_into_ring(raw.data(), q, out.data());
    parts[me] = out;
  }, 64);
  std::vector<u128> sum(N, 0);
  for (auto& p : parts)
    if (!p.empty())
      for (int i = 0; i < N; ++i) sum[i] = (sum[i] + p[i]) % q;
  return sum;
}

// rq.rs:226-256 (challenge_combination).
std::vector<u128> challenge_combination(const std::vector<u128>& cols, const std::vector<Challenge>& ch, u128 q) {
  std::vector<i128> raw(2 * N - 1, 0);
  for (size_t j = 0; j < ch.size(); ++j) {
    const u128* col = &cols[j * N];
    for (uint32_t t = 0; t < ch[j].weight; ++t) {
      int m = ch[j].positions[t];
      int sign = (1 - 2 * (int)((ch[j].signs >> t) & 1)) * (m % 2 == 0 ? 1 : -1);
      i128* w = &raw[4 * m];
      if (sign > 0)
        for (int i = 0; i < N; ++i) w[i] += (i128)col[i];
      else
        for (int i = 0; i < N; ++i) w[i] -= (i128)col[i];
    }
    if ((j + 1) % 64 == 0)
      for (auto& s : raw) s = rem_euclid(s, (i128)q);
  }
  std::vector<u128> out(N);
  fold_into_ring(raw.data(), q, out.data());
  return out;
}

// ---------------------------------------------------------------------------------------------
// The 3-prime transform commitment for Q = 3889 * 9721 * 17497
// (solution-arm/proof_generate/src/ntt.rs:26-272, 525-671), restated: modulo each prime,
// X^648 - X^324 + 1 splits along a tree (trinomial, radix 2, 2, 3, 3, 3, 3) into 648 linear
// factors; the product is slot-wise; the inverse tree and Garner's CRT give [0, Q).
// ---------------------------------------------------------------------------------------------
constexpr int ORDER = 1944;
const int RADICES[6] = {2, 2, 3, 3, 3, 3};
const uint32_t PRIMES3[3] = {3889, 9721, 17497};

uint64_t pow_mod(uint64_t b, uint64_t e, uint64_t p) {
  uint64_t r = 1 % p;
  b %= p;
  while (e) {
    if (e & 1) r = r * b % p;
    b = b * b % p;
    e >>= 1;
  }
  return r;
}

struct PrimeTree {
  uint64_t p;
  std::vector<uint64_t> pw;               // zeta^i
  std::vector<std::vector<uint32_t>> exps;  // node exponents after each level
  uint64_t inv_radix[4], inv_split;
  explicit PrimeTree(uint64_t prime) : p(prime) {
    uint64_t z = 0;
    for (uint64_t g = 2;; ++g) {  // ntt.rs:79-89: first g^((p-1)/1944) of order 1944
      z = pow_mod(g, (p - 1) / ORDER, p);
      if (pow_mod(z, 972, p) != 1 && pow_mod(z, 648, p) != 1) break;
    }
    pw.resize(ORDER);
    for (int i = 0; i < ORDER; ++i) pw[i] = pow_mod(z, i, p);
    exps.push_back({(uint32_t)SPLIT, (uint32_t)(5 * SPLIT)});
    for (int r : RADICES) {
      std::vector<uint32_t> next;
      for (uint32_t e : exps.back())
        for (int k = 0; k < r; ++k) next.push_back(e / r + k * ORDER / r);
      exps.push_back(next);
    }
    auto inv = [&](uint64_t x) { return pow_mod(x, p - 2, p); };
    inv_radix[0] = 0, inv_radix[1] = 1, inv_radix[2] = inv(2), inv_radix[3] = inv(3);
    inv_split = inv((pw[SPLIT] + p - pw[5 * SPLIT]) % p);
  }
  uint64_t root(uint64_t e) const { return pw[e % ORDER]; }
  void forward(uint64_t* x) const {
    uint64_t w = root(SPLIT), w5 = root(5 * SPLIT);
    for (int j = 0; j < SPLIT; ++j) {
      uint64_t a = x[j], b = x[j + SPLIT];
      x[j] = (a + w * b) % p;
      x[j + SPLIT] = (a + w5 * b) % p;
    }
    int len = SPLIT;
    for (int level = 0; level < 6; ++level) {
      int r = RADICES[level], sub = len / r;
      for (size_t node = 0; node < exps[level].size(); ++node) {
        int base = (int)node * len;
        uint64_t tau = exps[level][node] / r;
        for (int j = 0; j < sub; ++j) {
          uint64_t a[3];
          for (int i = 0; i < r; ++i) a[i] = x[base + j + i * sub] * root(tau * i) % p;
          for (int k = 0; k < r; ++k) {
            uint64_t acc = 0;
            for (int i = 0; i < r; ++i) acc += a[i] * root((uint64_t)k * i * (ORDER / r));
            x[base + j + k * sub] = acc % p;
          }
        }
      }
      len = sub;
    }
  }
  void inverse(uint64_t* x) const {
    int len = 1;
    for (int level = 5; level >= 0; --level) {
      int r = RADICES[level], parent = len * r;
      for (size_t node = 0; node < exps[level].size(); ++node) {
        int base = (int)node * parent;
        uint64_t tau = exps[level][node] / r;
        for (int j = 0; j < len; ++j) {
          uint64_t y[3];
          for (int k = 0; k < r; ++k) y[k] = x[base + j + k * len];
          for (int i = 0; i < r; ++i) {
            uint64_t acc = 0;
            for (int k = 0; k < r; ++k) acc += y[k] * root(ORDER - ((uint64_t)k * i * (ORDER / r)) % ORDER);
            uint64_t scale = root(ORDER - (tau * i) % ORDER) * inv_radix[r] % p;
            x[base + j + i * len] = acc % p * scale % p;
          }
        }
      }
      len = parent;
    }
    uint64_t w = root(SPLIT);
    for (int j = 0; j < SPLIT; ++j) {
      uint64_t u = x[j], v = x[j + SPLIT];
      uint64_t b = (u + p - v) * inv_split % p;
      x[j] = (u + p * p - w * b) % p;
      x[j + SPLIT] = b;
    }
  }
};

u128 crt3(const uint64_t r[3]) {  // ntt.rs:251-267 (Garner)
  const uint64_t P0 = PRIMES3[0], P1 = PRIMES3[1], P2 = PRIMES3[2];
  uint64_t inv01 = pow_mod(P0, P1 - 2, P1);
  uint64_t inv012 = pow_mod(P0 * P1 % P2, P2 - 2, P2);
  uint64_t x1 = (r[1] + P1 - r[0] % P1) % P1 * inv01 % P1;
  uint64_t low = r[0] + P0 * x1;
  uint64_t x2 = (r[2] + P2 - low % P2) % P2 * inv012 % P2;
  return (u128)(low + P0 * P1 * x2);
}

void commit_ntt(const Shape& s, const B128* table, const std::vector<u128>& matrix, std::vector<u128>& out) {
  std::vector<PrimeTree> trees;
  for (uint32_t p : PRIMES3) trees.emplace_back(p);
  size_t E = s.ring_elements;
  // The matrix in each prime's transform domain.
  std::vector<std::vector<uint32_t>> key(3, std::vector<uint32_t>(E * N));
  parallel_for(E, [&](size_t b, size_t e) {
    uint64_t x[N];
    for (size_t m = b; m < e; ++m)
      for (int i = 0; i < 3; ++i) {
        for (int t = 0; t < N; ++t) x[t] = (uint64_t)(matrix[m * N + t] % trees[i].p);
        trees[i].forward(x);
        for (int t = 0; t < N; ++t) key[i][m * N + t] = (uint32_t)x[t];
      }
  });
  out.assign((size_t)COLUMNS * N, 0);
  parallel_for(COLUMNS, [&](size_t b, size_t e) {
    uint64_t x[N], acc[3][N];
    for (size_t j = b; j < e; ++j) {
      memset(acc, 0, sizeof acc);
      for (size_t m = 0; m < E; ++m) {
        const B128* words = table + j * s.column_len + 4 * m;
        for (int i = 0; i < 3; ++i) {
          for (int p = 0; p < N / 4; ++p)
            for (int k = 0; k < 4; ++k) x[4 * p + k] = p < 128 ? (uint64_t)words[k].bit(p) : 0;
          trees[i].forward(x);
          const uint32_t* a = &key[i][m * N];
          for (int t = 0; t < N; ++t) acc[i][t] = (acc[i][t] + x[t] * a[t]) % trees[i].p;
        }
      }
      for (int i = 0; i < 3; ++i) trees[i].inverse(acc[i]);
      for (int t = 0; t < N; ++t) {
        uint64_t r[3] = {acc[0][t], acc[1][t], acc[2][t]};
        out[j * N + t] = crt3(r);
      }
    }
  });
}

void commit_schoolbook(const Shape& s, const B128* table, const std::vector<u128>& matrix, u128 q,
                       std::vector<u128>& out) {
  out.assign((size_t)COLUMNS * N, 0);
  parallel_for(COLUMNS, [&](size_t b, size_t e) {
    for (size_t j = b; j < e; ++j)
      commit_binary_column(matrix.data(), table + j * s.column_len, s.ring_elements, q, &out[j * N]);
  });
}

// ---------------------------------------------------------------------------------------------
// Partials and the switch (crossfield.rs:150-170, 548-701; sumcheck.rs:128-251).
// ---------------------------------------------------------------------------------------------
std::vector<B128> partial_evals(const B128* pi0, const B128* eq, size_t n) {  // crossfield.rs:714-724
  std::vector<std::vector<B128>> parts(threads(), std::vector<B128>(128, {0, 0}));
  std::atomic<int> slot{0};
  parallel_for(n, [&](size_t b, size_t e) {
    auto& v = parts[slot++];
    for (size_t j = b; j < e; ++j) {
      B128 p = pi0[j];
      for (int k = 0; k < 128; ++k)
        if (p.bit(k)) v[k] = badd(v[k], eq[j]);
    }
  }, 1 << 14);
  std::vector<B128> v(128, {0, 0});
  for (auto& p : parts)
    for (int k = 0; k < 128; ++k) v[k] = badd(v[k], p[k]);
  return v;
}

// psi_table / psi (crossfield.rs:150-170): sum_k bit_k(x) batch[k].
struct Psi {
  F162 t[16][256];
  explicit Psi(const std::vector<F162>& batch) {
    for (int c = 0; c < 16; ++c) {
      t[c][0] = F_ZERO;
      for (int m = 1; m < 256; ++m) {
        int b = __builtin_ctz(m);
        t[c][m] = fadd(t[c][m ^ (1 << b)], batch[c * 8 + b]);
      }
    }
  }
  F162 operator()(B128 x) const {
    F162 acc = F_ZERO;
    for (int c = 0; c < 16; ++c) {
      uint64_t byte = c < 8 ? (x.lo >> (8 * c)) & 0xff : (x.hi >> (8 * (c - 8))) & 0xff;
      acc = fadd(acc, t[c][byte]);
    }
    return acc;
  }
};

// The transparent coefficient (crossfield.rs:10-65, 139-148): the tensor prod_i (1 + v_i + h_i)
// in F162 (x) GHASH, folded against batch.
F162 transparent_coeff(const std::vector<B128>& r_hi, const std::vector<F162>& r_pp, const std::vector<F162>& batch) {
  std::vector<F162> t(128, F_ZERO);
  t[0] = F_ONE;
  auto shift_x = [](const std::vector<F162>& c) {
    std::vector<F162> o(128, F_ZERO);
    for (int i = 1; i < 128; ++i) o[i] = c[i - 1];
    F162 top = c[127];
    for (int k : {0, 1, 2, 7}) o[k] = fadd(o[k], top);
    return o;
  };
  for (size_t i = 0; i < r_pp.size(); ++i) {
    std::vector<F162> vs(128), hs(128, F_ZERO);
    for (int k = 0; k < 128; ++k) vs[k] = fmul(t[k], r_pp[i]);
    for (int k = 127; k >= 0; --k) {
      hs = shift_x(hs);
      if (r_hi[i].bit(k))
        for (int x = 0; x < 128; ++x) hs[x] = fadd(hs[x], t[x]);
    }
    for (int k = 0; k < 128; ++k) t[k] = fadd(fadd(t[k], vs[k]), hs[k]);
  }
  F162 acc = F_ZERO;
  for (int k = 0; k < 128; ++k) acc = fadd(acc, fmul(t[k], batch[k]));
  return acc;
}

// slice_sum (crossfield.rs:637-649)
F162 slice_sum(const std::vector<B128>& v, const std::vector<F162>& batch) {
  F162 s = F_ZERO;
  for (int k = 0; k < 128; ++k) {
    B128 u = {0, 0};
    for (int i = 0; i < 128; ++i)
      if (v[i].bit(k)) (i < 64 ? u.lo : u.hi) |= 1ull << (i & 63);
    s = fadd(s, fmul(lift(u), batch[k]));
  }
  return s;
}

B128 claim(const std::vector<B128>& partials, const std::vector<B128>& lo) {  // main.rs:184-189
  std::vector<B128> e = eq_expand_b128(lo.data(), (int)lo.size());
  B128 acc = {0, 0};
  for (int i = 0; i < 128; ++i) acc = badd(acc, bmul(partials[i], e[i]));
  return acc;
}

// ---------------------------------------------------------------------------------------------
// Row evaluation, fold, wire (reference.rs:50-133; wire/mod.rs:96-140, 445-457).
// ---------------------------------------------------------------------------------------------
std::vector<F162> row_evaluate(const Shape& s, const B128* table, const std::vector<F162>& p0) {
  std::vector<F162> eq = eq_table(p0.data(), (int)p0.size());
  std::vector<F162> out(COLUMNS, F_ZERO);
  parallel_for(COLUMNS, [&](size_t b, size_t e) {
    for (size_t j = b; j < e; ++j) {
      F162 acc = F_ZERO;
      for (size_t i = 0; i < s.column_len; ++i) acc = fadd(acc, fmul(eq[i], lift(table[j * s.column_len + i])));
      out[j] = acc;
    }
  });
  return out;
}

std::vector<uint8_t> pack_f162(const std::vector<F162>& v) {
  size_t bytes = (v.size() * 162 + 7) / 8;
  std::vector<uint8_t> out(bytes, 0);
  size_t bit = 0;
  auto put = [&](uint64_t x, int nbits) {
    for (int i = 0; i < nbits; ++i, ++bit)
      if ((x >> i) & 1) out[bit / 8] |= (uint8_t)(1u << (bit % 8));
  };
  for (auto& x : v) {
    put(x.w[0], 64);
    put(x.w[1], 64);
    put(x.w[2], 34);
  }
  return out;
}
bool unpack_f162(const uint8_t* b, size_t len, size_t count, std::vector<F162>& out) {
  if (len != (count * 162 + 7) / 8) return false;
  out.assign(count, F_ZERO);
  size_t bit = 0;
  auto get = [&](int nbits) {
    uint64_t x = 0;
    for (int i = 0; i < nbits; ++i, ++bit) x |= (uint64_t)((b[bit / 8] >> (bit % 8)) & 1) << i;
    return x;
  };
  for (size_t i = 0; i < count; ++i) {
    out[i].w[0] = get(64);
    out[i].w[1] = get(64);
    out[i].w[2] = get(34);
  }
  return true;
}

void absorb_row(Transcript& t, const std::vector<F162>& row) {  // scheme/commitment.rs:320-331
  const char* label = "labinius/row-evaluation";
  t.absorb_bytes(label, strlen(label));
  std::vector<uint8_t> b(24 * row.size());
  for (size_t i = 0; i < row.size(); ++i)
    for (int k = 0; k < 3; ++k) put_u64(&b[24 * i + 8 * k], row[i].w[k]);
  t.absorb_bytes(b.data(), b.size());
}

// reference.rs:78-115 (fold_element)
bool fold_element(const Shape& s, const B128* table, const std::vector<Challenge>& ch, size_t m, int16_t* out) {
  std::vector<int32_t> raw(2 * N - 1, 0);
  int32_t bits[N];
  for (size_t j = 0; j < ch.size(); ++j) {
    const B128* packed = table + j * s.column_len + 4 * m;
    for (int k = 0; k < 4; ++k)
      for (int p = 0; p < N / 4; ++p) bits[4 * p + k] = p < 128 ? (int32_t)packed[k].bit(p) : 0;
    for (uint32_t t = 0; t < ch[j].weight; ++t) {
      int pos = ch[j].positions[t];
      bool negative = (((ch[j].signs >> t) & 1) == 1) ^ (pos % 2 == 1);
      int32_t* w = &raw[4 * pos];
      if (negative)
        for (int i = 0; i < N; ++i) w[i] -= bits[i];
      else
        for (int i = 0; i < N; ++i) w[i] += bits[i];
    }
  }
  for (int k = 2 * N - 2; k >= N; --k) {
    int32_t v = raw[k];
    raw[k] = 0;
    raw[k - SPLIT] += v;
    raw[k - N] -= v;
  }
  for (int i = 0; i < N; ++i) {
    if (raw[i] < -32768 || raw[i] > 32767) return false;
    out[i] = (int16_t)raw[i];
  }
  return true;
}

// ---------------------------------------------------------------------------------------------
// Proof layout (main.rs:98-124; bincode fixint, no trailing bytes).
// ---------------------------------------------------------------------------------------------
struct Proof {
  u128 modulus;
  std::vector<uint8_t> commitment;
  std::vector<B128> partials;
  std::vector<F162> rounds;  // 2 per round
  F162 opened;
  std::vector<uint8_t> row;
  std::vector<uint8_t> folded;
};

size_t proof_size(u128 q, const Shape& s) {
  return 4 + 16 + 8 + coefficient_bytes(q) * COLUMNS * N + 8 + 16 * 128 + 8 + 48 * (size_t)s.lp + 24 + 8 +
         (COLUMNS * 162 + 7) / 8 + 8 + 4 * N * s.ring_elements;
}

std::vector<uint8_t> encode(const Proof& p) {
  std::vector<uint8_t> o;
  auto u64 = [&](uint64_t x) {
    uint8_t b[8];
    put_u64(b, x);
    o.insert(o.end(), b, b + 8);
  };
  o.push_back(1), o.push_back(0), o.push_back(0), o.push_back(0);
  for (int i = 0; i < 16; ++i) o.push_back((uint8_t)(p.modulus >> (8 * i)));
  u64(p.commitment.size());
  o.insert(o.end(), p.commitment.begin(), p.commitment.end());
  u64(p.partials.size());
  for (auto& x : p.partials) u64(x.lo), u64(x.hi);
  u64(p.rounds.size() / 2);
  for (auto& x : p.rounds)
    for (int k = 0; k < 3; ++k) u64(x.w[k]);
  for (int k = 0; k < 3; ++k) u64(p.opened.w[k]);
  u64(p.row.size());
  o.insert(o.end(), p.row.begin(), p.row.end());
  u64(p.folded.size());
  o.insert(o.end(), p.folded.begin(), p.folded.end());
  return o;
}

bool decode(const uint8_t* b, size_t len, Proof& p, std::string& err) {
  size_t at = 0;
  auto need = [&](size_t n) {
    if (len - at < n || at > len) {
      err = "truncated proof";
      return false;
    }
    return true;
  };
  if (!need(20)) return false;
  uint32_t version = (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
  if (version != 1) {
    err = "version";
    return false;
  }
  p.modulus = q_from_le(b + 4);
  at = 20;
  auto vec = [&](std::vector<uint8_t>& v) {
    if (!need(8)) return false;
    uint64_t n = get_u64(b + at);
    at += 8;
    if (!need(n)) return false;
    v.assign(b + at, b + at + n);
    at += n;
    return true;
  };
  if (!vec(p.commitment)) return false;
  if (!need(8)) return false;
  uint64_t np = get_u64(b + at);
  at += 8;
  if (np > (len - at) / 16 || !need(16 * np)) return false;
  p.partials.resize(np);
  for (uint64_t i = 0; i < np; ++i, at += 16) p.partials[i] = {get_u64(b + at), get_u64(b + at + 8)};
  if (!need(8)) return false;
  uint64_t nr = get_u64(b + at);
  at += 8;
  if (nr > (len - at) / 48 || !need(48 * nr)) return false;
  p.rounds.resize(2 * nr);
  for (uint64_t i = 0; i < 2 * nr; ++i, at += 24)
    p.rounds[i] = {{get_u64(b + at), get_u64(b + at + 8), get_u64(b + at + 16)}};
  if (!need(24)) return false;
  p.opened = {{get_u64(b + at), get_u64(b + at + 8), get_u64(b + at + 16)}};
  at += 24;
  if (!vec(p.row) || !vec(p.folded)) return false;
  if (at != len) {
    err = "trailing bytes";
    return false;
  }
  return true;
}

uint64_t fold_cap(const Shape& s) {  // main.rs:62-64 with recursion/mod.rs:81 (FOLD_CAP = 108.0)
  double x = 108.0 * (double)(((uint64_t)1 << s.lp) / 4 * N);
  return (uint64_t)std::ceil(x);
}
uint64_t isqrt_u64(uint64_t x) {
  uint64_t r = (uint64_t)std::sqrt((double)x);
  while (r * r > x) --r;
  while ((r + 1) * (r + 1) <= x) ++r;
  return r;
}
int accept_modulus(u128 q, const Shape& s) {  // main.rs:85-96
  if (q < MIN_MODULUS) return LFO_E_MODULUS;
  if (q <= (u128)2 * isqrt_u64(fold_cap(s))) return LFO_E_MODULUS;
  if (q >= MAX_MODULUS) return LFO_E_MODULUS;
  return LFO_OK;
}

Transcript transcript(const uint8_t seed[32], const Shape& s, u128 q, const std::vector<uint8_t>& commitment) {
  Transcript t("labinius-fast/v1");  // main.rs:166-174
  t.absorb_bytes(seed, 32);
  t.absorb_u64((uint64_t)s.log_vars);
  t.absorb_u64((uint64_t)COLUMN_LOG);
  uint8_t qb[16];
  for (int i = 0; i < 16; ++i) qb[i] = (uint8_t)(q >> (8 * i));
  t.absorb_bytes(qb, 16);
  t.absorb_bytes(commitment.data(), commitment.size());
  return t;
}

void split_point(const Shape& s, const std::vector<F162>& coords, std::vector<F162>& p0, std::vector<F162>& p1) {
  p0.assign(coords.rbegin(), coords.rend() - COLUMN_LOG);  // main.rs:257-264
  p1.assign(coords.rend() - COLUMN_LOG, coords.rend());
  (void)s;
}

std::vector<B128> table_words(const uint8_t* t, size_t n) {
  std::vector<B128> w(n);
  for (size_t i = 0; i < n; ++i) w[i] = {get_u64(t + 16 * i), get_u64(t + 16 * i + 8)};
  return w;
}

struct TraceWriter {
  uint8_t* p;
  size_t cap, at = 0;
  bool ok = true;
  void put(const void* x, size_t n) {
    if (!p) return;
    if (at + n > cap) {
      ok = false;
      return;
    }
    memcpy(p + at, x, n);
    at += n;
  }
  void b128(const std::vector<B128>& v) {
    for (auto& x : v) {
      uint8_t b[16];
      put_u64(b, x.lo), put_u64(b + 8, x.hi);
      put(b, 16);
    }
  }
  void f162(const std::vector<F162>& v) {
    for (auto& x : v) {
      uint8_t b[24];
      for (int k = 0; k < 3; ++k) put_u64(b + 8 * k, x.w[k]);
      put(b, 24);
    }
  }
};

}  // namespace

// =============================================================================================
// C ABI
// =============================================================================================
extern "C" {

void lfo_set_threads(int n) { g_threads = n; }

int lfo_blake3(const uint8_t* key32, const char* ctx, const uint8_t* in, size_t n, uint64_t seek, uint8_t* out,
               size_t n_out) {
  b3::Hasher h;
  if (key32 && ctx) return LFO_E_ARGS;
  if (key32)
    h.init_keyed(key32);
  else if (ctx)
    h.init_derive_key(ctx);
  else
    h.init_plain();
  h.update(in, n);
  h.finalize_node().root_bytes(seek, out, n_out);
  return LFO_OK;
}

int lfo_write_table(const uint8_t seed[32], uint32_t log_vars, uint8_t* out) {
  Shape s;
  if (!s.set(log_vars)) return LFO_E_SHAPE;
  b3::Hasher h;  // verifier/table_writer/src/main.rs:17-20; main.rs:135-141
  h.init_keyed(seed);
  const char* ctx = "labinius-fast/binary-table/v1";
  h.update(ctx, strlen(ctx));
  b3::Node node = h.finalize_node();
  size_t total = ((size_t)1 << log_vars) / 8;
  parallel_for(total / 64, [&](size_t b, size_t e) { node.root_bytes(64 * b, out + 64 * b, 64 * (e - b)); }, 1024);
  return LFO_OK;
}

int lfo_b128_mul(const uint8_t* a, const uint8_t* b, uint8_t* out, size_t n) {
  for (size_t i = 0; i < n; ++i) {
    B128 x = {get_u64(a + 16 * i), get_u64(a + 16 * i + 8)}, y = {get_u64(b + 16 * i), get_u64(b + 16 * i + 8)};
    B128 z = bmul(x, y);
    put_u64(out + 16 * i, z.lo), put_u64(out + 16 * i + 8, z.hi);
  }
  return LFO_OK;
}

int lfo_f162_mul(const uint8_t* a, const uint8_t* b, uint8_t* out, size_t n) {
  for (size_t i = 0; i < n; ++i) {
    F162 x, y;
    for (int k = 0; k < 3; ++k) x.w[k] = get_u64(a + 24 * i + 8 * k), y.w[k] = get_u64(b + 24 * i + 8 * k);
    F162 z = fmul(x, y);
    for (int k = 0; k < 3; ++k) put_u64(out + 24 * i + 8 * k, z.w[k]);
  }
  return LFO_OK;
}

int lfo_ajtai_matrix(const uint8_t q_le[16], uint64_t elements, uint8_t* out) {
  u128 q = q_from_le(q_le);
  if (q < 2) return LFO_E_MODULUS;
  std::vector<u128> m = ajtai_matrix(q, elements);
  for (size_t i = 0; i < m.size(); ++i)
    for (int b = 0; b < 16; ++b) out[16 * i + b] = (uint8_t)(m[i] >> (8 * b));
  return LFO_OK;
}

int lfo_a_times_v(const uint8_t q_le[16], uint64_t elements, const int16_t* v, uint8_t* out) {
  u128 q = q_from_le(q_le);
  if (q < 2 || (q >> 96)) return LFO_E_MODULUS;
  std::vector<u128> m = ajtai_matrix(q, elements);
  std::vector<int16_t> vv(v, v + elements * N);
  std::vector<u128> r = a_times_v(m, vv, q);
  for (int i = 0; i < N; ++i)
    for (int b = 0; b < 16; ++b) out[16 * i + b] = (uint8_t)(r[i] >> (8 * b));
  return LFO_OK;
}

size_t lfo_proof_size(const uint8_t q_le[16], uint32_t log_vars) {
  Shape s;
  if (!s.set(log_vars)) return 0;
  return proof_size(q_from_le(q_le), s);
}

uint64_t lfo_fold_cap(uint32_t log_vars) {
  Shape s;
  if (!s.set(log_vars)) return 0;
  return fold_cap(s);
}

int lfo_accept_modulus(const uint8_t q_le[16], uint32_t log_vars) {
  Shape s;
  if (!s.set(log_vars)) return LFO_E_SHAPE;
  return accept_modulus(q_from_le(q_le), s);
}

int lfo_commit(const uint8_t q_le[16], uint32_t log_vars, const uint8_t* table, int mode, uint8_t* out) {
  Shape s;
  if (!s.set(log_vars)) return LFO_E_SHAPE;
  u128 q = q_from_le(q_le);
  if (q < 2 || q >= MAX_MODULUS) return LFO_E_MODULUS;
  std::vector<B128> words = table_words(table, s.words);
  std::vector<u128> matrix = ajtai_matrix(q, s.ring_elements);
  std::vector<u128> cols;
  if (mode == 1) {
    if (q != BASELINE_Q) return LFO_E_MODULUS;
    commit_ntt(s, words.data(), matrix, cols);
  } else {
    if ((u128)(s.ring_elements * N) + 2 > (((u128)1 << 127) / q)) return LFO_E_MODULUS;
    commit_schoolbook(s, words.data(), matrix, q, cols);
  }
  pack_ring_elements(cols.data(), cols.size(), q, out);
  return LFO_OK;
}

// reference.rs:137-177 (prove). r_hi_at, when not NULL, replaces the sampled packed coordinates
// (lfo_prove_at_point); the transcript still draws them, so every later sample is the same.
static int prove_impl(const uint8_t seed[32], const uint8_t q_le[16], uint32_t log_vars, const uint8_t* table_bytes,
                      int commit_mode, uint8_t* proof_out, size_t cap, size_t* len, uint8_t* trace, size_t trace_cap,
                      const uint8_t* r_hi_at) {
  Shape s;
  if (!s.set(log_vars)) return LFO_E_SHAPE;
  u128 q = q_from_le(q_le);
  if (accept_modulus(q, s) != LFO_OK) return LFO_E_MODULUS;
  size_t need = proof_size(q, s);
  if (len) *len = need;
  if (!proof_out || cap < need) return LFO_E_CAP;
  TraceWriter tw{trace, trace_cap};
  std::vector<uint8_t> generated;
  if (!table_bytes) {
    generated.resize(s.words * 16);
    lfo_write_table(seed, log_vars, generated.data());
    table_bytes = generated.data();
  }
  std::vector<B128> values = table_words(table_bytes, s.words);
  Proof pr;
  pr.modulus = q;
  {
    std::vector<u128> matrix = ajtai_matrix(q, s.ring_elements);
    std::vector<u128> cols;
    if (commit_mode == 1 && q == BASELINE_Q)
      commit_ntt(s, values.data(), matrix, cols);
    else
      commit_schoolbook(s, values.data(), matrix, q, cols);
    pr.commitment.resize(coefficient_bytes(q) * cols.size());
    pack_ring_elements(cols.data(), cols.size(), q, pr.commitment.data());
  }
  Transcript t = transcript(seed, s, q, pr.commitment);
  std::vector<B128> lo = t.sample_b128("r-lo", 7);
  std::vector<B128> hi = t.sample_b128("r-hi", s.lp);
  if (r_hi_at) memcpy(hi.data(), r_hi_at, 16 * (size_t)s.lp);
  tw.b128(lo), tw.b128(hi);
  std::vector<B128> eq(s.words);
  eq_expand_b128_par(hi.data(), s.lp, eq.data());
  pr.partials = partial_evals(values.data(), eq.data(), s.words);
  B128 value = claim(pr.partials, lo);
  tw.b128(pr.partials), tw.b128({value});
  t.absorb_b128(&value, 1);
  t.absorb_b128(pr.partials.data(), 128);
  std::vector<F162> rb = t.sample_f162("switch-batch", 7);
  std::vector<F162> batch = eq_expand_f162(rb.data(), 7);
  tw.f162(rb);
  // SwitchProver::from_workspace with gammas = [ONE] (crossfield.rs:600-634).
  std::vector<F162> a(s.words), p(s.words);
  {
    Psi psi(batch);
    parallel_for(s.words, [&](size_t b, size_t e) {
      for (size_t j = b; j < e; ++j) a[j] = psi(eq[j]), p[j] = lift(values[j]);
    }, 1 << 14);
  }
  size_t half = s.words;
  std::vector<F162> coords;
  for (int round = 0; round < s.lp; ++round) {
    half /= 2;
    std::vector<std::pair<F162, F162>> parts(threads(), {F_ZERO, F_ZERO});
    std::atomic<int> slot{0};
    parallel_for(half, [&](size_t b, size_t e) {
      F162 e0 = F_ZERO, ei = F_ZERO;
      for (size_t j = b; j < e; ++j) {
        e0 = fadd(e0, fmul(a[j], p[j]));
        ei = fadd(ei, fmul(fadd(a[j], a[j + half]), fadd(p[j], p[j + half])));
      }
      parts[slot++] = {e0, ei};
    }, 1 << 12);
    F162 msg[2] = {F_ZERO, F_ZERO};
    for (auto& x : parts) msg[0] = fadd(msg[0], x.first), msg[1] = fadd(msg[1], x.second);
    t.absorb_f162(msg, 2);
    F162 r = t.sample_f162("switch-round", 1)[0];
    pr.rounds.push_back(msg[0]);
    pr.rounds.push_back(msg[1]);
    coords.push_back(r);
    parallel_for(half, [&](size_t b, size_t e) {
      for (size_t j = b; j < e; ++j) {
        a[j] = fadd(a[j], fmul(r, fadd(a[j], a[j + half])));
        p[j] = fadd(p[j], fmul(r, fadd(p[j], p[j + half])));
      }
    }, 1 << 12);
  }
  pr.opened = p[0];
  tw.f162(coords), tw.f162({pr.opened});
  std::vector<F162>().swap(a);
  std::vector<F162>().swap(p);
  t.absorb_f162(&pr.opened, 1);
  std::vector<F162> p0, p1;
  split_point(s, coords, p0, p1);
  std::vector<F162> row = row_evaluate(s, values.data(), p0);
  tw.f162(row);
  pr.row = pack_f162(row);
  absorb_row(t, row);  // main.rs:284-292
  std::vector<Challenge> ch = short_challenges(t, COLUMNS);
  for (auto& c : ch) tw.put(&c, sizeof c);
  pr.folded.resize(4 * N * s.ring_elements);
  std::atomic<bool> ok{true};
  parallel_for(s.ring_elements, [&](size_t b, size_t e) {
    int16_t v[N];
    for (size_t m = b; m < e; ++m) {
      if (!fold_element(s, values.data(), ch, m, v)) ok = false;
      for (int i = 0; i < N; ++i) {
        uint32_t x = (uint32_t)(int32_t)v[i];
        uint8_t* d = &pr.folded[4 * (m * N + i)];
        d[0] = (uint8_t)x, d[1] = (uint8_t)(x >> 8), d[2] = (uint8_t)(x >> 16), d[3] = (uint8_t)(x >> 24);
      }
    }
  });
  if (!ok) return LFO_E_ARGS;
  std::vector<uint8_t> bytes = encode(pr);
  if (bytes.size() != need) return LFO_E_ARGS;
  memcpy(proof_out, bytes.data(), need);
  if (trace && !tw.ok) return LFO_E_CAP;
  return LFO_OK;
}

int lfo_prove(const uint8_t seed[32], const uint8_t q_le[16], uint32_t log_vars, const uint8_t* table_bytes,
              int commit_mode, uint8_t* proof_out, size_t cap, size_t* len, uint8_t* trace, size_t trace_cap) {
  return prove_impl(seed, q_le, log_vars, table_bytes, commit_mode, proof_out, cap, len, trace, trace_cap, nullptr);
}

int lfo_prove_at_point(const uint8_t seed[32], const uint8_t q_le[16], uint32_t log_vars, const uint8_t* table_bytes,
                       const uint8_t* r_hi, uint8_t* proof_out, size_t cap, size_t* len) {
  if (!r_hi) return LFO_E_ARGS;
  return prove_impl(seed, q_le, log_vars, table_bytes, 1, proof_out, cap, len, nullptr, 0, r_hi);
}

// main.rs:293-409 (check_proof_shape, verify, check_field_switch, check_opening)
int lfo_verify(const uint8_t seed[32], uint32_t log_vars, const uint8_t* table_bytes, const uint8_t* proof,
               size_t len, char* err, size_t err_cap) {
  auto fail = [&](const char* m) {
    if (err && err_cap) snprintf(err, err_cap, "%s", m);
    return LFO_E_REJECT;
  };
  Shape s;
  if (!s.set(log_vars)) return LFO_E_SHAPE;
  if (len > 64u * 1024 * 1024) return fail("proof too large");
  Proof pr;
  std::string e;
  if (!decode(proof, len, pr, e)) return fail(e.c_str());
  if (pr.partials.size() != 128) return fail("128 partial evaluations");
  if (pr.rounds.size() != 2 * (size_t)s.lp) return fail("one switch round per packed coordinate");
  u128 q = pr.modulus;
  if (accept_modulus(q, s) != LFO_OK) return fail("invalid commitment modulus");
  std::vector<uint8_t> generated;
  if (!table_bytes) {
    generated.resize(s.words * 16);
    lfo_write_table(seed, log_vars, generated.data());
    table_bytes = generated.data();
  }
  std::vector<B128> values = table_words(table_bytes, s.words);
  Transcript t = transcript(seed, s, q, pr.commitment);
  // check_field_switch
  std::vector<B128> lo = t.sample_b128("r-lo", 7);
  std::vector<B128> hi = t.sample_b128("r-hi", s.lp);
  std::vector<B128> eq(s.words);
  eq_expand_b128_par(hi.data(), s.lp, eq.data());
  std::vector<B128> trusted = partial_evals(values.data(), eq.data(), s.words);
  std::vector<B128>().swap(eq);
  B128 value = claim(trusted, lo);
  t.absorb_b128(&value, 1);
  t.absorb_b128(pr.partials.data(), 128);
  std::vector<F162> rb = t.sample_f162("switch-batch", 7);
  std::vector<F162> batch = eq_expand_f162(rb.data(), 7);
  if (!(claim(pr.partials, lo) == value)) return fail("partial evaluation mismatch");
  F162 sum = slice_sum(pr.partials, batch);
  std::vector<F162> coords;
  for (int r = 0; r < s.lp; ++r) {
    F162 e0 = pr.rounds[2 * r], einf = pr.rounds[2 * r + 1];
    if ((e0.w[2] >> 34) || (einf.w[2] >> 34)) return fail("noncanonical F162 element");
    t.absorb_f162(&pr.rounds[2 * r], 2);
    F162 ch = t.sample_f162("switch-round", 1)[0];
    F162 e1 = fadd(sum, e0);
    sum = fadd(fadd(e0, fmul(ch, fadd(fadd(e0, e1), einf))), fmul(fmul(ch, ch), einf));
    coords.push_back(ch);
  }
  if (pr.opened.w[2] >> 34) return fail("noncanonical F162 element");
  F162 d = transparent_coeff(hi, coords, batch);
  if (d == F_ZERO) return fail("the switch left the opened value unbound");
  if (sum != fmul(d, pr.opened)) return fail("sumcheck final check failed");
  t.absorb_f162(&pr.opened, 1);
  // check_opening
  std::vector<F162> p0, p1;
  split_point(s, coords, p0, p1);
  std::vector<F162> row;
  if (!unpack_f162(pr.row.data(), pr.row.size(), COLUMNS, row)) return fail("malformed row evaluation");
  if (pr.folded.size() != 4 * (size_t)N * s.ring_elements) return fail("malformed folded witness");
  std::vector<int16_t> v(N * s.ring_elements);
  for (size_t i = 0; i < v.size(); ++i) {
    int32_t w = (int32_t)((uint32_t)pr.folded[4 * i] | ((uint32_t)pr.folded[4 * i + 1] << 8) |
                          ((uint32_t)pr.folded[4 * i + 2] << 16) | ((uint32_t)pr.folded[4 * i + 3] << 24));
    if (w < -32768 || w > 32767) return fail("malformed folded witness");
    v[i] = (int16_t)w;
  }
  absorb_row(t, row);
  std::vector<Challenge> ch = short_challenges(t, COLUMNS);
  {
    std::vector<F162> e1 = eq_table(p1.data(), (int)p1.size());
    F162 acc = F_ZERO;
    for (int j = 0; j < COLUMNS; ++j) acc = fadd(acc, fmul(e1[j], row[j]));
    if (acc != pr.opened) return fail("the row evaluation does not reduce to the opened value");
  }
  uint64_t normsq = 0;
  u128 worst = 0;
  for (int16_t c : v) {
    uint64_t m = (uint64_t)(c < 0 ? -(int32_t)c : c);
    normsq += m * m;
    worst = std::max<u128>(worst, m);
  }
  if (normsq > fold_cap(s)) return fail("the fold is longer than the cap");
  if (worst > (q - 1) / 2) return fail("the fold is not centered");
  size_t w = coefficient_bytes(q);
  if (pr.commitment.size() != w * COLUMNS * N) return fail("malformed commitment");
  std::vector<u128> cols(COLUMNS * N);
  for (size_t i = 0; i < cols.size(); ++i) {
    u128 x = 0;
    for (size_t b = w; b-- > 0;) x = (x << 8) | pr.commitment[i * w + b];
    if (x >= q) return fail("malformed commitment");
    cols[i] = x;
  }
  std::vector<u128> matrix = ajtai_matrix(q, s.ring_elements);
  if (a_times_v(matrix, v, q) != challenge_combination(cols, ch, q))
    return fail("the fold does not open the folded commitment");
  {
    std::vector<F162> e0 = eq_table(p0.data(), (int)p0.size());
    F162 left = F_ZERO, right = F_ZERO;
    for (size_t m = 0; m < s.ring_elements; ++m)
      for (int k = 0; k < 4; ++k) {
        F162 x = F_ZERO;  // components_mod_2 (main.rs:268-280)
        for (int pp = 0; pp < N / 4; ++pp)
          if (v[m * N + 4 * pp + k] & 1) x.w[pp >> 6] |= 1ull << (pp & 63);
        left = fadd(left, fmul(e0[4 * m + k], x));
      }
    for (int j = 0; j < COLUMNS; ++j) right = fadd(right, fmul(challenge_to_f162(ch[j]), row[j]));
    if (left != right) return fail("the fold does not match the folded row evaluation");
  }
  return LFO_OK;
}

int lfo_short_challenges(const char* domain, const uint8_t* prefix, size_t prefix_len, uint32_t n, uint8_t* out) {
  Transcript t(domain);
  t.absorb_bytes(prefix, prefix_len);
  std::vector<Challenge> ch = short_challenges(t, n);
  for (uint32_t i = 0; i < n; ++i) {
    memcpy(out + 40 * i, ch[i].positions, 32);
    memcpy(out + 40 * i + 32, &ch[i].signs, 4);
    memcpy(out + 40 * i + 36, &ch[i].weight, 4);
  }
  return LFO_OK;
}

double lfo_norm_blocked(const uint8_t positions[32], uint32_t signs, uint32_t weight) {
  Challenge c;
  memcpy(c.positions, positions, 32);
  c.signs = signs, c.weight = weight;
  return norm_blocked(c);
}
double lfo_norm_horner(const uint8_t positions[32], uint32_t signs, uint32_t weight) {
  Challenge c;
  memcpy(c.positions, positions, 32);
  c.signs = signs, c.weight = weight;
  return norm_horner(c);
}

}  // extern "C"
