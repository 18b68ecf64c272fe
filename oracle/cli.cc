// lf-oracle: command-line front end of the CPU oracle (TEST INFRASTRUCTURE).
//
//   LABINIUS_SEED=<64 hex> lf-oracle --write-table FILE [--log-vars L]
//   LABINIUS_SEED=<64 hex> lf-oracle --prove FILE --table FILE [--modulus Q] [--log-vars L] [--commit ntt|schoolbook]
//   LABINIUS_SEED=<64 hex> lf-oracle --verify FILE [--table FILE] [--log-vars L]
//
// Mirrors labinius-fast-verify (verifier/proof_verify/src/main.rs:411-458) with LOG_VARS as an option.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "oracle.h"

static bool parse_seed(uint8_t seed[32]) {
  const char* s = getenv("LABINIUS_SEED");
  if (!s || strlen(s) != 64) return false;
  for (int i = 0; i < 32; ++i) {
    char b[3] = {s[2 * i], s[2 * i + 1], 0};
    char* end;
    long v = strtol(b, &end, 16);
    if (*end) return false;
    seed[i] = (uint8_t)v;
  }
  return true;
}

static bool parse_q(const char* t, uint8_t q[16]) {
  unsigned __int128 x = 0;
  if (!*t) return false;
  for (const char* p = t; *p; ++p) {
    if (*p < '0' || *p > '9') return false;
    unsigned __int128 n = x * 10 + (unsigned)(*p - '0');
    if (n / 10 != x) return false;
    x = n;
  }
  for (int i = 0; i < 16; ++i) q[i] = (uint8_t)(x >> (8 * i));
  return true;
}

static std::vector<uint8_t> read_file(const char* path) {
  std::vector<uint8_t> v;
  FILE* f = fopen(path, "rb");
  if (!f) return v;
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  v.resize((size_t)n);
  if (n && fread(v.data(), 1, (size_t)n, f) != (size_t)n) v.clear();
  fclose(f);
  return v;
}

static bool write_file(const char* path, const uint8_t* p, size_t n) {
  FILE* f = fopen(path, "wb");
  if (!f) return false;
  bool ok = fwrite(p, 1, n, f) == n;
  return fclose(f) == 0 && ok;
}

int main(int argc, char** argv) {
  std::string cmd, target, table, commit = "ntt";
  uint32_t log_vars = 31;
  uint8_t q[16];
  parse_q("661473542593", q);
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    auto next = [&]() -> const char* {
      if (i + 1 >= argc) {
        fprintf(stderr, "missing value for %s\n", a.c_str());
        exit(2);
      }
      return argv[++i];
    };
    if (a == "--write-table" || a == "--prove" || a == "--verify")
      cmd = a, target = next();
    else if (a == "--table")
      table = next();
    else if (a == "--log-vars")
      log_vars = (uint32_t)atoi(next());
    else if (a == "--modulus") {
      if (!parse_q(next(), q)) return fprintf(stderr, "invalid modulus\n"), 2;
    } else if (a == "--commit")
      commit = next();
    else if (a == "--threads")
      lfo_set_threads(atoi(next()));
    else
      return fprintf(stderr, "unknown option %s\n", a.c_str()), 2;
  }
  uint8_t seed[32];
  if (!parse_seed(seed)) return fprintf(stderr, "LABINIUS_SEED is required (64 hex chars)\n"), 2;
  auto t0 = std::chrono::steady_clock::now();
  if (cmd == "--write-table") {
    std::vector<uint8_t> t(((size_t)1 << log_vars) / 8);
    if (lfo_write_table(seed, log_vars, t.data())) return fprintf(stderr, "bad shape\n"), 2;
    return write_file(target.c_str(), t.data(), t.size()) ? 0 : 1;
  }
  if (cmd == "--prove") {
    std::vector<uint8_t> t;
    if (!table.empty()) {
      t = read_file(table.c_str());
      if (t.size() != ((size_t)1 << log_vars) / 8) return fprintf(stderr, "witness table has the wrong length\n"), 1;
    }
    if (lfo_accept_modulus(q, log_vars)) return fprintf(stderr, "invalid commitment modulus\n"), 1;
    size_t n = lfo_proof_size(q, log_vars);
    std::vector<uint8_t> proof(n);
    size_t len = 0;
    int rc = lfo_prove(seed, q, log_vars, t.empty() ? nullptr : t.data(), commit == "ntt" ? 1 : 0, proof.data(),
                       proof.size(), &len, nullptr, 0);
    if (rc) return fprintf(stderr, "prove failed: %d\n", rc), 1;
    if (!write_file(target.c_str(), proof.data(), len)) return 1;
    double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    fprintf(stderr, "lf-oracle prove_ms=%.1f\n", ms);
    return 0;
  }
  if (cmd == "--verify") {
    std::vector<uint8_t> p = read_file(target.c_str());
    std::vector<uint8_t> t;
    if (!table.empty()) t = read_file(table.c_str());
    char err[256] = {0};
    int rc = lfo_verify(seed, log_vars, t.empty() ? nullptr : t.data(), p.data(), p.size(), err, sizeof err);
    if (rc) return fprintf(stderr, "rejected: %s\n", err), 1;
    uint64_t qq[2];
    memcpy(qq, p.data() + 4, 16);
    printf("{\"accepted\":true,\"polynomialSize\":%llu}\n", (unsigned long long)1 << log_vars);
    return 0;
  }
  fprintf(stderr, "usage: lf-oracle --write-table FILE | --prove FILE --table FILE [--modulus Q] | --verify FILE\n");
  return 2;
}
