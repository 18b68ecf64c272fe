// labinius-fast: the drop-in prover executable.
//
//   LABINIUS_SEED=<64 hex> labinius-fast --prove FILE --table FILE [--modulus Q]
//
// Same contract as solution/proof_generate/src/main.rs:2050-2090 (and the ARM track's
// solution-arm/proof_generate/src/main.rs:940-972): the table file must hold exactly
// 2^LOG_VARS / 8 bytes, the modulus passes the checker's gate, any failure exits nonzero.
// `--log-vars L` selects a smaller instance (default 31, the challenge's).
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <time.h>
#include <unistd.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "labinius_gpu.h"

// CLOCK_MONOTONIC in nanoseconds (the clock a harness timing the process from outside reads).
static long long mono_ns() {
  timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (long long)ts.tv_sec * 1000000000LL + ts.tv_nsec;
}

static int die(const char* msg) {
  fprintf(stderr, "labinius-fast: %s\n", msg);
  return 1;
}

int main(int argc, char** argv) {
  const long long main_ns = mono_ns();
  auto t0 = std::chrono::steady_clock::now();
  std::string proof_path, table_path, modulus = "661473542593";
  uint32_t log_vars = 31;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    if (i + 1 >= argc) return die("usage: labinius-fast --prove FILE --table FILE [--modulus Q]");
    if (a == "--prove")
      proof_path = argv[++i];
    else if (a == "--table")
      table_path = argv[++i];
    else if (a == "--modulus")
      modulus = argv[++i];
    else if (a == "--log-vars")
      log_vars = (uint32_t)atoi(argv[++i]);
    else
      return die("unknown option");
  }
  if (proof_path.empty() || table_path.empty()) return die("usage: labinius-fast --prove FILE --table FILE [--modulus Q]");
  const char* s = getenv("LABINIUS_SEED");
  if (!s || strlen(s) != 64) return die("LABINIUS_SEED is required (64 hex characters)");
  uint8_t seed[32];
  for (int i = 0; i < 32; ++i) {
    char b[3] = {s[2 * i], s[2 * i + 1], 0};
    char* end;
    seed[i] = (uint8_t)strtol(b, &end, 16);
    if (*end) return die("invalid seed");
  }
  unsigned __int128 q = 0;
  for (char ch : modulus) {
    if (ch < '0' || ch > '9') return die("invalid modulus");
    unsigned __int128 n = q * 10 + (unsigned)(ch - '0');
    if (n / 10 != q) return die("invalid modulus");
    q = n;
  }
  uint8_t q_le[16];
  for (int i = 0; i < 16; ++i) q_le[i] = (uint8_t)(q >> (8 * i));
  if (lf_accept_modulus(q_le, log_vars) != LF_OK) return die("invalid commitment modulus");

  // The CUDA context (most of a one-proof process's time) and the commitment key are made on a
  // thread while this one maps and checks the table and the proof file.
  auto ti = std::chrono::steady_clock::now();
  lf_ctx* ctx = nullptr;
  int ctx_rc = LF_OK, key_rc = LF_OK;
  std::chrono::steady_clock::time_point t_ctx, t_key;
  std::thread init([&] {
    lf_config cfg = {0, 0, 1};
    ctx_rc = lf_ctx_create(&cfg, &ctx);
    t_ctx = std::chrono::steady_clock::now();
    if (ctx_rc == LF_OK) key_rc = lf_key_prepare(ctx, q_le, log_vars);
    t_key = std::chrono::steady_clock::now();
  });
  // A failure below ends the process at once (_exit: no destructors run while the other thread
  // may still be inside the CUDA runtime).
  auto quit = [&](const char* msg) {
    die(msg);
    _exit(1);
    return 1;
  };

  int fd = open(table_path.c_str(), O_RDONLY);
  if (fd < 0) return quit("read witness table");
  struct stat st;
  if (fstat(fd, &st) != 0) return quit("read witness table");
  size_t want = ((size_t)1 << log_vars) / 8;
  if ((size_t)st.st_size != want) return quit("witness table has the wrong length");
  void* table = mmap(nullptr, want, PROT_READ, MAP_PRIVATE | MAP_POPULATE, fd, 0);
  if (table == MAP_FAILED) return quit("map witness table");
  // The proof is encoded straight into the output file, mapped and pre-faulted at its final size
  // (the reference maps its output the same way, solution/proof_generate/src/main.rs:1427-1569).
  size_t cap = lf_proof_size(q_le, log_vars);
  int pfd = open(proof_path.c_str(), O_RDWR | O_CREAT | O_TRUNC, 0644);
  if (pfd < 0 || ftruncate(pfd, (off_t)cap) != 0) return quit("write proof");
  void* pmap = mmap(nullptr, cap, PROT_READ | PROT_WRITE, MAP_SHARED | MAP_POPULATE, pfd, 0);
  if (pmap == MAP_FAILED) return quit("write proof");
  auto t1 = std::chrono::steady_clock::now();
  init.join();
  auto t2 = std::chrono::steady_clock::now();
  if (ctx_rc != LF_OK) {
    unlink(proof_path.c_str());
    return die("no CUDA device");
  }
  if (key_rc != LF_OK) {
    fprintf(stderr, "labinius-fast: %s: %s\n", lf_strerror(key_rc), lf_last_error(ctx));
    unlink(proof_path.c_str());
    return 1;
  }
  size_t len = 0;
  int rc = lf_prove(ctx, seed, q_le, log_vars, table, want, static_cast<uint8_t*>(pmap), cap, &len);
  if (rc != LF_OK) {
    fprintf(stderr, "labinius-fast: %s: %s\n", lf_strerror(rc), lf_last_error(ctx));
    unlink(proof_path.c_str());
    return 1;
  }
  auto t3 = std::chrono::steady_clock::now();
  if (len != cap && ftruncate(pfd, (off_t)len) != 0) return die("write proof");
  if (munmap(pmap, cap) != 0 || close(pfd) != 0) return die("write proof");
  auto t4 = std::chrono::steady_clock::now();
  lf_profile p;
  lf_last_profile(ctx, &p);
  auto ms = [](auto a, auto b) { return std::chrono::duration<double, std::milli>(b - a).count(); };
  // load: argument checks, table and proof file mapped (concurrent with ctx + key on the other
  // thread); wait: what was left of ctx + key after the mapping; then prove and write. main_ns and
  // end_ns are CLOCK_MONOTONIC stamps at the start of main and here, for a harness to split off
  // the process start and exit.
  fprintf(stderr,
          "labinius-gb300 load_ms=%.2f ctx_ms=%.2f key_ms=%.2f wait_ms=%.2f prove_ms=%.2f write_ms=%.2f "
          "upload_ms=%.2f commit_ms=%.3f transcript_ms=%.3f partials_ms=%.3f switch_ms=%.3f row_ms=%.3f "
          "challenges_ms=%.3f fold_ms=%.3f download_ms=%.3f main_ns=%lld end_ns=%lld\n",
          ms(t0, t1), ms(ti, t_ctx), ms(t_ctx, t_key), ms(t1, t2), ms(t2, t3), ms(t3, t4), p.upload_ms, p.commit_ms,
          p.transcript_ms, p.partials_ms, p.switch_ms, p.row_ms, p.challenges_ms, p.fold_ms, p.download_ms, main_ns,
          mono_ns());
  // The proof is on disk; leave teardown of the context and mappings to process exit.
  _exit(0);
}
