"""Python binding of liblabinius_gpu (ctypes over include/labinius_gpu.h).

The prover mirrors the reference's `prove(seed, Q, table) -> proof` boundary
(solution/proof_generate/src/main.rs:1692-2009) with the bincode proof layout of
verifier/proof_verify/src/main.rs:98-124. There is no CPU path: without the CUDA library or a
device every call raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblabinius_gpu.so")
CLI_PATH = os.path.join(HERE, "_build", "labinius-fast")
BASELINE_Q = 3889 * 9721 * 17497

LF_OK = 0
ERRORS = {
    -1: "LF_E_ARGS", -2: "LF_E_SHAPE", -3: "LF_E_MODULUS", -4: "LF_E_TABLE_LEN", -5: "LF_E_CAP",
    -6: "LF_E_OOM", -7: "LF_E_CUDA", -8: "LF_E_INTERNAL", -9: "LF_E_ADMISSION", -10: "LF_E_LIMIT",
    -11: "LF_E_TIMEOUT", -12: "LF_E_TICKET", -13: "LF_E_REJECT",
}
LF_E_ARGS = -1
LF_E_MODULUS = -3
LF_E_REJECT = -13
LF_E_TIMEOUT = -11
NOALLOC_MAX_CHALLENGES = 4096
EXPORTS = [
    "lf_ctx_create", "lf_ctx_destroy", "lf_ctx_stream", "lf_proof_size", "lf_accept_modulus", "lf_key_prepare", "lf_prove",
    "lf_prove_device", "lf_write_table_device", "lf_device_alloc", "lf_device_free", "lf_memcpy_h2d",
    "lf_last_profile", "lf_strerror", "lf_last_error", "lf_last_challenges",
    "lf_sample_challenges", "lf_sample_challenges_noalloc", "lf_prove_batch", "lf_submit", "lf_poll",
    "lf_verify", "lf_verify_device", "lf_request_footprint", "lf_ring_mul", "lf_ghash_mul", "lf_ajtai_matrix_device",
    "lf_a_times_v", "lf_tune", "lf_test_set_point", "lf_test_withhold_table_part", "lf_test_table_part_order",
]


class LfError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class TuneResult(ctypes.Structure):
    _fields_ = [("commit_splits", ctypes.c_int), ("commit_ms", ctypes.c_float), ("candidates", ctypes.c_int),
                ("fold_splits", ctypes.c_int), ("fold_ms", ctypes.c_float), ("fold_candidates", ctypes.c_int)]


class Config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("hbm_budget", ctypes.c_size_t), ("lanes", ctypes.c_int)]


class Job(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_char_p), ("q_le", ctypes.c_char_p), ("log_vars", ctypes.c_uint32),
                ("table_on_device", ctypes.c_int), ("table", ctypes.c_void_p), ("table_bytes", ctypes.c_size_t),
                ("proof", ctypes.POINTER(ctypes.c_uint8)), ("proof_cap", ctypes.c_size_t)]


class Result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("proof_len", ctypes.c_size_t), ("queue_ms", ctypes.c_double),
                ("run_ms", ctypes.c_double), ("device_ms", ctypes.c_double), ("commit_ms", ctypes.c_double),
                ("upload_ms", ctypes.c_double)]


class Profile(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in (
        "upload_ms", "key_ms", "commit_ms", "finish_ms", "transcript_ms", "partials_ms", "switch_ms", "row_ms",
        "challenges_ms", "fold_ms", "download_ms", "total_ms")] + [("launches", ctypes.c_int)] + [
        (n, ctypes.c_double) for n in ("switch_blocks_ms", "switch_materialize_ms", "switch_tail_ms")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


_lib = None


def load(path=LIB_PATH):
    """The shared library, loaded once. Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is missing: run labinius-fast-challenge_gb300/build.py")
    lib = ctypes.CDLL(path)
    p, u8p, sz = ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint8), ctypes.c_size_t
    lib.lf_ctx_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(p)]
    lib.lf_ctx_destroy.argtypes = [p]
    lib.lf_ctx_destroy.restype = None
    lib.lf_ctx_stream.argtypes = [p]
    lib.lf_ctx_stream.restype = p
    lib.lf_proof_size.argtypes = [ctypes.c_char_p, ctypes.c_uint32]
    lib.lf_proof_size.restype = sz
    lib.lf_accept_modulus.argtypes = [ctypes.c_char_p, ctypes.c_uint32]
    lib.lf_key_prepare.argtypes = [p, ctypes.c_char_p, ctypes.c_uint32]
    lib.lf_prove.argtypes = [p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint32, p, sz, u8p, sz,
                             ctypes.POINTER(sz)]
    lib.lf_prove_device.argtypes = [p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint32, p, u8p, sz,
                                    ctypes.POINTER(sz)]
    lib.lf_write_table_device.argtypes = [p, ctypes.c_char_p, ctypes.c_uint32, p]
    lib.lf_device_alloc.argtypes = [p, sz, ctypes.POINTER(p)]
    lib.lf_device_free.argtypes = [p, p]
    lib.lf_memcpy_h2d.argtypes = [p, p, p, sz]
    lib.lf_last_profile.argtypes = [p, ctypes.POINTER(Profile)]
    lib.lf_strerror.argtypes = [ctypes.c_int]
    lib.lf_strerror.restype = ctypes.c_char_p
    lib.lf_last_error.argtypes = [p]
    lib.lf_last_error.restype = ctypes.c_char_p
    lib.lf_last_challenges.argtypes = [p, u8p, sz]
    lib.lf_sample_challenges.argtypes = [p, ctypes.c_char_p, ctypes.c_char_p, sz, ctypes.c_uint32, u8p]
    lib.lf_verify.argtypes = [p, ctypes.c_char_p, ctypes.c_uint32, p, sz, ctypes.c_char_p, sz]
    lib.lf_verify_device.argtypes = [p, ctypes.c_char_p, ctypes.c_uint32, p, ctypes.c_char_p, sz]
    lib.lf_prove_batch.argtypes = [p, sz, ctypes.POINTER(Job), ctypes.POINTER(Result)]
    lib.lf_submit.argtypes = [p, ctypes.POINTER(Job), ctypes.POINTER(ctypes.c_uint64)]
    lib.lf_poll.argtypes = [p, ctypes.c_uint64, ctypes.c_uint32, ctypes.POINTER(Result)]
    lib.lf_request_footprint.argtypes = [p, ctypes.c_char_p, ctypes.c_uint32, ctypes.c_int]
    lib.lf_request_footprint.restype = sz
    lib.lf_tune.argtypes = [p, ctypes.c_char_p, ctypes.c_uint32, p, ctypes.POINTER(TuneResult)]
    lib.lf_ring_mul.argtypes = [p, ctypes.c_char_p, sz, p, p, p]
    lib.lf_ghash_mul.argtypes = [p, sz, p, p, p]
    lib.lf_ajtai_matrix_device.argtypes = [p, ctypes.c_char_p, ctypes.c_uint64, p]
    lib.lf_a_times_v.argtypes = [p, ctypes.c_char_p, ctypes.c_uint64, p, u8p]
    lib.lf_sample_challenges_noalloc.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p, sz, ctypes.c_uint32,
                                                 u8p, p]
    lib.lf_test_set_point.argtypes = [p, ctypes.c_char_p, ctypes.c_uint32]
    lib.lf_test_withhold_table_part.argtypes = [p, ctypes.c_int, ctypes.c_uint64]
    lib.lf_test_table_part_order.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_int, u8p,
                                             ctypes.POINTER(ctypes.c_int)]
    _lib = lib
    return lib


def _parse_challenges(raw, n):
    out = []
    for i in range(n):
        c = raw[40 * i:40 * i + 40]
        w = int.from_bytes(c[36:40], "little")
        out.append((list(c[:w]), int.from_bytes(c[32:36], "little"), w))
    return out


def sample_challenges_noalloc(domain, prefix, n, device=0, stream=None):
    """n challenges from lf_sample_challenges_noalloc: no context and no device allocation.
    `stream` is a cudaStream_t handle as an int (None = the legacy default stream)."""
    buf = (ctypes.c_uint8 * (40 * max(n, 1)))()
    rc = load().lf_sample_challenges_noalloc(device, domain.encode(), bytes(prefix), len(prefix), n, buf, stream)
    if rc != LF_OK:
        raise LfError(rc, load().lf_strerror(rc).decode())
    return _parse_challenges(bytes(buf), n)


def table_part_order(ring_elements, splits, blocks_per_split, sms):
    """lf_test_table_part_order (host only): the copy order lf_prove gives a streamed table's parts."""
    lib = load()
    buf = (ctypes.c_uint8 * 64)()
    n = ctypes.c_int()
    rc = lib.lf_test_table_part_order(ring_elements, splits, blocks_per_split, sms, buf, ctypes.byref(n))
    if rc != LF_OK:
        raise LfError(rc, "table part order")
    return list(buf[:n.value])


def q_bytes(q):
    return int(q).to_bytes(16, "little")


def proof_size(q, log_vars):
    return load().lf_proof_size(q_bytes(q), log_vars)


def accept_modulus(q, log_vars):
    return load().lf_accept_modulus(q_bytes(q), log_vars) == LF_OK


class Prover:
    """One device context (lf_ctx). Not thread-safe across calls; the C side serialises."""

    def __init__(self, device=0, hbm_budget=0, lanes=0):
        self.lib = load()
        self.ctx = ctypes.c_void_p()
        self.device, self.lanes = device, lanes
        cfg = Config(device, hbm_budget, lanes)
        rc = self.lib.lf_ctx_create(ctypes.byref(cfg), ctypes.byref(self.ctx))
        if rc != LF_OK:
            raise LfError(rc, "context creation failed (no CUDA device?)")

    def close(self):
        if self.ctx:
            self.lib.lf_ctx_destroy(self.ctx)
            self.ctx = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc != LF_OK:
            raise LfError(rc, self.lib.lf_last_error(self.ctx).decode())

    def prove(self, seed, table, log_vars, q=BASELINE_Q, out=None):
        """Proof bytes for a host table (bytes, bytearray, memoryview, numpy array or ctypes buffer).
        With `out` (a ctypes buffer of at least proof_size bytes, reused across calls) the proof is
        written there and (out, length) is returned instead of a bytes copy."""
        mv = memoryview(table).cast("B")
        cap = proof_size(q, log_vars)
        keep = out
        out = out if out is not None else (ctypes.c_uint8 * max(cap, 1))()
        n = ctypes.c_size_t()
        buf = (ctypes.c_uint8 * len(mv)).from_buffer_copy(mv) if mv.readonly else (ctypes.c_uint8 * len(mv)).from_buffer(mv)
        rc = self.lib.lf_prove(self.ctx, bytes(seed), q_bytes(q), log_vars, ctypes.cast(buf, ctypes.c_void_p),
                               len(mv), out, cap, ctypes.byref(n))
        self._check(rc)
        if keep is not None:
            return out, n.value
        return ctypes.string_at(out, n.value)

    def prove_device(self, seed, table_dev, log_vars, q=BASELINE_Q, out=None):
        cap = proof_size(q, log_vars)
        out = out if out is not None else (ctypes.c_uint8 * cap)()
        n = ctypes.c_size_t()
        rc = self.lib.lf_prove_device(self.ctx, bytes(seed), q_bytes(q), log_vars, ctypes.c_void_p(table_dev), out,
                                      cap, ctypes.byref(n))
        self._check(rc)
        return out, n.value

    def key_prepare(self, log_vars, q=BASELINE_Q):
        self._check(self.lib.lf_key_prepare(self.ctx, q_bytes(q), log_vars))

    def verify(self, seed, proof, log_vars, table=None):
        """(accepted, message) from the GPU checker. `table` is host bytes, or None to regenerate the
        seed's table on the device. Errors other than a rejection raise."""
        if table is None:
            rc = self.lib.lf_verify(self.ctx, bytes(seed), log_vars, None, 0, bytes(proof), len(proof))
        else:
            mv = memoryview(table).cast("B")
            buf = (ctypes.c_uint8 * len(mv)).from_buffer_copy(mv) if mv.readonly else (ctypes.c_uint8 * len(mv)).from_buffer(mv)
            rc = self.lib.lf_verify(self.ctx, bytes(seed), log_vars, ctypes.cast(buf, ctypes.c_void_p), len(mv),
                                    bytes(proof), len(proof))
        if rc == LF_OK:
            return True, ""
        if rc == LF_E_REJECT:
            return False, self.lib.lf_last_error(self.ctx).decode()
        self._check(rc)

    def verify_device(self, seed, proof, log_vars, table_dev):
        """(accepted, message) from the GPU checker for a device-resident table."""
        rc = self.lib.lf_verify_device(self.ctx, bytes(seed), log_vars, ctypes.c_void_p(table_dev), bytes(proof),
                                       len(proof))
        if rc == LF_OK:
            return True, ""
        if rc == LF_E_REJECT:
            return False, self.lib.lf_last_error(self.ctx).decode()
        self._check(rc)

    def make_job(self, seed, table, log_vars, q=BASELINE_Q, on_device=False, nbytes=None):
        """A job and the buffers it points to (kept alive on the returned object). `table` is bytes /
        a ctypes buffer / an int host address (host tables), or an int device pointer with
        on_device=True."""
        cap = proof_size(q, log_vars)
        keep = {"seed": bytes(seed), "q": q_bytes(q), "proof": (ctypes.c_uint8 * cap)()}
        if on_device:
            addr, n = int(table), 0
        elif isinstance(table, int):
            addr, n = table, nbytes
        else:
            buf = table if isinstance(table, ctypes.Array) else (ctypes.c_uint8 * len(table)).from_buffer_copy(table)
            keep["table"] = buf
            addr, n = ctypes.addressof(buf), ctypes.sizeof(buf)
        job = Job(keep["seed"], keep["q"], log_vars, 1 if on_device else 0, addr, n, keep["proof"], cap)
        job._keep = keep
        return job

    @staticmethod
    def job_proof(job, result):
        return ctypes.string_at(job._keep["proof"], result.proof_len)

    def prove_batch(self, jobs):
        """Results of lf_prove_batch, one per job (status checked by the caller)."""
        arr = (Job * len(jobs))(*jobs)
        res = (Result * len(jobs))()
        self.lib.lf_prove_batch(self.ctx, len(jobs), arr, res)
        return list(res)

    def submit(self, job):
        t = ctypes.c_uint64()
        self._check(self.lib.lf_submit(self.ctx, ctypes.byref(job), ctypes.byref(t)))
        return t.value

    def footprint(self, log_vars, q=BASELINE_Q, host_table=True):
        """Device bytes one request holds while proven (what admission compares with the budget)."""
        return self.lib.lf_request_footprint(self.ctx, q_bytes(q), log_vars, 1 if host_table else 0)

    def tune(self, log_vars, table_dev, q=BASELINE_Q):
        """lf_tune: the commitment's split count and the fold's column-run count measured for this
        shape; returns (commit splits, commit ms, candidates), the whole result in self.last_tune."""
        r = TuneResult()
        self._check(self.lib.lf_tune(self.ctx, q_bytes(q), log_vars, ctypes.c_void_p(table_dev), ctypes.byref(r)))
        self.last_tune = {f: getattr(r, f) for f, _ in TuneResult._fields_}
        return r.commit_splits, r.commit_ms, r.candidates

    def ring_mul(self, q, n, a_dev, b_dev, c_dev):
        """c = a * b in R_q for n pairs of device elements (648 u128 LE coefficients each)."""
        self._check(self.lib.lf_ring_mul(self.ctx, q_bytes(q), n, ctypes.c_void_p(a_dev), ctypes.c_void_p(b_dev),
                                         ctypes.c_void_p(c_dev)))

    def ghash_mul(self, n, a_dev, b_dev, c_dev):
        self._check(self.lib.lf_ghash_mul(self.ctx, n, ctypes.c_void_p(a_dev), ctypes.c_void_p(b_dev),
                                          ctypes.c_void_p(c_dev)))

    def ajtai_matrix_device(self, q, elements, out_dev):
        self._check(self.lib.lf_ajtai_matrix_device(self.ctx, q_bytes(q), elements, ctypes.c_void_p(out_dev)))

    def a_times_v(self, q, elements, v_dev):
        """rq::a_times_v of ajtai_matrix(q, elements) and the device int16 vector v: 648 ints."""
        out = (ctypes.c_uint8 * (16 * 648))()
        self._check(self.lib.lf_a_times_v(self.ctx, q_bytes(q), elements, ctypes.c_void_p(v_dev), out))
        raw = bytes(out)
        return [int.from_bytes(raw[16 * i:16 * i + 16], "little") for i in range(648)]

    def poll(self, ticket, wait_ms=0):
        """(code, Result): LF_OK with the result, LF_E_TIMEOUT while pending."""
        r = Result()
        rc = self.lib.lf_poll(self.ctx, ticket, wait_ms, ctypes.byref(r))
        return rc, r

    def stream(self):
        """The context's cudaStream_t as an int (every call of this prover runs on it)."""
        return self.lib.lf_ctx_stream(self.ctx) or 0

    def alloc(self, nbytes):
        p = ctypes.c_void_p()
        self._check(self.lib.lf_device_alloc(self.ctx, nbytes, ctypes.byref(p)))
        return p.value

    def free(self, dev):
        self._check(self.lib.lf_device_free(self.ctx, ctypes.c_void_p(dev)))

    def h2d(self, dev, data):
        mv = memoryview(data).cast("B")
        buf = (ctypes.c_uint8 * len(mv)).from_buffer_copy(mv)
        self._check(self.lib.lf_memcpy_h2d(self.ctx, ctypes.c_void_p(dev), buf, len(mv)))

    def write_table_device(self, seed, log_vars, dev):
        self._check(self.lib.lf_write_table_device(self.ctx, bytes(seed), log_vars, ctypes.c_void_p(dev)))

    def sample_challenges(self, domain, prefix, n):
        buf = (ctypes.c_uint8 * (40 * n))()
        self._check(self.lib.lf_sample_challenges(self.ctx, domain.encode(), bytes(prefix), len(prefix), n, buf))
        return _parse_challenges(bytes(buf), n)

    def last_challenges(self):
        """[(positions, signs, weight)] of the last proof's 1024 folding challenges."""
        buf = (ctypes.c_uint8 * (40 * 1024))()
        self._check(self.lib.lf_last_challenges(self.ctx, buf, 40 * 1024))
        return _parse_challenges(bytes(buf), 1024)

    def test_set_point(self, r_hi):
        """Test hook: the next proof uses r_hi (a list of 16-byte GHASH elements, or ints) as its
        packed point coordinates instead of sampling them."""
        raw = b"".join(x if isinstance(x, (bytes, bytearray)) else int(x).to_bytes(16, "little") for x in r_hi)
        self._check(self.lib.lf_test_set_point(self.ctx, raw, len(raw) // 16))

    def test_withhold_table_part(self, part, wait_cycles=0):
        """Test hook: the next streamed table upload leaves `part`'s ready flag unset; the commitment
        gives up after wait_cycles SM cycles and the proof returns LF_E_INTERNAL."""
        self._check(self.lib.lf_test_withhold_table_part(self.ctx, part, wait_cycles))

    def profile(self):
        p = Profile()
        self._check(self.lib.lf_last_profile(self.ctx, ctypes.byref(p)))
        return p.as_dict()
