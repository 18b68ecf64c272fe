"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, as the checker or the reported CPU baseline. The prover never imports it.
"""
import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
CLI = os.path.join(HERE, "_build", "lf-oracle")
BASELINE_Q = 3889 * 9721 * 17497
N = 648
COLUMNS = 1024

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "-j8"], check=True)


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        build()
    lib = ctypes.CDLL(LIB)
    c8 = ctypes.c_char_p
    u8p = ctypes.POINTER(ctypes.c_uint8)
    lib.lfo_blake3.argtypes = [c8, c8, c8, ctypes.c_size_t, ctypes.c_uint64, u8p, ctypes.c_size_t]
    lib.lfo_write_table.argtypes = [c8, ctypes.c_uint32, u8p]
    lib.lfo_b128_mul.argtypes = [c8, c8, u8p, ctypes.c_size_t]
    lib.lfo_f162_mul.argtypes = [c8, c8, u8p, ctypes.c_size_t]
    lib.lfo_ajtai_matrix.argtypes = [c8, ctypes.c_uint64, u8p]
    lib.lfo_a_times_v.argtypes = [c8, ctypes.c_uint64, ctypes.c_void_p, u8p]
    lib.lfo_proof_size.argtypes = [c8, ctypes.c_uint32]
    lib.lfo_proof_size.restype = ctypes.c_size_t
    lib.lfo_commit.argtypes = [c8, ctypes.c_uint32, c8, ctypes.c_int, u8p]
    lib.lfo_prove.argtypes = [c8, c8, ctypes.c_uint32, c8, ctypes.c_int, u8p, ctypes.c_size_t,
                              ctypes.POINTER(ctypes.c_size_t), u8p, ctypes.c_size_t]
    lib.lfo_prove_at_point.argtypes = [c8, c8, ctypes.c_uint32, c8, c8, u8p, ctypes.c_size_t,
                                       ctypes.POINTER(ctypes.c_size_t)]
    lib.lfo_verify.argtypes = [c8, ctypes.c_uint32, c8, c8, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t]
    lib.lfo_accept_modulus.argtypes = [c8, ctypes.c_uint32]
    lib.lfo_fold_cap.argtypes = [ctypes.c_uint32]
    lib.lfo_fold_cap.restype = ctypes.c_uint64
    lib.lfo_short_challenges.argtypes = [c8, c8, ctypes.c_size_t, ctypes.c_uint32, u8p]
    lib.lfo_norm_blocked.argtypes = [c8, ctypes.c_uint32, ctypes.c_uint32]
    lib.lfo_norm_blocked.restype = ctypes.c_double
    lib.lfo_norm_horner.argtypes = [c8, ctypes.c_uint32, ctypes.c_uint32]
    lib.lfo_norm_horner.restype = ctypes.c_double
    lib.lfo_set_threads.argtypes = [ctypes.c_int]
    lib.lfo_set_threads.restype = None
    _lib = lib
    return lib


def qb(q):
    return int(q).to_bytes(16, "little")


def _buf(n):
    return (ctypes.c_uint8 * max(n, 1))()


def blake3(data=b"", key=None, derive=None, n=32, seek=0):
    out = _buf(n)
    rc = load().lfo_blake3(key, derive.encode() if derive else None, bytes(data), len(data), seek, out, n)
    assert rc == 0
    return bytes(out[:n])


def write_table(seed, log_vars):
    n = (1 << log_vars) // 8
    out = _buf(n)
    assert load().lfo_write_table(bytes(seed), log_vars, out) == 0
    return bytes(out[:n])


def b128_mul(a, b):
    n = len(a) // 16
    out = _buf(16 * n)
    load().lfo_b128_mul(bytes(a), bytes(b), out, n)
    return bytes(out[: 16 * n])


def f162_mul(a, b):
    n = len(a) // 24
    out = _buf(24 * n)
    load().lfo_f162_mul(bytes(a), bytes(b), out, n)
    return bytes(out[: 24 * n])


def ajtai_matrix(q, elements):
    out = _buf(16 * N * elements)
    assert load().lfo_ajtai_matrix(qb(q), elements, out) == 0
    raw = bytes(out[: 16 * N * elements])
    return [int.from_bytes(raw[16 * i:16 * i + 16], "little") for i in range(N * elements)]


def a_times_v(q, elements, v):
    """rq::a_times_v (rq.rs:188-217) of ajtai_matrix(q, elements) and the signed vector v
    (elements * 648 values in i16), through the C oracle; 648 ints in [0, q)."""
    import array

    vv = array.array("h", v)
    assert len(vv) == elements * N
    out = _buf(16 * N)
    assert load().lfo_a_times_v(qb(q), elements, vv.buffer_info()[0], out) == 0
    raw = bytes(out[: 16 * N])
    return [int.from_bytes(raw[16 * i:16 * i + 16], "little") for i in range(N)]


def fold_into_ring(raw, q):
    """rq.rs:146-164: X^648 = X^324 - 1 from the top coefficient down, each reduced before it is
    folded, then every coefficient into [0, q)."""
    raw = list(raw)
    assert len(raw) == 2 * N - 1
    for k in range(2 * N - 2, N - 1, -1):
        value = raw[k] % q
        raw[k] = 0
        raw[k - N // 2] += value
        raw[k - N] -= value
    return [x % q for x in raw[:N]]


def ring_mul_schoolbook(a, b, q):
    """rq::mul (rq.rs:171-186): the schoolbook raw product, then fold_into_ring. Pure Python,
    for a handful of products."""
    raw = [0] * (2 * N - 1)
    for j, c in enumerate(b):
        if c:
            for i, x in enumerate(a):
                raw[i + j] += x * c
    return fold_into_ring(raw, q)


def ring_mul(a, b, q):
    """The same product with the raw coefficients from one big-integer multiplication (Kronecker
    substitution: slots wide enough that no coefficient carries into the next)."""
    slot = 8 * ((2 * (max(q, 2) - 1).bit_length() + 12) // 8 + 1)
    big_a = int.from_bytes(b"".join(int(x).to_bytes(slot // 8, "little") for x in a), "little")
    big_b = int.from_bytes(b"".join(int(x).to_bytes(slot // 8, "little") for x in b), "little")
    prod = (big_a * big_b).to_bytes(slot // 8 * (2 * N), "little")
    raw = [int.from_bytes(prod[i * slot // 8:(i + 1) * slot // 8], "little") for i in range(2 * N - 1)]
    return fold_into_ring(raw, q)


def proof_size(q, log_vars):
    return load().lfo_proof_size(qb(q), log_vars)


def commit(table, log_vars, q=BASELINE_Q, mode=1):
    w = (int(q - 1).bit_length() + 7) // 8
    out = _buf(w * COLUMNS * N)
    rc = load().lfo_commit(qb(q), log_vars, bytes(table), mode, out)
    if rc != 0:
        raise ValueError(f"commit failed {rc}")
    return bytes(out[: w * COLUMNS * N])


def trace_size(log_vars):
    lp = log_vars - 7
    return 112 + 16 * lp + 2048 + 16 + 168 + 24 * lp + 24 + 24 * COLUMNS + 40 * COLUMNS


def prove(seed, table, log_vars, q=BASELINE_Q, commit_mode=1, trace=False):
    cap = proof_size(q, log_vars)
    out = _buf(cap)
    n = ctypes.c_size_t()
    tcap = trace_size(log_vars) if trace else 0
    tb = _buf(tcap) if trace else None
    rc = load().lfo_prove(bytes(seed), qb(q), log_vars, bytes(table) if table is not None else None, commit_mode,
                          out, cap, ctypes.byref(n), tb, tcap)
    if rc != 0:
        raise ValueError(f"oracle prove failed {rc}")
    proof = bytes(out[: n.value])
    if trace:
        return proof, bytes(tb[:tcap])
    return proof


def prove_at_point(seed, table, log_vars, r_hi, q=BASELINE_Q):
    """The proof with the packed point coordinates r_hi (list of 16-byte elements or ints) in place of
    the sampled ones."""
    raw = b"".join(x if isinstance(x, (bytes, bytearray)) else int(x).to_bytes(16, "little") for x in r_hi)
    assert len(raw) == 16 * (log_vars - 7)
    cap = proof_size(q, log_vars)
    out = _buf(cap)
    n = ctypes.c_size_t()
    rc = load().lfo_prove_at_point(bytes(seed), qb(q), log_vars, bytes(table), raw, out, cap, ctypes.byref(n))
    if rc != 0:
        raise ValueError(f"oracle prove failed {rc}")
    return bytes(out[: n.value])


def verify(seed, proof, log_vars, table=None):
    """(accepted, message)."""
    err = ctypes.create_string_buffer(256)
    rc = load().lfo_verify(bytes(seed), log_vars, bytes(table) if table is not None else None, bytes(proof), len(proof),
                           err, 256)
    return rc == 0, err.value.decode()


def accept_modulus(q, log_vars=31):
    return load().lfo_accept_modulus(qb(q), log_vars) == 0


def fold_cap(log_vars=31):
    return load().lfo_fold_cap(log_vars)


def short_challenges(domain, prefix, n):
    out = _buf(40 * n)
    load().lfo_short_challenges(domain.encode(), bytes(prefix), len(prefix), n, out)
    raw = bytes(out[: 40 * n])
    res = []
    for i in range(n):
        c = raw[40 * i:40 * i + 40]
        w = int.from_bytes(c[36:40], "little")
        res.append((list(c[:w]), int.from_bytes(c[32:36], "little"), w))
    return res


def norms(positions, signs):
    pos = bytes(positions) + bytes(32 - len(positions))
    return load().lfo_norm_blocked(pos, signs, len(positions)), load().lfo_norm_horner(pos, signs, len(positions))


def set_threads(n):
    load().lfo_set_threads(n)


def parse_proof(proof, log_vars):
    """Split a proof into its bincode fields (main.rs:99-117)."""
    lp = log_vars - 7
    o = {}
    at = 0
    o["version"] = int.from_bytes(proof[0:4], "little")
    o["modulus"] = int.from_bytes(proof[4:20], "little")
    at = 20

    def vec():
        nonlocal at
        n = int.from_bytes(proof[at:at + 8], "little")
        at += 8
        v = proof[at:at + n]
        at += n
        return v

    o["commitment"] = vec()
    n = int.from_bytes(proof[at:at + 8], "little")
    at += 8
    o["partials"] = proof[at:at + 16 * n]
    at += 16 * n
    n = int.from_bytes(proof[at:at + 8], "little")
    at += 8
    o["rounds"] = proof[at:at + 48 * n]
    at += 48 * n
    o["opened"] = proof[at:at + 24]
    at += 24
    o["row"] = vec()
    o["folded"] = vec()
    o["trailing"] = len(proof) - at
    assert len(o["rounds"]) == 48 * lp
    return o
