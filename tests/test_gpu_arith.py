"""The arithmetic under the commitment, batched on the device, against the oracle: ring products
in R_Q (rq.rs:146-186) for the moduli of the kernel microbenchmark (the baseline prime product,
2^64, a three-prime product near 2^93) and others, the public matrix (rq.rs:114-148), the key
product a_times_v (rq.rs:188-217) and GHASH products (fields/scalar.rs:61-72)."""
import random

import pytest

pytestmark = pytest.mark.gpu

N = 648
BASELINE_Q = 3889 * 9721 * 17497
Q93 = 2147478481 * 2147449321 * 2147429881  # three primes = 1 (mod 1944) below 2^31
RING_Q = [BASELINE_Q, 1 << 64, Q93, 55_144_219_393, (1 << 96) - 17, 1 << 36, 3889, 2917, 19441, 2, 1944 * 5 + 1]


def _torch():
    return pytest.importorskip("torch")


def _dev(torch, data):
    t = torch.frombuffer(bytearray(data), dtype=torch.uint8).cuda()
    torch.cuda.synchronize()
    return t


def _pack(vals):
    return b"".join(int(v).to_bytes(16, "little") for v in vals)


def _unpack(raw):
    return [int.from_bytes(raw[16 * i:16 * i + 16], "little") for i in range(len(raw) // 16)]


def _ring_case(prover, torch, q, a, b):
    n = len(a) // N
    da, db = _dev(torch, _pack(a)), _dev(torch, _pack(b))
    dc = torch.zeros(16 * N * n, dtype=torch.uint8, device="cuda")
    prover.ring_mul(q, n, da.data_ptr(), db.data_ptr(), dc.data_ptr())
    return _unpack(dc.cpu().numpy().tobytes())


@pytest.mark.parametrize("q", RING_Q, ids=[str(q) if q < 1 << 20 else hex(q) for q in RING_Q])
def test_ring_products_match_oracle(prover, oracle, q):
    torch = _torch()
    r = random.Random(q % 100003)
    n = 12
    a = [r.randrange(q) for _ in range(N * n)]
    b = [r.randrange(q) for _ in range(N * n)]
    # edge elements: all zero, all q - 1, the monomials 1 and X^647
    a[:N] = [0] * N
    b[N:2 * N] = [q - 1] * N
    a[2 * N:3 * N] = [q - 1] * N
    b[2 * N:3 * N] = [q - 1] * N
    a[3 * N:4 * N] = [1] + [0] * (N - 1)
    b[4 * N:5 * N] = [0] * (N - 1) + [1]
    a[4 * N:5 * N] = [0] * (N - 1) + [1 % q]
    got = _ring_case(prover, torch, q, a, b)
    for i in range(n):
        want = oracle.ring_mul(a[i * N:(i + 1) * N], b[i * N:(i + 1) * N], q)
        assert got[i * N:(i + 1) * N] == want, f"product {i} differs"


def test_ring_products_on_reference_test_inputs(prover, oracle):
    # rq.rs:346-386: values(label) = u128 LE words of BLAKE3(label)'s output, reduced mod q; the
    # signed case centres b in [-300, 300] (taken mod q here: the product is the same).
    torch = _torch()

    def values(label, n):
        raw = oracle.blake3(label, n=16 * n)
        return _unpack(raw)

    for q in (3889, 2917, 19441):
        a = [x % q for x in values(b"rq/a", N)]
        b = [x % q for x in values(b"rq/b", N)]
        assert _ring_case(prover, torch, q, a, b) == oracle.ring_mul_schoolbook(a, b, q)
    q = 3889
    a = [x % q for x in values(b"rq/a2", N)]
    b = [((x % 601) - 300) % q for x in values(b"rq/b2", N)]
    assert _ring_case(prover, torch, q, a, b) == oracle.ring_mul_schoolbook(a, b, q)


def test_ring_operand_out_of_range_is_refused(prover, gpu_lib):
    torch = _torch()
    q = BASELINE_Q
    a = [1] * N
    b = [2] * (N - 1) + [q]
    with pytest.raises(gpu_lib.LfError) as e:
        _ring_case(prover, torch, q, a, b)
    assert e.value.code == gpu_lib.LF_E_ARGS
    with pytest.raises(gpu_lib.LfError) as e:
        _ring_case(prover, torch, 1 << 96, a, a)
    assert e.value.code == gpu_lib.LF_E_MODULUS


@pytest.mark.parametrize("q", [BASELINE_Q, 1 << 64, Q93, 1 << 100])
def test_matrix_on_device_matches_oracle(prover, oracle, q):
    torch = _torch()
    elements = 24
    out = torch.zeros(16 * N * elements, dtype=torch.uint8, device="cuda")
    prover.ajtai_matrix_device(q, elements, out.data_ptr())
    assert _unpack(out.cpu().numpy().tobytes()) == oracle.ajtai_matrix(q, elements)


@pytest.mark.parametrize("q", [BASELINE_Q, 1 << 64, Q93])
def test_matrix_products_at_scale(prover, oracle, q):
    # operands from the device's public-matrix expansion (uniform in [0, q) by rejection), 2^12
    # products; a sample of them against the oracle, and c(a, b) == c(b, a) for all.
    torch = _torch()
    n = 1 << 12
    m = torch.zeros(16 * N * 2 * n, dtype=torch.uint8, device="cuda")
    prover.ajtai_matrix_device(q, 2 * n, m.data_ptr())
    half = 16 * N * n
    c1 = torch.zeros(half, dtype=torch.uint8, device="cuda")
    c2 = torch.zeros(half, dtype=torch.uint8, device="cuda")
    prover.ring_mul(q, n, m.data_ptr(), m.data_ptr() + half, c1.data_ptr())
    prover.ring_mul(q, n, m.data_ptr() + half, m.data_ptr(), c2.data_ptr())
    assert torch.equal(c1, c2)
    host = m.cpu().numpy().tobytes()
    got = c1.cpu().numpy().tobytes()
    for i in (0, 1, n // 2, n - 1):
        a = _unpack(host[16 * N * i:16 * N * (i + 1)])
        b = _unpack(host[half + 16 * N * i:half + 16 * N * (i + 1)])
        assert _unpack(got[16 * N * i:16 * N * (i + 1)]) == oracle.ring_mul(a, b, q)


@pytest.mark.parametrize("q,elements", [(BASELINE_Q, 64), (1 << 64, 16), (Q93, 16), (55_144_219_393, 8),
                                        (BASELINE_Q, 4096)])
def test_a_times_v_matches_oracle(prover, oracle, q, elements):
    torch = _torch()
    r = random.Random(elements)
    lo, hi = (-(1 << 10), 1 << 10) if elements == 4096 else (-(1 << 15), (1 << 15) - 1)
    v = [r.randint(lo, hi) for _ in range(elements * N)]
    v[:N] = [0] * N
    v[N] = -(1 << 15) if elements < 4096 else -(1 << 10)
    vd = torch.tensor(v, dtype=torch.int16, device="cuda")
    torch.cuda.synchronize()
    assert prover.a_times_v(q, elements, vd.data_ptr()) == oracle.a_times_v(q, elements, v)


def test_ghash_products_match_oracle(prover, oracle):
    torch = _torch()
    r = random.Random(7)
    n = 1 << 16
    a = bytes(r.getrandbits(8) for _ in range(16 * n))
    b = bytes(r.getrandbits(8) for _ in range(16 * n))
    # edges: zero, one, x^127 times x^127, all ones
    a = bytes(16) + (1).to_bytes(16, "little") + (1 << 127).to_bytes(16, "little") + b"\xff" * 16 + a[64:]
    b = b"\xff" * 16 + b"\x07" * 16 + (1 << 127).to_bytes(16, "little") + b"\xff" * 16 + b[64:]
    da, db = _dev(torch, a), _dev(torch, b)
    dc = torch.zeros(16 * n, dtype=torch.uint8, device="cuda")
    prover.ghash_mul(n, da.data_ptr(), db.data_ptr(), dc.data_ptr())
    assert dc.cpu().numpy().tobytes() == oracle.b128_mul(a, b)


def test_ghash_products_distribute_at_scale(prover):
    # a (b + c) == a b + a c over 2^24 random triples (XOR is the addition)
    torch = _torch()
    g = torch.Generator(device="cuda").manual_seed(11)
    n = 1 << 24
    a, b, c = (torch.randint(-2 ** 63, 2 ** 63 - 1, (2 * n,), dtype=torch.int64, device="cuda", generator=g)
               for _ in range(3))
    bc = b ^ c
    out = [torch.empty_like(a) for _ in range(3)]
    torch.cuda.synchronize()
    prover.ghash_mul(n, a.data_ptr(), bc.data_ptr(), out[0].data_ptr())
    prover.ghash_mul(n, a.data_ptr(), b.data_ptr(), out[1].data_ptr())
    prover.ghash_mul(n, a.data_ptr(), c.data_ptr(), out[2].data_ptr())
    assert torch.equal(out[0], out[1] ^ out[2])
