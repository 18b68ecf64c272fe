"""The CPU oracle against the properties the reference's own tests pin (there are no golden
vectors in the reference; see tests/golden/README.md for what is and is not pinned)."""
import hashlib

import pytest

Q = 3889 * 9721 * 17497
MIN_MODULUS = 34_816_965_049


def test_fold_cap_matches_the_library(oracle):
    # verifier/proof_verify/src/main.rs:467-480
    assert oracle.fold_cap(31) == 293_534_171_136
    import math

    assert math.isqrt(oracle.fold_cap(31)) == 541_787


def test_the_gate_is_two_size_conditions(oracle):
    # verifier/proof_verify/src/main.rs:485-492
    assert oracle.accept_modulus(1 << 36)
    assert oracle.accept_modulus(MIN_MODULUS)
    assert not oracle.accept_modulus(MIN_MODULUS - 1)
    assert oracle.accept_modulus(55_144_219_393)
    assert not oracle.accept_modulus(1 << 96)
    assert 2 * 541_787 < MIN_MODULUS


def test_table_is_the_keyed_xof(oracle):
    # verifier/proof_verify/src/main.rs:135-141 and :494-521
    seed = bytes([9] * 32)
    t = oracle.write_table(seed, 19)
    assert t[:4096] == oracle.blake3(b"labinius-fast/binary-table/v1", key=seed, n=4096)
    assert t[-64:] == oracle.blake3(b"labinius-fast/binary-table/v1", key=seed, n=64, seek=len(t) - 64)
    assert t[:32] != oracle.write_table(bytes([8] * 32), 19)[:32]


def test_blake3_tree_and_modes_are_consistent(oracle):
    data = hashlib.sha512(b"x").digest() * 200  # 12800 bytes, 13 chunks
    full = oracle.blake3(data, n=256)
    assert oracle.blake3(data, n=64, seek=192) == full[192:]
    assert oracle.blake3(data, n=32) == full[:32]
    assert oracle.blake3(data, key=bytes(32), n=32) != full[:32]
    assert oracle.blake3(data, derive="ctx", n=32) != full[:32]
    assert len({oracle.blake3(data[:n]) for n in (0, 1, 64, 1024, 1025, 2048, 12800)}) == 7


def test_power_of_two_matrix_is_the_raw_stream(oracle):
    # verifier/proof_verify/src/rq.rs:467-479
    q = 1 << 36
    m = oracle.ajtai_matrix(q, 3)
    for i in range(3):
        msg = b"labinius-fast/ajtai-matrix/v1" + q.to_bytes(16, "little") + (3).to_bytes(8, "little") + i.to_bytes(
            8, "little")
        stream = oracle.blake3(msg, key=bytes([0x5A] * 32), n=5 * 648)
        want = [int.from_bytes(stream[5 * t:5 * t + 5], "little") & (q - 1) for t in range(648)]
        assert m[648 * i:648 * (i + 1)] == want
    assert all(x < q for x in m)


def test_the_matrix_is_element_by_element(oracle):
    # verifier/proof_verify/src/rq.rs:482-489
    q = 55_144_219_393
    wide = oracle.ajtai_matrix(q, 64)
    assert oracle.ajtai_matrix(q, 64)[:648] == wide[:648]
    assert oracle.ajtai_matrix(q, 65)[:648] != wide[:648]
    assert oracle.ajtai_matrix(q + 2, 64)[:648] != wide[:648]
    assert all(x < q for x in wide)


@pytest.mark.parametrize("log_vars", [19, 20])
def test_transform_commitment_is_the_schoolbook_product(oracle, log_vars):
    # solution-arm/proof_generate/src/main.rs:1241-1290 (NTT commit == schoolbook)
    table = oracle.write_table(bytes([3] * 32), log_vars)
    assert oracle.commit(table, log_vars, Q, mode=1) == oracle.commit(table, log_vars, Q, mode=0)


def test_commitment_edge_columns(oracle):
    # solution-arm/proof_generate/src/main.rs:1211-1237: zeros, all ones, single bits.
    log_vars = 19
    n = (1 << log_vars) // 8
    for table in (bytes(n), b"\xff" * n, (b"\x01" + bytes(15)) * (n // 16), (bytes(15) + b"\x80") * (n // 16)):
        assert oracle.commit(table, log_vars, Q, 1) == oracle.commit(table, log_vars, Q, 0)
    assert set(oracle.commit(bytes(n), log_vars, Q, 1)) == {0}


def test_challenges_are_short_and_well_formed(oracle):
    cs = oracle.short_challenges("labinius/test/batch", b"lf", 64)
    for pos, signs, w in cs:
        assert w == 28
        assert pos == sorted(pos) and len(set(pos)) == 28 and max(pos) < 162
        assert signs < (1 << 28)
        blocked, horner = oracle.norms(pos, signs)
        assert blocked <= 144.0 + 1e-12
        assert abs(blocked - horner) < 1e-9 * max(1.0, horner)
    assert len({tuple(c[0]) for c in cs}) == 64


def test_norm_blocked_is_horner(oracle):
    # solution/labinius/crates/pcs/tests/challenge.rs:128-143
    import random

    r = random.Random(7)
    for _ in range(50):
        pos = sorted(r.sample(range(162), 28))
        signs = r.getrandbits(28)
        b, h = oracle.norms(pos, signs)
        assert abs(b - h) < 1e-9 * max(1.0, h)


@pytest.mark.parametrize("log_vars", [19, 20])
def test_round_trip_and_reject_wrong_instance(oracle, log_vars):
    # solution/proof_generate/src/main.rs:2244-2253
    seed = bytes([42] * 32)
    table = oracle.write_table(seed, log_vars)
    proof = oracle.prove(seed, table, log_vars)
    assert len(proof) == oracle.proof_size(Q, log_vars)
    ok, msg = oracle.verify(seed, proof, log_vars)
    assert ok, msg
    ok, _ = oracle.verify(bytes([43] * 32), proof, log_vars)
    assert not ok


def test_tampered_fields_are_rejected(oracle):
    log_vars = 19
    seed = bytes([5] * 32)
    table = oracle.write_table(seed, log_vars)
    proof = bytearray(oracle.prove(seed, table, log_vars))
    parts = oracle.parse_proof(bytes(proof), log_vars)
    offsets = {
        "commitment": 28 + 3,
        "partials": 28 + len(parts["commitment"]) + 8 + 5,
        "rounds": 28 + len(parts["commitment"]) + 8 + 2048 + 8 + 1,
        "opened": 28 + len(parts["commitment"]) + 8 + 2048 + 8 + len(parts["rounds"]) + 2,
        "row": len(proof) - len(parts["folded"]) - 8 - len(parts["row"]) + 7,
        "folded": len(proof) - len(parts["folded"]) + 4,
    }
    for name, at in offsets.items():
        bad = bytearray(proof)
        bad[at] ^= 0x01
        ok, msg = oracle.verify(seed, bytes(bad), log_vars, table)
        assert not ok, f"tampered {name} accepted"
    ok, _ = oracle.verify(seed, bytes(proof) + b"\x00", log_vars, table)
    assert not ok
    ok, _ = oracle.verify(seed, bytes(proof[:-1]), log_vars, table)
    assert not ok


def test_other_moduli(oracle):
    # solution/proof_generate/src/main.rs:2255-2266 (Q = 9721*2917*4861) and a power of two.
    log_vars = 19
    seed = bytes([7] * 32)
    table = oracle.write_table(seed, log_vars)
    for q in (9721 * 2917 * 4861, 1 << 40):
        proof = oracle.prove(seed, table, log_vars, q=q)
        assert oracle.parse_proof(proof, log_vars)["modulus"] == q
        ok, msg = oracle.verify(seed, proof, log_vars, table)
        assert ok, msg


def test_full_size_layout(oracle):
    assert oracle.proof_size(Q, 31) == 13_958_612


def test_prove_at_the_sampled_point_is_the_proof(oracle):
    # lfo_prove_at_point only replaces the sampled r_hi: at the sampled coordinates (read from the
    # prover's trace, after the 7 r_lo elements) it is the proof itself, and any other point
    # changes the switch and every field after it, not the commitment or the partials' point.
    log_vars = 20
    seed = bytes([9] * 32)
    table = oracle.write_table(seed, log_vars)
    proof, trace = oracle.prove(seed, table, log_vars, trace=True)
    lp = log_vars - 7
    hi = [trace[112 + 16 * i:112 + 16 * (i + 1)] for i in range(lp)]
    assert oracle.prove_at_point(seed, table, log_vars, hi) == proof
    other = oracle.prove_at_point(seed, table, log_vars, [1] * lp)
    a, b = oracle.parse_proof(proof, log_vars), oracle.parse_proof(other, log_vars)
    assert a["commitment"] == b["commitment"]
    assert a["rounds"] != b["rounds"] and a["folded"] != b["folded"]
