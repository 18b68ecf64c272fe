"""The GPU checker (lf_verify) against the oracle's: the same accept / reject decision on valid
proofs, on proofs under other moduli and on proofs with one field tampered (the tampering cases of
the reference's own tests: verifier/proof_verify/src/main.rs:430-520)."""
import pytest

pytestmark = pytest.mark.gpu

SEED = bytes([42] * 32)


@pytest.mark.parametrize("log_vars", [19, 20, 22])
def test_valid_proofs_verify(prover, oracle, log_vars):
    table = oracle.write_table(SEED, log_vars)
    proof = prover.prove(SEED, table, log_vars)
    assert prover.verify(SEED, proof, log_vars, table) == (True, "")
    assert prover.verify(SEED, proof, log_vars) == (True, "")  # table regenerated from the seed


@pytest.mark.parametrize("q", [9721 * 2917 * 4861, (1 << 64) - 59, (1 << 96) - 17])
def test_other_moduli_verify(prover, oracle, q):
    table = oracle.write_table(SEED, 19)
    proof = prover.prove(SEED, table, 19, q=q)
    assert prover.verify(SEED, proof, 19, table) == (True, "")


def _fields(oracle, proof, log_vars):
    """Byte offsets of each field of the bincode layout (main.rs:98-124)."""
    w = (int.from_bytes(proof[4:20], "little") - 1).bit_length()
    w = (w + 7) // 8
    lp = log_vars - 7
    at_commit = 28
    commit_len = w * 1024 * 648
    at_partials = at_commit + commit_len + 8
    at_rounds = at_partials + 128 * 16 + 8
    at_opened = at_rounds + 48 * lp
    at_row = at_opened + 24 + 8
    row_len = (1024 * 162 + 7) // 8
    at_fold = at_row + row_len + 8
    return {"commitment": at_commit + 5, "partials": at_partials + 3, "rounds": at_rounds + 7,
            "opened": at_opened + 2, "row": at_row + 11, "folded": at_fold + 4 * 77}


@pytest.mark.parametrize("field", ["commitment", "partials", "rounds", "opened", "row", "folded"])
def test_tampered_field_rejected_like_the_oracle(prover, oracle, field):
    log_vars = 19
    table = oracle.write_table(SEED, log_vars)
    proof = bytearray(prover.prove(SEED, table, log_vars))
    at = _fields(oracle, proof, log_vars)[field]
    proof[at] ^= 0x01
    ok, msg = prover.verify(SEED, bytes(proof), log_vars, table)
    ok_o, msg_o = oracle.verify(SEED, bytes(proof), log_vars, table)
    assert not ok and not ok_o
    assert msg == msg_o, (msg, msg_o)


def test_wrong_seed_and_truncation_rejected(prover, oracle):
    table = oracle.write_table(SEED, 19)
    proof = prover.prove(SEED, table, 19)
    assert not prover.verify(bytes([43] * 32), proof, 19, table)[0]
    assert prover.verify(SEED, proof[:-1], 19, table) == (False, "truncated proof")
    assert prover.verify(SEED, proof + b"\0", 19, table) == (False, "trailing bytes")


def test_full_size_prove_and_verify_on_device(prover, gpu_lib):
    """The 2^31-bit instance: device table, device proof, GPU checker; a flipped fold byte is
    rejected."""
    import ctypes

    log_vars = 31
    seed = bytes(range(32))
    dev = prover.alloc((1 << log_vars) // 8)
    try:
        prover.write_table_device(seed, log_vars, dev)
        out, n = prover.prove_device(seed, dev, log_vars)
        proof = ctypes.string_at(out, n)
        assert n == 13_958_612
        assert prover.verify_device(seed, proof, log_vars, dev) == (True, "")
        bad = bytearray(proof)
        bad[-40] ^= 0x02
        assert not prover.verify_device(seed, bytes(bad), log_vars, dev)[0]
    finally:
        prover.free(dev)
