"""GPU prover vs the CPU oracle: byte-identical proofs on the same (seed, table, Q), and the
oracle's checker accepting the GPU proof (verifier/proof_verify/src/main.rs:402-409).

Every shape is compared byte for byte, the full 2^31-bit instance included (the oracle proves it
on all host cores in about half a minute), through the library and through the drop-in
`labinius-fast` executable. Edge tables, the reference's moduli and degenerate points are in
test_gpu_edges.py."""
import hashlib
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

SEEDS = [bytes([42] * 32), bytes([44] * 32), hashlib.sha256(b"lf-test/seed/0").digest()]


def _first_diff(a, b, log_vars, oracle):
    pa, pb = oracle.parse_proof(a, log_vars), oracle.parse_proof(b, log_vars)
    return [k for k in pa if pa[k] != pb[k]]


@pytest.mark.parametrize("log_vars", [19, 20, 22])
@pytest.mark.parametrize("seed", SEEDS[:2])
def test_proof_matches_oracle(prover, oracle, log_vars, seed):
    table = oracle.write_table(seed, log_vars)
    got = prover.prove(seed, table, log_vars)
    want = oracle.prove(seed, table, log_vars)
    assert len(got) == len(want)
    assert got == want, f"fields differ: {_first_diff(got, want, log_vars, oracle)}"
    ok, msg = oracle.verify(seed, got, log_vars, table)
    assert ok, msg


# Moduli other than 3889*9721*17497 commit through an exact integer lift over more transform
# primes (main.rs:2255-2266 proves under 9721*2917*4861; the gate admits any 35..96-bit Q).
OTHER_Q = [9721 * 2917 * 4861, 1 << 40, (1 << 64) - 59, (1 << 96) - 17]


@pytest.mark.parametrize("q", OTHER_Q, ids=["3primes", "2^40", "2^64-59", "2^96-17"])
@pytest.mark.parametrize("log_vars", [19, 20])
def test_other_moduli_match_oracle(prover, oracle, log_vars, q):
    seed = SEEDS[2]
    table = oracle.write_table(seed, log_vars)
    got = prover.prove(seed, table, log_vars, q=q)
    want = oracle.prove(seed, table, log_vars, q=q)
    assert got == want, f"fields differ: {_first_diff(got, want, log_vars, oracle)}"
    ok, msg = oracle.verify(seed, got, log_vars, table)
    assert ok, msg


def test_wrong_seed_rejected(prover, oracle):
    # solution/proof_generate/src/main.rs:2244-2253: a proof for seed 42 fails under seed 43.
    log_vars = 20
    seed = bytes([42] * 32)
    table = oracle.write_table(seed, log_vars)
    proof = prover.prove(seed, table, log_vars)
    ok, _ = oracle.verify(bytes([43] * 32), proof, log_vars)
    assert not ok


def test_device_table_writer_matches_oracle(prover, oracle):
    log_vars = 22
    seed = SEEDS[2]
    n = (1 << log_vars) // 8
    dev = prover.alloc(n)
    try:
        prover.write_table_device(seed, log_vars, dev)
        proof_dev, n_dev = prover.prove_device(seed, dev, log_vars)
        table = oracle.write_table(seed, log_vars)
        assert bytes(proof_dev[:n_dev]) == oracle.prove(seed, table, log_vars)
    finally:
        prover.free(dev)


@pytest.mark.parametrize("log_vars", [23, 27, 31])
def test_page_locked_table_streams_into_the_commitment(prover, oracle, log_vars):
    # lf_prove from page-locked host memory copies the table in up to 64 element ranges, in the
    # order the commitment's blocks reach them, while the commitment already runs, each block
    # waiting for its range (tables of at least 16 ring elements per column: 2^23 bits and up):
    # the proof is the one of the same table proven from device memory (and, at 2^23 bits, the
    # oracle's).
    torch = pytest.importorskip("torch")
    seed = SEEDS[0]
    n = (1 << log_vars) // 8
    dev = torch.empty(n, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    prover.write_table_device(seed, log_vars, dev.data_ptr())
    proof_dev, n_dev = prover.prove_device(seed, dev.data_ptr(), log_vars)
    torch.cuda.synchronize()
    host = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    host.copy_(dev)
    torch.cuda.synchronize()
    for _ in range(2):  # the second run finds the ready flags set by the first, under a new epoch
        got = prover.prove(seed, host.numpy(), log_vars)
        assert got == bytes(proof_dev[:n_dev])
    if log_vars == 23:
        assert got == oracle.prove(seed, oracle.write_table(seed, log_vars), log_vars)


@pytest.mark.parametrize("q", [(1 << 64) - 59, (1 << 96) - 17], ids=["2^64-59", "2^96-17"])
def test_page_locked_table_streams_under_other_moduli(prover, oracle, q):
    # the exact-lift commitment (more transform primes, hence more blocks per element range)
    # reading a table that is still arriving
    torch = pytest.importorskip("torch")
    log_vars, seed = 23, SEEDS[2]
    table = oracle.write_table(seed, log_vars)
    host = torch.empty(len(table), dtype=torch.uint8, pin_memory=True)
    host.numpy()[:] = bytearray(table)
    assert prover.prove(seed, host.numpy(), log_vars, q=q) == oracle.prove(seed, table, log_vars, q=q)


def test_repeatable(prover, oracle):
    log_vars = 20
    seed = SEEDS[1]
    table = oracle.write_table(seed, log_vars)
    assert prover.prove(seed, table, log_vars) == prover.prove(seed, table, log_vars)


@pytest.mark.parametrize("log_vars", [27, 29])
def test_repeatable_over_several_waves(prover, log_vars):
    # Grids of several waves of blocks per SM (2^28 bits and up for the partial sums) start their
    # blocks at staggered times, the schedule under which a missing ordering between a ring slot's
    # read and its refill once changed the partial sums from one proof to the next: six proofs of
    # one device table, byte-identical.
    seed = SEEDS[0]
    dev = prover.alloc((1 << log_vars) // 8)
    try:
        prover.write_table_device(seed, log_vars, dev)
        proofs = set()
        for _ in range(6):
            proof, plen = prover.prove_device(seed, dev, log_vars)
            proofs.add(bytes(proof[:plen]))
    finally:
        prover.free(dev)
    assert len(proofs) == 1


@pytest.mark.parametrize("prefix", [b"", b"lfchk", bytes(range(256)) * 13], ids=["empty", "short", "3328B"])
def test_device_challenges_match_oracle(prover, oracle, prefix):
    want = oracle.short_challenges("labinius/test/batch", prefix, 64)
    got = prover.sample_challenges("labinius/test/batch", prefix, 64)
    assert got == want


@pytest.mark.parametrize("prefix", [b"many", bytes(range(200))], ids=["4-byte", "200B"])
def test_many_device_challenges_match_oracle(prover, oracle, prefix):
    # 4096 challenges: about half a million norm evaluations, a few of them inside the band
    # around the bound where the sampler repeats the f64 arithmetic.
    want = oracle.short_challenges("labinius/test/many", prefix, 4096)
    got = prover.sample_challenges("labinius/test/many", prefix, 4096)
    assert got == want


def test_tuned_split_count_keeps_the_proof(gpu_lib, oracle):
    # lf_tune changes only the commitment's grid depth and the fold's column-run count; the proof
    # must stay the oracle's
    seed = SEEDS[0]
    log_vars = 21
    table = oracle.write_table(seed, log_vars)
    with gpu_lib.Prover(0, lanes=2) as p:
        dev = p.alloc(len(table))
        try:
            p.h2d(dev, table)
            splits, ms, tried = p.tune(log_vars, dev)
            assert splits >= 1 and ms > 0 and tried >= 1
            assert p.last_tune["fold_splits"] >= 1 and p.last_tune["fold_ms"] > 0
            assert p.last_tune["fold_candidates"] >= 1
            got = p.prove(seed, table, log_vars)
        finally:
            p.free(dev)
    assert got == oracle.prove(seed, table, log_vars)


def test_full_instance_matches_oracle(prover, oracle):
    # The challenge's own instance: 2^31 bits, baseline Q. The table is written on the device by
    # the table PRG, proven from device memory, and the oracle proves the same bytes on the host.
    log_vars, seed = 31, SEEDS[2]
    n = (1 << log_vars) // 8
    dev = prover.alloc(n)
    try:
        prover.write_table_device(seed, log_vars, dev)
        proof, plen = prover.prove_device(seed, dev, log_vars)
        got = bytes(proof[:plen])
    finally:
        prover.free(dev)
    assert plen == 13_958_612
    table = oracle.write_table(seed, log_vars)
    want = oracle.prove(seed, table, log_vars)
    assert got == want, f"fields differ: {_first_diff(got, want, log_vars, oracle)}"
    ok, msg = oracle.verify(seed, got, log_vars, table)
    assert ok, msg


@pytest.mark.parametrize("modulus", [None, 35_039_150_080, 55_144_219_393, (1 << 96) - 17],
                         ids=["default", "x86-default", "recorded-run", "2^96-17"])
@pytest.mark.parametrize("log_vars", [20, 22])
def test_cli_proof_file_matches_oracle(gpu_lib, oracle, tmp_path, log_vars, modulus):
    # The drop-in boundary (solution/proof_generate/src/main.rs:2050-2090): the table file, the
    # seed in LABINIUS_SEED, the proof file; without --modulus the proof is made (and carries) the
    # baseline Q 3889 * 9721 * 17497.
    seed = hashlib.sha256(b"lf-test/cli").digest()
    table = oracle.write_table(seed, log_vars)
    tpath, ppath = tmp_path / "witness-table.bin", tmp_path / "proof.bin"
    tpath.write_bytes(table)
    args = [gpu_lib.CLI_PATH, "--prove", str(ppath), "--table", str(tpath), "--log-vars", str(log_vars)]
    if modulus is not None:
        args += ["--modulus", str(modulus)]
    env = dict(os.environ, LABINIUS_SEED=seed.hex())
    r = subprocess.run(args, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "labinius-gb300" in r.stderr  # the phase line
    got = ppath.read_bytes()
    q = modulus if modulus is not None else 3889 * 9721 * 17497
    assert got == oracle.prove(seed, table, log_vars, q=q)
    assert oracle.verify(seed, got, log_vars, table)[0]


def test_cli_rejects_bad_inputs(gpu_lib, oracle, tmp_path):
    # any failure exits nonzero and leaves no proof file (main.rs:2056-2069, 391-392)
    seed = bytes(range(32))
    tpath, ppath = tmp_path / "t.bin", tmp_path / "p.bin"
    tpath.write_bytes(oracle.write_table(seed, 20)[:-16])
    env = dict(os.environ, LABINIUS_SEED=seed.hex())
    base = [gpu_lib.CLI_PATH, "--prove", str(ppath), "--table", str(tpath), "--log-vars", "20"]
    r = subprocess.run(base, env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode != 0 and "wrong length" in r.stderr
    tpath.write_bytes(oracle.write_table(seed, 20))
    r = subprocess.run(base + ["--modulus", "34816965048"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode != 0 and "modulus" in r.stderr
    r = subprocess.run(base, env=dict(os.environ, LABINIUS_SEED="zz" * 32), capture_output=True, text=True, timeout=120)
    assert r.returncode != 0
    assert not ppath.exists()
