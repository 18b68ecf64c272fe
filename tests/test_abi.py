"""The C ABI without a GPU: the library builds for sm_103a, loads, exports every entry point the
header declares, and its host-only entry points agree with the oracle."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "labinius_gpu.h")


def declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(lf_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(gpu_lib):
    lib = gpu_lib.load()
    names = declared()
    assert len(names) >= 14
    for n in names:
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", gpu_lib.LIB_PATH], capture_output=True, text=True).stdout
    for n in names:
        assert re.search(rf"\bT {n}\b", out), n


def test_proof_size_and_gate_match_oracle(gpu_lib, oracle):
    for log_vars in (19, 20, 22, 31):
        for q in (3889 * 9721 * 17497, 1 << 36, 55_144_219_393, (1 << 96) - 1):
            assert gpu_lib.proof_size(q, log_vars) == oracle.proof_size(q, log_vars)
            assert gpu_lib.accept_modulus(q, log_vars) == oracle.accept_modulus(q, log_vars)
    assert gpu_lib.proof_size(3889 * 9721 * 17497, 31) == 13_958_612
    assert not gpu_lib.accept_modulus(34_816_965_048, 31)


def test_cli_built_and_usage(gpu_lib):
    assert os.path.exists(gpu_lib.CLI_PATH)
    p = subprocess.run([gpu_lib.CLI_PATH], capture_output=True, text=True)
    assert p.returncode != 0 and "usage" in p.stderr


def test_no_device_fails_loudly(gpu_lib):
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a device is present")
    except ImportError:
        pass
    with pytest.raises(gpu_lib.LfError):
        gpu_lib.Prover(0)


def test_noalloc_sampler_limits_checked_on_the_host(gpu_lib):
    """Argument and size checks return before any device work, so they hold without a GPU."""
    lib = gpu_lib.load()
    import ctypes

    buf = (ctypes.c_uint8 * 40)()
    n_max = gpu_lib.NOALLOC_MAX_CHALLENGES
    assert lib.lf_sample_challenges_noalloc(0, b"d", b"", 0, n_max + 1, buf, None) == -10
    assert lib.lf_sample_challenges_noalloc(0, b"d", b"", 0, 0, buf, None) == -1
    assert lib.lf_sample_challenges_noalloc(-1, b"d", b"", 0, 1, buf, None) == -1
    assert lib.lf_sample_challenges_noalloc(64, b"d", b"", 0, 1, buf, None) == -1
    assert lib.lf_sample_challenges_noalloc(0, None, b"", 0, 1, buf, None) == -1
    assert b"4096" in lib.lf_strerror(-10)


def test_test_hooks_check_their_arguments(gpu_lib):
    lib = gpu_lib.load()
    assert lib.lf_test_set_point(None, b"", 0) == -1
    assert lib.lf_test_withhold_table_part(None, 0, 0) == -1
    assert lib.lf_test_table_part_order(0, 1, 1, 1, None, None) == -1


def test_streamed_table_parts_go_up_in_the_order_the_commitment_reads_them(gpu_lib):
    # 2^31 bits: 4096 ring elements per column in 64 parts of 64; the commitment's grid runs 21
    # element splits of 196 elements, 72 blocks each (3 primes x 3 leaf thirds x 8 column groups),
    # 152 at a time. Splits 0, 1 and 2 start in the first wave at elements 0, 196 and 392 (parts 0,
    # 3 and 6); then each part by when a split's blocks reach it (448, 256, 64: parts 7, 4, 1).
    order = gpu_lib.table_part_order(4096, 21, 72, 152)
    assert sorted(order) == list(range(64))
    assert order[:3] == [0, 3, 6]
    assert order[3:6] == [7, 4, 1]
    # parts of at least 16 elements: a 2^24-bit table (64 elements) goes up in 4 parts, 2^23 in 2,
    # a table of fewer than 32 elements in one
    assert sorted(gpu_lib.table_part_order(64, 4, 72, 152)) == [0, 1, 2, 3]
    assert gpu_lib.table_part_order(32, 1, 72, 152) == [0, 1]
    assert gpu_lib.table_part_order(20, 1, 72, 152) == [0]
    # one split, one wave: the parts in index order
    assert gpu_lib.table_part_order(1024, 1, 72, 152) == list(range(64))
