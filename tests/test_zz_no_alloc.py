"""lf_sample_challenges_noalloc: the sampler with its scratch in a fixed device array, no context
and no device allocation. Collected last, so it runs both alone and after every other test has
used the device; it must agree with lf_sample_challenges, the context-based entry point."""
import pytest

pytestmark = pytest.mark.gpu

DOMAIN = "labinius/test/batch"


def test_two_consecutive_calls_match_context_sampler(gpu_lib, prover):
    cases = [(b"lfchk", 64), (bytes(range(256)) * 13, 1024)]
    got = [gpu_lib.sample_challenges_noalloc(DOMAIN, prefix, n) for prefix, n in cases]
    want = [prover.sample_challenges(DOMAIN, prefix, n) for prefix, n in cases]
    assert got[0] == want[0]
    assert got[1] == want[1]
    assert got[0] != got[1][:64]


def test_matches_oracle_and_fills_the_whole_scratch(gpu_lib, prover, oracle):
    n = gpu_lib.NOALLOC_MAX_CHALLENGES
    got = gpu_lib.sample_challenges_noalloc(DOMAIN, b"", n)
    assert got == prover.sample_challenges(DOMAIN, b"", n)
    assert got[:64] == oracle.short_challenges(DOMAIN, b"", 64)
    # a smaller request right after a full one sees none of the earlier challenges
    assert gpu_lib.sample_challenges_noalloc(DOMAIN, b"x", 3) == prover.sample_challenges(DOMAIN, b"x", 3)


def test_oversized_request_rejected(gpu_lib):
    with pytest.raises(gpu_lib.LfError) as e:
        gpu_lib.sample_challenges_noalloc(DOMAIN, b"", gpu_lib.NOALLOC_MAX_CHALLENGES + 1)
    assert e.value.code == -10
