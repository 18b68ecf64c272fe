"""The oracle against its committed digests (tests/golden/make_golden.py). A regression pin of the
checker, not a reference vector: the reference ships no golden vectors."""
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def test_oracle_matches_committed_digests(oracle):
    import sys

    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_golden

    want = json.load(open(os.path.join(HERE, "golden", "oracle_digests.json")))
    assert make_golden.digests() == want
