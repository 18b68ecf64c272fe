"""Regenerate tests/golden/oracle_digests.json from the CPU oracle.

These digests pin the oracle against its own earlier output (a regression guard for the
checker). They are NOT reference vectors: the reference ships none, and BLAKE3 parity with the
reference's `blake3` crate is unpinned in this environment.

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import pyoracle  # noqa: E402

CASES = [(19, bytes([42] * 32)), (20, bytes([44] * 32)), (20, bytes(range(32)))]


def digests():
    out = {
        "blake3_empty": pyoracle.blake3(b"").hex(),
        "blake3_abc_keyed": pyoracle.blake3(b"abc", key=bytes(range(32))).hex(),
        "blake3_derive": pyoracle.blake3(b"material", derive="lf golden context").hex(),
        "blake3_xof_1025_at_4000": pyoracle.blake3(bytes(1025), n=64, seek=4000).hex(),
        "proofs": [],
    }
    for log_vars, seed in CASES:
        table = pyoracle.write_table(seed, log_vars)
        proof = pyoracle.prove(seed, table, log_vars)
        out["proofs"].append({"log_vars": log_vars, "seed": seed.hex(),
                              "table_sha256": hashlib.sha256(table).hexdigest(),
                              "proof_sha256": hashlib.sha256(proof).hexdigest(), "proof_len": len(proof)})
    return out


if __name__ == "__main__":
    pyoracle.build()
    with open(os.path.join(HERE, "oracle_digests.json"), "w") as f:
        json.dump(digests(), f, indent=1)
    print("wrote oracle_digests.json")
