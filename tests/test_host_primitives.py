"""The prover's shared host/device primitives (field products, BLAKE3, the device-style subtree
absorb of the transcript), compiled for the host and checked against the independent oracle."""
import os
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_primitives_agree_with_oracle(oracle):
    lib = os.path.join(ROOT, "oracle", "_build")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "prim_check")
        subprocess.run(["g++", "-O2", "-std=c++17", os.path.join(ROOT, "tests", "prim_check.cc"), "-I",
                        os.path.join(ROOT, "oracle"), "-L", lib, "-loracle", f"-Wl,-rpath,{lib}", "-o", exe],
                       check=True)
        p = subprocess.run([exe], capture_output=True, text=True)
    assert p.returncode == 0, p.stdout
    assert p.stdout.startswith("OK")
