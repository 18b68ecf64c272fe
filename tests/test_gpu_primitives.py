"""Device builds of the shared BLAKE3 and binary-field code against their host builds
(tests/dev_blake3_check.cu): hashing in every mode across block and chunk boundaries, a hasher
image copied to the device and extended there (the challenge derivation), and the field products."""
import os
import shutil
import subprocess
import tempfile

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("flags", [[], ["-lineinfo", "-Xcompiler", "-ffp-contract=off"]])
def test_device_primitives_match_host(flags):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "dev_check")
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", *flags,
                        os.path.join(ROOT, "tests", "dev_blake3_check.cu"), "-o", exe], check=True)
        p = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stdout + p.stderr
    assert p.stdout.strip().startswith("OK")
