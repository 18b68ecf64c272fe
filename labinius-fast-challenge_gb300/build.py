"""Build liblabinius_gpu.so (sm_103a) and the labinius-fast command, in-tree.

    python labinius-fast-challenge_gb300/build.py [--verbose-ptxas]

Translation units compile in parallel with one -gencode; outputs go to
labinius-fast-challenge_gb300/_build/.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(OUT, "liblabinius_gpu.so")
CLI = os.path.join(OUT, "labinius-fast")
UNITS = ["lf_commit.cu", "lf_switch.cu", "lf_open.cu", "lf_ring.cu", "lf_api.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    return p.stdout + p.stderr


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(verbose_ptxas=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "labinius_gpu.h"))
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE,
                    "-Xcompiler", "-ffp-contract=off"]
    if verbose_ptxas:
        flags += ["-Xptxas", "-v"]
    jobs = []
    for u in UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(OUT, u.replace(".cu", ".o"))
        if force or verbose_ptxas or _stale(obj, [src] + headers):
            jobs.append([nvcc(), *flags, "-c", src, "-o", obj])
    logs = []
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    objs = [os.path.join(OUT, u.replace(".cu", ".o")) for u in UNITS]
    if force or _stale(LIB, objs):
        _run([nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    cli_src = os.path.join(HERE, "cli", "labinius_fast.cpp")
    if os.path.exists(cli_src) and (force or _stale(CLI, [cli_src, LIB])):
        _run(["g++", "-O2", "-std=c++17", "-I", INCLUDE, cli_src, "-o", CLI, "-L", OUT, "-llabinius_gpu",
              "-Wl,-rpath,$ORIGIN"])
    return "\n".join(logs)


if __name__ == "__main__":
    log = build(verbose_ptxas="--verbose-ptxas" in sys.argv, force="--force" in sys.argv)
    if log.strip():
        print(log)
    print(LIB)
