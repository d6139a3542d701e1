"""Build the CPU oracle `oracle/_build/liboracle.so` (test infrastructure).

The oracle is the checker for the CUDA engine and the timed CPU baseline; it
is never part of the product path.  -ffp-contract=off keeps its FP64 results
independent of whether the host compiler fuses multiply-adds, so x86 and Arm
builds agree.
"""

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "oracle.c")
OUT = os.path.join(HERE, "_build", "liboracle.so")


def stale():
    if not os.path.exists(OUT):
        return True
    t = os.path.getmtime(OUT)
    deps = [SRC, os.path.join(ROOT, "include", "acc_gb300.h"),
            os.path.abspath(__file__)]
    return any(os.path.getmtime(f) > t for f in deps)


def build(force=False):
    if not force and not stale():
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    tmp = OUT + ".tmp"
    cmd = [os.environ.get("CC", "gcc"), "-O2", "-std=c11", "-D_GNU_SOURCE",
           "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-Wall",
           "-Wextra", "-Wno-unused-parameter", SRC, "-o", tmp, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
