"""Build the CPU oracle (test infrastructure).

The oracle is the checker for the CUDA engine and the timed CPU baseline; it
is never part of the product path.  Two builds of the same source:

* `oracle/_build/liboracle.so`, the checker: -O2 -ffp-contract=off, so that
  its FP64 results do not depend on whether the host compiler fuses
  multiply-adds and x86 and Arm builds agree;
* `oracle/_build/liboracle_timing.so`, the timed CPU baseline: -O3 with
  multiply-add contraction allowed (-ffp-contract=fast), the fastest
  portable build (no -march/-mcpu=native: the same flags on both hosts).
"""

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "oracle.c")
OUT = os.path.join(HERE, "_build", "liboracle.so")
OUT_TIMING = os.path.join(HERE, "_build", "liboracle_timing.so")
FLAGS = {OUT: ["-O2", "-ffp-contract=off"],
         OUT_TIMING: ["-O3", "-ffp-contract=fast"]}


def stale(out=OUT):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    deps = [SRC, os.path.join(ROOT, "include", "acc_gb300.h"),
            os.path.abspath(__file__)]
    return any(os.path.getmtime(f) > t for f in deps)


def build(force=False, timing=False):
    """Build (when stale) and return the checker, or with `timing` the
    timed-baseline build."""
    out = OUT_TIMING if timing else OUT
    if not force and not stale(out):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    tmp = out + ".tmp"
    cmd = [os.environ.get("CC", "gcc"), *FLAGS[out], "-std=c11",
           "-D_GNU_SOURCE", "-fPIC", "-shared", "-fopenmp", "-Wall",
           "-Wextra", "-Wno-unused-parameter", SRC, "-o", tmp, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    return out


def describe(timing=False):
    """The compiler flags of a build, for reports."""
    out = OUT_TIMING if timing else OUT
    return " ".join([os.environ.get("CC", "gcc"), *FLAGS[out], "-fopenmp"])


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    print(build(force="--force" in sys.argv, timing=True))
