"""Build the in-tree CUDA engine `acc_gb300/libacc_gb300.so` for sm_103a.

One nvcc invocation per translation unit, run in parallel, then one link.
The library statically links the CUDA runtime so that it loads (and reports
"no device") on a machine without a GPU.
"""

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libacc_gb300.so")

SOURCES = ["engine.cu", "launch_fp32.cu", "launch_fp64.cu",
           "launch_fp64_fma.cu", "probe.cu", "noalloc.cu"]
HEADERS = ["common.cuh", "components.cuh", "sample.cuh", "monitors.cuh",
           "kernels.cuh", "ms.cuh", "track.cuh"]
# per-source extra flags: the FP64 kernels round every multiply and add
# separately, like the CPU restatement they are checked against; the
# contracted FP64 chain kernel lives in a namespace of its own
EXTRA_FLAGS = {"launch_fp64.cu": ["--fmad=false"],
               "launch_fp64_fma.cu": ["-Dmcv=mcv_fma"]}

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# FP32 code paths are written for approximate division and square root;
# neither flag changes FP64 arithmetic.  Denormals are kept (no --ftz): a
# flush would also zero float32 table entries converted to double and the
# squares of small float weights.
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--prec-div=false",
              "--prec-sqrt=false", "-Xcompiler", "-fPIC", "-Xcompiler",
              "-Wall"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _inputs():
    files = [os.path.join(CSRC, s) for s in SOURCES + HEADERS]
    files.append(os.path.join(ROOT, "include", "acc_gb300.h"))
    files.append(os.path.join(ROOT, "include", "acc_gb300_probe.h"))
    files.append(os.path.abspath(__file__))
    return files


def stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in _inputs())


def _compile(src):
    obj = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *EXTRA_FLAGS.get(src, []), "-c",
           os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build_engine(force=False, verbose=False):
    """Compile and link the engine if any source changed; return its path."""
    if not force and not stale():
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build_engine(force="--force" in sys.argv, verbose=True)
