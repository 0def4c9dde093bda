"""Build recipe for libiskra_gpu.so (sm_103a) -- nvcc only, no cmake.

Each .cu under csrc/ compiles to an object in parallel, then one nvcc link
produces iskra_gb300/lib/libiskra_gpu.so in the source tree.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(OUT_DIR, "libiskra_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
         "-Xptxas", "-v" if os.environ.get("ISKRA_PTXAS_V") else "-O3"]
# extra nvcc flags for tuning builds, e.g. ISKRA_NVCC_FLAGS="-DISKRA_PUSH_MIN_BLOCKS=6"
FLAGS += os.environ.get("ISKRA_NVCC_FLAGS", "").split()


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _compile(src, obj):
    cmd = [nvcc(), *ARCH, *FLAGS, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    srcs = sources()
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    hdrs.append(os.path.join(os.path.dirname(HERE), "include", "iskra_gpu.h"))
    stamp = os.path.join(OUT_DIR, ".flags")
    flags = " ".join(ARCH + FLAGS)
    old = open(stamp).read() if os.path.exists(stamp) else ""
    if not force and os.path.exists(LIB) and old == flags:
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(f) < t for f in srcs + hdrs + [__file__]):
            return LIB
    obj_dir = os.path.join(HERE, "_build")
    os.makedirs(obj_dir, exist_ok=True)
    os.makedirs(OUT_DIR, exist_ok=True)
    objs = [os.path.join(obj_dir, os.path.basename(s)[:-3] + ".o") for s in srcs]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        logs = list(ex.map(_compile, srcs, objs))
    if verbose:
        for l in logs:
            if l:
                print(l, file=sys.stderr)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(flags)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
