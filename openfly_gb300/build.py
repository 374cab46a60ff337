"""Build libflygpu.so in-tree for sm_103a (GB300).

Every translation unit is compiled in parallel with one -gencode. The neighbour-list and binary64 EAM
units use -fmad=false so their arithmetic matches the reference's binary64 operations exactly; host
code uses -ffp-contract=off for the same reason (spline coefficients, search drivers).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libflygpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-Wall"]
EXACT = {"nlist.cu", "eam_fp64.cu", "noalloc.cu", "env.cu", "hessian.cu"}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libflygpu")


def sources() -> list[str]:
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _compile(nvcc: str, src: str, verbose: bool) -> str:
    obj = os.path.join(OUT_DIR, src + ".o")
    path = os.path.join(CSRC, src)
    hdrs = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".hpp", ".cuh"))]
    hdrs.append(os.path.join(HERE, "..", "include", "flygpu.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(p) for p in [path, *hdrs]):
        return obj
    cmd = [nvcc, *ARCH, *COMMON, "-c", path, "-o", obj]
    if src in EXACT:
        cmd.insert(1, "-fmad=false")
    if src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"] if verbose else []
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False) -> str:
    """Compile all sources and link libflygpu.so; returns its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    srcs = sources()
    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 8))) as ex:
        objs = list(ex.map(lambda s: _compile(nvcc, s, verbose), srcs))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
