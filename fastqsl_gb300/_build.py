"""Builds libfastqsl_gb300.so (all CUDA kernels + the C ABI) for sm_103a.

Each translation unit is compiled by nvcc in parallel and linked into one
shared object next to this file.  trace_exact.cu and qassembly.cu are
compiled with -fmad=false: their kernels reproduce the reference's rounding
and must not have multiplies and adds fused.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfastqsl_gb300.so")
NVCC = os.environ.get("NVCC", os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc"))
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-I", os.path.join(ROOT, "include"), "-I", CSRC]
NO_FMA = {"trace_exact.cu", "qassembly.cu", "curl.cu", "path.cu"}
SOURCES = ["capi.cu", "trace_exact.cu", "trace_fast_soa.cu", "trace_fast_f4.cu", "trace_fast_h4b.cu",
           "trace_fast_h4bw.cu", "trace_fast_h8c.cu", "trace_fast_stretch.cu", "trace_fast_stretch_packed.cu",
           "trace_fast_stretch_packed_uni.cu", "field_store.cu",
           "qassembly.cu", "hybrid.cu", "curl.cu", "path.cu", "noalloc.cu", "probe.cu", "seeds.cu",
           "qmap_batch.cu"]


def _deps():
    out = []
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".h")):
                out.append(os.path.join(d, f))
    return out


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, extra=()):
    obj = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    flags = list(COMMON) + list(ARCH) + list(extra)
    if src in NO_FMA:
        flags.append("-fmad=false")
    cmd = [NVCC, *flags, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force=False, verbose=False, extra=()):
    deps = _deps() + [__file__]
    if not force and not _stale(LIB, deps):
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    if verbose:
        for _, err in results:
            if err.strip():
                print(err)
    tmp = LIB + ".tmp"
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *[o for o, _ in results], "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    extra = ["-Xptxas", "-v"] if "-v" in sys.argv else []
    print(build(force=True, verbose=bool(extra), extra=extra))
