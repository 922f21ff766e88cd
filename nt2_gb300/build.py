"""Build the nt2cuda shared library (sm_103a) in-tree.

Each translation unit under csrc/ is compiled by nvcc in parallel into
_build/, then linked into nt2_gb300/libnt2cuda.so.  A unit is rebuilt only
when it or any header under csrc/ or include/ is newer than its object.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnt2cuda.so")

SOURCES = [
    "capi_core.cu",
    "capi_transform.cu",
    "capi_fold.cu",
    "capi_sigmadelta.cu",
    "capi_mandelbrot.cu",
    "capi_reduce_f32.cu",
    "capi_reduce_f64.cu",
    "capi_scan.cu",
    "server.cu",
    "capi_noalloc.cu",
    "capi_selftest.cu",
    "capi_trig_f32.cu",
    "capi_trig_f64.cu",
    "capi_expfam_f32.cu",
    "capi_expfam_f64.cu",
    "capi_trigx_f32.cu",
    "capi_trigx_f64.cu",
    "capi_trigx_fwd_f32.cu",
    "capi_trigx_fwd_f64.cu",
    "capi_trigx_fwd128_f32.cu",
    "capi_trigx_fwd128_f64.cu",
]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-lineinfo", "-O3", "-std=c++17",
    "-Xcompiler", "-fPIC",
    "-I", os.path.join(ROOT, "include"),
    "-I", CSRC,
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _headers() -> list[str]:
    out = []
    for d in (CSRC, os.path.join(ROOT, "include")):
        for base, _, files in os.walk(d):
            out += [os.path.join(base, f) for f in files if f.endswith((".cuh", ".h", ".hpp"))]
    return out


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile and link; return the library path.  Raises RuntimeError on failure."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in srcs]

    def compile_one(i: int):
        src = os.path.join(CSRC, srcs[i])
        if not _stale(objs[i], [src] + headers):
            return None
        cmd = [nvcc] + NVCC_FLAGS + ["-c", src, "-o", objs[i]]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            return f"{srcs[i]}:\n{r.stdout}\n{r.stderr}"
        return None

    n = jobs or min(len(srcs), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=max(1, n)) as ex:
        errs = [e for e in ex.map(compile_one, range(len(srcs))) if e]
    if errs:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errs))
    if _stale(LIB, objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread", "-ldl"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
