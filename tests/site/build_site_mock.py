"""Compile the mock-tree site program (nt2_site_mock.cu) with nvcc for sm_103a."""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "_build", "nt2_site_mock")


def build() -> str:
    src = os.path.join(HERE, "nt2_site_mock.cu")
    deps = [src]
    for d in (os.path.join(ROOT, "include"), os.path.join(ROOT, "nt2_gb300", "csrc", "nt2cuda")):
        for base, _, files in os.walk(d):
            deps += [os.path.join(base, f) for f in files]
    if os.path.exists(OUT) and all(os.path.getmtime(OUT) > os.path.getmtime(d) for d in deps):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = [os.environ.get("NVCC", "nvcc"), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "nt2_gb300", "csrc"), src, "-o", OUT]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"site mock build failed:\n{r.stdout}\n{r.stderr}")
    return OUT


if __name__ == "__main__":
    print(build())
