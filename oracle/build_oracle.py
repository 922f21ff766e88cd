"""Build recipe for the CPU oracle (test infrastructure only).

Produces, under oracle/_build/:
  libnt2oracle.so      -O2 -fno-tree-vectorize: NT2's scalar+OpenMP path, which is
                       what NT2 runs on a CPU without a Boost.SIMD backend
                       (aarch64 falls back to simd_emulation_, scalar loops);
  libnt2oracle_vec.so  -O3 with the compiler's auto-vectorisation, an upper bound
                       for a vectorised CPU build of the same loops.
Both use -ffp-contract=off because NT2's fma/fnms round twice.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
SRCS = [os.path.join(HERE, "nt2_oracle.c"), os.path.join(HERE, "nt2_oracle_trig.c")]

VARIANTS = {
    "libnt2oracle.so": ["-O2", "-fno-tree-vectorize"],
    "libnt2oracle_vec.so": ["-O3"],
}


def build(verbose: bool = False) -> dict[str, str]:
    os.makedirs(OUT, exist_ok=True)
    cc = os.environ.get("CC", "gcc")
    out = {}
    for name, opt in VARIANTS.items():
        lib = os.path.join(OUT, name)
        out[name] = lib
        if os.path.exists(lib) and all(os.path.getmtime(lib) > os.path.getmtime(src) for src in SRCS):
            continue
        cmd = [cc, *opt, "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
               "-shared", *SRCS, "-o", lib, "-lm"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
