"""Build the oracle's C restatement (TEST INFRASTRUCTURE: parity oracle and CPU baseline only).

Produces oracle/_build/liboracle_lbm_f32.so and liboracle_lbm_f64.so from
oracle/lbm_oracle.c with gcc.  -ffp-contract=off keeps the arithmetic
identical on x86-64 and aarch64 (no implicit FMA); -fopenmp parallelises the
cell loops for the timed CPU baseline.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "lbm_oracle.c")
FLAGS = ["-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-std=c11"]


def lib_path(real: str) -> str:
    return os.path.join(OUT, f"liboracle_lbm_{real}.so")


def build(verbose: bool = False) -> dict:
    os.makedirs(OUT, exist_ok=True)
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    out = {}
    for tag, real in (("f32", "float"), ("f64", "double")):
        dst = lib_path(tag)
        if os.path.exists(dst) and os.path.getmtime(dst) >= os.path.getmtime(SRC):
            out[tag] = dst
            continue
        cmd = [cc, *FLAGS, f"-DREAL={real}", SRC, "-o", dst + ".tmp", "-lm"]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stderr}")
        os.replace(dst + ".tmp", dst)
        out[tag] = dst
    return out


if __name__ == "__main__":
    print(build(verbose=True))
