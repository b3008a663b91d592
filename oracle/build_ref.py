"""Build the reference's own plain kernels for the CPU (TEST INFRASTRUCTURE: the pinning reference).

The reference's lattice and thermal kernels are CUDA with a torch host part, and the
reference tree is not present where the device tests run, so they are run here, on the
host, from their unmodified text, to write golden fixtures:
  1. the device part of solver/lbm_kernels.cu (its constant tables, device helpers and
     the kernels defined before its host code, plus lbm_zou_he_bc_kernel,
     lbm_macro_collide_mrt_smag_kernel, lbm_convective_bc_reduce_kernel and
     lbm_convective_mass_correct_kernel) is cut out of the file as text, by brace
     matching, with no edit;
  2. one translation unit oracle/_ref/ref_lbm_host.cpp is written: oracle/ref_shim.h
     (host stand-ins for the CUDA built-ins), the cut text, oracle/ref_launch.inc (C
     entry points that run each kernel over the reference's launch grid);
  3. g++ -std=c++20 -O2 -ffp-contract=off -> oracle/_ref/libref_lbm_host.so.
The same recipe builds oracle/_ref/libref_thermal_host.so from solver/thermal_kernels.cu
(thermal_reconstruct_kernel and physics_check_kernel, compiled with double in place of
float, plus oracle/ref_thermal_launch.inc), so that the reference's fused thermal step can
run in FP64 with its torch multigrid on the host.
Everything written goes to oracle/_ref/ (git-ignored).  The libraries are loaded only by
the fixture scripts tests/golden/make_ref_fixtures.py (tests/golden/ref_lbm.npz) and
tests/golden/make_golden.py (tests/golden/thermal_steady.npz).

Usage:  python oracle/build_ref.py /path/to/fluxcore3D
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libref_lbm_host.so")
THERMAL_LIB = os.path.join(OUT, "libref_thermal_host.so")
KERNELS = ("lbm_zou_he_bc_kernel", "lbm_macro_collide_mrt_smag_kernel", "lbm_convective_bc_reduce_kernel",
           "lbm_convective_mass_correct_kernel")
THERMAL_KERNELS = ("thermal_reconstruct_kernel", "physics_check_kernel")


def function_text(src: str, name: str) -> str:
    """The full text of the __global__ function `name` (signature through its closing brace)."""
    m = re.search(r"__global__\s+void\s+" + re.escape(name) + r"\s*\(", src)
    if not m:
        raise RuntimeError(f"{name} not found")
    i = src.index("{", m.end())
    depth = 0
    for j in range(i, len(src)):
        if src[j] == "{":
            depth += 1
        elif src[j] == "}":
            depth -= 1
            if depth == 0:
                return src[m.start():j + 1]
    raise RuntimeError(f"unbalanced braces in {name}")


def lbm_device_part(src: str) -> str:
    """Everything before the host code (which starts at the BLOCK macro) without #include lines,
    plus the kernels defined after it."""
    host = src.index("#define BLOCK")
    head = "\n".join(ln for ln in src[:host].splitlines() if not ln.lstrip().startswith("#include"))
    return head + "\n\n" + "\n\n".join(function_text(src, k) for k in KERNELS) + "\n"


def _compile(tu: str, lib: str, verbose: bool) -> None:
    cxx = os.environ.get("CXX") or shutil.which("g++") or "c++"
    cmd = [cxx, "-std=c++20", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
           "-Wno-unknown-pragmas", tu, "-o", lib + ".tmp"]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building the reference kernels for the host failed:\n{r.stderr[-4000:]}")
    os.replace(lib + ".tmp", lib)


def _read(ref_root: str, rel: str) -> str:
    with open(os.path.join(ref_root, rel)) as fh:
        return fh.read()


def build(ref_root: str, verbose: bool = False) -> str:
    """Compile the lattice kernels; returns the library path."""
    os.makedirs(OUT, exist_ok=True)
    body = lbm_device_part(_read(ref_root, os.path.join("solver", "lbm_kernels.cu")))
    tu = os.path.join(OUT, "ref_lbm_host.cpp")
    with open(tu, "w") as fh:
        fh.write('#include "%s"\n' % os.path.join(HERE, "ref_shim.h"))
        fh.write("// ---- text of solver/lbm_kernels.cu (device part) ----\n")
        fh.write(body)
        fh.write('\n#include "%s"\n' % os.path.join(HERE, "ref_launch.inc"))
    _compile(tu, LIB, verbose)
    return LIB


def build_thermal(ref_root: str, verbose: bool = False) -> str:
    """Compile the thermal kernels in FP64 (float -> double); returns the library path."""
    os.makedirs(OUT, exist_ok=True)
    src = _read(ref_root, os.path.join("solver", "thermal_kernels.cu"))
    body = "\n\n".join(function_text(src, k) for k in THERMAL_KERNELS)
    tu = os.path.join(OUT, "ref_thermal_host.cpp")
    with open(tu, "w") as fh:
        fh.write('#include "%s"\n' % os.path.join(HERE, "ref_shim.h"))
        fh.write("#define float double\n// ---- text of solver/thermal_kernels.cu (two kernels) ----\n")
        fh.write(body)
        fh.write('\n#undef float\n#include "%s"\n' % os.path.join(HERE, "ref_thermal_launch.inc"))
    _compile(tu, THERMAL_LIB, verbose)
    return THERMAL_LIB


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else None
    if not root:
        sys.exit("usage: python oracle/build_ref.py /path/to/fluxcore3D")
    print(build(root, verbose=True))
    print(build_thermal(root, verbose=True))
