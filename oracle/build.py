"""Build recipe for the CPU oracle (test infrastructure, not product code).

Compiles ``getm_oracle.c`` to ``oracle/_build/libgetm_oracle.so`` with
``-O2 -ffp-contract=off`` (no fused multiply-add, matching gfortran's
default code generation on generic x86-64 for the reference Fortran).
``variant="omp"`` builds the same source with OpenMP for the timed CPU
baseline (the per-row loops carry ``omp`` pragmas that are inert otherwise).
``variant="fma"`` lets the compiler contract multiply-adds into fused
multiply-adds (``-ffp-contract=fast``; on x86-64 with ``-mfma`` so that the
instruction exists), as gfortran does by default for the reference on
aarch64: the two builds are the reference's own spread between two valid
compilations, against which the GPU's rounding differences are measured.
"""

from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
SRC = HERE / "getm_oracle.c"


def lib_path(variant: str = "serial") -> Path:
    return BUILD / ("libgetm_oracle.so" if variant == "serial" else f"libgetm_oracle_{variant}.so")


def build(variant: str = "serial", force: bool = False) -> Path:
    out = lib_path(variant)
    if out.exists() and not force and out.stat().st_mtime > max(SRC.stat().st_mtime, Path(__file__).stat().st_mtime):
        return out
    BUILD.mkdir(exist_ok=True)
    flags = ["-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11"]
    if variant == "omp":
        flags = ["-O3", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11", "-fopenmp"]
    elif variant == "fma":
        import platform

        flags = ["-O2", "-ffp-contract=fast", "-fPIC", "-shared", "-std=c11"]
        if platform.machine() in ("x86_64", "AMD64"):
            flags.append("-mfma")
    elif variant != "serial":
        raise ValueError(f"unknown oracle variant {variant!r}")
    tmp = out.with_suffix(".tmp")
    cmd = [os.environ.get("CC", "gcc")] + flags + [str(SRC), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    for v in ("serial", "omp", "fma"):
        print(build(v, force="--force" in sys.argv))
