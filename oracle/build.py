"""Builds the CPU oracle (oracle.c) into oracle/_build/liboracle.so with gcc.

Test infrastructure only.  -ffp-contract=off keeps gcc from fusing
multiply-adds on its own (the oracle places every FMA explicitly), and no
fast-math flags are used, so results are identical on x86-64 and aarch64.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.abspath(__file__))):
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler found for the oracle")
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp"
    base = [cc, "-O2", "-std=c11", "-D_DEFAULT_SOURCE", "-fPIC", "-shared", "-ffp-contract=off",
            "-fno-fast-math", "-fno-strict-aliasing", SRC, "-o", tmp, "-lm"]
    # OpenMP only spreads the timed CPU baseline over the host cores; without
    # it the oracle builds serial.
    r = subprocess.run(base + ["-fopenmp"], capture_output=True, text=True)
    if r.returncode != 0:
        r = subprocess.run(base, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
