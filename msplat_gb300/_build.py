"""Builds the native library ``libmsplat_gb300.so`` in-tree with nvcc.

Every translation unit in ``csrc/`` is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``) with the same floating-point
flags as the reference build (``-O3 --use_fast_math``, reference
``setup.py:39``), in parallel, then linked into one shared object that
exports the C ABI declared in ``include/msplat_gb300.h``.

Kernel shape parameters chosen by the autotuner (``msplat_gb300/autotune.py``)
are read from ``msplat_gb300/tuning.json`` when it exists and passed as -D
flags; without it the sources' defaults apply.

Run ``python -m msplat_gb300._build`` (or ``__graft_entry__.build()``).
"""
from __future__ import annotations

import concurrent.futures as cf
import json
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libmsplat_gb300.so")
TUNING_PATH = os.path.join(PKG_DIR, "tuning.json")

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH_FLAGS + [
    "-O3",
    "--use_fast_math",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-fvisibility=hidden",
    "--expt-relaxed-constexpr",
]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build msplat_gb300")
    return cand


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def tuned_defines(path: str = TUNING_PATH) -> dict:
    """The autotuner's choices {macro: value} -- the frame's and every other
    workload's (their macros are disjoint) -- or {} without a tuning file."""
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        data = json.load(f)
    out = {str(k): int(v) for k, v in data.get("defines", {}).items()}
    for w in data.get("workloads", {}).values():
        out.update({str(k): int(v) for k, v in w.get("defines", {}).items()})
    return out


def define_flags(defines: dict) -> list[str]:
    return [f"-D{k}={v}" for k, v in sorted(defines.items())]


def _needs_build(lib_path: str) -> bool:
    if not os.path.exists(lib_path):
        return True
    lib_m = os.path.getmtime(lib_path)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(INCLUDE, "msplat_gb300.h"))
    deps.append(os.path.abspath(__file__))
    if os.path.exists(TUNING_PATH):
        deps.append(TUNING_PATH)
    return any(os.path.getmtime(d) > lib_m for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None,
          defines: dict | None = None, lib_path: str | None = None, build_dir: str | None = None) -> str:
    """Compiles and links the library; returns its path.  `defines`
    replaces the tuning file's macros (the autotuner builds its variants this
    way, into their own `lib_path` / `build_dir`)."""
    lib_path = lib_path or LIB_PATH
    build_dir = build_dir or BUILD_DIR
    srcs = sources()
    os.makedirs(build_dir, exist_ok=True)
    objs = [os.path.join(build_dir, os.path.basename(s)[:-3] + ".o") for s in srcs]
    if not force and not _needs_build(lib_path):
        return lib_path
    nvcc = _nvcc()
    macros = tuned_defines() if defines is None else dict(defines)
    flags = NVCC_FLAGS + ["-I", INCLUDE, "-I", CSRC] + define_flags(macros) + list(extra_flags or [])

    def compile_one(pair):
        src, obj = pair
        cmd = [nvcc, *flags, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stderr}")
        return r.stderr

    workers = min(len(srcs), max(1, os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        for msg in ex.map(compile_one, zip(srcs, objs)):
            if verbose and msg:
                print(msg, file=sys.stderr)
    tmp = lib_path + ".tmp"
    cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stderr}")
    os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
