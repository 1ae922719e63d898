"""Autotuner for the kernels' shape parameters.

The blend and sort kernels have compile-time shape parameters: pixels per
thread in the blend forward and backward (which also sets the block shape,
256 / NPIX threads per 16x16 tile), the number of contributing lanes below
which the backward sends a Gaussian's gradients as direct atomics instead
of a warp reduction, and the keys per thread of a radix tile (which sets
the tile size, 256 x items), optional register caps of the two blend
kernels (more resident blocks per SM against spills) and whether a tile is
blended by one block or by two of 8 rows each.  The tuner builds a variant of the library for
each candidate setting (into its own directory), times a forward + backward
frame of the benchmark's synthetic scene (``synthetic.training_scene``)
with it in a separate process, searches the settings by coordinate descent
from the current defaults, and writes the best to
``msplat_gb300/tuning.json``, which the build then applies.

    python -m msplat_gb300.autotune [--gaussians N --width W --height H]
                                    [--params MACRO,MACRO...]

(``--params`` searches only the named parameters, the others staying at
their current tuned values.)

Results are those of any setting (all are parity-tested); only speed
differs.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys

from . import _build

SPACE = {
    "MSPLAT_BLEND_NPIX_FWD": [1, 2],
    "MSPLAT_BLEND_NPIX_BWD": [1, 2, 4],
    "MSPLAT_FEW_LANES": [8, 12, 16],
    "MSPLAT_SORT_ITEMS": [8, 12, 16],
    "MSPLAT_BLEND_FWD_REGS": [0, 40],
    "MSPLAT_BLEND_BWD_REGS": [0, 64, 72],
    "MSPLAT_BLEND_SPLIT_FWD": [1, 2],
    "MSPLAT_BLEND_SPLIT_BWD": [1, 2],
}
DEFAULTS = {"MSPLAT_BLEND_NPIX_FWD": 1, "MSPLAT_BLEND_NPIX_BWD": 2, "MSPLAT_FEW_LANES": 12,
            "MSPLAT_SORT_ITEMS": 12, "MSPLAT_BLEND_FWD_REGS": 0, "MSPLAT_BLEND_BWD_REGS": 0,
            "MSPLAT_BLEND_SPLIT_FWD": 1, "MSPLAT_BLEND_SPLIT_BWD": 1}
TUNE_DIR = os.path.join(_build.PKG_DIR, "_build", "tune")


def coordinate_descent(space: dict, start: dict, objective, rounds: int = 2):
    """Minimises objective(setting) one parameter at a time (each tried at
    every value with the others fixed), for up to `rounds` sweeps or until a
    sweep changes nothing.  Returns (best setting, its value, {setting: value}
    for every setting evaluated)."""
    seen: dict = {}

    def f(setting):
        key = tuple(sorted(setting.items()))
        if key not in seen:
            seen[key] = objective(dict(setting))
        return seen[key]

    best = dict(start)
    best_v = f(best)
    for _ in range(rounds):
        changed = False
        for name, values in space.items():
            for v in values:
                if v == best[name]:
                    continue
                cand = dict(best, **{name: v})
                cv = f(cand)
                if cv < best_v:
                    best, best_v, changed = cand, cv, True
        if not changed:
            break
    return best, best_v, {k: v for k, v in seen.items()}


def make_objective(build_variant, time_library, log=print):
    """objective(setting) -> ms for coordinate_descent: builds the variant
    with build_variant(setting) -> library path and times it with
    time_library(path) -> ms.  A setting whose build fails (a combination
    the kernels reject at compile time) scores infinity instead of ending
    the search."""
    def objective(setting):
        try:
            lib = build_variant(setting)
        except RuntimeError as e:
            log(f"{setting} -> does not build ({str(e).splitlines()[0][:120] if str(e) else 'error'})")
            return float("inf")
        ms = time_library(lib)
        log(f"{setting} -> {ms:.4f} ms")
        return ms
    return objective


def variant_library(defines: dict) -> str:
    """Builds (once) the library with `defines` into its own directory."""
    tag = hashlib.sha1(json.dumps(sorted(defines.items())).encode()).hexdigest()[:12]
    d = os.path.join(TUNE_DIR, tag)
    return _build.build(defines=defines, lib_path=os.path.join(d, "libmsplat_gb300.so"), build_dir=d)


def time_variant(lib: str, gaussians: int, width: int, height: int, steps: int, warmup: int) -> float:
    """Median ms of a forward + backward frame with the library at `lib`,
    measured in a fresh process (the library is loaded once per process)."""
    env = dict(os.environ, MSPLAT_GB300_LIB=lib)
    cmd = [sys.executable, "-m", "msplat_gb300.autotune", "--time", "--gaussians", str(gaussians), "--width",
           str(width), "--height", str(height), "--steps", str(steps), "--warmup", str(warmup)]
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, cwd=_build.ROOT, timeout=600)
    if r.returncode != 0:
        raise RuntimeError(f"timing run failed:\n{r.stderr[-2000:]}")
    return float(r.stdout.strip().splitlines()[-1])


def _time_here(gaussians: int, width: int, height: int, steps: int, warmup: int) -> float:
    import numpy as np
    import torch

    import msplat_gb300 as ms
    from .synthetic import training_scene
    dev = torch.device("cuda")
    sc = training_scene(gaussians, width, height, 1500.0 * width / 1920.0, seed=0)
    p = [sc[k].to(dev).contiguous().requires_grad_() for k in ("xyz", "scale", "rot", "opacity", "shs")]
    intr, extr, w = sc["intr"].to(dev), sc["extr"].to(dev), sc["weights"].to(dev)

    def step():
        for t in p:
            t.grad = None
        img = ms.rasterization_sh(*p, intr, extr, width, height, 0.0)
        (img * w).sum().backward()

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        step()
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    return float(np.median(times))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gaussians", type=int, default=1_000_000)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--rounds", type=int, default=1)
    ap.add_argument("--params", default="", help="comma-separated subset of the parameters to search")
    ap.add_argument("--time", action="store_true", help="(internal) time the library of this process")
    ap.add_argument("--out", default=_build.TUNING_PATH)
    a = ap.parse_args()
    if a.time:
        print(_time_here(a.gaussians, a.width, a.height, a.steps, a.warmup))
        return

    objective = make_objective(
        variant_library, lambda lib: time_variant(lib, a.gaussians, a.width, a.height, a.steps, a.warmup),
        log=lambda msg: print(msg, flush=True))

    start = dict(DEFAULTS, **{k: v for k, v in _build.tuned_defines().items() if k in SPACE})
    space = SPACE
    if a.params:
        names = [n.strip() for n in a.params.split(",") if n.strip()]
        unknown = [n for n in names if n not in SPACE]
        if unknown:
            raise SystemExit(f"unknown parameters: {unknown}")
        space = {n: SPACE[n] for n in names}
    best, best_ms, seen = coordinate_descent(space, start, objective, rounds=a.rounds)
    out = {"defines": best, "ms_per_frame": round(best_ms, 4),
           "workload": {"gaussians": a.gaussians, "width": a.width, "height": a.height},
           "evaluated": [{"defines": dict(k), "ms_per_frame": round(v, 4)} for k, v in seen.items()]}
    with open(a.out, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps({"defines": best, "ms_per_frame": round(best_ms, 4)}))


if __name__ == "__main__":
    main()
