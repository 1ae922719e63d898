"""Autotuner for the kernels' shape parameters, per workload.

The blend and sort kernels have compile-time shape parameters: pixels per
thread in the blend forward and backward (which sets the block shape, 256 /
NPIX threads per 16x16 tile), the Gaussians per shared-memory batch (entries
gathered per thread x threads), the number of contributing lanes below
which the backward sends a Gaussian's gradients as direct atomics instead
of a warp reduction, the keys per thread of a radix tile (which sets the
sort tile, 256 x items), optional register caps of the two blend kernels
(more resident blocks per SM against spills), whether a tile is blended
by one block or by two of 8 rows each, and whether the forward runs as a
producer / consumer ring, with how many producer warps and with what
minimum of resident ring blocks per SM, and whether the backward runs as
a ring and with how many producer warps.  The tile itself stays 16x16: it is
part of the reference's outputs (tiles_touched, tile_range).  The
multi-camera blend grid has its own pixels-per-thread and batch parameters.

The tuner builds a variant of the library for each candidate setting (into
its own directory), times it in a separate process on the workload --
``frame``: a forward + backward frame of the benchmark's training scene
(``synthetic.training_scene``); ``batch``: a forward + backward batch of
sphere cameras of one scene through ``rasterization_sh_batch`` -- searches
the workload's parameters by coordinate descent from the current values,
and writes the best into ``msplat_gb300/tuning.json`` (its own section per
workload), which the build then applies: the single-camera kernels take
the frame's values, the multi-camera grid the batch's.

    python -m msplat_gb300.autotune [--workload frame|batch]
                                    [--gaussians N --width W --height H --cameras B]
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
    "MSPLAT_BLEND_GATHER_FWD": [1, 2],
    "MSPLAT_BLEND_GATHER_BWD": [1, 2, 4],
    "MSPLAT_FEW_LANES": [8, 12, 16],
    "MSPLAT_SORT_ITEMS": [8, 12, 16],
    "MSPLAT_BLEND_FWD_REGS": [0, 40],
    "MSPLAT_BLEND_BWD_REGS": [0, 64, 72],
    "MSPLAT_BLEND_SPLIT_FWD": [1, 2],
    "MSPLAT_BLEND_SPLIT_BWD": [1, 2],
    "MSPLAT_BLEND_RING_FWD": [0, 2, 4],
    "MSPLAT_RING_MIN_BLOCKS": [0, 5],
    "MSPLAT_BLEND_RING_BWD": [0, 1, 2],
}
DEFAULTS = {"MSPLAT_BLEND_NPIX_FWD": 1, "MSPLAT_BLEND_NPIX_BWD": 2, "MSPLAT_BLEND_GATHER_FWD": 1,
            "MSPLAT_BLEND_GATHER_BWD": 2, "MSPLAT_FEW_LANES": 12, "MSPLAT_SORT_ITEMS": 12,
            "MSPLAT_BLEND_FWD_REGS": 0, "MSPLAT_BLEND_BWD_REGS": 0, "MSPLAT_BLEND_SPLIT_FWD": 1,
            "MSPLAT_BLEND_SPLIT_BWD": 1, "MSPLAT_BLEND_RING_FWD": 0, "MSPLAT_RING_MIN_BLOCKS": 0,
            "MSPLAT_BLEND_RING_BWD": 0}
# the multi-camera blend grid's own parameters (workload "batch")
BATCH_SPACE = {
    "MSPLAT_BATCH_BLEND_NPIX_FWD": [1, 2],
    "MSPLAT_BATCH_BLEND_NPIX_BWD": [1, 2, 4],
    "MSPLAT_BATCH_BLEND_GATHER_FWD": [1, 2],
    "MSPLAT_BATCH_BLEND_GATHER_BWD": [1, 2, 4],
    "MSPLAT_BATCH_BLEND_RING_FWD": [0, 2, 4],
    "MSPLAT_BATCH_BLEND_RING_BWD": [0, 1, 2],
}
BATCH_DEFAULTS = {"MSPLAT_BATCH_BLEND_NPIX_FWD": 1, "MSPLAT_BATCH_BLEND_NPIX_BWD": 2,
                  "MSPLAT_BATCH_BLEND_GATHER_FWD": 1, "MSPLAT_BATCH_BLEND_GATHER_BWD": 2,
                  "MSPLAT_BATCH_BLEND_RING_FWD": 0, "MSPLAT_BATCH_BLEND_RING_BWD": 0}
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


def time_variant(lib: str, gaussians: int, width: int, height: int, steps: int, warmup: int,
                 workload: str = "frame", cameras: int = 16) -> float:
    """Median ms of a forward + backward frame (or batch) with the library at
    `lib`, measured in a fresh process (the library is loaded once per
    process)."""
    env = dict(os.environ, MSPLAT_GB300_LIB=lib)
    cmd = [sys.executable, "-m", "msplat_gb300.autotune", "--time", "--gaussians", str(gaussians), "--width",
           str(width), "--height", str(height), "--steps", str(steps), "--warmup", str(warmup), "--workload",
           workload, "--cameras", str(cameras)]
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


def _time_batch_here(gaussians: int, cameras: int, steps: int, warmup: int) -> float:
    """Median ms of a forward + backward batch of `cameras` sphere cameras
    (sizes drawn from 256^2, 512^2, 1280x720, 1920x1080, the 1080p field of
    view) of one training scene, through rasterization_sh_batch."""
    import numpy as np
    import torch

    import msplat_gb300 as ms
    from .synthetic import training_scene
    dev = torch.device("cuda")
    sc = training_scene(gaussians, 1920, 1080, 1500.0, seed=0)
    p = [sc[k].to(dev).contiguous().requires_grad_() for k in ("xyz", "scale", "rot", "opacity", "shs")]
    rng = np.random.default_rng(0)
    choices = [(256, 256), (512, 512), (1280, 720), (1920, 1080)]
    sizes = [choices[i] for i in rng.integers(0, len(choices), cameras)]
    intrs, extrs = [], []
    for w, h in sizes:
        f = 1500.0 * w / 1920.0
        intrs.append([f, f, w / 2, h / 2])
        v = rng.normal(size=3)
        eye = v / np.linalg.norm(v) * 4.0
        fw = -eye / np.linalg.norm(eye)
        r = np.cross(fw, [0.0, 1.0, 0.0])
        r /= np.linalg.norm(r)
        R = np.stack([r, np.cross(fw, r), fw])
        extrs.append(np.concatenate([R, (-R @ eye)[:, None]], 1))
    intrs = torch.tensor(intrs, dtype=torch.float32, device=dev)
    extrs = torch.tensor(np.stack(extrs), dtype=torch.float32, device=dev)
    ws = [torch.randn(3, h, w, device=dev) for w, h in sizes]

    def step():
        for t in p:
            t.grad = None
        imgs = ms.rasterization_sh_batch(*p, intrs, extrs, sizes, 0.0)
        sum((i * w).sum() for i, w in zip(imgs, ws)).backward()

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
    ap.add_argument("--workload", default="frame", choices=["frame", "batch"])
    ap.add_argument("--cameras", type=int, default=16, help="batch workload: cameras per batch")
    ap.add_argument("--params", default="", help="comma-separated subset of the parameters to search")
    ap.add_argument("--time", action="store_true", help="(internal) time the library of this process")
    ap.add_argument("--out", default=_build.TUNING_PATH)
    a = ap.parse_args()
    if a.time:
        if a.workload == "batch":
            print(_time_batch_here(a.gaussians, a.cameras, a.steps, a.warmup))
        else:
            print(_time_here(a.gaussians, a.width, a.height, a.steps, a.warmup))
        return

    tuned = _build.tuned_defines(a.out)
    full_space, defaults = (BATCH_SPACE, BATCH_DEFAULTS) if a.workload == "batch" else (SPACE, DEFAULTS)
    fixed = {k: v for k, v in tuned.items() if k not in full_space}  # the other workload's choices stay
    objective = make_objective(
        lambda setting: variant_library(dict(fixed, **setting)),
        lambda lib: time_variant(lib, a.gaussians, a.width, a.height, a.steps, a.warmup, a.workload, a.cameras),
        log=lambda msg: print(msg, flush=True))
    start = dict(defaults, **{k: v for k, v in tuned.items() if k in full_space})
    space = full_space
    if a.params:
        names = [n.strip() for n in a.params.split(",") if n.strip()]
        unknown = [n for n in names if n not in full_space]
        if unknown:
            raise SystemExit(f"unknown parameters for workload {a.workload}: {unknown}")
        space = {n: full_space[n] for n in names}
    best, best_ms, seen = coordinate_descent(space, start, objective, rounds=a.rounds)
    write_tuning(a.out, a.workload, best, best_ms,
                 {"gaussians": a.gaussians, "width": a.width, "height": a.height, "cameras": a.cameras},
                 [{"defines": dict(k), "ms": round(v, 4)} for k, v in seen.items()])
    print(json.dumps({"workload": a.workload, "defines": best, "ms": round(best_ms, 4)}))


def write_tuning(path: str, workload: str, best: dict, best_ms: float, shape: dict, evaluated: list) -> None:
    """Stores a workload's choice in the tuning file: the frame's under
    "defines" (the single-camera kernels), every other workload's under
    "workloads"[name]["defines"]; the other sections are kept, and so are
    the settings earlier searches of the workload evaluated (a setting timed
    again keeps its new time)."""
    data = {}
    if os.path.exists(path):
        with open(path) as f:
            data = json.load(f)
    before = data.get("evaluated", []) if workload == "frame" else \
        data.get("workloads", {}).get(workload, {}).get("evaluated", [])
    fresh = {json.dumps(e["defines"], sort_keys=True) for e in evaluated}
    evaluated = [e for e in before if json.dumps(e["defines"], sort_keys=True) not in fresh] + list(evaluated)
    if workload == "frame":
        data.update({"defines": best, "ms_per_frame": round(best_ms, 4),
                     "workload": {k: shape[k] for k in ("gaussians", "width", "height")}, "evaluated": evaluated})
    else:
        data.setdefault("workloads", {})[workload] = {"defines": best, "ms": round(best_ms, 4), "workload": shape,
                                                      "evaluated": evaluated}
    with open(path, "w") as f:
        json.dump(data, f, indent=1)


if __name__ == "__main__":
    main()
