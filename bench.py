"""Benchmark: differentiable render (forward + backward) of 1M Gaussians at
1920x1080, colour from SH degree 3, loss = sum(W * image), gradients for
xyz / scales / rotations / opacity / SH / intr / extr.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` is device time per frame with the
scene resident in HBM; `e2e` is the same step through the public API with
the scene and loss weights copied from pinned host memory every step and the
loss read back.  Inputs (236 MB of parameters + 25 MB of loss weights) are
larger than L2, so no explicit flush is done between steps.

`--impl reference` times the reference algorithm on the host CPU (the CPU
oracle port of the reference, all host threads) on a bounded sample of the
same frame: the full projection / covariance / SH / EWA / sort for all
Gaussians plus the forward and backward blend of a band of tile rows, the
band's time scaled to the whole frame.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np
import torch

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fwd+bwd ms/frame @1M Gauss 1080p"
N_GAUSS = 1_000_000
W_IMG, H_IMG = 1920, 1080
FOCAL = 1500.0
SH_DEG = 3


# ------------------------------------------------------------------ scene
def make_scene(seed: int = 0):
    g = torch.Generator().manual_seed(seed)
    n = N_GAUSS
    xyz = torch.rand(n, 3, generator=g) * 2 - 1
    scale = torch.exp(torch.rand(n, 3, generator=g) * 2 - 5)
    rot = torch.randn(n, 4, generator=g)
    rot = rot / rot.norm(dim=-1, keepdim=True)
    opacity = torch.sigmoid(torch.randn(n, 1, generator=g))
    shs = torch.randn(n, 3, (SH_DEG + 1) ** 2, generator=g) * 0.3
    # random look-at camera on a radius-4 sphere (OpenCV: right, down, forward)
    v = torch.randn(3, generator=g, dtype=torch.float64)
    eye = (v / v.norm() * 4.0).numpy()
    f = -eye / np.linalg.norm(eye)
    r = np.cross(f, [0.0, 1.0, 0.0])
    r /= np.linalg.norm(r)
    d = np.cross(f, r)
    R = np.stack([r, d, f])
    extr = torch.tensor(np.concatenate([R, (-R @ eye)[:, None]], 1), dtype=torch.float32)
    intr = torch.tensor([FOCAL, FOCAL, W_IMG / 2, H_IMG / 2], dtype=torch.float32)
    weights = torch.randn(3, H_IMG, W_IMG, generator=g)
    return dict(xyz=xyz, scale=scale, rot=rot, opacity=opacity, shs=shs, intr=intr, extr=extr, weights=weights)


PARAMS = ["xyz", "scale", "rot", "opacity", "shs", "intr", "extr"]


def view_dirs(xyz, extr):
    R, t = extr[:, :3], extr[:, 3]
    cam = -(R.transpose(0, 1) @ t)
    d = xyz - cam
    return d / d.norm(dim=-1, keepdim=True)


def train_step(ms, p, weights):
    """One fwd+bwd frame through the public API (reference call sequence:
    compute_sh -> rasterization -> loss -> backward)."""
    color = ms.compute_sh(p["shs"], view_dirs(p["xyz"], p["extr"]))
    img = ms.rasterization(p["xyz"], p["scale"], p["rot"], p["opacity"], color, p["intr"], p["extr"],
                           W_IMG, H_IMG, 0.0)
    loss = (img * weights).sum()
    loss.backward()
    return loss


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- roofline
def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def fp32_peak_tflops(sm_mhz):
    # 152 SMs x 128 FP32 lanes x 2 flop/FMA at the sampled SM clock (nominal
    # rate; no measured FP32 peak exists for this machine).
    mhz = sm_mhz or 2070.0
    return 152 * 128 * 2 * mhz * 1e6 / 1e12


def blend_pairs(ms, p, color_dim=3):
    """Pixel-Gaussian pairs the forward blend evaluates (sum of ncontrib),
    from one forward on the device outside the timed region."""
    from msplat_gb300 import _lib
    with torch.no_grad():
        uv, depth = ms.project_point(p["xyz"], p["intr"], p["extr"], W_IMG, H_IMG)
        vis = depth != 0
        cov = ms.compute_cov3d(p["scale"], p["rot"], vis)
        conic, radius, tiles = ms.ewa_project(p["xyz"], cov, p["intr"], p["extr"], uv, W_IMG, H_IMG, vis)
        idx, tr = ms.sort_gaussian(uv, depth, W_IMG, H_IMG, radius, tiles)
        col = torch.ones(p["xyz"].shape[0], color_dim, device=uv.device)
        lib = _lib.load()
        out = torch.empty(color_dim, H_IMG, W_IMG, device=uv.device)
        T = torch.empty(H_IMG, W_IMG, device=uv.device)
        nc = torch.empty(H_IMG, W_IMG, dtype=torch.int32, device=uv.device)
        _lib.check(lib.msplat_alpha_blending_forward(
            p["xyz"].shape[0], color_dim, uv.data_ptr(), conic.data_ptr(), p["opacity"].data_ptr(),
            col.data_ptr(), idx.data_ptr(), tr.data_ptr(), 0.0, W_IMG, H_IMG, out.data_ptr(), T.data_ptr(),
            nc.data_ptr(), _lib.stream()), "blend")
        torch.cuda.synchronize()
        return int(nc.sum().item()), int(idx.numel()), int((radius > 0).sum().item())


def roofline(stages, steps, pairs, inter, nvis, sm_mhz, peaks, peak_kind):
    """Roofline entry for the stage with the largest share of the step."""
    name, (calls, total) = max(stages.items(), key=lambda kv: kv[1][1])
    per_launch_ms = total / max(calls, 1)
    C = 3
    if name.startswith("alpha_blending"):
        fl = (12 + 2 * C) if name.endswith("forward") else (30 + 8 * C)
        flops = pairs * (fl + 1)  # + one exponential per pair
        ach = flops / (per_launch_ms * 1e-3) / 1e12
        peak = fp32_peak_tflops(sm_mhz)
        return name, {"bound": "fp32", "achieved": round(ach, 3), "peak": round(peak, 2), "unit": "TFLOP/s",
                      "frac": round(ach / peak, 4), "traffic": None,
                      "peak_source": "nominal FP32 lanes x sampled SM clock (not measured)",
                      "kernel": name, "per_launch_ms": round(per_launch_ms, 4)}
    bytes_per = {
        "sort_gaussian_finish": inter * 52.0,
        "sort_gaussian_prepare": N_GAUSS * 100.0,
        "compute_sh_forward": N_GAUSS * (4 * 3 * 16 + 12 + 1 + 12),
        "compute_sh_backward": N_GAUSS * (2 * 4 * 3 * 16 + 12 + 12 + 12 + 1),
        "ewa_project_forward": N_GAUSS * 65.0,
        "ewa_project_backward": N_GAUSS * 88.0,
        "compute_cov3d_forward": N_GAUSS * 53.0,
        "compute_cov3d_backward": N_GAUSS * 81.0,
        "project_point_forward": N_GAUSS * 24.0,
        "project_point_backward": N_GAUSS * 48.0,
    }.get(name, 0.0)
    ach = bytes_per / (per_launch_ms * 1e-3) / 1e9
    peak = peaks.get("hbm_gbs", 6800.0)
    return name, {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                  "frac": round(ach / peak, 4), "traffic": None, "peak_source": peak_kind,
                  "kernel": name, "per_launch_ms": round(per_launch_ms, 4)}


# ------------------------------------------------------------- our arm
def run_ours(args, rank, world, device):
    import msplat_gb300 as ms
    from msplat_gb300 import _lib

    scene = make_scene(seed=rank)
    p = {k: scene[k].to(device).contiguous().requires_grad_() for k in PARAMS}
    weights = scene["weights"].to(device)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        for t in p.values():
            t.grad = None
        train_step(ms, p, weights)
    barrier()

    clocks = ClockSampler(torch.cuda.current_device() if "CUDA_VISIBLE_DEVICES" not in os.environ
                          else int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    _lib.profile_start()
    barrier()
    ev0.record(stream)
    for _ in range(args.steps):
        for t in p.values():
            t.grad = None
        train_step(ms, p, weights)
    ev1.record(stream)
    barrier()
    stages = _lib.profile_stop()
    clk = clocks.stop()
    ms_step = ev0.elapsed_time(ev1) / args.steps
    t = torch.tensor([ms_step], device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    ms_step = float(t.item())

    # e2e: the same step with host inputs copied in and the loss read back.
    if args.no_e2e:
        return _finish(args, rank, world, ms, p, stages, clk, ms_step, None, 0)
    host = {k: scene[k].pin_memory() for k in PARAMS}
    host_w = scene["weights"].pin_memory()
    h2d = sum(v.numel() * v.element_size() for v in host.values()) + host_w.numel() * host_w.element_size()
    for _ in range(max(1, args.warmup // 2)):
        pe = {k: v.to(device, non_blocking=True).requires_grad_() for k, v in host.items()}
        train_step(ms, pe, host_w.to(device, non_blocking=True)).item()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        pe = {k: v.to(device, non_blocking=True).requires_grad_() for k, v in host.items()}
        loss = train_step(ms, pe, host_w.to(device, non_blocking=True))
        loss.item()
    e1.record(stream)
    barrier()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    t = torch.tensor([e2e_ms], device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    e2e_ms = float(t.item())
    return _finish(args, rank, world, ms, p, stages, clk, ms_step, e2e_ms, h2d)


def _finish(args, rank, world, ms, p, stages, clk, ms_step, e2e_ms, h2d):
    if rank != 0:
        return None
    pairs, inter, nvis = blend_pairs(ms, p)
    peaks, peak_kind = measured_peaks()
    dom, roof = roofline(stages, args.steps, pairs, inter, nvis, clk.get("sm_mhz"), peaks, peak_kind)
    stage_ms = {k: round(v[1] / args.steps, 4) for k, v in sorted(stages.items(), key=lambda kv: -kv[1][1])}
    out = {
        "metric": METRIC,
        "value": round(ms_step / world, 4),
        "unit": "ms/frame",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_step, 4),
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded; config distributions, random look-at camera on a radius-4 sphere)",
        "config": {"workload": "1M Gaussians, 1920x1080, SH deg 3, fwd+bwd, loss sum(W*img)",
                   "n_gaussians": N_GAUSS, "width": W_IMG, "height": H_IMG, "sh_degree": SH_DEG,
                   "focal": FOCAL, "intersections": inter, "visible_gaussians": nvis, "blend_pairs": pairs,
                   "parallelism": "replicas" if world > 1 else "single",
                   "l2": "inputs (261 MB) larger than L2; no flush"},
        "e2e": None if e2e_ms is None else {"value": round(e2e_ms / world, 4), "unit": "ms/frame",
                                            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": 4},
        "gpu_launches": None,
        "stage_ms_per_step": stage_ms,
        "roofline": roof,
        "clocks": clk,
    }
    out["gpu_launches"] = int(launches_per_step(stages, args.steps) * args.steps)
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(threads=1)
    return out


# Native kernels each native call launches (counted from the C sources).
KERNELS_PER_CALL = {
    "project_point_forward": 1, "project_point_backward": 2, "compute_cov3d_forward": 1,
    "compute_cov3d_backward": 1, "compute_sh_forward": 1, "compute_sh_backward": 1,
    "ewa_project_forward": 1, "ewa_project_backward": 2, "sort_gaussian_prepare": 1 + 4 * 3 + 1 + 3,
    "sort_gaussian_finish": 1 + 2 * 3 + 1, "alpha_blending_forward": 1, "alpha_blending_backward": 1,
}


def launches_per_step(stages, steps):
    return sum(KERNELS_PER_CALL.get(k, 1) * c for k, (c, _) in stages.items()) / steps


# ------------------------------------------------------------- CPU (oracle)
def cpu_frame(scene, band_rows=8, threads=1):
    """Wall time of one frame of the reference algorithm on the CPU oracle,
    with the blend measured on `band_rows` tile rows and scaled."""
    import oracle
    os.environ["OMP_NUM_THREADS"] = str(threads)
    s = {k: v.numpy() for k, v in scene.items()}
    W, H = W_IMG, H_IMG
    t0 = time.perf_counter()
    dirs = s["xyz"] - (-(s["extr"][:, :3].T @ s["extr"][:, 3]))
    dirs = (dirs / np.linalg.norm(dirs, axis=1, keepdims=True)).astype(np.float32)
    color = oracle.compute_sh_forward(s["shs"], dirs).astype(np.float32)
    uv, depth = oracle.project_point_forward(s["xyz"], s["intr"], s["extr"], W, H)
    vis = (depth != 0).reshape(-1)
    cov = oracle.compute_cov3d_forward(s["scale"], s["rot"], vis)
    conic, radius, tiles, _ = oracle.ewa_project_forward(s["xyz"], cov, s["intr"], s["extr"], uv, W, H, vis)
    idx, tr = oracle.sort_gaussian(uv, depth, W, H, radius, tiles)
    t_pre = time.perf_counter() - t0
    # band of tile rows in the middle of the image
    gx, gy = (W + 15) // 16, (H + 15) // 16
    r0 = gy // 2 - band_rows // 2
    h = band_rows * 16
    uvb = uv.copy()
    uvb[:, 1] -= r0 * 16
    trb = tr.reshape(gy, gx, 2)[r0:r0 + band_rows].reshape(-1, 2)
    wb = s["weights"][:, r0 * 16:r0 * 16 + h]
    t1 = time.perf_counter()
    out, T, nc, _ = oracle.alpha_blending_forward(uvb, conic, s["opacity"], color, idx, trb, 0.0, W, h)
    grads = oracle.alpha_blending_backward(uvb, conic, s["opacity"], color, idx, trb, 0.0, W, h, T, nc, wb)
    t_blend = (time.perf_counter() - t1) * gy / band_rows
    t2 = time.perf_counter()
    duv, dcon, dop, dcol = grads
    dcol = dcol.astype(np.float32)
    oracle.ewa_project_backward(s["xyz"], cov, s["intr"], s["extr"], radius, dcon.astype(np.float32))
    oracle.compute_cov3d_backward(s["scale"], s["rot"], vis, np.zeros_like(cov))
    oracle.project_point_backward(s["xyz"], s["intr"], s["extr"], depth, duv.astype(np.float32),
                                  np.zeros_like(depth))
    oracle.compute_sh_backward(s["shs"], dirs, None, dcol)
    t_post = time.perf_counter() - t2
    return (t_pre + t_blend + t_post) * 1e3, band_rows, gy


def cpu_baseline(threads=1):
    scene = make_scene(0)
    ms_frame, band, gy = cpu_frame(scene, threads=threads)
    return {"value": round(ms_frame, 1), "unit": "ms/frame", "cores": threads, "kind": "port",
            "sample": f"all 1M Gaussians through projection/cov3d/SH/EWA/sort and their adjoints; blend fwd+bwd "
                      f"on {band} of {gy} tile rows (1920x{band * 16} band), scaled to the frame"}


# ------------------------------------------------------------- reference arm
def run_reference(args):
    threads = os.cpu_count() or 1
    base = cpu_baseline(threads=threads)
    return {
        "impl": "reference", "metric": METRIC, "value": base["value"], "unit": "ms/frame", "n_gpus": args.gpus,
        "steps": 1, "warmup": 0, "ms_per_step": base["value"], "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": "1M Gaussians, 1920x1080, SH deg 3, fwd+bwd, loss sum(W*img)"},
        "cpu_baseline": base,
        "e2e": {"value": base["value"], "unit": "ms/frame", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer (e2e) loop")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)), flush=True)
        return
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    if world > 1:
        torch.distributed.init_process_group("nccl", device_id=device)
    from msplat_gb300 import _build
    _build.build()
    out = run_ours(args, rank, world, device)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
