"""A render server over scenes resident in device memory.

Requests (a scene, a camera, an image size, forward-only or forward +
backward) arrive over time.  The server admits them in arrival order while
the device memory they need fits in a budget, groups admitted forward-only
requests of the same scene into one multi-camera call
(``rasterization_sh_batch``), runs each forward + backward request on its
own (its gradients are its own), and executes the jobs on several CUDA
streams from worker threads, so work admitted while other work is on the
GPU overlaps with it.  Memory is returned to the budget as jobs finish.
Every result equals the request served alone: batching evaluates the same
per-camera arithmetic (images bit-identical), and a backward request's
gradients come from its own graph.

``serve_one_by_one`` serves the same requests one at a time, in arrival
order, on one stream: the baseline for throughput and latency.
"""
from __future__ import annotations

import queue
import threading
import time
from dataclasses import dataclass

import torch

from .batch import rasterization_sh_batch
from .rasterize import rasterization_sh

PARAMS = ("xyz", "scale", "rot", "opacity", "shs")


@dataclass
class Request:
    scene: int
    intr: torch.Tensor          # [4] fx, fy, cx, cy
    extr: torch.Tensor          # [3, 4] world-to-camera
    W: int
    H: int
    backward: bool = False
    weights: torch.Tensor | None = None  # [C, H, W]: loss = sum(weights * image) for backward requests
    arrival: float = 0.0        # seconds after the start of serving
    bg: float = 0.0
    # results
    image: torch.Tensor | None = None
    grads: dict | None = None
    start: float | None = None
    done: float | None = None
    batch: int = 0              # size of the job it ran in

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def request_bytes(P: int, W: int, H: int, C: int, D: int, backward: bool) -> int:
    """Device memory a request may hold while it runs (an upper estimate):
    per-Gaussian preprocess outputs and sort scratch, the intersections
    (about 29 tiles per Gaussian at 1080p and f = 1500, scaling with the
    image area), the image and blend state, and for a backward request the
    per-Gaussian gradients."""
    tiles_per = max(2.0, 29.0 * (W * H) / (1920 * 1080)) * 1.5
    inter = int(P * tiles_per)
    b = P * (44 + 4 * C + 48) + inter * 20 + W * H * (4 * C + 8)
    if backward:
        b += P * (4 * (6 + C) + 4 * (14 + C * D)) + W * H * 4 * C
    return int(b)


class Server:
    def __init__(self, scenes: list, hbm_budget: int, streams: int = 4, max_batch: int = 16, device="cuda"):
        self.scenes = scenes
        self.budget = int(hbm_budget)
        self.max_batch = max_batch
        dev = torch.device(device)
        self.device = torch.device("cuda", dev.index if dev.index is not None else torch.cuda.current_device())
        self.n_workers = streams
        self._free = self.budget
        self._cv = threading.Condition()

    # ---------------------------------------------------------------- jobs
    def _run_job(self, reqs: list, stream: torch.cuda.Stream) -> None:
        sc = self.scenes[reqs[0].scene]
        with torch.cuda.stream(stream):
            if reqs[0].backward:
                r = reqs[0]
                leaves = {k: sc[k].detach().requires_grad_() for k in PARAMS}
                img = rasterization_sh(leaves["xyz"], leaves["scale"], leaves["rot"], leaves["opacity"],
                                       leaves["shs"], r.intr, r.extr, r.W, r.H, r.bg)
                loss = (img * r.weights).sum()
                g = torch.autograd.grad(loss, [leaves[k] for k in PARAMS])
                r.image, r.grads = img.detach(), dict(zip(PARAMS, g))
            else:
                intrs = torch.stack([r.intr for r in reqs])
                extrs = torch.stack([r.extr for r in reqs])
                with torch.no_grad():
                    imgs = rasterization_sh_batch(sc["xyz"], sc["scale"], sc["rot"], sc["opacity"], sc["shs"],
                                                  intrs, extrs, [(r.W, r.H) for r in reqs], reqs[0].bg)
                for r, img in zip(reqs, imgs):
                    r.image = img
            ev = torch.cuda.Event()
            ev.record(stream)
        ev.synchronize()

    def _worker_stream(self):
        """The CUDA stream of a worker thread (called on that thread)."""
        torch.cuda.set_device(self.device)
        return torch.cuda.Stream(device=self.device)

    def _bytes(self, r: Request) -> int:
        sc = self.scenes[r.scene]
        P, C, D = sc["shs"].shape
        return request_bytes(P, r.W, r.H, C, D, r.backward)

    # -------------------------------------------------------------- serving
    def serve(self, requests: list, timeout: float = 600.0) -> list:
        """Serves `requests` (arrival times relative to now) and returns them
        with image, gradients (backward requests), start and done times.

        Arrived requests are admitted in arrival order while their memory
        fits in the budget; a job is formed whenever a worker is idle, from
        the oldest admitted request: a backward request alone, or all
        admitted forward-only requests of its scene (up to max_batch).  So
        requests that arrive while the workers are busy accumulate into
        larger multi-camera jobs.  Raises if a job fails or if serving takes
        longer than `timeout` seconds."""
        order = sorted(requests, key=lambda r: r.arrival)
        need = {id(r): self._bytes(r) for r in order}
        for r in order:
            if need[id(r)] > self.budget:
                raise RuntimeError(f"a request needs {need[id(r)]} bytes, more than the budget {self.budget}")
        jobs: queue.Queue = queue.Queue()
        errors: list = []
        state = {"idle": self.n_workers}
        t0 = time.perf_counter()

        def worker():
            try:
                stream = self._worker_stream()
            except Exception as e:  # re-raised by serve()
                errors.append(e)
                return
            while True:
                job = jobs.get()
                if job is None:
                    return
                try:
                    now = time.perf_counter() - t0
                    for r in job:
                        r.start, r.batch = now, len(job)
                    self._run_job(job, stream)
                    now = time.perf_counter() - t0
                    for r in job:
                        r.done = now
                except Exception as e:  # re-raised by serve()
                    errors.append(e)
                finally:
                    with self._cv:
                        self._free += sum(need[id(r)] for r in job)
                        state["idle"] += 1
                        self._cv.notify_all()

        threads = [threading.Thread(target=worker, daemon=True) for _ in range(self.n_workers)]
        for t in threads:
            t.start()
        pending: list = []   # arrived, waiting for memory
        ready: list = []     # admitted, waiting for a worker
        nxt = finished = 0
        try:
            while finished < len(order):
                now = time.perf_counter() - t0
                while nxt < len(order) and order[nxt].arrival <= now:
                    pending.append(order[nxt])
                    nxt += 1
                with self._cv:
                    while pending and need[id(pending[0])] <= self._free:
                        r = pending.pop(0)
                        self._free -= need[id(r)]
                        ready.append(r)
                    dispatched = False
                    while state["idle"] > 0 and ready:
                        job = self._take_job(ready)
                        state["idle"] -= 1
                        jobs.put(job)
                        dispatched = True
                    if errors:
                        break
                    if time.perf_counter() - t0 > timeout:
                        errors.append(RuntimeError(f"serving did not finish within {timeout} s"))
                        break
                    finished = sum(1 for r in order if r.done is not None)
                    if not dispatched and finished < len(order):
                        wait = 0.002 if nxt >= len(order) else min(0.002, max(0.0, order[nxt].arrival - now))
                        self._cv.wait(timeout=wait)
        finally:
            for _ in threads:
                jobs.put(None)
            for t in threads:
                t.join()
        if errors:
            raise errors[0]
        return order

    def _take_job(self, ready: list) -> list:
        """The oldest ready request's job: itself if it is a backward
        request, else every ready forward-only request of its scene (oldest
        first, up to max_batch).  Removes the job's requests from `ready`."""
        head = ready[0]
        if head.backward:
            return [ready.pop(0)]
        job = [r for r in ready if not r.backward and r.scene == head.scene][:self.max_batch]
        taken = {id(r) for r in job}
        ready[:] = [r for r in ready if id(r) not in taken]
        return job


def serve_one_by_one(scenes: list, requests: list, device="cuda") -> list:
    """The baseline: each request alone, in arrival order, on one stream,
    waiting for its arrival; latency includes the time spent queued."""
    order = sorted(requests, key=lambda r: r.arrival)
    srv = Server(scenes, hbm_budget=1 << 62, streams=1, device=device)
    stream = torch.cuda.current_stream(srv.device)
    t0 = time.perf_counter()
    for r in order:
        now = time.perf_counter() - t0
        if r.arrival > now:
            time.sleep(r.arrival - now)
        r.start, r.batch = time.perf_counter() - t0, 1
        srv._run_job([r], stream)
        r.done = time.perf_counter() - t0
    return order
