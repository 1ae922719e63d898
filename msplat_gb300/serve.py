"""A render server over scenes resident in device memory.

Requests (a scene, a camera, an image size, forward-only or forward +
backward) arrive over time.  The server admits them in arrival order while
the device memory they need fits in a budget (an estimate per request,
checked against the memory the device actually has allocated), and forms
jobs whenever a worker is idle: all admitted forward-only requests (of any
scene, up to max_batch) in one multi-camera, multi-scene call, or all
admitted forward + backward requests (up to max_backward) in one call in
which every request is its own scene (the same resident tensors, separate
autograd leaves), so each request gets its own gradients while the sort and
the blends of all of them run as one batch.  Jobs run on several CUDA
streams from worker threads, so work admitted while other work is on the
GPU overlaps with it.  Memory is returned to the budget as jobs finish.
Every result equals the request served alone: batching evaluates the same
per-camera arithmetic (images bit-identical), and a backward request's
gradients come from its own leaves.

``serve_one_by_one`` serves the same requests one at a time, in arrival
order, on one stream: the baseline for throughput and latency.
"""
from __future__ import annotations

import queue
import threading
import time
from dataclasses import dataclass

import torch

from .batch import rasterization_sh_scenes
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
    per-Gaussian preprocess outputs and sort scratch (keys, ids, the
    rectangle records and the per-row reach records), the intersections
    (about 29 tiles per Gaussian at 1080p and f = 1500, scaling with the
    image area), the image and blend state, and for a backward request the
    per-Gaussian gradients."""
    tiles_per = max(2.0, 29.0 * (W * H) / (1920 * 1080)) * 1.5
    inter = int(P * tiles_per)
    b = P * (44 + 4 * C + 100) + inter * 20 + W * H * (4 * C + 8)
    if backward:
        b += P * (4 * (6 + C) + 4 * (14 + C * D)) + W * H * 4 * C
    return int(b)


class Server:
    def __init__(self, scenes: list, hbm_budget: int, streams: int = 4, max_batch: int = 16, device="cuda",
                 max_backward: int = 8):
        self.scenes = scenes
        self.budget = int(hbm_budget)
        self.max_batch = max_batch
        self.max_backward = max_backward
        self.peak_allocated = 0  # device memory above the resident scenes, peak while serving (bytes)
        self.peak_reserved = 0   # the same for the caching allocator's reserved memory
        dev = torch.device(device)
        self.device = torch.device("cuda", dev.index if dev.index is not None else torch.cuda.current_device())
        self.n_workers = streams
        self._free = self.budget
        self._cv = threading.Condition()

    # ---------------------------------------------------------------- jobs
    def _run_job(self, reqs: list, stream: torch.cuda.Stream) -> None:
        with torch.cuda.stream(stream):
            intrs = torch.stack([r.intr for r in reqs])
            extrs = torch.stack([r.extr for r in reqs])
            sizes = [(r.W, r.H) for r in reqs]
            if reqs[0].backward:
                # every request its own scene: separate leaves, separate gradients
                leaves = [{k: self.scenes[r.scene][k].detach().requires_grad_() for k in PARAMS} for r in reqs]
                imgs = rasterization_sh_scenes([tuple(lv[k] for k in PARAMS) for lv in leaves], range(len(reqs)),
                                               intrs, extrs, sizes, reqs[0].bg)
                loss = sum((img * r.weights).sum() for img, r in zip(imgs, reqs))
                g = torch.autograd.grad(loss, [lv[k] for lv in leaves for k in PARAMS])
                for i, (r, img) in enumerate(zip(reqs, imgs)):
                    r.image, r.grads = img.detach(), dict(zip(PARAMS, g[len(PARAMS) * i:len(PARAMS) * (i + 1)]))
            else:
                used = sorted({r.scene for r in reqs})
                slot = {s: i for i, s in enumerate(used)}
                with torch.no_grad():
                    imgs = rasterization_sh_scenes([tuple(self.scenes[s][k] for k in PARAMS) for s in used],
                                                   [slot[r.scene] for r in reqs], intrs, extrs, sizes, reqs[0].bg)
                for r, img in zip(reqs, imgs):
                    r.image = img
            ev = torch.cuda.Event()
            ev.record(stream)
        ev.synchronize()

    def _device_memory(self):
        """(allocated, reserved) bytes on the server's device."""
        return torch.cuda.memory_allocated(self.device), torch.cuda.memory_reserved(self.device)

    def _worker_stream(self):
        """The CUDA stream of a worker thread (called on that thread)."""
        torch.cuda.set_device(self.device)
        return torch.cuda.Stream(device=self.device)

    def _bytes(self, r: Request) -> int:
        sc = self.scenes[r.scene]
        P, C, D = sc["shs"].shape
        return request_bytes(P, r.W, r.H, C, D, r.backward)

    # -------------------------------------------------------------- serving
    def serve(self, requests: list, timeout: float = 600.0, on_done=None) -> list:
        """Serves `requests` (arrival times relative to now) and returns them
        with image, gradients (backward requests), start and done times.
        on_done(request), when given, is called on the worker thread as each
        request finishes (to hand its results on and release them).

        Arrived requests are admitted in arrival order while their memory
        fits in the budget -- the estimates of the admitted requests, and the
        device memory actually allocated above what it was when serving
        started plus the next request's estimate; a job is formed whenever a
        worker is idle, from the oldest admitted request: all admitted
        backward requests (up to max_backward) if it is one, else all
        admitted forward-only requests (up to max_batch), with its
        background value.  So requests that arrive while the workers are
        busy accumulate into larger multi-camera jobs.  The peak device
        memory above the starting point (allocated and reserved) is kept in
        peak_allocated / peak_reserved.  Raises if a job fails or if serving
        takes longer than `timeout` seconds."""
        order = sorted(requests, key=lambda r: r.arrival)
        need = {id(r): self._bytes(r) for r in order}
        for r in order:
            if need[id(r)] > self.budget:
                raise RuntimeError(f"a request needs {need[id(r)]} bytes, more than the budget {self.budget}")
        jobs: queue.Queue = queue.Queue()
        errors: list = []
        state = {"idle": self.n_workers, "finished": 0}  # (finished: requests done, kept by the workers)
        base_alloc, base_res = self._device_memory()
        self.peak_allocated = self.peak_reserved = 0
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
                        if on_done is not None:
                            on_done(r)
                    done = len(job)
                except Exception as e:  # re-raised by serve()
                    errors.append(e)
                    done = 0
                finally:
                    with self._cv:
                        self._free += sum(need[id(r)] for r in job)
                        state["idle"] += 1
                        state["finished"] += done
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
                    alloc, res = self._device_memory()
                    self.peak_allocated = max(self.peak_allocated, alloc - base_alloc)
                    self.peak_reserved = max(self.peak_reserved, res - base_res)
                    while pending and need[id(pending[0])] <= self._free and (
                            alloc - base_alloc + need[id(pending[0])] <= self.budget or self._free == self.budget):
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
                    finished = state["finished"]
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
        """The oldest ready request's job: every ready request of its kind
        (forward-only, or forward + backward) with its background value,
        oldest first, up to max_batch (forward-only) or max_backward.
        Removes the job's requests from `ready`."""
        head = ready[0]
        cap = self.max_backward if head.backward else self.max_batch
        job = [r for r in ready if r.backward == head.backward and r.bg == head.bg][:cap]
        taken = {id(r) for r in job}
        ready[:] = [r for r in ready if id(r) not in taken]
        return job


def serve_alone(scene: dict, r: Request) -> None:
    """One request through the single-camera call (rasterization_sh), its
    gradients from its own leaves; waits for the result."""
    if r.backward:
        leaves = {k: scene[k].detach().requires_grad_() for k in PARAMS}
        img = rasterization_sh(leaves["xyz"], leaves["scale"], leaves["rot"], leaves["opacity"], leaves["shs"],
                               r.intr, r.extr, r.W, r.H, r.bg)
        g = torch.autograd.grad((img * r.weights).sum(), [leaves[k] for k in PARAMS])
        r.image, r.grads = img.detach(), dict(zip(PARAMS, g))
    else:
        with torch.no_grad():
            r.image = rasterization_sh(scene["xyz"], scene["scale"], scene["rot"], scene["opacity"], scene["shs"],
                                       r.intr, r.extr, r.W, r.H, r.bg)
    torch.cuda.current_stream().synchronize()


def serve_one_by_one(scenes: list, requests: list, device="cuda", on_done=None) -> list:
    """The baseline: each request alone through the single-camera call, in
    arrival order, on one stream, waiting for its arrival; latency includes
    the time spent queued."""
    order = sorted(requests, key=lambda r: r.arrival)
    dev = torch.device(device)
    with torch.cuda.device(dev.index if dev.index is not None else torch.cuda.current_device()):
        t0 = time.perf_counter()
        for r in order:
            now = time.perf_counter() - t0
            if r.arrival > now:
                time.sleep(r.arrival - now)
            r.start, r.batch = time.perf_counter() - t0, 1
            serve_alone(scenes[r.scene], r)
            r.done = time.perf_counter() - t0
            if on_done is not None:
                on_done(r)
    return order
