"""Double-buffered staging of per-step inputs from pinned host memory.

A training or serving loop whose scene parameters (or loss targets) live in
host memory copies them to the device every step.  Done inline, the copy
and the step run one after the other; with `HostStager` the copy of step
k + 1 runs on a separate stream while step k computes:

    stager = HostStager({"xyz": xyz_pinned, ...}, device)
    stager.prefetch(0)
    for k in range(n):
        if k + 1 < n:
            stager.prefetch(k + 1)        # waits until step k - 1 released the slot
        inputs = stager.get(k)            # the current stream waits for the copy
        ... run step k on inputs ...
        stager.release(k)                 # the slot may be overwritten from now on

`get` returns leaf tensors (fresh `.grad` per step is the caller's choice);
`prefetch` optionally takes new host tensors for that step (same shapes).
"""
from __future__ import annotations

import torch


class HostStager:
    def __init__(self, host: dict, device, slots: int = 2):
        for k, v in host.items():
            if not v.is_pinned():
                raise RuntimeError(f"host tensor {k!r} must be in pinned memory")
        self.host = dict(host)
        self.device = torch.device(device)
        self.slots = [{k: torch.empty(v.shape, dtype=v.dtype, device=self.device) for k, v in host.items()}
                      for _ in range(slots)]
        self.copy_stream = torch.cuda.Stream(device=self.device)
        self.copied = [torch.cuda.Event() for _ in range(slots)]
        self.released = [None] * slots

    def _slot(self, step: int) -> int:
        return step % len(self.slots)

    def prefetch(self, step: int, host: dict | None = None) -> None:
        """Enqueues the host->device copy of `step`'s inputs on the copy
        stream, after the compute that last used the slot."""
        s = self._slot(step)
        src = self.host if host is None else host
        with torch.cuda.stream(self.copy_stream), torch.no_grad():
            if self.released[s] is not None:
                self.copy_stream.wait_event(self.released[s])
            for k, dst in self.slots[s].items():
                dst.copy_(src[k], non_blocking=True)
            self.copied[s].record(self.copy_stream)

    def get(self, step: int) -> dict:
        """Device tensors of `step`; the current stream waits for their copy."""
        s = self._slot(step)
        torch.cuda.current_stream(self.device).wait_event(self.copied[s])
        return self.slots[s]

    def release(self, step: int) -> None:
        """Marks the end of the work (on the current stream) that reads the
        slot of `step`."""
        s = self._slot(step)
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream(self.device))
        self.released[s] = ev

    def nbytes(self) -> int:
        return sum(v.numel() * v.element_size() for v in self.host.values())
