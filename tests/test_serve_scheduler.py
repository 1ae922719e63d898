"""The server's scheduling on CPU, with simulated jobs: every request is
served once, admitted memory never exceeds the budget (the estimates and
the simulated device memory), forward-only requests are batched (up to
max_batch, any scene), backward requests are batched among themselves (up
to max_backward), and a failing job surfaces as an exception instead of a
hang."""
import threading
import time

import pytest
import torch




def make(budget, streams, max_batch, job_time=0.004, fail=False, max_backward=3):
    from msplat_gb300.serve import Server

    class Sim(Server):
        def __init__(self):
            super().__init__([{"shs": torch.zeros(1000, 3, 16)} for _ in range(3)], budget, streams, max_batch,
                             device="cuda:0", max_backward=max_backward)
            self.lock = threading.Lock()
            self.in_use = 0
            self.peak = 0
            self.jobs = []

        def _worker_stream(self):
            return None

        def _device_memory(self):
            with self.lock:
                return self.in_use, self.in_use

        def _bytes(self, r):
            return 100 if r.backward else 60

        def _run_job(self, reqs, stream):
            if fail:
                raise ValueError("simulated job failure")
            with self.lock:
                self.in_use += sum(self._bytes(r) for r in reqs)
                self.peak = max(self.peak, self.in_use)
                self.jobs.append([(r.scene, r.backward) for r in reqs])
            time.sleep(job_time)
            for r in reqs:
                r.image = torch.zeros(1)
            with self.lock:
                self.in_use -= sum(self._bytes(r) for r in reqs)

    return Sim()


def reqs(n, seed=0):
    import numpy as np
    from msplat_gb300.serve import Request
    rng = np.random.default_rng(seed)
    return [Request(scene=int(rng.integers(3)), intr=None, extr=None, W=8, H=8, backward=bool(rng.random() < 0.2),
                    arrival=float(rng.uniform(0, 0.05))) for _ in range(n)]


@pytest.mark.timeout(60)
def test_every_request_served_within_budget_and_batched():
    srv = make(budget=600, streams=3, max_batch=4)
    rs = reqs(120)
    done = []
    out = srv.serve(rs, timeout=30, on_done=done.append)
    assert len(out) == 120 and all(r.done is not None and r.done >= r.arrival for r in out)
    assert sorted(map(id, done)) == sorted(map(id, rs))
    assert srv.peak <= 600 and srv.peak_allocated <= 600
    for job in srv.jobs:
        kinds = {b for _, b in job}
        assert len(kinds) == 1  # forward-only and backward requests never share a job
        assert len(job) <= (3 if kinds == {True} else 4)
    assert max(len(j) for j in srv.jobs if not j[0][1]) > 1
    assert max(len(j) for j in srv.jobs if j[0][1]) > 1
    assert sum(len(j) for j in srv.jobs) == 120


@pytest.mark.timeout(60)
def test_failing_job_raises():
    srv = make(budget=600, streams=2, max_batch=4, fail=True)
    with pytest.raises(ValueError, match="simulated"):
        srv.serve(reqs(10), timeout=30)


@pytest.mark.timeout(60)
def test_oversized_request_is_rejected():
    srv = make(budget=50, streams=1, max_batch=1)
    with pytest.raises(RuntimeError, match="budget"):
        srv.serve(reqs(3), timeout=5)
