"""HostStager: each step sees exactly its own host inputs although the copy
of the next step overlaps the current step's work."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_each_step_sees_its_own_inputs():
    from msplat_gb300.pipeline import HostStager
    n = 6
    hosts = [{"a": torch.full((1 << 20,), float(k)).pin_memory(), "b": (torch.arange(7.0) * k).pin_memory()}
             for k in range(n)]
    st = HostStager(hosts[0], "cuda")
    out = torch.empty(n, 2, device="cuda")
    st.prefetch(0, hosts[0])
    for k in range(n):
        if k + 1 < n:
            st.prefetch(k + 1, hosts[k + 1])
        d = st.get(k)
        # a long kernel chain on the slot so the next copy would overrun an
        # unguarded buffer
        x = d["a"]
        for _ in range(20):
            x = x * 1.0 + 0.0
        out[k, 0] = x.mean()
        out[k, 1] = d["b"].sum()
        st.release(k)
    torch.cuda.synchronize()
    for k in range(n):
        assert out[k, 0].item() == float(k)
        assert out[k, 1].item() == 21.0 * k


def test_rejects_pageable_memory():
    from msplat_gb300.pipeline import HostStager
    with pytest.raises(RuntimeError, match="pinned"):
        HostStager({"a": torch.zeros(4)}, "cuda")
