"""The allocation-free root half-width (ag2_root_radius_noalloc) against the
context path (ag2_build_tree + ag2_root_radius), called through the C-ABI.

Callers that cannot allocate device memory (a host code that has reserved the
GPU's memory for its own pools, or code capturing a CUDA stream) hand in their
own device buffers; the entry point's scratch is a fixed array inside the
library.  Two calls in a row must both reproduce the context path bit for bit,
and sizes beyond the stated maximum must be refused without a launch."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_root_radius_matches_context_path():
    import torch

    import ag2
    import build
    import ics

    build.build()
    L = ag2.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for n in (5000, 100000):  # sequential sums, then per-block partial sums
        d = ics.plummer(n, seed=21)
        c = ag2.Context(n)
        c.upload(d["pos"], d["mass"], d["type"])
        c.build_tree()
        want = c.root_radius()
        c.close()
        pos = torch.tensor(d["pos"], dtype=torch.float64, device="cuda").contiguous()
        out = torch.zeros(1, dtype=torch.float64, device="cuda")
        for _ in range(2):
            out.fill_(-1.0)
            rc = L.ag2_root_radius_noalloc(ctypes.c_void_p(pos.data_ptr()), n, ctypes.c_void_p(out.data_ptr()),
                                           stream)
            assert rc == ag2.OK
            torch.cuda.synchronize()
            assert out.item() == want
    rc = L.ag2_root_radius_noalloc(ctypes.c_void_p(pos.data_ptr()), 8355840 + 1, ctypes.c_void_p(out.data_ptr()),
                                   stream)
    assert rc == ag2.E_CAPACITY
