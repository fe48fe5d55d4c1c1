"""The allocation-free root half-width (ag2_root_radius_noalloc) against the
context path (ag2_build_tree + ag2_root_radius), called through the C-ABI.

Callers that cannot allocate device memory (a host code that has reserved the
GPU's memory for its own pools, or code capturing a CUDA stream) hand in their
own device buffers; the entry point's scratch is a fixed array inside the
library.  Two calls in a row must both reproduce the context path bit for bit,
and sizes beyond the stated maximum must be refused without a launch.

The sizes cover each path of the entry point:
  1, 3000, 4096  one sequential sum over all particles (n <= 4096), as the
                 context path sums up to that size;
  4097, 100000   the first size past that boundary, and a 64-ary sum tree
                 whose second level (one pair per 4096 particles, 1 and 25
                 entries) the final kernel adds in one run;
  300000         74 second-level entries: the final kernel reduces in place
                 over two levels (runs of 64, then the two run sums);
  8355840        the largest accepted size (2040 entries, the whole scratch).
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu

MAX_N = 8355840  # AG2_NOALLOC_MAX_PARTICLES


@pytest.mark.parametrize("n", [1, 3000, 4096, 4097, 100000, 300000, MAX_N])
def test_noalloc_root_radius_matches_context_path(n):
    import torch

    import ag2
    import build
    import ics

    build.build()
    L = ag2.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    d = ics.plummer(n, seed=21)
    c = ag2.Context(n)
    c.upload(d["pos"], d["mass"], d["type"])
    c.build_tree()
    want = c.root_radius()
    c.close()
    pos = torch.tensor(d["pos"], dtype=torch.float64, device="cuda").contiguous()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    for _ in range(2):  # the second call starts from the scratch the first one left
        out.fill_(-1.0)
        rc = L.ag2_root_radius_noalloc(ctypes.c_void_p(pos.data_ptr()), n, ctypes.c_void_p(out.data_ptr()), stream)
        assert rc == ag2.OK
        torch.cuda.synchronize()
        assert out.item() == want
    del pos
    torch.cuda.empty_cache()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch

    import ag2
    import build

    build.build()
    L = ag2.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    pos = torch.zeros(3, dtype=torch.float64, device="cuda")
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    rc = L.ag2_root_radius_noalloc(ctypes.c_void_p(pos.data_ptr()), MAX_N + 1, ctypes.c_void_p(out.data_ptr()),
                                   stream)
    assert rc == ag2.E_CAPACITY
    rc = L.ag2_root_radius_noalloc(ctypes.c_void_p(pos.data_ptr()), 0, ctypes.c_void_p(out.data_ptr()), stream)
    assert rc == ag2.E_INVALID
    torch.cuda.synchronize()
    assert out.item() == -1.0  # nothing was launched
