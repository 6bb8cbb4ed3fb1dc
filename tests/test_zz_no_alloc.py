"""lsdtt_gpu_fill_pits_noalloc -- the fill for callers that must not have
the library allocate device memory (a framework that has reserved the device
for its own allocator, or a latency-critical loop).

Called through the C ABI, twice in a row on different surfaces (the fixed
scratch array keeps the previous call's contents, so the second call checks
that everything that must start from a known state is reset), and compared
with the allocating entry point lsdtt_gpu_fill_pits. Both run the same
kernels, so the tolerance is zero: identical bits. Also checks that a grid
larger than the fixed scratch is refused with a clear message, and that a
call on a capturing stream is refused before it enqueues anything.

Named test_zz_* so pytest collects it after every other test file; it also
passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from tests import surfaces

pytestmark = pytest.mark.gpu


def _abi():
    import lsdtt_gb300 as G
    L = G.lib()
    f = L.lsdtt_gpu_fill_pits_noalloc
    f.argtypes = [ctypes.POINTER(G.Grid), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float, ctypes.c_void_p,
                  ctypes.c_void_p]
    f.restype = ctypes.c_int
    return G, L


def _run(G, L, fn, z, m, cell, bc, eps):
    import torch
    zt = torch.from_numpy(np.ascontiguousarray(z)).cuda()
    mt = torch.from_numpy(np.ascontiguousarray(m)).cuda()
    out = torch.full_like(zt, float("nan"))
    g = G.make_grid(z.shape[0], z.shape[1], cell, bc)
    st = fn(ctypes.byref(g), ctypes.c_void_p(zt.data_ptr()), ctypes.c_void_p(mt.data_ptr()), ctypes.c_float(eps),
            ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return st, out.cpu().numpy()


def test_noalloc_fill_matches_allocating_fill_twice_in_a_row():
    import torch
    G, L = _abi()
    rng = np.random.default_rng(5)
    z1 = surfaces.fractal_pits(512)
    m1 = np.ones_like(z1, np.uint8)
    z2 = surfaces.fractal(300, 420, 200.0, 9)
    m2 = (rng.random(z2.shape) > 0.02).astype(np.uint8)
    z2[m2 == 0] = -9999.0
    for z, m, cell, bc, eps in ((z1, m1, 10.0, "oooo", 1e-4), (z2, m2, 5.0, "popo", 1e-4)):
        st_a, want = _run(G, L, L.lsdtt_gpu_fill_pits, z, m, cell, bc, eps)
        st_b, got = _run(G, L, L.lsdtt_gpu_fill_pits_noalloc, z, m, cell, bc, eps)
        assert st_a == 0 and st_b == 0, G.lib().lsdtt_gpu_last_error()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    torch.cuda.synchronize()


def test_noalloc_fill_refuses_grids_beyond_its_scratch():
    G, L = _abi()
    import torch
    n_rows, n_cols = 4200, 4200
    zt = torch.zeros((n_rows, n_cols), dtype=torch.float32, device="cuda")
    mt = torch.ones((n_rows, n_cols), dtype=torch.uint8, device="cuda")
    g = G.make_grid(n_rows, n_cols, 10.0, "oooo")
    st = L.lsdtt_gpu_fill_pits_noalloc(ctypes.byref(g), ctypes.c_void_p(zt.data_ptr()),
                                       ctypes.c_void_p(mt.data_ptr()), ctypes.c_float(1e-4),
                                       ctypes.c_void_p(zt.data_ptr()), None)
    assert st == G.EINVAL
    assert b"fixed scratch" in L.lsdtt_gpu_last_error()


def test_noalloc_fill_refuses_a_capturing_stream():
    """The call reads flags back to the host between passes, so it cannot be
    captured: on a stream that is capturing it returns EINVAL before it
    enqueues anything, and the capture stays valid."""
    G, L = _abi()
    import torch
    z = surfaces.fractal_pits(128)
    zt = torch.from_numpy(z).cuda()
    mt = torch.ones_like(zt, dtype=torch.uint8)
    out = torch.empty_like(zt)
    g = G.make_grid(128, 128, 10.0, "oooo")
    s = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(graph, stream=s):
        st = L.lsdtt_gpu_fill_pits_noalloc(ctypes.byref(g), ctypes.c_void_p(zt.data_ptr()),
                                           ctypes.c_void_p(mt.data_ptr()), ctypes.c_float(1e-4),
                                           ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(s.cuda_stream))
        out.add_(0.0)  # something for the capture to hold
    assert st == G.EINVAL
    assert b"capturing" in L.lsdtt_gpu_last_error()
    graph.replay()
    torch.cuda.synchronize()
