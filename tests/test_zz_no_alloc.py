"""Allocation-free filter entry point (collected last on purpose).

Some callers of this library cannot allocate device memory at call time:
their device heap belongs to a pool they reserved at start-up, or the call
sits on a latency-critical path where a cudaMalloc/cudaFree pair (which may
synchronize the device) is not acceptable.  gbpt_bilateral_noalloc() serves
them: it runs the same bilateral filter as gbpt_bilateral() on device arrays
but keeps its weight table in a file-scope device array.  This test drives
both through the C ABI on identical device inputs and requires identical
bits, on two calls in a row with different radii and inputs (the second
call must not see anything left over from the first).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class _Dev:
    """Minimal device buffers through the CUDA runtime already loaded by libgbpt.so."""

    def __init__(self):
        self.rt = ctypes.CDLL("libcudart.so.13")
        self.bufs = []

    def put(self, a):
        a = np.ascontiguousarray(a, np.float32)
        p = ctypes.c_void_p()
        assert self.rt.cudaMalloc(ctypes.byref(p), ctypes.c_size_t(max(a.nbytes, 4))) == 0
        assert self.rt.cudaMemcpy(p, a.ctypes.data, ctypes.c_size_t(a.nbytes), 1) == 0
        self.bufs.append(p)
        return p

    def get(self, p, n):
        out = np.zeros(n, np.float32)
        assert self.rt.cudaMemcpy(out.ctypes.data, p, ctypes.c_size_t(out.nbytes), 2) == 0
        return out

    def free(self):
        for p in self.bufs:
            self.rt.cudaFree(p)
        self.bufs = []


def test_noalloc_matches_allocating_entry_point(gbdev):
    L = gbdev._native.load()
    ck = gbdev._native.check
    dev = _Dev()
    try:
        rng = np.random.Generator(np.random.PCG64(77))
        for call, (W, H, radius, emit, delta) in enumerate(((53, 37, 5, True, 50.0), (64, 48, 2, False, 1.5))):
            planes = [dev.put(rng.random(W * H * 3)) for _ in range(4)]
            out_ref = dev.put(np.zeros(W * H * 3))
            out_new = dev.put(np.full(W * H * 3, np.nan))
            g = np.zeros(64, np.float32)
            ck(L.gbpt_gaussian_table(delta, radius, g.ctypes.data))
            e = planes[3] if emit else None
            args = (planes[0], planes[1], planes[2], e, W, H, 0.5, 1.0, 0.25, 0.1, radius, g.ctypes.data)
            ck(L.gbpt_bilateral(*args, out_ref, 1))
            ck(L.gbpt_bilateral_noalloc(*args, out_new, None))
            a = dev.get(out_ref, W * H * 3)
            b = dev.get(out_new, W * H * 3)
            assert np.isfinite(a).all()
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), f"call {call}"
        # sizes beyond the 64-entry table are refused on the host, including radii
        # whose 2*radius+1 wraps around in 32-bit arithmetic
        for bad in (32, 0x80000000, 0xFFFFFFFF):
            with pytest.raises(gbdev.GbptError, match="radius") as e:
                ck(L.gbpt_bilateral_noalloc(planes[0], planes[1], planes[2], None, 8, 8, 1.0, 1.0, 1.0, 1.0, bad,
                                            g.ctypes.data, out_new, None))
            assert e.value.status == 1
    finally:
        dev.free()
