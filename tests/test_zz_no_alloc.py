"""The allocation-free surface entry point (ima_gpu_surface_fp64_noalloc) for
callers that may not allocate device memory, e.g. a plugin inside a host
application that owns every device allocation through its own pool.

It is called through the C ABI on device buffers the test owns, twice in a
row with different point sets (the fixed scratch array it shares across calls
keeps the previous call's contents), and each result is compared with the
existing FP64 entry point, ima_gpu_surface_eval(IMA_SURF_FP64), at the 1e-12
relative tolerance the surface tests use.  This file sorts last so a run that
stops at the first failure has already run every other test.
"""
import ctypes
import ctypes.util

import numpy as np
import pytest

from ima2p_gb300 import api, synth

pytestmark = pytest.mark.gpu


class DeviceBuffers:
    """Test-owned device memory (the entry point itself allocates nothing)."""

    def __init__(self):
        try:
            import torch

            if not torch.cuda.is_available():
                raise ImportError
            self.torch = torch
            self.rt = None
        except ImportError:
            self.torch = None
            name = ctypes.util.find_library("cudart") or "/usr/local/cuda/lib64/libcudart.so"
            self.rt = ctypes.CDLL(name)
        self.keep = []

    def put(self, a):
        a = np.ascontiguousarray(a)
        if self.torch is not None:
            t = self.torch.from_numpy(a.copy()).to("cuda")
            self.keep.append(t)
            return t.data_ptr()
        p = ctypes.c_void_p()
        assert self.rt.cudaMalloc(ctypes.byref(p), ctypes.c_size_t(a.nbytes)) == 0
        assert self.rt.cudaMemcpy(p, a.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(a.nbytes), 1) == 0
        self.keep.append(p)
        return p.value

    def zeros(self, n):
        return self.put(np.zeros(n))

    def get(self, ptr, n):
        out = np.zeros(n)
        if self.torch is not None:
            self.torch.cuda.synchronize()
            for t in self.keep:
                if t.data_ptr() == ptr:
                    return t.cpu().numpy()[:n].copy()
        assert self.rt.cudaDeviceSynchronize() == 0
        assert self.rt.cudaMemcpy(out.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(ptr),
                                  ctypes.c_size_t(out.nbytes), 2) == 0
        return out

    def close(self):
        if self.rt is not None:
            for p in self.keep:
                self.rt.cudaFree(p)
        self.keep = []


def test_noalloc_surface_matches_existing_entry_point():
    rng = np.random.default_rng(77)
    G = 70000  # two genealogy chunks
    rows, lognorm, _ = synth.surface_stats(rng, G, 5, 8, 2)
    calls = [(synth.surface_points(rng, 37), 0), (synth.surface_points(rng, 129), 1)]

    ctx = api.Context(0)
    ctx.surface_load(rows, 5, 8, 3, lognorm=lognorm)
    dev = DeviceBuffers()
    try:
        d_rows = dev.put(rows.astype(np.float32))
        d_lognorm = dev.put(lognorm)
        for pts, mt in calls:  # two calls in a row
            want_q, want_ess = ctx.surface_eval(pts, modeltype=mt, method=api.SURF_FP64)
            d_x = dev.put(pts)
            d_q = dev.zeros(len(pts))
            d_ess = dev.zeros(len(pts))
            rc = api.surface_fp64_noalloc(d_rows, G, rows.shape[1], 5, 8, 3, d_lognorm, d_x,
                                          len(pts), mt, d_q, d_ess, None)
            assert rc == api.IMA_OK
            q = dev.get(d_q, len(pts))
            ess = dev.get(d_ess, len(pts))
            np.testing.assert_allclose(q, want_q, rtol=1e-12, atol=0)
            np.testing.assert_allclose(ess, want_ess, rtol=1e-9, atol=0)
        # beyond the fixed scratch: rejected before anything is launched
        rc = api.surface_fp64_noalloc(d_rows, G, rows.shape[1], 5, 8, 3, d_lognorm, d_x,
                                      200000, 0, d_q, d_ess, None)
        assert rc == api.IMA_ERR_TOO_LARGE
    finally:
        dev.close()
        ctx.close()


def test_noalloc_surface_fewer_chunks_when_the_array_is_full():
    """Enough points that the fixed array holds fewer genealogy chunks than
    the FP64 form would use (300,000 genealogies are 5 chunks; 40,000 points
    leave room for 4): the result still matches the existing entry point."""
    rng = np.random.default_rng(78)
    G = 300000
    rows, lognorm, _ = synth.surface_stats(rng, G, 5, 8, 2)
    pts = synth.surface_points(rng, 40000)
    ctx = api.Context(0)
    ctx.surface_load(rows, 5, 8, 3, lognorm=lognorm)
    dev = DeviceBuffers()
    try:
        d_rows = dev.put(rows.astype(np.float32))
        d_lognorm = dev.put(lognorm)
        want_q, want_ess = ctx.surface_eval(pts, modeltype=0, method=api.SURF_FP64)
        d_x = dev.put(pts)
        d_q = dev.zeros(len(pts))
        d_ess = dev.zeros(len(pts))
        rc = api.surface_fp64_noalloc(d_rows, G, rows.shape[1], 5, 8, 3, d_lognorm, d_x,
                                      len(pts), 0, d_q, d_ess, None)
        assert rc == api.IMA_OK
        np.testing.assert_allclose(dev.get(d_q, len(pts)), want_q, rtol=1e-12, atol=0)
        np.testing.assert_allclose(dev.get(d_ess, len(pts)), want_ess, rtol=1e-9, atol=0)
    finally:
        dev.close()
        ctx.close()
