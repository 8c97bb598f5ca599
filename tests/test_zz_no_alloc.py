"""The allocation-free tricubic sampler, through the C ABI.

gfs_tricubic_interpolate_noalloc serves callers that cannot allocate device
memory (hosts that own all device memory through their own allocator, or code
where cudaMalloc is not allowed): they pass their own device buffers and a
stream, and the entry point's scratch lives in a fixed array inside libgfs.
This test gives it device buffers (allocated here by torch, standing in for the
caller's allocator) and checks its output against the allocating entry point
gfs_tricubic_interpolate on the same inputs, within the tolerance the other
sampler tests use (relative 1e-5, absolute 1e-6 of the field scale), on two
calls in a row: the second call uses a smaller grid, so it also shows that the
shared scratch left over from the first call does not leak into the result.
"""
import ctypes

import numpy as np
import pytest

from gridfluidsim3d_gb300 import GFSError, MACVelocityField, ParticleAdvector, _lib

pytestmark = pytest.mark.gpu


def _field(dims, dx, seed):
    rng = np.random.default_rng(seed)
    ni, nj, nk = dims
    return MACVelocityField(ni, nj, nk, dx,
                            rng.normal(size=(nk, nj, ni + 1)).astype(np.float32),
                            rng.normal(size=(nk, nj + 1, ni)).astype(np.float32),
                            rng.normal(size=(nk + 1, nj, ni)).astype(np.float32))


def _call(torch, f, pts):
    dev = torch.device("cuda", 0)
    du, dv, dw = (torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (f.u, f.v, f.w))
    dp = torch.from_numpy(pts).to(dev)
    out = torch.full((len(pts), 3), float("nan"), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    _lib.lib().gfs_tricubic_interpolate_noalloc(f.isize, f.jsize, f.ksize, f.dx, ctypes.c_void_p(du.data_ptr()),
                                                ctypes.c_void_p(dv.data_ptr()), ctypes.c_void_p(dw.data_ptr()),
                                                ctypes.c_void_p(dp.data_ptr()), len(pts),
                                                ctypes.c_void_p(out.data_ptr()), None)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_matches_allocating_entry_point(gpu_ctx):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    for dims, dx, seed in (((40, 36, 30), 0.125, 1), ((17, 23, 11), 0.25, 2)):
        f = _field(dims, dx, seed)
        ext = np.array(dims) * dx
        pts = (rng.random((6000, 3)) * ext * 1.1 - 0.05 * ext).astype(np.float32)
        want = ParticleAdvector(gpu_ctx).tricubic_interpolate(pts, f)
        got = _call(torch, f, pts)
        np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-6 * 4.0)


def test_noalloc_rejects_oversized_grid(gpu_ctx):
    with pytest.raises(GFSError):
        _lib.lib().gfs_tricubic_interpolate_noalloc(400, 400, 400, 0.1, ctypes.c_void_p(16), ctypes.c_void_p(16),
                                                    ctypes.c_void_p(16), ctypes.c_void_p(16), 0, None, None)
