"""kdgr_render_batch_noalloc, the batched render call for callers that cannot
allocate device memory (a host that owns the whole device-memory budget, or a
frame loop that must never enter the allocator).

It renders with the same kernel as kdgr_render_batch, but takes its scratch
(view table and work-queue counter) from a fixed file-scope device array
instead of the allocator.  Called here through the C ABI, twice in a row with
different view sets -- the shared array keeps the previous call's contents,
so each call must rewrite the table and zero the counter -- and checked
against kdgr_render_batch within the parity tolerance of the tests (1e-5
absolute).  A third test checks the defining property itself: around a
warmed-up call, the high-water mark of the device's default stream-ordered
pool does not rise and the device's free memory does not change, while the
same probe does see one stream-ordered allocation from that pool.  The file sorts last so that a run stopping
at the first failure has already run every other test; it also passes alone
in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-5
MAX_VIEWS = 256


def _noalloc(pkg):
    L = pkg.capi.lib()
    F = pkg.renderer
    fn = L.kdgr_render_batch_noalloc
    vp = ctypes.c_void_p
    fn.argtypes = [vp, ctypes.POINTER(F.View), ctypes.c_int, vp, vp, vp, ctypes.POINTER(F.BatchConfig), vp]
    fn.restype = ctypes.c_int
    return fn


def test_noalloc_matches_batch_two_calls(pkg, cuda, fixtures):
    F = pkg.renderer
    fx = fixtures["dense800"]
    scene = F.Scene(fx.tree, fx.rec)
    fn = _noalloc(pkg)
    stream = torch.cuda.current_stream().cuda_stream
    view_sets = [
        pkg.scenes.sphere_cameras(5, seed=21, resolutions=[(48, 40), (33, 17)]),
        pkg.scenes.sphere_cameras(3, seed=22, resolutions=[(64, 48)]),
    ]
    for cams in view_sets:
        views, total, _ = F.make_views(cams)
        ref_rgb = torch.zeros(total * 3, device=cuda)
        ref_a = torch.zeros(total, device=cuda)
        scene.render_batch(views, len(cams), ref_rgb, ref_a)
        rgb = torch.full((total * 3,), -1.0, device=cuda)
        alpha = torch.full((total,), -1.0, device=cuda)
        rc = fn(scene.handle, views, len(cams), rgb.data_ptr(), alpha.data_ptr(), None, None, stream)
        assert rc == 0, pkg.capi.lib().kdgr_last_error()
        torch.cuda.synchronize()
        assert scene.status() == 0
        np.testing.assert_allclose(rgb.cpu().numpy(), ref_rgb.cpu().numpy(), rtol=0, atol=TOL)
        np.testing.assert_allclose(alpha.cpu().numpy(), ref_a.cpu().numpy(), rtol=0, atol=TOL)
        assert float(ref_a.max()) > 0.0  # the views see the scene
    scene.close()


# CUmemPool_attribute values (cuda.h)
_USED_MEM_CURRENT = 7
_USED_MEM_HIGH = 8


class _DefaultPool:
    """High-water mark of the current device's default memory pool, read
    through the driver API (libcuda), reset before each probe."""

    def __init__(self, index):
        cu = ctypes.CDLL("libcuda.so.1")
        dev = ctypes.c_int()
        assert cu.cuDeviceGet(ctypes.byref(dev), index) == 0
        self.pool = ctypes.c_void_p()
        assert cu.cuDeviceGetDefaultMemPool(ctypes.byref(self.pool), dev) == 0
        self.cu = cu

    def _attr(self, a):
        v = ctypes.c_uint64()
        assert self.cu.cuMemPoolGetAttribute(self.pool, a, ctypes.byref(v)) == 0
        return v.value

    def reset(self):
        zero = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, _USED_MEM_HIGH, ctypes.byref(zero)) == 0
        return self._attr(_USED_MEM_CURRENT)

    def high(self):
        return self._attr(_USED_MEM_HIGH)

    def alloc_free(self, nbytes, stream):
        """One stream-ordered allocation and free from this pool."""
        p = ctypes.c_uint64()
        assert self.cu.cuMemAllocAsync(ctypes.byref(p), ctypes.c_size_t(nbytes), ctypes.c_void_p(stream)) == 0
        assert self.cu.cuMemFreeAsync(p, ctypes.c_void_p(stream)) == 0


def test_noalloc_takes_no_device_memory(pkg, cuda, fixtures):
    F = pkg.renderer
    fx = fixtures["cluster2k"]
    scene = F.Scene(fx.tree, fx.rec)
    fn = _noalloc(pkg)
    stream = torch.cuda.current_stream().cuda_stream
    cams = pkg.scenes.sphere_cameras(4, seed=23, resolutions=[(40, 32)])
    views, total, _ = F.make_views(cams)
    rgb = torch.zeros(total * 3, device=cuda)
    ref = torch.zeros(total * 3, device=cuda)
    pool = _DefaultPool(cuda.index)
    for _ in range(2):  # warm-up: modules loaded, scratch address looked up
        assert fn(scene.handle, views, len(cams), rgb.data_ptr(), None, None, None, stream) == 0
        scene.render_batch(views, len(cams), ref)
    torch.cuda.synchronize()
    # positive control: an allocation from the pool raises its high-water mark
    base = pool.reset()
    pool.alloc_free(1 << 20, stream)
    torch.cuda.synchronize()
    assert pool.high() > base
    free0 = torch.cuda.mem_get_info(cuda)[0]
    base = pool.reset()
    rc = fn(scene.handle, views, len(cams), rgb.data_ptr(), None, None, None, stream)
    assert rc == 0, pkg.capi.lib().kdgr_last_error()
    torch.cuda.synchronize()
    assert pool.high() == base
    assert torch.cuda.mem_get_info(cuda)[0] == free0
    np.testing.assert_allclose(rgb.cpu().numpy(), ref.cpu().numpy(), rtol=0, atol=TOL)
    scene.close()


def test_noalloc_rejects_more_views_than_its_scratch_holds(pkg, cuda, fixtures):
    F = pkg.renderer
    fx = fixtures["uniform2k"]
    scene = F.Scene(fx.tree, fx.rec)
    fn = _noalloc(pkg)
    cams = [(pkg.scenes.front_camera(8, 8), 8, 8)] * (MAX_VIEWS + 1)
    views, total, _ = F.make_views(cams)
    rgb = torch.zeros(total * 3, device=cuda)
    rc = fn(scene.handle, views, len(cams), rgb.data_ptr(), None, None, None,
            torch.cuda.current_stream().cuda_stream)
    assert rc == 10  # KDGR_ERR_LIMIT
    assert b"256" in pkg.capi.lib().kdgr_last_error()
    scene.close()
