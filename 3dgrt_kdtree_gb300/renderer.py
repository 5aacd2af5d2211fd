"""Python host mirror of the render surface (over the libkdgr C ABI).

Device buffers are torch CUDA tensors (torch is used only for device memory
and streams); every render call goes to the sm_103a kernels in libkdgr.so.
There is no CPU fallback: a missing library raises.

Reference surface (cudaRenderer.h:60-109) and where it maps:

====================================  =====================================
renderGaussianWithCudaSetup           Scene(tree, gaussians, ...)
renderGaussianWithCudaFrame           Scene.render(camera, W, H, rgb, ...)
cleanupCudaResources                  Scene.close()
(none: batching / precision forms)    Scene.render_batch / Batch / autotune
====================================  =====================================
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np

from . import capi
from .kdtree import KdTree

FORM_EXACT, FORM_FAST, FORM_PACKED = 0x10, 0x20, 0x40
SCHED_WARP_TILES, SCHED_CTA_BLOCKS = 0, 1
SCALES_INVERTED = 0x1


class SceneInfo(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_uint32), ("n_offsets", ctypes.c_uint32), ("n_gaussians", ctypes.c_uint32),
                ("depth", ctypes.c_uint32), ("n_leaves", ctypes.c_uint32), ("max_leaf", ctypes.c_uint32),
                ("forms", ctypes.c_uint32), ("top_nodes", ctypes.c_uint32), ("n_aniso", ctypes.c_uint32),
                ("device_bytes", ctypes.c_uint64)]


class View(ctypes.Structure):
    _fields_ = [("cam", capi.Camera), ("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("out_offset", ctypes.c_uint64)]


class BatchConfig(ctypes.Structure):
    _fields_ = [("schedule", ctypes.c_int32), ("min_blocks", ctypes.c_int32), ("blocks_per_sm", ctypes.c_int32),
                ("chunk", ctypes.c_int32), ("precision", ctypes.c_int32)]

    def as_dict(self) -> dict:
        return {k: int(getattr(self, k)) for k, _ in self._fields_}

    @classmethod
    def default(cls) -> "BatchConfig":
        c = cls()
        capi.lib().kdgr_batch_config_default(ctypes.byref(c))
        return c


vp = ctypes.c_void_p
capi._EXTRA_SIGS.update({
    "kdgr_init": [ctypes.c_int],
    "kdgr_scene_create": [vp, ctypes.c_uint32, vp, ctypes.c_uint32, vp, vp, ctypes.c_uint32, ctypes.c_uint32,
                          ctypes.POINTER(vp)],
    "kdgr_scene_destroy": [vp],
    "kdgr_scene_info_get": [vp, ctypes.POINTER(SceneInfo)],
    "kdgr_scene_status": [vp, ctypes.POINTER(ctypes.c_uint32), ctypes.c_int],
    "kdgr_render": [vp, ctypes.POINTER(capi.Camera), ctypes.c_int, ctypes.c_int, vp, vp, vp, vp,
                    ctypes.POINTER(ctypes.c_float)],
    "kdgr_render_trace": [vp, ctypes.POINTER(capi.Camera), ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, vp],
    "kdgr_render_fast": [vp, ctypes.POINTER(capi.Camera), ctypes.c_int, ctypes.c_int, vp, vp, vp, ctypes.c_int,
                         vp, ctypes.POINTER(ctypes.c_float)],
    "kdgr_batch_config_default": [ctypes.POINTER(BatchConfig)],
    "kdgr_render_batch": [vp, ctypes.POINTER(View), ctypes.c_int, vp, vp, vp, ctypes.POINTER(BatchConfig), vp,
                          ctypes.POINTER(ctypes.c_float)],
    "kdgr_batch_create": [vp, ctypes.POINTER(View), ctypes.c_int, vp, vp, vp, ctypes.POINTER(BatchConfig),
                          ctypes.POINTER(vp)],
    "kdgr_batch_run": [vp, vp],
    "kdgr_batch_destroy": [vp],
    "kdgr_autotune": [vp, ctypes.POINTER(View), ctypes.c_int, ctypes.c_int, vp, ctypes.POINTER(BatchConfig),
                      ctypes.c_char_p, ctypes.c_int],
})


def _ptr(t) -> Optional[int]:
    if t is None:
        return None
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("device buffers must be contiguous CUDA tensors")
    return t.data_ptr()


def _stream(stream) -> Optional[int]:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return getattr(stream, "cuda_stream", stream)


def init(device: int = 0) -> None:
    capi.check(capi.lib().kdgr_init(device), "kdgr_init")


def make_views(cams: Sequence) -> tuple:
    """[(Camera, W, H)] -> (ctypes View array, total pixels, per-view offsets)."""
    arr = (View * len(cams))()
    off = 0
    offs = []
    for i, (cam, w, h) in enumerate(cams):
        arr[i].cam = capi.Camera.from_scene_camera(cam)
        arr[i].width, arr[i].height, arr[i].out_offset = w, h, off
        offs.append(off)
        off += w * h
    return arr, off, offs


class Scene:
    """A tree plus Gaussians resident on the device (renderGaussianWithCudaSetup)."""

    def __init__(self, tree: KdTree, gaussians: np.ndarray, forms: int = FORM_EXACT | FORM_FAST,
                 scales_inverted: bool = False):
        L = capi.lib()
        nodes = np.ascontiguousarray(tree.nodes, dtype=np.uint32)
        offs = np.ascontiguousarray(tree.offsets, dtype=np.uint32)
        aabb = np.ascontiguousarray(tree.aabb, dtype=np.float32)
        rec = np.ascontiguousarray(gaussians, dtype=np.float32)
        if rec.ndim != 2 or rec.shape[1] != 64:
            raise ValueError("gaussians must be (n, 64) float32 records")
        h = ctypes.c_void_p()
        flags = forms | (SCALES_INVERTED if scales_inverted else 0)
        capi.check(L.kdgr_scene_create(nodes.ctypes.data, nodes.shape[0], offs.ctypes.data if offs.size else None,
                                       offs.shape[0], aabb.ctypes.data, rec.ctypes.data, rec.shape[0], flags,
                                       ctypes.byref(h)), "kdgr_scene_create")
        self.handle = h
        self.n_gaussians = rec.shape[0]

    def info(self) -> dict:
        i = SceneInfo()
        capi.check(capi.lib().kdgr_scene_info_get(self.handle, ctypes.byref(i)), "kdgr_scene_info_get")
        return {k: int(getattr(i, k)) for k, _ in i._fields_}

    def status(self, clear: bool = True) -> int:
        b = ctypes.c_uint32()
        capi.check(capi.lib().kdgr_scene_status(self.handle, ctypes.byref(b), int(clear)), "kdgr_scene_status")
        return int(b.value)

    def render(self, cam, width: int, height: int, rgb, alpha=None, depth=None, stream=None,
               timed: bool = False) -> Optional[float]:
        """Plain drop-in form (oracle-matching).  Returns kernel ms when timed."""
        c = capi.Camera.from_scene_camera(cam)
        ms = ctypes.c_float()
        capi.check(capi.lib().kdgr_render(self.handle, ctypes.byref(c), width, height, _ptr(rgb), _ptr(alpha),
                                          _ptr(depth), _stream(stream), ctypes.byref(ms) if timed else None),
                   "kdgr_render")
        return float(ms.value) if timed else None

    def render_trace(self, cam, width: int, height: int, rgb, alpha, depth, trace, stream=None) -> None:
        c = capi.Camera.from_scene_camera(cam)
        capi.check(capi.lib().kdgr_render_trace(self.handle, ctypes.byref(c), width, height, _ptr(rgb),
                                                _ptr(alpha), _ptr(depth), _ptr(trace), _stream(stream)),
                   "kdgr_render_trace")

    def render_fast(self, cam, width: int, height: int, rgb, alpha=None, depth=None, precision: int = 0,
                    stream=None, timed: bool = False) -> Optional[float]:
        c = capi.Camera.from_scene_camera(cam)
        ms = ctypes.c_float()
        capi.check(capi.lib().kdgr_render_fast(self.handle, ctypes.byref(c), width, height, _ptr(rgb), _ptr(alpha),
                                               _ptr(depth), precision, _stream(stream),
                                               ctypes.byref(ms) if timed else None), "kdgr_render_fast")
        return float(ms.value) if timed else None

    def render_batch(self, views, n_views: int, rgb, alpha=None, depth=None, cfg: BatchConfig | None = None,
                     stream=None, timed: bool = False) -> Optional[float]:
        ms = ctypes.c_float()
        capi.check(capi.lib().kdgr_render_batch(self.handle, views, n_views, _ptr(rgb), _ptr(alpha), _ptr(depth),
                                                ctypes.byref(cfg) if cfg is not None else None, _stream(stream),
                                                ctypes.byref(ms) if timed else None), "kdgr_render_batch")
        return float(ms.value) if timed else None

    def autotune(self, views, n_views: int, rgb, precision: int = 0) -> tuple:
        best = BatchConfig()
        buf = ctypes.create_string_buffer(1 << 16)
        capi.check(capi.lib().kdgr_autotune(self.handle, views, n_views, precision, _ptr(rgb), ctypes.byref(best),
                                            buf, len(buf)), "kdgr_autotune")
        return best, buf.value.decode()

    def close(self) -> None:
        if getattr(self, "handle", None):
            capi.check(capi.lib().kdgr_scene_destroy(self.handle), "kdgr_scene_destroy")
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """A fixed batch of views captured as a CUDA graph (kdgr_batch_create)."""

    def __init__(self, scene: Scene, views, n_views: int, rgb, alpha=None, depth=None,
                 cfg: BatchConfig | None = None):
        h = ctypes.c_void_p()
        capi.check(capi.lib().kdgr_batch_create(scene.handle, views, n_views, _ptr(rgb), _ptr(alpha), _ptr(depth),
                                                ctypes.byref(cfg) if cfg is not None else None, ctypes.byref(h)),
                   "kdgr_batch_create")
        self.handle = h
        self._keep = (scene, rgb, alpha, depth)

    def run(self, stream=None) -> None:
        capi.check(capi.lib().kdgr_batch_run(self.handle, _stream(stream)), "kdgr_batch_run")

    def close(self) -> None:
        if getattr(self, "handle", None):
            capi.lib().kdgr_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
