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
SCHED_WARP_TILES, SCHED_CTA_BLOCKS, SCHED_SM_STRIPS, SCHED_WARP_STRIPS = 0, 1, 2, 3
TRAV_PACKET, TRAV_RAY = 0, 1
TILE_8X4, TILE_4X8, TILE_16X2 = 0, 1, 2
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
                ("chunk", ctypes.c_int32), ("precision", ctypes.c_int32), ("hit_buffer", ctypes.c_int32),
                ("traversal", ctypes.c_int32), ("tile_shape", ctypes.c_int32), ("rays_per_warp", ctypes.c_int32)]

    def as_dict(self) -> dict:
        return {k: int(getattr(self, k)) for k, _ in self._fields_}

    @classmethod
    def default(cls) -> "BatchConfig":
        c = cls()
        capi.lib().kdgr_batch_config_default(ctypes.byref(c))
        return c


class DebugStats(ctypes.Structure):
    _fields_ = [("avg", ctypes.c_float * 6), ("total", ctypes.c_float * 6), ("max", ctypes.c_int32 * 6),
                ("n_pixels", ctypes.c_uint32)]


class Material(ctypes.Structure):
    _fields_ = [("material", ctypes.c_int32), ("reflectivity", ctypes.c_float), ("ior", ctypes.c_float),
                ("color", ctypes.c_float * 3)]


class Sphere(ctypes.Structure):
    _fields_ = [("center", ctypes.c_float * 3), ("radius", ctypes.c_float), ("material", Material)]


OPAQUE, MIRROR, GLASS = 0, 1, 2

DEBUG_COUNTERS = ("node_visits", "leaf_visits", "intersection_tests", "hits_found", "blend_ops", "max_sort_size")


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("arena_bytes", ctypes.c_uint64),
                ("max_views_per_launch", ctypes.c_int32), ("lanes", ctypes.c_int32), ("precision", ctypes.c_int32)]


class RequestStats(ctypes.Structure):
    _fields_ = [("latency_ms", ctypes.c_double), ("queue_ms", ctypes.c_double), ("rays", ctypes.c_uint64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_uint64), ("cancelled", ctypes.c_uint64), ("queued", ctypes.c_uint64),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double), ("mean_ms", ctypes.c_double),
                ("max_ms", ctypes.c_double), ("mrays_per_s", ctypes.c_double), ("rays", ctypes.c_uint64),
                ("launches", ctypes.c_uint64), ("views_launched", ctypes.c_uint64),
                ("max_views_per_launch", ctypes.c_uint64), ("resident_bytes", ctypes.c_uint64)]


vp = ctypes.c_void_p
capi._EXTRA_SIGS.update({
    "kdgr_server_config_default": [ctypes.POINTER(ServerConfig)],
    "kdgr_server_create": [ctypes.POINTER(ServerConfig), ctypes.POINTER(vp)],
    "kdgr_server_add_scene": [vp, vp, ctypes.c_uint32, vp, ctypes.c_uint32, vp, vp, ctypes.c_uint32, ctypes.c_uint32,
                              ctypes.POINTER(ctypes.c_int)],
    "kdgr_server_remove_scene": [vp, ctypes.c_int],
    "kdgr_server_submit": [vp, ctypes.c_int, ctypes.POINTER(View), ctypes.c_int, vp,
                           ctypes.POINTER(ctypes.c_uint64)],
    "kdgr_server_wait": [vp, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(RequestStats)],
    "kdgr_server_cancel": [vp, ctypes.c_uint64],
    "kdgr_server_stats_get": [vp, ctypes.POINTER(ServerStats)],
    "kdgr_server_reset_stats": [vp],
    "kdgr_server_destroy": [vp],
    "kdgr_init": [ctypes.c_int],
    "kdgr_scene_create": [vp, ctypes.c_uint32, vp, ctypes.c_uint32, vp, vp, ctypes.c_uint32, ctypes.c_uint32,
                          ctypes.POINTER(vp)],
    "kdgr_scene_create_device": [vp, ctypes.c_uint32, vp, ctypes.c_uint32, vp, vp, ctypes.c_uint32,
                                 ctypes.c_uint32, ctypes.POINTER(vp)],
    "kdgr_scene_create_from_files": [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint32, ctypes.POINTER(vp)],
    "kdgr_read_ply_device": [ctypes.c_char_p, vp, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32), vp],
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
    "kdgr_demo_spheres": [ctypes.POINTER(Sphere)],
    "kdgr_secondary_mesh_material_default": [ctypes.POINTER(Material)],
    "kdgr_read_obj": [ctypes.c_char_p, ctypes.POINTER(ctypes.POINTER(ctypes.c_float)),
                      ctypes.POINTER(ctypes.c_uint32)],
    "kdgr_free": [vp],
    "kdgr_secondary_create": [ctypes.POINTER(Sphere), ctypes.c_int, vp, ctypes.c_uint32, ctypes.POINTER(Material),
                              ctypes.POINTER(vp)],
    "kdgr_secondary_destroy": [vp],
    "kdgr_render_hybrid": [vp, ctypes.POINTER(capi.Camera), ctypes.c_int, ctypes.c_int, vp, vp, vp,
                           ctypes.POINTER(ctypes.c_float)],
    "kdgr_debug_report": [vp, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_float,
                          ctypes.POINTER(DebugStats)],
    "kdgr_autotune": [vp, ctypes.POINTER(View), ctypes.c_int, ctypes.c_int, vp, ctypes.POINTER(BatchConfig),
                      ctypes.c_char_p, ctypes.c_int],
})


def _ptr(t) -> Optional[int]:
    """Address of a contiguous CUDA tensor, or of a contiguous pinned CPU
    tensor (page-locked host memory is addressable from the device at the
    same address, so a kernel can write its output straight into it)."""
    if t is None:
        return None
    if not t.is_contiguous() or not (t.is_cuda or t.is_pinned()):
        raise ValueError("buffers must be contiguous CUDA tensors or pinned host tensors")
    return t.data_ptr()


def _stream(stream) -> Optional[int]:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return getattr(stream, "cuda_stream", stream)


def init(device: int = 0) -> None:
    capi.check(capi.lib().kdgr_init(device), "kdgr_init")


def material(kind: int, reflectivity: float = 1.0, ior: float = 1.0, color=(1.0, 1.0, 1.0)) -> Material:
    return Material(kind, reflectivity, ior, (ctypes.c_float * 3)(*color))


def sphere(center, radius: float, mat: Material) -> Sphere:
    return Sphere((ctypes.c_float * 3)(*center), radius, mat)


def demo_spheres() -> list:
    """The reference's two demo spheres: glass at (0,1,0), mirror at (0.8,1,1.2)."""
    arr = (Sphere * 2)()
    capi.check(capi.lib().kdgr_demo_spheres(arr), "kdgr_demo_spheres")
    return list(arr)


def mesh_material_default() -> Material:
    m = Material()
    capi.lib().kdgr_secondary_mesh_material_default(ctypes.byref(m))
    return m


def read_obj(path: str):
    """loadSecondaryMesh: (n, 9) float32 triangles, axes mapped (x, -z, y)."""
    import numpy as np
    p = ctypes.POINTER(ctypes.c_float)()
    n = ctypes.c_uint32()
    capi.check(capi.lib().kdgr_read_obj(path.encode(), ctypes.byref(p), ctypes.byref(n)), "kdgr_read_obj")
    try:
        return np.ctypeslib.as_array(p, shape=(n.value, 9)).copy()
    finally:
        capi.lib().kdgr_free(p)


class Secondary:
    """Secondary primitives on the device (kdgr_secondary_create)."""

    def __init__(self, spheres=(), tris=None, tri_material: Optional[Material] = None):
        import numpy as np
        arr = (Sphere * max(1, len(spheres)))(*spheres)
        self._tris = np.ascontiguousarray(tris if tris is not None else np.zeros((0, 9)), np.float32)
        m = tri_material if tri_material is not None else mesh_material_default()
        h = ctypes.c_void_p()
        capi.check(capi.lib().kdgr_secondary_create(arr, len(spheres),
                                                    self._tris.ctypes.data if self._tris.shape[0] else None,
                                                    self._tris.shape[0], ctypes.byref(m), ctypes.byref(h)),
                   "kdgr_secondary_create")
        self.handle = h.value

    def close(self):
        if self.handle:
            capi.lib().kdgr_secondary_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def debug_report(trace, width: int, height: int, out_dir: Optional[str] = None,
                 heat_max: float = 120.0) -> dict:
    """The reference's HIT_AND_NODE_COUNT_DEBUG report over host traces (a
    numpy array of capi.TRACE_DTYPE records in y*W + x order): returns
    {counter: {"avg", "max", "total"}, "n_pixels"} and, with out_dir, writes
    the reference's files there (kdgr_debug_report).  Host only."""
    import numpy as np
    tr = np.ascontiguousarray(trace)
    if tr.dtype != np.dtype(capi.TRACE_DTYPE) or tr.size != width * height:
        raise ValueError("trace must hold width*height records of capi.TRACE_DTYPE")
    st = DebugStats()
    capi.check(capi.lib().kdgr_debug_report(tr.ctypes.data, width, height,
                                            out_dir.encode() if out_dir else None, heat_max, ctypes.byref(st)),
               "kdgr_debug_report")
    out = {name: {"avg": st.avg[k], "max": st.max[k], "total": st.total[k]}
           for k, name in enumerate(DEBUG_COUNTERS)}
    out["n_pixels"] = st.n_pixels
    return out


def read_ply_device(path: str, device=None):
    """kdgr_read_ply_device: the activated (n, 64) float32 records of a 3DGS
    .ply as a CUDA tensor, activated on the device."""
    import torch
    n = ctypes.c_uint32()
    L = capi.lib()
    capi.check(L.kdgr_read_ply_device(path.encode(), None, 0, ctypes.byref(n), None), "kdgr_read_ply_device")
    out = torch.empty((n.value, 64), dtype=torch.float32, device=device or "cuda")
    capi.check(L.kdgr_read_ply_device(path.encode(), _ptr(out), n.value, ctypes.byref(n), _stream(None)),
               "kdgr_read_ply_device")
    return out


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

    @classmethod
    def _adopt(cls, handle, n: int) -> "Scene":
        sc = cls.__new__(cls)
        sc.handle = handle
        sc.n_gaussians = n
        return sc

    @classmethod
    def from_device(cls, tree: KdTree, d_gaussians, forms: int = FORM_EXACT | FORM_FAST,
                    scales_inverted: bool = False) -> "Scene":
        """kdgr_scene_create_device: records already on the device, a CUDA
        tensor of shape (n, 64) float32 (e.g. from read_ply_device)."""
        nodes = np.ascontiguousarray(tree.nodes, dtype=np.uint32)
        offs = np.ascontiguousarray(tree.offsets, dtype=np.uint32)
        aabb = np.ascontiguousarray(tree.aabb, dtype=np.float32)
        if d_gaussians.dim() != 2 or d_gaussians.shape[1] != 64:
            raise ValueError("device records must be an (n, 64) float32 CUDA tensor")
        h = ctypes.c_void_p()
        flags = forms | (SCALES_INVERTED if scales_inverted else 0)
        capi.check(capi.lib().kdgr_scene_create_device(
            nodes.ctypes.data, nodes.shape[0], offs.ctypes.data if offs.size else None, offs.shape[0],
            aabb.ctypes.data, _ptr(d_gaussians), d_gaussians.shape[0], flags, ctypes.byref(h)),
            "kdgr_scene_create_device")
        return cls._adopt(h, int(d_gaussians.shape[0]))

    @classmethod
    def from_files(cls, ply_path: str, kdt_path: str, forms: int = FORM_EXACT | FORM_FAST) -> "Scene":
        """kdgr_scene_create_from_files: a 3DGS .ply activated on the device
        and a binary .kdt tree."""
        h = ctypes.c_void_p()
        capi.check(capi.lib().kdgr_scene_create_from_files(ply_path.encode(), kdt_path.encode(), forms,
                                                            ctypes.byref(h)), "kdgr_scene_create_from_files")
        sc = cls._adopt(h, 0)
        sc.n_gaussians = sc.info()["n_gaussians"]
        return sc

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

    def render_hybrid(self, cam, width: int, height: int, secondary: "Secondary", rgb, stream=None) -> float:
        """Secondary-ray kernel (kdgr_render_hybrid); returns kernel ms."""
        c = capi.Camera.from_scene_camera(cam)
        ms = ctypes.c_float()
        capi.check(capi.lib().kdgr_render_hybrid(self.handle, ctypes.byref(c), width, height, secondary.handle,
                                                 _ptr(rgb), _stream(stream), ctypes.byref(ms)),
                   "kdgr_render_hybrid")
        return ms.value

    def debug_counters(self, cam, width: int, height: int):
        """Per-pixel traces of the oracle-matching kernel, copied to the host
        (numpy, capi.TRACE_DTYPE, y*W + x): the input of debug_report."""
        import numpy as np
        import torch
        dev = torch.device("cuda", torch.cuda.current_device())
        rgb = torch.empty(width * height * 3, device=dev)
        tr = torch.empty(width * height * np.dtype(capi.TRACE_DTYPE).itemsize, dtype=torch.uint8, device=dev)
        self.render_trace(cam, width, height, rgb, None, None, tr)
        torch.cuda.current_stream().synchronize()
        return np.frombuffer(tr.cpu().numpy().tobytes(), dtype=np.dtype(capi.TRACE_DTYPE))

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


class Server:
    """The serving loop (kdgr_server_*): resident scenes under an HBM budget,
    continuous batching of requests into persistent multi-scene launches."""

    def __init__(self, hbm_budget_bytes: int | None = None, arena_bytes: int | None = None,
                 max_views_per_launch: int | None = None, lanes: int | None = None, precision: int = 0):
        L = capi.lib()
        c = ServerConfig()
        L.kdgr_server_config_default(ctypes.byref(c))
        if hbm_budget_bytes is not None:
            c.hbm_budget_bytes = hbm_budget_bytes
        if arena_bytes is not None:
            c.arena_bytes = arena_bytes
        if max_views_per_launch is not None:
            c.max_views_per_launch = max_views_per_launch
        if lanes is not None:
            c.lanes = lanes
        c.precision = precision
        h = ctypes.c_void_p()
        capi.check(L.kdgr_server_create(ctypes.byref(c), ctypes.byref(h)), "kdgr_server_create")
        self.handle = h
        self.config = c

    def add_scene(self, tree: KdTree, gaussians: np.ndarray, scales_inverted: bool = False) -> int:
        nodes = np.ascontiguousarray(tree.nodes, dtype=np.uint32)
        offs = np.ascontiguousarray(tree.offsets, dtype=np.uint32)
        aabb = np.ascontiguousarray(tree.aabb, dtype=np.float32)
        rec = np.ascontiguousarray(gaussians, dtype=np.float32)
        slot = ctypes.c_int()
        capi.check(capi.lib().kdgr_server_add_scene(self.handle, nodes.ctypes.data, nodes.shape[0],
                                                    offs.ctypes.data if offs.size else None, offs.shape[0],
                                                    aabb.ctypes.data, rec.ctypes.data, rec.shape[0],
                                                    SCALES_INVERTED if scales_inverted else 0, ctypes.byref(slot)),
                   "kdgr_server_add_scene")
        return int(slot.value)

    def remove_scene(self, slot: int) -> None:
        capi.check(capi.lib().kdgr_server_remove_scene(self.handle, slot), "kdgr_server_remove_scene")

    def submit(self, slot: int, views, n_views: int, host_rgb) -> int:
        """host_rgb: a (pinned) CPU torch tensor or numpy array with 3 floats per pixel."""
        ptr = host_rgb.data_ptr() if hasattr(host_rgb, "data_ptr") else host_rgb.ctypes.data
        t = ctypes.c_uint64()
        capi.check(capi.lib().kdgr_server_submit(self.handle, slot, views, n_views, ptr, ctypes.byref(t)),
                   "kdgr_server_submit")
        return int(t.value)

    def wait(self, ticket: int, timeout_ms: int = 60_000) -> tuple:
        """Returns (status, stats dict); status 0 = done, 9 = cancelled, 7 = timeout."""
        st = RequestStats()
        rc = capi.lib().kdgr_server_wait(self.handle, ticket, timeout_ms, ctypes.byref(st))
        return rc, {"latency_ms": st.latency_ms, "queue_ms": st.queue_ms, "rays": int(st.rays)}

    def cancel(self, ticket: int) -> int:
        return capi.lib().kdgr_server_cancel(self.handle, ticket)

    def stats(self) -> dict:
        s = ServerStats()
        capi.check(capi.lib().kdgr_server_stats_get(self.handle, ctypes.byref(s)), "kdgr_server_stats_get")
        return {k: (float(getattr(s, k)) if isinstance(getattr(s, k), float) else int(getattr(s, k)))
                for k, _ in s._fields_}

    def reset_stats(self) -> None:
        capi.lib().kdgr_server_reset_stats(self.handle)

    def close(self) -> None:
        if getattr(self, "handle", None):
            capi.lib().kdgr_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
