"""ctypes wrapper of liboracle (oracle/oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg.  Nothing in the product imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
LIB = os.path.join(HERE, "_build", "liboracle.so")

TRACE_DTYPE = np.dtype([("n_inner", "<u4"), ("n_leaf", "<u4"), ("n_cand", "<u4"), ("n_hit", "<u4"),
                        ("n_blend", "<u4"), ("n_restart", "<u4"), ("n_found", "<u4"), ("max_sort", "<u4"), ("h_leaf", "<u8"), ("h_hit", "<u8"),
                        ("h_blend", "<u8")])


def build(cxx: str = "g++") -> str:
    """Compile liboracle with the flags the transcription requires."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           "-I" + os.path.join(REPO, "include"), os.path.join(HERE, "oracle.cpp"), "-o", LIB]
    subprocess.run(cmd, check=True)
    return LIB


class _Scene(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_void_p), ("n_nodes", ctypes.c_uint32), ("offsets", ctypes.c_void_p),
                ("n_offsets", ctypes.c_uint32), ("aabb", ctypes.c_float * 6), ("gauss", ctypes.c_void_p),
                ("n_gauss", ctypes.c_uint32)]


class CamInfo(ctypes.Structure):
    _fields_ = [("eye", ctypes.c_float * 3), ("u", ctypes.c_float * 3), ("v", ctypes.c_float * 3),
                ("start", ctypes.c_float * 3), ("step_x", ctypes.c_float), ("step_y", ctypes.c_float)]


class _Camera(ctypes.Structure):
    _fields_ = [("pos", ctypes.c_float * 3), ("uaxis", ctypes.c_float * 3), ("vaxis", ctypes.c_float * 3),
                ("naxis", ctypes.c_float * 3), ("fovy", ctypes.c_double), ("aspect", ctypes.c_double),
                ("near_c", ctypes.c_double)]


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        vp = ctypes.c_void_p
        L.orc_caminfo_from_camera.argtypes = [ctypes.POINTER(_Camera), ctypes.c_int, ctypes.c_int,
                                              ctypes.POINTER(CamInfo)]
        L.orc_caminfo_from_camera.restype = None
        for n in ("orc_render_f32", "orc_render_f64"):
            getattr(L, n).argtypes = [ctypes.POINTER(_Scene), ctypes.POINTER(CamInfo), ctypes.c_int, ctypes.c_int,
                                      vp, ctypes.c_uint32, vp, vp, vp, vp, ctypes.c_int]
        vp = ctypes.c_void_p
        L.orc_render_hybrid_f32.argtypes = [ctypes.POINTER(_Scene), ctypes.POINTER(CamInfo), ctypes.c_int,
                                            ctypes.c_int, vp, ctypes.c_uint32, vp, ctypes.c_int, vp,
                                            ctypes.c_uint32, vp, vp, ctypes.c_int]
        L.orc_expf.argtypes = [ctypes.c_float]
        L.orc_expf.restype = ctypes.c_float
        L.orc_expf_n.argtypes = [vp, vp, ctypes.c_uint32]
        L.orc_expf_n.restype = None
        _lib = L
    return _lib


def invert_scales(rec: np.ndarray) -> np.ndarray:
    """The caller-side inversion the reference performs before upload
    (Kd-treeConverterMain.cpp:3636-3650): scale <- 1/scale, k_scale <- 1/k_scale,
    in float32."""
    out = np.array(rec, dtype=np.float32, copy=True)
    one = np.float32(1.0)
    out[:, 4:7] = one / out[:, 4:7]
    out[:, 7] = one / out[:, 7]
    return out


def caminfo(cam, width: int, height: int) -> CamInfo:
    c = _Camera()
    c.pos[:] = list(cam.pos)
    c.uaxis[:] = list(cam.uaxis)
    c.vaxis[:] = list(cam.vaxis)
    c.naxis[:] = list(cam.naxis)
    c.fovy, c.aspect, c.near_c = cam.fovy, cam.aspect, cam.near_c
    ci = CamInfo()
    lib().orc_caminfo_from_camera(ctypes.byref(c), width, height, ctypes.byref(ci))
    return ci


class OracleScene:
    """Holds numpy arrays alive for the oracle.  ``gauss_inv`` must hold
    inverted scales (see :func:`invert_scales`)."""

    def __init__(self, nodes: np.ndarray, offsets: np.ndarray, aabb, gauss_inv: np.ndarray):
        self.nodes = np.ascontiguousarray(nodes, dtype=np.uint32).reshape(-1)
        self.offsets = np.ascontiguousarray(offsets, dtype=np.uint32)
        self.gauss = np.ascontiguousarray(gauss_inv, dtype=np.float32)
        s = _Scene()
        s.nodes = self.nodes.ctypes.data
        s.n_nodes = self.nodes.shape[0] // 2
        s.offsets = self.offsets.ctypes.data if self.offsets.size else None
        s.n_offsets = self.offsets.shape[0]
        s.aabb[:] = [float(x) for x in aabb]
        s.gauss = self.gauss.ctypes.data
        s.n_gauss = self.gauss.shape[0]
        self.s = s


def render(scene: OracleScene, cam, width: int, height: int, pixels: np.ndarray | None = None,
           precision: str = "f32", trace: bool = False, threads: int = 0):
    """Render listed pixels (y*width + x; all pixels when None).  Returns
    (rgb (n,3), alpha (n,), depth (n,), trace or None) in list order."""
    if pixels is None:
        pixels = np.arange(width * height, dtype=np.uint32)
    pixels = np.ascontiguousarray(pixels, dtype=np.uint32)
    n = pixels.shape[0]
    dt = np.float32 if precision == "f32" else np.float64
    rgb = np.zeros((n, 3), dt)
    alpha = np.zeros(n, dt)
    depth = np.zeros(n, dt)
    tr = np.zeros(n, TRACE_DTYPE) if trace else None
    ci = cam if isinstance(cam, CamInfo) else caminfo(cam, width, height)
    fn = lib().orc_render_f32 if precision == "f32" else lib().orc_render_f64
    rc = fn(ctypes.byref(scene.s), ctypes.byref(ci), width, height, pixels.ctypes.data, n, rgb.ctypes.data,
            alpha.ctypes.data, depth.ctypes.data, tr.ctypes.data if trace else None, threads)
    if rc != 0:
        raise RuntimeError(f"oracle render failed ({rc})")
    return rgb, alpha, depth, tr


def pack_spheres(spheres) -> np.ndarray:
    """[(center(3), radius, material, reflectivity, ior, color(3))] -> the
    10-float layout with the material as int bits."""
    out = np.zeros((len(spheres), 10), np.float32)
    for i, (ctr, rad, mat, refl, ior, col) in enumerate(spheres):
        out[i, 0:3] = ctr
        out[i, 3] = rad
        out[i, 4] = np.array([mat], np.int32).view(np.float32)[0]
        out[i, 5:7] = (refl, ior)
        out[i, 7:10] = col
    return out


def pack_material(mat, refl, ior, col) -> np.ndarray:
    out = np.zeros(6, np.float32)
    out[0] = np.array([mat], np.int32).view(np.float32)[0]
    out[1:3] = (refl, ior)
    out[3:6] = col
    return out


def render_hybrid(scene: OracleScene, cam, width: int, height: int, spheres=(), tris=None, tri_material=None,
                  pixels: np.ndarray | None = None, threads: int = 0) -> np.ndarray:
    """The secondary-ray kernel (FP32, oracle-matching).  spheres: list as in
    pack_spheres; tris: (n, 9) float32; tri_material: (material, reflectivity,
    ior, color).  Returns rgb (n, 3) in list order."""
    if pixels is None:
        pixels = np.arange(width * height, dtype=np.uint32)
    pixels = np.ascontiguousarray(pixels, dtype=np.uint32)
    sph = pack_spheres(spheres)
    tri = np.ascontiguousarray(tris if tris is not None else np.zeros((0, 9)), np.float32)
    tm = pack_material(*tri_material) if tri_material is not None else np.zeros(6, np.float32)
    rgb = np.zeros((pixels.shape[0], 3), np.float32)
    ci = cam if isinstance(cam, CamInfo) else caminfo(cam, width, height)
    rc = lib().orc_render_hybrid_f32(ctypes.byref(scene.s), ctypes.byref(ci), width, height, pixels.ctypes.data,
                                     pixels.shape[0], sph.ctypes.data if len(sph) else None, len(sph),
                                     tri.ctypes.data if tri.shape[0] else None, tri.shape[0], tm.ctypes.data,
                                     rgb.ctypes.data, threads)
    if rc != 0:
        raise RuntimeError(f"oracle hybrid render failed ({rc})")
    return rgb


def read_kdt(path: str):
    """read_kd_tree_from_file(obj, path, KD_TREE_DUMP_IN_BINARY)
    (Kd-treeConverter.cpp:444-495) restated in numpy: f32 version (0.1),
    f32 aabb[6] (xmin, ymin, zmin, xmax, ymax, zmax), i32 node count, 8-byte
    nodes, i32 offset count, u32 offsets.  Returns (nodes (n, 2) uint32,
    offsets uint32, aabb float32[6]).  Lets a checker load a tree without
    the product library."""
    raw = open(path, "rb").read()
    hdr = np.frombuffer(raw, dtype="<f4", count=7)
    if hdr[0] != np.float32(0.1):
        raise ValueError(f"{path}: unsupported .kdt version {hdr[0]}")
    pos = 28
    nn = int(np.frombuffer(raw, dtype="<i4", count=1, offset=pos)[0])
    pos += 4
    if nn <= 0 or pos + 8 * nn + 4 > len(raw):
        raise ValueError(f"{path}: bad node count {nn}")
    nodes = np.frombuffer(raw, dtype="<u4", count=2 * nn, offset=pos).reshape(nn, 2).copy()
    pos += 8 * nn
    no = int(np.frombuffer(raw, dtype="<i4", count=1, offset=pos)[0])
    pos += 4
    if no < 0 or pos + 4 * no > len(raw):
        raise ValueError(f"{path}: bad offset count {no}")
    offsets = np.frombuffer(raw, dtype="<u4", count=no, offset=pos).copy()
    return nodes, offsets, hdr[1:7].astype(np.float32)


def to_image(values: np.ndarray, width: int, height: int) -> np.ndarray:
    """Arrange per-pixel values of a full render (pixel y*width+x in kernel
    row order) into the reference's framebuffer layout, rows flipped
    (cudaRenderer.cu:2370): out[(H-1-y), x]."""
    v = values.reshape(height, width, *values.shape[1:])
    return v[::-1].copy()
