"""ctypes declarations of the libkdgr C ABI (include/kdgr.h).

Loading is strict: when ``libkdgr.so`` is absent or fails to load,
:func:`lib` raises -- there is no fallback render path.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libkdgr.so")

c_u32p = ctypes.POINTER(ctypes.c_uint32)


class Camera(ctypes.Structure):
    _fields_ = [("pos", ctypes.c_float * 3), ("uaxis", ctypes.c_float * 3), ("vaxis", ctypes.c_float * 3),
                ("naxis", ctypes.c_float * 3), ("fovy", ctypes.c_double), ("aspect", ctypes.c_double),
                ("near_c", ctypes.c_double)]

    @classmethod
    def from_scene_camera(cls, cam) -> "Camera":
        c = cls()
        c.pos[:] = list(cam.pos)
        c.uaxis[:] = list(cam.uaxis)
        c.vaxis[:] = list(cam.vaxis)
        c.naxis[:] = list(cam.naxis)
        c.fovy, c.aspect, c.near_c = float(cam.fovy), float(cam.aspect), float(cam.near_c)
        return c


class BuildParams(ctypes.Structure):
    _fields_ = [("max_level", ctypes.c_int32), ("force_split", ctypes.c_int32), ("isect_cost", ctypes.c_float),
                ("sah_mode", ctypes.c_int32), ("sort_cost", ctypes.c_float), ("threads", ctypes.c_int32)]


class Tree(ctypes.Structure):
    _fields_ = [("nodes", c_u32p), ("n_nodes", ctypes.c_uint32), ("offsets", c_u32p),
                ("n_offsets", ctypes.c_uint32), ("aabb", ctypes.c_float * 6), ("depth", ctypes.c_uint32),
                ("n_leaves", ctypes.c_uint32), ("max_leaf", ctypes.c_uint32),
                ("valid", ctypes.POINTER(ctypes.c_uint8)), ("n_gaussians", ctypes.c_uint32)]


class Gaussians(ctypes.Structure):
    _fields_ = [("records", ctypes.POINTER(ctypes.c_float)), ("n", ctypes.c_uint32)]


class BuildStats(ctypes.Structure):
    _fields_ = [("proxy_s", ctypes.c_double), ("build_s", ctypes.c_double), ("n_triangles", ctypes.c_uint64),
                ("n_valid", ctypes.c_uint32), ("serialize_s", ctypes.c_double)]


class RayTrace(ctypes.Structure):
    _fields_ = [("n_inner", ctypes.c_uint32), ("n_leaf", ctypes.c_uint32), ("n_cand", ctypes.c_uint32),
                ("n_hit", ctypes.c_uint32), ("n_blend", ctypes.c_uint32), ("n_restart", ctypes.c_uint32),
                ("n_found", ctypes.c_uint32), ("max_sort", ctypes.c_uint32),
                ("h_leaf", ctypes.c_uint64), ("h_hit", ctypes.c_uint64), ("h_blend", ctypes.c_uint64)]


TRACE_DTYPE = [("n_inner", "<u4"), ("n_leaf", "<u4"), ("n_cand", "<u4"), ("n_hit", "<u4"),
               ("n_blend", "<u4"), ("n_restart", "<u4"), ("n_found", "<u4"), ("max_sort", "<u4"), ("h_leaf", "<u8"), ("h_hit", "<u8"),
               ("h_blend", "<u8")]

_lib = None


def lib() -> ctypes.CDLL:
    """The loaded libkdgr.  Raises RuntimeError when the library is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libkdgr.so not built ({LIB_PATH}); run __graft_entry__.build()")
        _lib = ctypes.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


def _declare(L: ctypes.CDLL) -> None:
    vp = ctypes.c_void_p
    L.kdgr_last_error.restype = ctypes.c_char_p
    L.kdgr_build_params_default.argtypes = [ctypes.POINTER(BuildParams)]
    L.kdgr_build_params_default.restype = None
    L.kdgr_build_tree.argtypes = [vp, ctypes.c_uint32, ctypes.POINTER(BuildParams), ctypes.POINTER(Tree),
                                  ctypes.POINTER(BuildStats)]
    L.kdgr_build_tree_gpu.argtypes = L.kdgr_build_tree.argtypes
    L.kdgr_read_kdt.argtypes = [ctypes.c_char_p, ctypes.POINTER(Tree)]
    L.kdgr_write_kdt.argtypes = [ctypes.POINTER(Tree), ctypes.c_char_p]
    L.kdgr_validate_tree.argtypes = [vp, ctypes.c_uint32, vp, ctypes.c_uint32, ctypes.c_uint32]
    L.kdgr_tree_free.argtypes = [ctypes.POINTER(Tree)]
    L.kdgr_read_kdt_ascii.argtypes = [ctypes.c_char_p, ctypes.POINTER(Tree)]
    L.kdgr_write_kdt_ascii.argtypes = [ctypes.POINTER(Tree), ctypes.c_char_p]
    L.kdgr_read_ply.argtypes = [ctypes.c_char_p, ctypes.POINTER(Gaussians)]
    L.kdgr_gaussians_free.argtypes = [ctypes.POINTER(Gaussians)]
    L.kdgr_gaussians_free.restype = None
    L.kdgr_tree_free.restype = None
    for name, args in _EXTRA_SIGS.items():
        fn = getattr(L, name, None)
        if fn is not None:
            fn.argtypes = args


_EXTRA_SIGS: dict = {}


class KdgrError(RuntimeError):
    def __init__(self, status: int, where: str):
        msg = lib().kdgr_last_error()
        super().__init__(f"{where} failed with status {status}: {msg.decode() if msg else ''}")
        self.status = status


def check(status: int, where: str) -> None:
    if status != 0:
        raise KdgrError(status, where)
