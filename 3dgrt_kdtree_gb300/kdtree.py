"""Host-side kd-tree handling: build, `.kdt` read/write, validation.

Mirrors the reference's tree surface -- build_kd_tree_for_composite_object
(Kd-treeConverter.cpp:22), dump_kd_tree_for_composite_object (:297) and
read_kd_tree_from_file (:444) -- over the libkdgr C ABI.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import capi


@dataclass
class KdTree:
    nodes: np.ndarray          # (n_nodes, 2) uint32: reference KdTreeNode words
    offsets: np.ndarray        # (n_offsets,) uint32: leaf Gaussian IDs
    aabb: np.ndarray           # (6,) float32, .kdt order (xmin,ymin,zmin,xmax,ymax,zmax)
    depth: int = 0
    n_leaves: int = 0
    max_leaf: int = 0
    valid: np.ndarray | None = None   # per Gaussian, for built trees
    stats: dict = field(default_factory=dict)

    @property
    def n_nodes(self) -> int:
        return int(self.nodes.shape[0])


def _take(t: capi.Tree) -> KdTree:
    nodes = np.ctypeslib.as_array(t.nodes, shape=(t.n_nodes * 2,)).copy().reshape(t.n_nodes, 2)
    offsets = (np.ctypeslib.as_array(t.offsets, shape=(t.n_offsets,)).copy() if t.n_offsets
               else np.zeros(0, np.uint32))
    valid = (np.ctypeslib.as_array(t.valid, shape=(t.n_gaussians,)).copy() if t.n_gaussians else None)
    out = KdTree(nodes, offsets, np.array(list(t.aabb), np.float32), int(t.depth), int(t.n_leaves),
                 int(t.max_leaf), valid)
    capi.lib().kdgr_tree_free(ctypes.byref(t))
    return out


def build(gaussians: np.ndarray, max_level: int = 24, force_split: int = 16, isect_cost: float = 5.0,
          sah_mode: int = 1, sort_cost: float = 0.5, threads: int = 0, device: str = "cpu") -> KdTree:
    """Proxy mesh + SAH kd-tree over activated (non-inverted) records, on the
    host (device="cpu", kdgr_build_tree) or on the current CUDA device
    (device="cuda", kdgr_build_tree_gpu); both give the same tree."""
    if device not in ("cpu", "cuda"):
        raise ValueError("device must be 'cpu' or 'cuda'")
    L = capi.lib()
    rec = np.ascontiguousarray(gaussians, dtype=np.float32)
    if rec.ndim != 2 or rec.shape[1] != 64:
        raise ValueError("gaussians must be an (n, 64) float32 record array")
    p = capi.BuildParams(max_level, force_split, isect_cost, sah_mode, sort_cost, threads)
    t = capi.Tree()
    s = capi.BuildStats()
    fn = "kdgr_build_tree" if device == "cpu" else "kdgr_build_tree_gpu"
    capi.check(getattr(L, fn)(rec.ctypes.data, rec.shape[0], ctypes.byref(p), ctypes.byref(t), ctypes.byref(s)),
               fn)
    tree = _take(t)
    tree.stats = {"proxy_s": s.proxy_s, "build_s": s.build_s, "serialize_s": s.serialize_s,
                  "n_triangles": int(s.n_triangles),
                  "n_valid": int(s.n_valid)}
    return tree


def read_kdt(path: str, ascii: bool = False) -> KdTree:
    """read_kd_tree_from_file (Kd-treeConverter.cpp:444-541), binary or ASCII
    format; the ASCII format has no scene box (aabb comes back zero)."""
    t = capi.Tree()
    fn = "kdgr_read_kdt_ascii" if ascii else "kdgr_read_kdt"
    capi.check(getattr(capi.lib(), fn)(path.encode(), ctypes.byref(t)), fn)
    return _take(t)


def write_kdt(tree: KdTree, path: str, ascii: bool = False) -> None:
    """dump_kd_tree_for_composite_object (Kd-treeConverter.cpp:297-380)."""
    nodes = np.ascontiguousarray(tree.nodes, dtype=np.uint32)
    offs = np.ascontiguousarray(tree.offsets, dtype=np.uint32)
    t = capi.Tree()
    t.nodes = nodes.ctypes.data_as(capi.c_u32p)
    t.n_nodes = nodes.shape[0]
    t.offsets = offs.ctypes.data_as(capi.c_u32p)
    t.n_offsets = offs.shape[0]
    t.aabb[:] = [float(x) for x in tree.aabb]
    fn = "kdgr_write_kdt_ascii" if ascii else "kdgr_write_kdt"
    capi.check(getattr(capi.lib(), fn)(ctypes.byref(t), path.encode()), fn)


def read_ply(path: str) -> np.ndarray:
    """loadGaussiansFromPly (Kd-treeConverterMain.cpp:1652-1769): activated
    (n, 64) float32 records from a binary 3DGS .ply (kdgr_read_ply)."""
    g = capi.Gaussians()
    capi.check(capi.lib().kdgr_read_ply(path.encode(), ctypes.byref(g)), "kdgr_read_ply")
    try:
        return np.ctypeslib.as_array(g.records, shape=(g.n, 64)).copy()
    finally:
        capi.lib().kdgr_gaussians_free(ctypes.byref(g))


def validate(tree: KdTree, n_gaussians: int) -> None:
    nodes = np.ascontiguousarray(tree.nodes, dtype=np.uint32)
    offs = np.ascontiguousarray(tree.offsets, dtype=np.uint32)
    capi.check(capi.lib().kdgr_validate_tree(nodes.ctypes.data, nodes.shape[0], offs.ctypes.data,
                                             offs.shape[0], n_gaussians), "kdgr_validate_tree")
