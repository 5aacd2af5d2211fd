"""The device kd-tree builder (kdgr_build_tree_gpu) against the host builder
and the reference builder's committed trees: the same nodes, split bits, leaf
ID lists, scene box and depth, for the golden scenes, fresh scenes under
every SAH mode and flag, and the 100k-Gaussian uniform workload."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

sc = importlib.import_module("3dgrt_kdtree_gb300.scenes")


def _same(a, b):
    np.testing.assert_array_equal(a.nodes, b.nodes)
    np.testing.assert_array_equal(a.offsets, b.offsets)
    np.testing.assert_array_equal(np.asarray(a.aabb, np.float32).view(np.uint32),
                                  np.asarray(b.aabb, np.float32).view(np.uint32))
    assert a.depth == b.depth


@pytest.mark.parametrize("name", ["uniform2k", "cluster2k", "dense800"])
def test_gpu_build_matches_reference_golden(pkg, cuda, fixtures, name):
    fx = fixtures[name]
    t = pkg.kdtree.build(fx.rec, device="cuda")
    np.testing.assert_array_equal(t.nodes, fx.tree.nodes)
    np.testing.assert_array_equal(t.offsets, fx.tree.offsets)
    np.testing.assert_array_equal(np.asarray(t.aabb, np.float32), np.asarray(fx.tree.aabb, np.float32))


@pytest.mark.parametrize("kind,seed,n,flags", [
    ("uniform", 11, 3000, dict()),
    ("cluster", 12, 5000, dict(sah_mode=0)),
    ("cluster", 13, 4000, dict(sah_mode=4)),
    ("uniform", 14, 3000, dict(sah_mode=7, sort_cost=0.25)),
    ("cluster", 15, 6000, dict(force_split=0)),
    ("uniform", 16, 2500, dict(max_level=9, isect_cost=3.0)),
    ("dense", 17, 3000, dict()),
])
def test_gpu_build_matches_host_build(pkg, cuda, kind, seed, n, flags):
    if kind == "uniform":
        rec = sc.uniform_cube(n, seed=seed, scale=0.03)
    elif kind == "cluster":
        rec = sc.cluster_shell(n, seed=seed, n_clusters=6)
    else:  # two tight clusters: deep trees, many straddling triangles
        rec = sc.cluster_shell(n, seed=seed, n_clusters=2)
    _same(pkg.kdtree.build(rec, device="cuda", **flags), pkg.kdtree.build(rec, **flags))


def test_gpu_build_100k_uniform_workload(pkg, cuda):
    rec = sc.uniform_cube(100_000, seed=0)
    g = pkg.kdtree.build(rec, device="cuda")
    h = pkg.kdtree.build(rec)
    _same(g, h)
    assert g.stats["n_triangles"] == h.stats["n_triangles"]


def test_gpu_build_degenerate_inputs(pkg, cuda):
    rec = sc.uniform_cube(40, seed=3)
    _same(pkg.kdtree.build(rec, device="cuda"), pkg.kdtree.build(rec))  # root stays a leaf (<= 16 IDs)
    dup = np.repeat(sc.uniform_cube(1, seed=4), 50, axis=0)  # 50 identical Gaussians
    _same(pkg.kdtree.build(dup, device="cuda"), pkg.kdtree.build(dup))
    faint = sc.uniform_cube(100, seed=5)
    faint[:, 3] = 0.001  # every Gaussian below the opacity cut
    with pytest.raises(pkg.capi.KdgrError):
        pkg.kdtree.build(faint, device="cuda")
