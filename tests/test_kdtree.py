"""The product kd-tree builder against the reference builder, `.kdt` I/O and
tree validation.  CPU only."""
import os
import struct
import subprocess

import numpy as np
import pytest

from conftest import FIXTURE_NAMES, REPO

REF_BIN = os.path.join(REPO, "oracle", "_ref", "ref_kdbuild")


@pytest.mark.parametrize("name", FIXTURE_NAMES)
def test_builder_matches_reference_golden(pkg, fixtures, name, tmp_path):
    """Bit-identical to the tree the reference's own Kd-treeConstructor.cpp
    wrote for the same scene (committed fixture)."""
    fx = fixtures[name]
    t = pkg.kdtree.build(fx.rec, max_level=24, force_split=16)
    np.testing.assert_array_equal(t.nodes, fx.tree.nodes)
    np.testing.assert_array_equal(t.offsets, fx.tree.offsets)
    np.testing.assert_array_equal(t.aabb, fx.tree.aabb)
    out = tmp_path / "mine.kdt"
    pkg.kdtree.write_kdt(t, str(out))
    assert out.read_bytes() == open(fx.kdt, "rb").read()


@pytest.mark.skipif(not os.path.exists(REF_BIN), reason="reference builder not built here")
@pytest.mark.parametrize("kind,seed,n,flags", [
    ("uniform", 11, 1500, ["-m", "24", "-f", "16"]),
    ("cluster", 12, 3000, ["-m", "24", "-f", "16"]),
    ("uniform", 13, 1200, ["-m", "12", "-f", "0"]),
    ("cluster", 14, 2500, ["-m", "24", "-f", "16", "-s", "0"]),
    ("cluster", 15, 2500, ["-m", "20", "-f", "32", "-s", "7", "-sc", "0.25"]),
    ("uniform", 16, 1500, ["-m", "24", "-f", "16", "-s", "4", "-i", "3"]),
])
def test_builder_matches_reference_live(pkg, tmp_path, kind, seed, n, flags):
    """Fresh scenes and non-default build flags against the reference binary."""
    sc = pkg.scenes
    rec = sc.uniform_cube(n, seed) if kind == "uniform" else sc.cluster_shell(n, seed, n_clusters=6)
    kdgs = tmp_path / "s.kdgs"
    sc.write_kdgs(str(kdgs), rec)
    ref = tmp_path / "ref.kdt"
    subprocess.run([REF_BIN, str(kdgs), str(ref), *flags], check=True, capture_output=True)
    kw = dict(zip(flags[0::2], flags[1::2]))
    t = pkg.kdtree.build(rec, max_level=int(kw["-m"]), force_split=int(kw["-f"]),
                         sah_mode=int(kw.get("-s", 1)), isect_cost=float(kw.get("-i", 5.0)),
                         sort_cost=float(kw.get("-sc", 0.5)))
    mine = tmp_path / "mine.kdt"
    pkg.kdtree.write_kdt(t, str(mine))
    assert mine.read_bytes() == ref.read_bytes()


def test_kdt_roundtrip_and_stats(pkg, fixtures, tmp_path):
    fx = fixtures["cluster2k"]
    p = tmp_path / "x.kdt"
    pkg.kdtree.write_kdt(fx.tree, str(p))
    t2 = pkg.kdtree.read_kdt(str(p))
    np.testing.assert_array_equal(t2.nodes, fx.tree.nodes)
    np.testing.assert_array_equal(t2.offsets, fx.tree.offsets)
    leaves = (fx.tree.nodes[:, 0] & 7) == 3
    assert t2.n_leaves == int(leaves.sum())
    assert t2.max_leaf == int((fx.tree.nodes[leaves, 0] >> 3).max())


def _write_raw(path, nodes, offsets, version=0.1, aabb=(-1, -1, -1, 1, 1, 1), truncate=0):
    b = struct.pack("<f6f", version, *aabb) + struct.pack("<i", len(nodes)) + np.array(
        nodes, np.uint32).tobytes() + struct.pack("<i", len(offsets)) + np.array(offsets, np.uint32).tobytes()
    with open(path, "wb") as f:
        f.write(b[:len(b) - truncate])


@pytest.mark.parametrize("case,status", [
    ("child_out_of_range", 5), ("leaf_range", 5), ("cycle", 5), ("truncated", 5), ("version", 5),
])
def test_corrupt_kdt_rejected(pkg, tmp_path, case, status):
    p = str(tmp_path / "bad.kdt")
    if case == "child_out_of_range":
        _write_raw(p, [[(7 << 3) | 0, 0], [3, 0], [3, 0]], [])
    elif case == "leaf_range":
        _write_raw(p, [[(5 << 3) | 3, 2]], [0, 1, 2])
    elif case == "cycle":
        _write_raw(p, [[(1 << 3) | 0, 0], [(1 << 3) | 1, 0], [3, 0]], [])
    elif case == "truncated":
        _write_raw(p, [[(1 << 3) | 3, 0]], [0], truncate=2)
    else:
        _write_raw(p, [[3, 0]], [], version=0.2)
    with pytest.raises(pkg.capi.KdgrError) as e:
        pkg.kdtree.read_kdt(p)
    assert e.value.status == status


def test_validate_rejects_bad_gaussian_id(pkg):
    t = pkg.kdtree.KdTree(np.array([[(2 << 3) | 3, 0]], np.uint32), np.array([0, 9], np.uint32),
                          np.zeros(6, np.float32))
    pkg.kdtree.validate(t, 10)
    with pytest.raises(pkg.capi.KdgrError):
        pkg.kdtree.validate(t, 9)


def test_builder_params_and_errors(pkg):
    rec = pkg.scenes.uniform_cube(800, seed=2)
    t = pkg.kdtree.build(rec, max_level=5, force_split=16)
    assert t.depth <= 5
    pkg.kdtree.validate(t, rec.shape[0])
    with pytest.raises(pkg.capi.KdgrError):
        pkg.kdtree.build(rec, sah_mode=3)
    dim = rec.copy()
    dim[:, 3] = 0.001  # every Gaussian below the opacity cut
    with pytest.raises(pkg.capi.KdgrError):
        pkg.kdtree.build(dim)


def test_builder_thread_count_does_not_change_tree(pkg):
    rec = pkg.scenes.cluster_shell(20000, seed=4, n_clusters=8)
    a = pkg.kdtree.build(rec, threads=1)
    b = pkg.kdtree.build(rec, threads=8)
    np.testing.assert_array_equal(a.nodes, b.nodes)
    np.testing.assert_array_equal(a.offsets, b.offsets)
