"""Scene ingest: kdgr_read_ply against the restatement of the reference's
loadGaussiansFromPly (oracle/ply_ref.py), and the ASCII .kdt format of
read_kd_tree_from_file / dump_kd_tree_for_composite_object.  Host only."""
import importlib
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import ply_ref  # noqa: E402

sc = importlib.import_module("3dgrt_kdtree_gb300.scenes")


def _assert_records_equal(got, want):
    """Bit-exact on every field the render path and the builder read; k_scale
    (field 7, read by neither) within 1 ulp-scale of float."""
    assert got.shape == want.shape
    cols = [i for i in range(64) if i != 7]
    np.testing.assert_array_equal(got[:, cols], want[:, cols])
    np.testing.assert_allclose(got[:, 7], want[:, 7], rtol=2e-7)


def test_ply_3dgs_layout_matches_reference_loader(pkg, tmp_path):
    raw = sc.raw_gaussians(5000, seed=3)
    raw["rot_0"][:7] = 0.0  # quaternions below the normalisation threshold stay as stored
    raw["rot_1"][:7] = 1e-3
    raw["rot_2"][:7] = 0.0
    raw["rot_3"][:7] = 0.0
    path = str(tmp_path / "scene.ply")
    sc.write_ply(path, raw)
    got = pkg.kdtree.read_ply(path)
    want = ply_ref.load_gaussians_from_ply(path)
    _assert_records_equal(got, want)
    np.testing.assert_array_equal(got[:7, 8:12], np.tile([0, 1e-3, 0, 0], (7, 1)).astype(np.float32))
    q = got[7:, 8:12].astype(np.float64)
    np.testing.assert_allclose((q * q).sum(1), 1.0, atol=1e-6)
    assert (got[:, 60:] == 0).all()


def test_ply_property_order_and_extra_properties(pkg, tmp_path):
    """Fields are found by name wherever the header puts them; properties of
    other sizes (uchar, double, int) shift the offsets."""
    raw = sc.raw_gaussians(777, seed=4)
    rng = np.random.default_rng(0)
    head = ["opacity", "rot_0", "rot_1", "rot_2", "rot_3", "z", "y", "x", "scale_0", "scale_1", "scale_2"]
    rest = [f"f_rest_{i}" for i in range(45)]
    order = head + ["f_dc_0", "f_dc_1", "f_dc_2"] + rest
    path = str(tmp_path / "shuffled.ply")
    sc.write_ply(path, raw, order=order,
                 extra=[("uchar", "red", rng.integers(0, 255, 777)), ("double", "weight", rng.normal(size=777))])
    ref_path = str(tmp_path / "std.ply")
    sc.write_ply(ref_path, raw)
    _assert_records_equal(pkg.kdtree.read_ply(path), pkg.kdtree.read_ply(ref_path))
    # x, y, z written in reverse order: the reference would copy three floats
    # from the offset of x, so compare with the restatement on the standard file
    _assert_records_equal(pkg.kdtree.read_ply(path), ply_ref.load_gaussians_from_ply(ref_path))


def test_ply_without_higher_sh(pkg, tmp_path):
    raw = sc.raw_gaussians(100, seed=5)
    order = [f for f in sc.PLY_FIELDS if not f.startswith("f_rest")]
    path = str(tmp_path / "dc_only.ply")
    sc.write_ply(path, raw, order=order)
    got = pkg.kdtree.read_ply(path)
    _assert_records_equal(got, ply_ref.load_gaussians_from_ply(path))
    assert (got[:, 15:60] == 0).all()


@pytest.mark.parametrize("case", ["ascii", "missing_field", "truncated", "not_ply", "no_vertices", "list_prop"])
def test_ply_rejects_malformed_files(pkg, tmp_path, case):
    raw = sc.raw_gaussians(10, seed=6)
    path = str(tmp_path / f"{case}.ply")
    sc.write_ply(path, raw)
    data = open(path, "rb").read()
    if case == "ascii":
        data = data.replace(b"binary_little_endian", b"ascii")
    elif case == "missing_field":
        data = data.replace(b"property float rot_3\n", b"property float rot_x\n")
    elif case == "truncated":
        data = data[:-100]
    elif case == "not_ply":
        data = b"plx" + data[3:]
    elif case == "no_vertices":
        data = data.replace(b"element vertex 10\n", b"element vertex 0\n")
    elif case == "list_prop":
        data = data.replace(b"property float nx\n", b"property list uchar int nx\n")
    open(path, "wb").write(data)
    with pytest.raises(pkg.capi.KdgrError) as e:
        pkg.kdtree.read_ply(path)
    assert e.value.status == 5  # KDGR_ERR_FORMAT
    with pytest.raises(pkg.capi.KdgrError) as e:
        pkg.kdtree.read_ply(str(tmp_path / "absent.ply"))
    assert e.value.status == 4  # KDGR_ERR_IO


def test_ply_to_tree_to_oracle_image(pkg, O, tmp_path):
    """The ingest path end to end on the host: PLY -> records -> builder ->
    .kdt round trip -> oracle render sees the scene."""
    raw = sc.raw_gaussians(1500, seed=7)
    path = str(tmp_path / "s.ply")
    sc.write_ply(path, raw)
    rec = pkg.kdtree.read_ply(path)
    tree = pkg.kdtree.build(rec)
    kdt = str(tmp_path / "s.kdt")
    pkg.kdtree.write_kdt(tree, kdt)
    t2 = pkg.kdtree.read_kdt(kdt)
    np.testing.assert_array_equal(t2.nodes, tree.nodes)
    S = O.OracleScene(t2.nodes, t2.offsets, t2.aabb, O.invert_scales(rec))
    rgb, a, _, _ = O.render(S, sc.front_camera(32, 32), 32, 32)
    assert a.max() > 0.5


def _ascii_expected(tree):
    lines = [f"n{tree.nodes.shape[0]}"]
    for x, y in tree.nodes:
        x, y = int(x), int(y)
        if x & 7 == 3:
            lines.append(f"L cnt:{x >> 3} off:{y}")
        else:
            split = float(np.array([y], np.uint32).view(np.float32)[0])
            lines.append("%s|%f %d<>%d" % ("XYZ"[x & 3], split, x >> 3, (x >> 3) + 1))
    lines.append(f"o{tree.offsets.shape[0]}")
    lines += [str(int(i)) for i in tree.offsets]
    return "\n".join(lines) + "\n"


def test_kdt_ascii_format(pkg, fixtures, tmp_path):
    fx = fixtures["cluster2k"]
    p = str(tmp_path / "t.txt")
    pkg.kdtree.write_kdt(fx.tree, p, ascii=True)
    assert open(p).read() == _ascii_expected(fx.tree)
    t = pkg.kdtree.read_kdt(p, ascii=True)
    assert (np.asarray(t.aabb) == 0).all()
    # topology and IDs survive; split planes are rounded to six decimals
    np.testing.assert_array_equal(t.nodes[:, 0], fx.tree.nodes[:, 0])
    np.testing.assert_array_equal(t.offsets, fx.tree.offsets)
    inner = (fx.tree.nodes[:, 0] & 7) != 3
    a = fx.tree.nodes[inner, 1].view(np.float32).astype(np.float64)
    b = t.nodes[inner, 1].view(np.float32).astype(np.float64)
    assert np.abs(a - b).max() <= 5e-7 + 1e-6 * np.abs(a).max()
    np.testing.assert_array_equal(t.nodes[~inner], fx.tree.nodes[~inner])
    # a second round trip is stable
    p2 = str(tmp_path / "t2.txt")
    pkg.kdtree.write_kdt(t, p2, ascii=True)
    assert open(p2).read() == open(p).read()


def test_kdt_ascii_rejects_malformed(pkg, fixtures, tmp_path):
    p = str(tmp_path / "t.txt")
    pkg.kdtree.write_kdt(fixtures["uniform2k"].tree, p, ascii=True)
    lines = open(p).read().splitlines()
    for bad in (["x5"] + lines[1:], lines[:3], lines[:1] + ["Q|0.5 1<>2"] + lines[2:]):
        open(p, "w").write("\n".join(bad) + "\n")
        with pytest.raises(pkg.capi.KdgrError) as e:
            pkg.kdtree.read_kdt(p, ascii=True)
        assert e.value.status == 5
