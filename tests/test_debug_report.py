"""kdgr_debug_report: the reference's HIT_AND_NODE_COUNT_DEBUG report
(cudaRenderer.cu:3173-3400) over per-pixel traces, checked file by file
against a restatement of the reference's host code in numpy (FP32 sums in
pixel order, the Turbo polynomial in FP32, the CSV/text/binary layouts).
Host only: the traces are the committed oracle traces of the golden scenes.
"""
import os
import struct
import zlib

import numpy as np
import pytest

NAMES = ("node_visits", "leaf_visits", "intersection", "hits_found", "blend_ops", "max_sort_size")
FIELDS = ("n_inner", "n_leaf", "n_cand", "n_found", "n_blend", "max_sort")
STAT = ("node_visits", "leaf_visits", "intersection_tests", "hits_found", "blend_ops", "max_sort_size")
TABS = (2, 2, 1, 2, 2, 1)
f32 = np.float32

# Turbo polynomial approximation (published), as the reference's host helper
# evaluates it (cudaRenderer.cu:2985-3007)
K4 = [(0.13572138, 4.61539260, -42.66032258, 132.13108234),
      (0.09140261, 2.19418839, 4.84296658, -14.18503333),
      (0.10667330, 12.64194608, -60.58204836, 110.36276771)]
K2 = [(-152.94239396, 59.28637943), (4.27729857, 2.82956604), (-89.90310912, 27.34824973)]


def turbo_bytes(v, max_val):
    x = f32(v) / f32(max_val)
    x = min(max(x, f32(0)), f32(1))
    p = [f32(1), x, x * x, x * x * x]
    q = [p[2] * p[2], p[3] * p[2]]
    out = []
    for c in range(3):
        k4 = [f32(k) for k in K4[c]]
        k2 = [f32(k) for k in K2[c]]
        s = ((k4[0] * p[0] + k4[1] * p[1]) + k4[2] * p[2]) + k4[3] * p[3]
        s = s + (k2[0] * q[0] + k2[1] * q[1])
        b = s * f32(255) + f32(0.5)
        out.append(int(min(max(b, f32(0)), f32(255))))
    return out


def read_png_rgb(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", None, None
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(typ + body) & 0xFFFFFFFF
        if typ == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert (depth, ctype) == (8, 2)
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(h, 3 * w + 1)
    assert (rows[:, 0] == 0).all()
    return rows[:, 1:].reshape(h, w, 3)


def expected_report(tr, W, H):
    sums = [f32(0)] * 6
    n = 0
    mx = [0] * 6
    hist_node, hist_leaf = {}, {}
    for i in range(W * H):
        vals = [int(tr[f][i]) for f in FIELDS]
        mx = [max(a, b) for a, b in zip(mx, vals)]
        if vals[4] != 0:
            sums = [s + f32(v) for s, v in zip(sums, vals)]
            n += 1
            hist_node[vals[0]] = hist_node.get(vals[0], 0) + 1
            hist_leaf[vals[1]] = hist_leaf.get(vals[1], 0) + 1
    rule = "===========================================\n"
    txt = "\n" + rule
    txt += "".join(f"avg_{s}" + "\t" * t + ": %f\n" % float(sums[k] / f32(n)) for k, (s, t) in enumerate(zip(STAT, TABS)))
    txt += rule + "".join(f"max_{s}" + "\t" * t + f": {mx[k]}\n" for k, (s, t) in enumerate(zip(STAT, TABS)))
    txt += rule + "".join(f"tot_{s}" + "\t" * t + ": %f\n" % float(sums[k]) for k, (s, t) in enumerate(zip(STAT, TABS)))
    txt += rule
    hist = "Value,Node_Visits,Leaf_Visits\n" + "".join(
        f"{v},{hist_node.get(v, 0)},{hist_leaf.get(v, 0)}\n" for v in sorted(set(hist_node) | set(hist_leaf)))
    return sums, n, mx, txt, hist


@pytest.mark.parametrize("fixture", ["dense800", "uniform2k"])
def test_report_matches_reference_restatement(pkg, fixtures, fixture, tmp_path):
    fx = fixtures[fixture]
    F = pkg.renderer
    for cname, cam, W, H, _ in fx.cameras():
        tr = fx.out[f"{cname}_trace"]
        d = tmp_path / cname
        d.mkdir()
        st = F.debug_report(tr, W, H, out_dir=str(d))
        sums, n, mx, txt, hist = expected_report(tr, W, H)
        assert st["n_pixels"] == n > 0
        for k, name in enumerate(F.DEBUG_COUNTERS):
            assert st[name]["total"] == sums[k]
            assert st[name]["avg"] == f32(sums[k] / f32(n))
            assert st[name]["max"] == mx[k]
        assert (d / "renderStats.txt").read_text() == txt
        assert (d / "render_stats.csv").read_text() == hist
        for k, (name, field) in enumerate(zip(NAMES, FIELDS)):
            v = tr[field].astype(np.int64).reshape(H, W)
            csv = "".join(",".join(str(x) for x in row) + "\n" for row in v)
            assert (d / f"heatmap_{name}.csv").read_text() == csv
            img = read_png_rgb(str(d / f"heatmap_{name}.png"))
            assert img.shape == (H, W, 3)
            want = np.zeros((H, W, 3), np.uint8)
            for val in np.unique(v):
                if val > 0:
                    want[v == val] = turbo_bytes(val, 120.0)
            np.testing.assert_array_equal(img, want)
        assert np.array_equal(np.fromfile(d / "isectCnt_kd.bin", "<u4"), tr["n_found"])
        assert np.array_equal(np.fromfile(d / "blendCnt_kd.bin", "<u4"), tr["n_blend"])


def test_counter_semantics_on_oracle_traces(fixtures):
    """n_found counts every accepted hit of each visited leaf, n_hit only those
    the compositing loop reached before saturating, so n_found >= n_hit;
    max_sort is a per-leaf count, bounded by n_found."""
    for fx in fixtures.values():
        for cname in ("front", "orbit"):
            tr = fx.out[f"{cname}_trace"]
            assert (tr["n_found"] >= tr["n_hit"]).all()
            assert (tr["max_sort"] <= tr["n_found"]).all()
            assert ((tr["max_sort"] > 0) == (tr["n_found"] > 0)).all()
            assert (tr["n_found"] <= tr["n_cand"]).all()


def test_report_stats_only_and_bad_args(pkg, fixtures, tmp_path):
    F = pkg.renderer
    tr = fixtures["cluster2k"].out["front_trace"]
    st = F.debug_report(tr, 48, 40)
    assert st["blend_ops"]["max"] >= 1 and not os.listdir(tmp_path)
    empty = np.zeros(4, dtype=np.dtype(pkg.capi.TRACE_DTYPE))
    st = F.debug_report(empty, 2, 2, out_dir=str(tmp_path))
    assert st["n_pixels"] == 0 and np.isnan(st["node_visits"]["avg"])
    assert "avg_node_visits\t\t: nan" in (tmp_path / "renderStats.txt").read_text()
    with pytest.raises(pkg.capi.KdgrError):
        F.debug_report(tr, 48, 40, heat_max=0.0)
    with pytest.raises(pkg.capi.KdgrError):
        F.debug_report(tr, 48, 40, out_dir=str(tmp_path / "missing_dir"))


@pytest.mark.gpu
def test_kernel_counters_feed_the_same_report(pkg, cuda, fixtures, tmp_path):
    """Scene.debug_counters (the oracle-matching kernel in trace mode) gives
    the oracle's counters, so the report is the oracle's report."""
    F = pkg.renderer
    fx = fixtures["dense800"]
    scene = F.Scene(fx.tree, fx.rec)
    for cname, cam, W, H, _ in fx.cameras():
        tr = scene.debug_counters(cam, W, H)
        np.testing.assert_array_equal(tr, fx.out[f"{cname}_trace"])
        assert F.debug_report(tr, W, H) == F.debug_report(fx.out[f"{cname}_trace"], W, H)
    scene.close()
