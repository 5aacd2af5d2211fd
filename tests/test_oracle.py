"""The CPU oracle, pinned: golden outputs, known-answer scenes, the project
exponential.  CPU only."""
import os

import numpy as np
import pytest

import kat


def caminfo_from_words(O, w):
    ci = O.CamInfo()
    ci.eye[:] = list(w[0:3])
    ci.u[:] = list(w[3:6])
    ci.v[:] = list(w[6:9])
    ci.start[:] = list(w[9:12])
    ci.step_x, ci.step_y = float(w[12]), float(w[13])
    return ci


def oscene(O, tree, rec):
    return O.OracleScene(tree.nodes, tree.offsets, tree.aabb, O.invert_scales(rec))


def test_expf_error_bound(O):
    """The oracle's exponential against double exp: <= 2 ulp on [-87, 0],
    and the relative error on the response domain [-3.6, 0] stays below
    2.5e-7."""
    xs = np.linspace(-87.0, 0.0, 200_001, dtype=np.float32)
    got = np.array([O.lib().orc_expf(float(x)) for x in xs[::7]], np.float32)
    ref = np.exp(xs[::7].astype(np.float64))
    ulp = np.abs(got.astype(np.float64) - ref) / np.spacing(ref.astype(np.float32)).astype(np.float64)
    assert ulp.max() <= 2.0, ulp.max()
    xs = np.linspace(-3.6, 0.0, 50_001, dtype=np.float32)
    got = np.array([O.lib().orc_expf(float(x)) for x in xs], np.float64)
    rel = np.abs(got - np.exp(xs.astype(np.float64))) / np.exp(xs.astype(np.float64))
    assert rel.max() < 2.5e-7, rel.max()
    assert O.lib().orc_expf(0.0) == 1.0
    assert O.lib().orc_expf(-100.0) == 0.0


def test_oracle_expf_equals_the_kernels(O, tmp_path):
    """The oracle restates the project exponential in its own code; the plain
    kernel calls the product's (3dgrt_kdtree_gb300/csrc/kdgr_math.h).  Both
    give the same bits: every float of the response domain's tail below
    -3.6 at a stride, all floats in [-3.6, 0] at a finer stride, and the
    edges of the domain."""
    import ctypes
    import subprocess
    here = os.path.dirname(os.path.abspath(__file__))
    so = str(tmp_path / "probe.so")
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-shared", "-fPIC",
                    "-I" + os.path.join(os.path.dirname(here), "3dgrt_kdtree_gb300", "csrc"),
                    os.path.join(here, "cpp", "expf_probe.c"), "-o", so, "-lm"], check=True)
    probe = ctypes.CDLL(so)
    lo = np.float32(-3.6).view(np.uint32)  # negative floats: bits grow with magnitude
    dense = np.arange(0x80000000, lo, 97, dtype=np.uint32).view(np.float32)
    tail = np.arange(lo, np.float32(-87.3).view(np.uint32), 1009, dtype=np.uint32).view(np.float32)
    edges = np.array([0.0, -0.0, -87.29, -87.3, -87.31, -100.0, 1.0, 10.0, 88.0, 88.5, np.nan], np.float32)
    xs = np.ascontiguousarray(np.concatenate([dense, tail, edges]))
    a = np.empty_like(xs)
    b = np.empty_like(xs)
    O.lib().orc_expf_n(xs.ctypes.data, a.ctypes.data, xs.size)
    probe.probe_expf_n(ctypes.c_void_p(xs.ctypes.data), ctypes.c_void_p(b.ctypes.data), ctypes.c_uint32(xs.size))
    assert xs.size > 2_000_000
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("name", ["uniform2k", "cluster2k", "dense800"])
def test_oracle_matches_golden(O, fixtures, name):
    fx = fixtures[name]
    S = oscene(O, fx.tree, fx.rec)
    for cname, cam, w, h, words in fx.cameras():
        ci = caminfo_from_words(O, words)
        rgb, a, d, tr = O.render(S, ci, w, h, trace=True)
        assert np.array_equal(rgb, fx.out[f"{cname}_rgb"])
        assert np.array_equal(a, fx.out[f"{cname}_alpha"])
        assert np.array_equal(d, fx.out[f"{cname}_depth"])
        assert np.array_equal(tr, fx.out[f"{cname}_trace"])
        r64, _, _, _ = O.render(S, ci, w, h, precision="f64")
        np.testing.assert_allclose(r64, fx.out[f"{cname}_rgb64"], rtol=0, atol=1e-12)


def test_caminfo_matches_golden(O, fixtures):
    """Host camera set-up (renderGaussianWithCudaFrame's CameraInfo) within
    one ulp of the committed words (tanf may differ by an ulp across libms)."""
    for cname, cam, w, h, words in fixtures["uniform2k"].cameras():
        ci = O.caminfo(cam, w, h)
        got = np.array(list(ci.eye) + list(ci.u) + list(ci.v) + list(ci.start) + [ci.step_x, ci.step_y],
                       np.float32)
        diff = np.abs(got.view(np.int32).astype(np.int64) - words.view(np.int32).astype(np.int64))
        assert diff.max() <= 1


def test_analytic_single_gaussian(O):
    """One Gaussian, one leaf: rgb, alpha and depth against the closed form
    t* = (mu-o)^T S^-1 d / d^T S^-1 d, response exp(-g^2/18) with g the
    squared Mahalanobis distance of the closest point, SH DC band + 0.5."""
    tree, rec, cam = kat.analytic_single()
    W, H = 32, 24
    S = oscene(O, tree, rec)
    ci = O.caminfo(cam, W, H)
    rgb, a, d, _ = O.render(S, ci, W, H)
    eye = np.array(list(ci.eye), np.float64)
    st = np.array(list(ci.start), np.float64)
    u = np.array(list(ci.u), np.float64)
    v = np.array(list(ci.v), np.float64)
    mu = rec[0, 0:3].astype(np.float64)
    s = rec[0, 4:7].astype(np.float64)
    op = float(rec[0, 3])
    col = np.maximum(0.28209479177387814 * rec[0, 12:15].astype(np.float64) + 0.5, 0.0)
    exp_rgb = np.zeros((H * W, 3))
    exp_a = np.zeros(H * W)
    exp_d = np.zeros(H * W)
    for y in range(H):
        for x in range(W):
            dirv = st + u * (x + 0.5) * ci.step_x - v * (y + 0.5) * ci.step_y - eye
            dirv /= np.linalg.norm(dirv)
            gro = (eye - mu) / s
            grd = dirv / s
            tstar = -np.dot(gro, grd) / np.dot(grd, grd)
            p = gro + tstar * grd
            g = np.dot(p, p)
            if g >= 8.0 or tstar < 0.01:
                continue
            gres = np.exp(-g * g / 18.0)
            al = min(0.99, op * gres)
            if gres < 0.0113 or al < 1 / 255:
                continue
            i = y * W + x
            exp_rgb[i] = col * al
            exp_a[i] = al
            exp_d[i] = tstar * al
    assert (exp_a > 0).sum() > 20
    np.testing.assert_allclose(rgb, exp_rgb, atol=2e-6)
    np.testing.assert_allclose(a, exp_a, atol=2e-6)
    np.testing.assert_allclose(d, exp_d, atol=1e-5)


def test_straddling_gaussian_composited_once(O):
    tree, flat, rec, cam = kat.straddle()
    W = H = 16
    rgb, a, d, tr = O.render(oscene(O, tree, rec), cam, W, H, trace=True)
    rgb_f, a_f, d_f, _ = O.render(oscene(O, flat, rec), cam, W, H)
    assert tr["n_leaf"].max() == 2 and tr["n_blend"].max() == 1
    assert (tr["n_blend"] == 1).sum() > 10
    np.testing.assert_array_equal(rgb, rgb_f)
    np.testing.assert_array_equal(a, a_f)


def test_short_stack_restart_matches_flat_tree(O):
    """20 pending far children overflow the 12-entry ring; the restart from
    the root must visit the same leaves in the same order, so the image
    equals the single-leaf render bit for bit."""
    tree, flat, rec, cam = kat.comb(20)
    W = H = 8
    rgb, a, d, tr = O.render(oscene(O, tree, rec), cam, W, H, trace=True)
    rgb_f, a_f, d_f, tr_f = O.render(oscene(O, flat, rec), cam, W, H, trace=True)
    assert tr["n_restart"].min() >= 1
    assert tr["n_leaf"].min() == 21
    np.testing.assert_array_equal(rgb, rgb_f)
    np.testing.assert_array_equal(a, a_f)
    np.testing.assert_array_equal(d, d_f)
    np.testing.assert_array_equal(tr["h_blend"], tr_f["h_blend"])


def _fnv(ids):
    h = 14695981039346656037
    for v in ids:
        for i in range(4):
            h ^= (v >> (8 * i)) & 0xFF
            h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


@pytest.mark.parametrize("order", [None, [5, 3, 19, 0, 1, 2, 4, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18]])
def test_equal_t_keeps_leaf_order(O, order):
    tree, rec, cam = kat.ties(20, order)
    W = H = 8
    _, a, _, tr = O.render(oscene(O, tree, rec), cam, W, H, trace=True)
    c = (H // 2) * W + W // 2
    expect = list(range(20)) if order is None else order
    assert tr["n_blend"][c] == 20
    assert int(tr["h_hit"][c]) == _fnv(expect)


def test_empty_scene_and_miss(O):
    tree, rec, cam = kat.empty()
    rgb, a, d, tr = O.render(oscene(O, tree, rec), cam, 8, 8, trace=True)
    assert not rgb.any() and not a.any() and tr["n_leaf"].max() == 1 and tr["n_cand"].max() == 0
    tree, rec, cam = kat.miss()
    rgb, a, d, tr = O.render(oscene(O, tree, rec), cam, 8, 8, trace=True)
    assert not rgb.any() and not a.any() and tr["n_leaf"].max() == 0


def test_fp32_vs_fp64_close(O, fixtures):
    fx = fixtures["dense800"]
    S = oscene(O, fx.tree, fx.rec)
    cname, cam, w, h, words = fx.cameras()[0]
    r32, _, _, _ = O.render(S, cam, w, h)
    r64, _, _, _ = O.render(S, cam, w, h, precision="f64")
    assert np.sqrt(((r32 - r64) ** 2).mean()) < 1e-4


def test_thin_gaussians_fp32_vs_fp64(O):
    """Very thin Gaussians (scale ratio 2000) seen edge-on and face-on: the
    FP32 transcription of the reference test stays within the fast forms'
    accuracy bar of the FP64 twin, and both composite the same leaves."""
    tree, rec, cam = kat.mixed_aniso()
    S = oscene(O, tree, rec)
    r32, a32, _, tr = O.render(S, cam, 16, 16, trace=True)
    r64, a64, _, _ = O.render(S, cam, 16, 16, precision="f64")
    assert np.sqrt(((r32 - r64) ** 2).mean()) < 1e-3
    assert np.sqrt(((a32 - a64) ** 2).mean()) < 1e-3
    assert tr["n_leaf"].max() == 2 and tr["n_blend"].max() > 0
