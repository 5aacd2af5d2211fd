"""The render oracle pinned to mathematics, not to its own transcription.

Each known-answer scene's expected image comes from tests/closed_form.py:
real spherical harmonics from the associated-Legendre closed form, ray
geometry and the front-to-back recurrence in double precision.  The same
expectations then pin the plain GPU kernel (bit-exact to the oracle) and the
fast forms (-m gpu tests at the end of this file).

* every SH basis function of bands 1-3 alone, for each colour channel, at
  ray directions covering the sphere (the normalisation constants of
  cudaRenderer.h:33-48 and the terms of cudaRenderer.cu:519-551 must
  reproduce the closed form);
* five Gaussians on one ray in a shuffled leaf: front-to-back order, the
  0.99 alpha cap and the 1/255 skip (cudaRenderer.cu:1608-1688);
* accumulated opacity reaching exactly 0.99: the walk goes on inside a leaf
  (stops only when A > 0.99, :1683) and stops at a leaf boundary
  (while A < 0.99, :1552, 1694).
"""
import numpy as np
import pytest

import closed_form as CF
import kat

# FP32 transcription against the double-precision closed form (whose ray
# directions are formed in FP32 like the reference's).  The colour term is
# compared at the render's own alpha (rgb = colour x alpha for one
# Gaussian); alpha to 5e-5 relative (the FP32 |grd x gro|^2 of the reference
# cancels when the eye is many sigma away); composites to 2e-5, and their
# structure exactly (Gaussians accepted and blended per ray, A == 0.99).
COL_TOL = 2e-6
ALPHA_RTOL = 5e-5
COMP_TOL = 2e-5
DEPTH_TOL = 1e-4
FAST_TOL = 2e-4  # fast forms, colour term: FMA, fast reciprocal and exponential


def oscene(O, tree, rec):
    return O.OracleScene(tree.nodes, tree.offsets, tree.aabb, O.invert_scales(rec))


def sh_expect(O, rec, cam, w, h):
    """(colour (n,3), alpha (n,)) where alpha is the closed-form alpha of the
    single Gaussian (rays that do not accept it have alpha 0)."""
    ci = O.caminfo(cam, w, h)
    eye, d = CF.ray_dirs(ci, w, h)
    tn, tf = CF.slab(rec_aabb(), eye, d)
    out = CF.composite(rec, [([0], tn, tf)], eye, d, None)
    return CF.colour(rec[0], d), out["alpha"], out["g"][0]


def rec_aabb():
    return (-1.0, -1.0, -1.0, 1.0, 1.0, 1.0)


SH_CASES = [(k, c) for k in range(1, 16) for c in range(3)]


def check_sh(rgb, alpha, want_col, want_a, g, tol=COL_TOL):
    keep = (want_a > 0) & (np.abs(g - 8.0) > 1e-3)
    assert keep.sum() > 100
    np.testing.assert_allclose(alpha[keep], want_a[keep], rtol=ALPHA_RTOL, atol=1e-7)
    np.testing.assert_allclose(rgb[keep], want_col[keep] * alpha[keep, None], rtol=0, atol=tol)


@pytest.mark.parametrize("k,channel", SH_CASES)
def test_oracle_sh_basis_closed_form(O, k, channel):
    coef = 0.45 if k % 2 else -0.4
    tree, rec, cams = kat.sh_probe(k, channel, coef)
    S = oscene(O, tree, rec)
    dirs = []
    for cam, w, h in cams:
        rgb, a, _, _ = O.render(S, cam, w, h)
        want_col, want_a, g = sh_expect(O, rec, cam, w, h)
        check_sh(rgb, a, want_col, want_a, g)
        dirs.append(CF.ray_dirs(O.caminfo(cam, w, h), w, h)[1][want_a > 0])
    # the directions seen cover the sphere: every octant
    dirs = np.concatenate(dirs)
    octants = {tuple(s) for s in (dirs > 0).astype(int)}
    assert len(octants) == 8


def test_sh_constants_are_the_closed_form():
    """The degree-3 normalisation constants of the reference's SH table
    (cudaRenderer.h:33-48), with the sign of each basis polynomial, equal the
    closed form at a generic direction."""
    d = np.array([[0.3, -0.5, 0.8]])
    d /= np.linalg.norm(d)
    x, y, z = d[0]
    poly = [1.0, y, z, x, x * y, y * z, 2 * z * z - x * x - y * y, x * z, x * x - y * y,
            y * (3 * x * x - y * y), x * y * z, y * (4 * z * z - x * x - y * y),
            z * (2 * z * z - 3 * x * x - 3 * y * y), x * (4 * z * z - x * x - y * y), z * (x * x - y * y),
            x * (x * x - 3 * y * y)]
    table = [0.28209479177387814, -0.4886025119029199, 0.4886025119029199, -0.4886025119029199,
             1.0925484305920792, -1.0925484305920792, 0.31539156525252005, -1.0925484305920792,
             0.5462742152960396, -0.5900435899266435, 2.890611442640554, -0.4570457994644658,
             0.3731763325901154, -0.4570457994644658, 1.445305721320277, -0.5900435899266435]
    for k in range(16):
        l, m = CF.sh_index(k)
        assert abs(CF.real_sh(l, m, d)[0] - table[k] * poly[k]) < 1e-14, k


def row_expect(O, tree, rec, cam, w, h, split_z=None):
    ci = O.caminfo(cam, w, h)
    eye, d = CF.ray_dirs(ci, w, h)
    tn, tf = CF.slab(tree.aabb, eye, d)
    if split_z is None:
        leaves = [(list(range(rec.shape[0])), tn, tf)]
    else:
        ts = (split_z - eye[2]) / d[:, 2]
        front = [i for i in range(rec.shape[0]) if rec[i, 2] > split_z]
        back = [i for i in range(rec.shape[0]) if rec[i, 2] <= split_z]
        leaves = [(front, tn, np.minimum(ts, tf)), (back, np.maximum(ts, tn), tf)]
    return CF.composite(rec, leaves, eye, d, None)


def check_composite(rgb, a, dep, want, tol=COMP_TOL, dtol=DEPTH_TOL):
    keep = (np.abs(want["g"] - 8.0) > 1e-3).all(0)
    assert keep.mean() > 0.95
    np.testing.assert_allclose(a[keep], want["alpha"][keep], rtol=0, atol=tol)
    np.testing.assert_allclose(rgb[keep], want["rgb"][keep], rtol=0, atol=tol)
    np.testing.assert_allclose(dep[keep], want["depth"][keep], rtol=0, atol=dtol)
    return keep


def test_oracle_row_front_to_back(O):
    tree, rec, cam = kat.row()
    w = h = 32
    rgb, a, dep, tr = O.render(oscene(O, tree, rec), cam, w, h, trace=True)
    want = row_expect(O, tree, rec, cam, w, h)
    keep = check_composite(rgb, a, dep, want)
    # composite structure exactly: Gaussians accepted and blended per ray
    assert np.array_equal(tr["n_found"][keep], want["n_accept"][keep])
    assert np.array_equal(tr["n_blend"][keep], want["n_blend"][keep])
    # the scene exercises what it is meant to: >= 3 Gaussians blended on most
    # rays, the 0.99 cap near the axis, the 1/255 skip of the third Gaussian
    assert (want["n_blend"][keep] >= 3).mean() > 0.5
    assert (np.exp(-want["g"][3] ** 2 / 18.0) >= 0.99).sum() > 10
    assert (want["n_accept"] > want["n_blend"]).sum() > 100


@pytest.mark.parametrize("split", [False, True])
def test_oracle_opacity_exactly_099(O, split):
    tree, rec, cam = kat.exact_099(split)
    w = h = 24
    rgb, a, dep, tr = O.render(oscene(O, tree, rec), cam, w, h, trace=True)
    want = row_expect(O, tree, rec, cam, w, h, split_z=0.0 if split else None)
    keep = check_composite(rgb, a, dep, want)
    assert np.array_equal(tr["n_blend"][keep], want["n_blend"][keep])
    capped = np.exp(-want["g"][0] ** 2 / 18.0) >= 0.99 + 1e-6
    assert capped.sum() > 10
    # P alone brings A to exactly 0.99 (FP32 0.99f)
    if split:
        assert (a[capped] == np.float32(0.99)).all()
        assert (tr["n_blend"][capped] == 1).all()
    else:
        assert (a[capped] > np.float32(0.99)).all()
        assert (tr["n_blend"][capped] == 2).all()


# ------------------------------------------------------------------ GPU
def _gpu_images(pkg, dev, tree, rec, cams):
    """Per (camera, W, H): the plain kernel, the fast FP32 and the precision
    form, each (rgb, alpha, depth) in kernel pixel order (y*W + x)."""
    import torch
    F = pkg.renderer
    scene = F.Scene(tree, rec, forms=F.FORM_EXACT | F.FORM_FAST | F.FORM_PACKED)
    res = []
    for cam, w, h in cams:
        out = {}
        for name in ("plain", "fast", "packed"):
            rgb = torch.zeros(w * h * 3, device=dev)
            a = torch.zeros(w * h, device=dev)
            dep = torch.zeros(w * h, device=dev)
            if name == "plain":
                scene.render(cam, w, h, rgb, a, dep)
            else:
                scene.render_fast(cam, w, h, rgb, a, dep, precision=1 if name == "packed" else 0)
            torch.cuda.synchronize()
            assert scene.status() == 0
            flip = lambda t, c: t.cpu().numpy().reshape(h, w, *c)[::-1].reshape(w * h, *c)
            out[name] = (flip(rgb, (3,)), flip(a, ()), flip(dep, ()))
        res.append(out)
    scene.close()
    return res


@pytest.mark.gpu
@pytest.mark.parametrize("k", range(1, 16))
def test_gpu_sh_basis_closed_form(pkg, O, cuda, k):
    for channel in range(3):
        tree, rec, cams = kat.sh_probe(k, channel, 0.45 if k % 2 else -0.4)
        for (cam, w, h), imgs in zip(cams, _gpu_images(pkg, cuda, tree, rec, cams)):
            want_col, want_a, g = sh_expect(O, rec, cam, w, h)
            check_sh(imgs["plain"][0], imgs["plain"][1], want_col, want_a, g)
            keep = (want_a > 0) & (np.abs(g - 8.0) > 1e-3)
            for form in ("fast", "packed"):
                rgb, a, _ = imgs[form]
                tol = FAST_TOL if form == "fast" else 4e-3  # BF16 coefficients: 2^-9 relative
                np.testing.assert_allclose(rgb[keep], want_col[keep] * a[keep, None], rtol=0, atol=tol)
                np.testing.assert_allclose(a[keep], want_a[keep], rtol=2e-3, atol=1e-6)


@pytest.mark.gpu
def test_gpu_row_front_to_back(pkg, O, cuda):
    tree, rec, cam = kat.row()
    w = h = 32
    imgs = _gpu_images(pkg, cuda, tree, rec, [(cam, w, h)])[0]
    want = row_expect(O, tree, rec, cam, w, h)
    check_composite(*imgs["plain"], want)
    check_composite(*imgs["fast"], want, tol=FAST_TOL, dtol=1e-3)
    check_composite(*imgs["packed"], want, tol=4e-3, dtol=1e-2)


@pytest.mark.gpu
@pytest.mark.parametrize("split", [False, True])
def test_gpu_opacity_exactly_099(pkg, O, cuda, split):
    tree, rec, cam = kat.exact_099(split)
    w = h = 24
    imgs = _gpu_images(pkg, cuda, tree, rec, [(cam, w, h)])[0]
    want = row_expect(O, tree, rec, cam, w, h, split_z=0.0 if split else None)
    capped = np.exp(-want["g"][0] ** 2 / 18.0) >= 0.99 + 1e-6
    check_composite(*imgs["plain"], want)
    for form in ("plain", "fast", "packed"):
        a = imgs[form][1]
        if split:
            assert (a[capped] == np.float32(0.99)).all(), form
        else:
            assert (a[capped] > np.float32(0.99)).all(), form
    check_composite(*imgs["fast"], want, tol=FAST_TOL, dtol=1e-3)
