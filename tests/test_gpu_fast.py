"""Batching and precision forms against the FP64 oracle (<= 1e-3 RMSE),
batch/graph/single-view equivalence, autotuner.  Through the C ABI."""
import numpy as np
import pytest
import torch

from gpu_util import oracle_image

pytestmark = pytest.mark.gpu

RMSE_TOL = 1e-3  # the fast forms' accuracy bar against the FP64 oracle


def fast_image(pkg, dev, scene, cam, W, H, precision=0):
    rgb = torch.zeros(W * H * 3, device=dev)
    alpha = torch.zeros(W * H, device=dev)
    scene.render_fast(cam, W, H, rgb, alpha, precision=precision)
    torch.cuda.synchronize()
    assert scene.status() == 0
    return rgb.cpu().numpy().reshape(H, W, 3), alpha.cpu().numpy().reshape(H, W)


def rmse(a, b):
    return float(np.sqrt(((a.astype(np.float64) - b) ** 2).mean()))


@pytest.mark.parametrize("name", ["uniform2k", "cluster2k", "dense800"])
def test_fast_forms_vs_fp64(pkg, O, cuda, fixtures, name):
    fx = fixtures[name]
    F = pkg.renderer
    scene = F.Scene(fx.tree, fx.rec, forms=F.FORM_FAST | F.FORM_PACKED)
    for _, cam, w, h, _ in fx.cameras():
        r64, a64, _, _ = oracle_image(O, fx.tree, fx.rec, cam, w, h, precision="f64")
        for prec in (0, 1):
            rgb, a = fast_image(pkg, cuda, scene, cam, w, h, prec)
            assert rmse(rgb, r64) <= RMSE_TOL, (prec, rmse(rgb, r64))
            assert rmse(a, a64) <= RMSE_TOL
    scene.close()


def test_fast_forms_at_scale_vs_fp64(pkg, O, cuda):
    """A 300k-Gaussian cluster+shell scene with the 5% anisotropic tail (some
    Gaussians above scale ratio 1e3 take the FP64-precomputed factors)."""
    sc = pkg.scenes
    rec = sc.cluster_shell(300_000, seed=2, n_clusters=32)
    tree = pkg.kdtree.build(rec)
    F = pkg.renderer
    scene = F.Scene(tree, rec, forms=F.FORM_FAST | F.FORM_PACKED)
    n_aniso = scene.info()["n_aniso"]
    assert n_aniso > 0 and abs(n_aniso - int((sc.scale_ratio(rec) > 1e3).sum())) <= 2
    W, H = 320, 180
    cam = sc.front_camera(W, H)
    r64, _, _, _ = oracle_image(O, tree, rec, cam, W, H, precision="f64")
    for prec in (0, 1):
        rgb, _ = fast_image(pkg, cuda, scene, cam, W, H, prec)
        assert rmse(rgb, r64) <= RMSE_TOL, (prec, rmse(rgb, r64))
    scene.close()


def test_batch_equals_single_views_and_graph(pkg, cuda, fixtures):
    fx = fixtures["dense800"]
    F = pkg.renderer
    sc = pkg.scenes
    scene = F.Scene(fx.tree, fx.rec)
    cams = sc.sphere_cameras(6, seed=3, resolutions=[(40, 30), (64, 48), (17, 9)])
    views, total, offs = F.make_views(cams)
    rgb = torch.zeros(total * 3, device=cuda)
    alpha = torch.zeros(total, device=cuda)
    scene.render_batch(views, len(cams), rgb, alpha)
    torch.cuda.synchronize()
    batch = rgb.cpu().numpy().copy()
    for (cam, w, h), off in zip(cams, offs):
        single, _ = fast_image(pkg, cuda, scene, cam, w, h)
        np.testing.assert_array_equal(batch[3 * off:3 * (off + w * h)].reshape(h, w, 3), single)
    rgb2 = torch.zeros_like(rgb)
    g = F.Batch(scene, views, len(cams), rgb2, None, None)
    for _ in range(3):
        g.run()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(rgb2.cpu().numpy(), batch)
    g.close()
    scene.close()


def test_batch_output_in_pinned_host_memory(pkg, cuda, fixtures):
    """Output buffers may be pinned host memory: the kernel writes the frame
    straight into it, bit-identical to a device buffer."""
    fx = fixtures["cluster2k"]
    F = pkg.renderer
    scene = F.Scene(fx.tree, fx.rec)
    cams = pkg.scenes.sphere_cameras(3, seed=14, resolutions=[(64, 48), (17, 9)])
    views, total, _ = F.make_views(cams)
    dev_rgb = torch.zeros(total * 3, device=cuda)
    dev_a = torch.zeros(total, device=cuda)
    scene.render_batch(views, len(cams), dev_rgb, dev_a)
    host_rgb = torch.full((total * 3,), -1.0).pin_memory()
    host_a = torch.full((total,), -1.0).pin_memory()
    scene.render_batch(views, len(cams), host_rgb, host_a)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(host_rgb.numpy(), dev_rgb.cpu().numpy())
    np.testing.assert_array_equal(host_a.numpy(), dev_a.cpu().numpy())
    assert scene.status() == 0
    scene.close()


@pytest.mark.parametrize("n_views", [1, 256, 257, 300])
def test_view_table_sizes(pkg, cuda, fixtures, n_views):
    """kdgr_render_batch stages up to 256 views through a kernel's parameters
    and copies larger tables; both give the frames of the graph-captured
    batch, which uploads its table once at creation, and the calls stay
    repeatable (the scratch comes back from the library's pool)."""
    fx = fixtures["dense800"]
    F = pkg.renderer
    scene = F.Scene(fx.tree, fx.rec)
    cams = pkg.scenes.sphere_cameras(n_views, seed=31, resolutions=[(16, 16), (24, 8)])
    views, total, _ = F.make_views(cams)
    ref = torch.zeros(total * 3, device=cuda)
    b = F.Batch(scene, views, n_views, ref, None, None, F.BatchConfig.default())
    b.run()
    for _ in range(2):
        rgb = torch.full((total * 3,), -1.0, device=cuda)
        scene.render_batch(views, n_views, rgb)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(rgb.cpu().numpy(), ref.cpu().numpy())
    assert float(ref.abs().sum()) > 0
    assert scene.status() == 0
    b.close()
    scene.close()


def test_every_schedule_renders_the_same_pixels(pkg, cuda, fixtures):
    """Warp tiles, CTA blocks, SM strips and warp strips (with several chunk sizes and
    register caps) only change which lane renders which pixel; warp packets
    and per-ray traversal give every ray the same leaves and intervals, for
    every warp tile shape."""
    fx = fixtures["cluster2k"]
    F = pkg.renderer
    scene = F.Scene(fx.tree, fx.rec)
    cams = pkg.scenes.sphere_cameras(5, seed=12, resolutions=[(67, 41), (96, 64), (8, 3)])
    views, total, _ = F.make_views(cams)
    ref = torch.zeros(total * 3, device=cuda)
    ref_a = torch.zeros(total, device=cuda)
    scene.render_batch(views, len(cams), ref, ref_a)
    for sched, chunk, minb, kb, trav, tile in [(0, 1, 0, 4, 0, 0), (0, 3, 8, 8, 0, 0), (0, 7, 6, 4, 1, 0),
                                               (1, 1, 6, 8, 0, 1), (1, 2, 0, 4, 1, 2), (1, 5, 8, 4, 0, 0),
                                               (2, 1, 0, 8, 1, 0), (2, 1, 8, 4, 0, 2), (1, 1, 8, 4, 1, 1),
                                               (2, 1, 8, 8, 1, 1), (3, 1, 8, 4, 0, 0), (3, 1, 0, 8, 1, 2),
                                               (3, 1, 6, 4, 0, 1)]:
        cfg = F.BatchConfig(sched, minb, 0, chunk, 0, kb, trav, tile, 32)
        out = torch.full_like(ref, -1.0)
        out_a = torch.full_like(ref_a, -1.0)
        scene.render_batch(views, len(cams), out, out_a, cfg=cfg)
        torch.cuda.synchronize()
        assert float((out - ref).abs().max()) <= 1e-5, (sched, chunk, minb, trav, tile)
        assert float((out_a - ref_a).abs().max()) <= 1e-5, (sched, chunk, minb, trav, tile)
    scene.close()


@pytest.mark.parametrize("name", ["cluster2k", "dense800", "uniform2k"])
def test_rays_per_warp_renders_the_same_pixels(pkg, cuda, fixtures, name):
    """16 or 8 rays per warp (2 or 4 lanes sharing each ray, each testing
    every 2nd or 4th candidate pair, hits merged in key order across the
    lanes) composite exactly the hits of 32 rays per warp in the same order:
    the pixels, alpha and depth are bit-identical, for both forms, both
    traversals, both hit buffer sizes and every register cap."""
    fx = fixtures[name]
    F = pkg.renderer
    scene = F.Scene(fx.tree, fx.rec, forms=F.FORM_FAST | F.FORM_PACKED)
    cams = pkg.scenes.sphere_cameras(5, seed=13, resolutions=[(67, 41), (96, 64), (8, 3)])
    views, total, _ = F.make_views(cams)
    for prec in (0, 1):
        ref = [torch.zeros(total * 3, device=cuda), torch.zeros(total, device=cuda), torch.zeros(total, device=cuda)]
        scene.render_batch(views, len(cams), *ref, cfg=F.BatchConfig(3, 8, 0, 1, prec, 4, 0, 0, 32))
        for rpw, minb, kb, trav in [(16, 8, 4, 0), (8, 8, 4, 0), (16, 0, 8, 0), (8, 6, 8, 0), (16, 8, 4, 1),
                                    (8, 8, 4, 1), (8, 0, 8, 1)]:
            out = [torch.full_like(t, -1.0) for t in ref]
            scene.render_batch(views, len(cams), *out, cfg=F.BatchConfig(3, minb, 0, 1, prec, kb, trav, 0, rpw))
            torch.cuda.synchronize()
            for a, b in zip(out, ref):
                np.testing.assert_array_equal(a.cpu().numpy(), b.cpu().numpy())
    assert scene.status() == 0
    scene.close()


def test_autotune_picks_a_valid_config(pkg, cuda, fixtures):
    fx = fixtures["cluster2k"]
    F = pkg.renderer
    scene = F.Scene(fx.tree, fx.rec)
    cams = pkg.scenes.sphere_cameras(4, seed=9, resolutions=[(64, 64)])
    views, total, _ = F.make_views(cams)
    rgb = torch.zeros(total * 3, device=cuda)
    best, report = scene.autotune(views, len(cams), rgb)
    assert best.schedule in (0, 1, 2, 3) and best.chunk in (1, 2) and best.min_blocks in (0, 6, 8)
    # 18 stage-1 lines, then 8-entry buffer, per-ray traversal, (unless the
    # warp-tile schedule won stage 1) the 4x8 and 16x2 tile shapes, and 16 and
    # 8 rays per warp with either traversal
    assert len(report.strip().splitlines()) in (24, 26)
    assert best.hit_buffer in (4, 8) and best.traversal in (F.TRAV_PACKET, F.TRAV_RAY)
    assert best.tile_shape in (F.TILE_8X4, F.TILE_4X8, F.TILE_16X2) and best.rays_per_warp in (32, 16, 8)
    ref = torch.zeros_like(rgb)
    scene.render_batch(views, len(cams), ref)
    out = torch.zeros_like(rgb)
    scene.render_batch(views, len(cams), out, cfg=best)
    torch.cuda.synchronize()
    assert float((out - ref).abs().max()) < 1e-4
    scene.close()


def test_batch_config_errors(pkg, cuda, fixtures):
    fx = fixtures["uniform2k"]
    F = pkg.renderer
    scene = F.Scene(fx.tree, fx.rec, forms=F.FORM_EXACT)
    views, total, _ = F.make_views(pkg.scenes.sphere_cameras(1, seed=1, resolutions=[(8, 8)]))
    rgb = torch.zeros(total * 3, device=cuda)
    with pytest.raises(pkg.capi.KdgrError):
        scene.render_batch(views, 1, rgb)  # no fast arrays materialised
    scene.close()
    scene = F.Scene(fx.tree, fx.rec)
    for bad in (F.BatchConfig(0, 8, 0, 1, 0, 4, 0, F.TILE_4X8),  # warp tiles are 8x4 only
                F.BatchConfig(1, 8, 0, 1, 0, 4, 0, 7), F.BatchConfig(1, 8, 0, 1, 0, 4, 5, 0),
                F.BatchConfig(3, 8, 0, 1, 0, 4, 0, 0, 12),  # 32, 16 or 8 rays per warp
                F.BatchConfig(1, 8, 0, 1, 0, 4, 0, 0, 16),  # fewer rays per warp need warp strips
                F.BatchConfig(3, 8, 0, 1, 0, 4, 1, 2, 8)):  # ... and 8x4 tiles
        with pytest.raises(pkg.capi.KdgrError):
            scene.render_batch(views, 1, rgb, cfg=bad)
    scene.close()


KAT_CASES = {
    "analytic": lambda kat: (kat.analytic_single(), 32, 24),
    "straddle": lambda kat: ((lambda t: (t[0], t[2], t[3]))(kat.straddle()), 16, 16),
    "comb": lambda kat: ((lambda t: (t[0], t[2], t[3]))(kat.comb(20)), 8, 8),
    "ties": lambda kat: (kat.ties(20), 8, 8),
    "big_leaf": lambda kat: (kat.big_leaf(100), 16, 16),
    "empty": lambda kat: (kat.empty(), 8, 8),
    "miss": lambda kat: (kat.miss(), 8, 8),
    "mixed_aniso": lambda kat: (kat.mixed_aniso(), 16, 16),
}


@pytest.mark.parametrize("case", sorted(KAT_CASES))
def test_fast_forms_on_known_answer_scenes(pkg, O, cuda, case):
    """The batching and precision forms on the hand-built scenes: a stack
    deeper than the ring (restarts), 20 equal-t hits in one leaf (more than
    the hit buffer: re-scan passes), a 100-candidate leaf, a Gaussian across
    a split, an empty scene, a missed box, and leaves mixing very thin
    Gaussians (the precision form's FP32 stream) with plain ones; both forms
    within the accuracy bar of the FP64 oracle and equal across every
    schedule, tile shape, both traversals and 32, 16 or 8 rays per warp."""
    import kat
    (tree, rec, cam), W, H = KAT_CASES[case](kat)
    F = pkg.renderer
    scene = F.Scene(tree, rec, forms=F.FORM_FAST | F.FORM_PACKED)
    r64, a64, _, _ = oracle_image(O, tree, rec, cam, W, H, precision="f64")
    for prec in (0, 1):
        rgb, a = fast_image(pkg, cuda, scene, cam, W, H, prec)
        assert rmse(rgb, r64) <= RMSE_TOL, (prec, rmse(rgb, r64))
        assert rmse(a, a64) <= RMSE_TOL
    views, total, _ = F.make_views([(cam, W, H)])
    if case == "mixed_aniso":
        assert scene.info()["n_aniso"] == 21  # 14 thin in the front leaf, 7 in the back
    for prec in (0, 1):
        ref = torch.zeros(total * 3, device=cuda)
        scene.render_batch(views, 1, ref, cfg=F.BatchConfig(1, 8, 0, 1, prec, 4, 0, 0))
        for sched, kb, trav, tile, rpw in [(0, 4, 0, 0, 32), (1, 8, 0, 1, 32), (2, 4, 0, 2, 32), (3, 4, 0, 1, 32),
                                           (0, 4, 1, 0, 32), (1, 8, 1, 2, 32), (3, 8, 1, 0, 32), (3, 4, 0, 0, 16),
                                           (3, 8, 0, 0, 8), (3, 4, 0, 0, 8), (3, 4, 1, 0, 16), (3, 8, 1, 0, 8)]:
            out = torch.full_like(ref, -1.0)
            scene.render_batch(views, 1, out, cfg=F.BatchConfig(sched, 8, 0, 1, prec, kb, trav, tile, rpw))
            torch.cuda.synchronize()
            np.testing.assert_array_equal(out.cpu().numpy(), ref.cpu().numpy())
    assert scene.status() == 0
    scene.close()
