"""Serving form (kdgr_server_*): admission under an HBM budget, continuous
batching, cancellation, eviction, bounded waits, and the same frames alone and
in a mix.  Page-locked output buffers are written by the kernel directly;
pageable ones go through the device arena (the arena tests use pageable
buffers).  Through the C ABI."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

RMSE_TOL = 1e-3


def _views(pkg, cams):
    return pkg.renderer.make_views(cams)


def _request(pkg, server, slot, cams, pinned=True):
    views, total, _ = _views(pkg, cams)
    out = torch.zeros(total * 3, dtype=torch.float32)
    if pinned:
        out = out.pin_memory()
    t = server.submit(slot, views, len(cams), out)
    return t, out


@pytest.fixture(scope="module")
def two_scenes(pkg):
    import numpy as np  # noqa: F401
    sc = pkg.scenes
    a = sc.uniform_cube(20000, seed=31, scale=0.02)
    b = sc.cluster_shell(30000, seed=32, n_clusters=8)
    return [(a, pkg.kdtree.build(a)), (b, pkg.kdtree.build(b))]


def test_request_alone_equals_request_in_a_mix(pkg, cuda, two_scenes):
    F = pkg.renderer
    sc = pkg.scenes
    srv = F.Server(hbm_budget_bytes=8 << 30, arena_bytes=1 << 30, lanes=3)
    slots = [srv.add_scene(t, rec) for rec, t in two_scenes]
    probe = sc.sphere_cameras(3, seed=41, resolutions=[(96, 64), (40, 40), (128, 72)])
    t, alone = _request(pkg, srv, slots[1], probe)
    rc, st = srv.wait(t)
    assert rc == 0 and st["latency_ms"] > 0
    # the same request submitted in the middle of 30 others on both scenes
    rng = np.random.default_rng(5)
    others = []
    for i in range(30):
        cams = sc.sphere_cameras(int(rng.integers(1, 5)), seed=100 + i,
                                 resolutions=[(64, 48), (128, 96), (200, 100)])
        others.append(_request(pkg, srv, slots[i % 2], cams, pinned=(i % 3 != 0)))
        if i == 15:
            t2, mixed = _request(pkg, srv, slots[1], probe, pinned=False)  # arena path
    for tk, _ in others:
        assert srv.wait(tk)[0] == 0
    assert srv.wait(t2)[0] == 0
    np.testing.assert_array_equal(alone.numpy(), mixed.numpy())
    assert float(alone.abs().sum()) > 0
    stats = srv.stats()
    assert stats["completed"] == 32 and stats["launches"] >= 2
    assert stats["p99_ms"] >= stats["p50_ms"] > 0 and stats["mrays_per_s"] > 0
    srv.close()


def test_served_frames_match_batch_kernel_and_fp64(pkg, O, cuda, two_scenes):
    F = pkg.renderer
    rec, tree = two_scenes[0]
    srv = F.Server(hbm_budget_bytes=4 << 30, arena_bytes=256 << 20)
    slot = srv.add_scene(tree, rec)
    cams = pkg.scenes.sphere_cameras(2, seed=7, resolutions=[(80, 60)])
    t, served = _request(pkg, srv, slot, cams)
    assert srv.wait(t)[0] == 0
    scene = F.Scene(tree, rec)
    views, total, offs = _views(pkg, cams)
    ref = torch.zeros(total * 3, device=cuda)
    scene.render_batch(views, len(cams), ref)
    torch.cuda.synchronize()
    np.testing.assert_allclose(served.numpy(), ref.cpu().numpy(), rtol=0, atol=1e-5)
    S = O.OracleScene(tree.nodes, tree.offsets, tree.aabb, O.invert_scales(rec))
    for (cam, w, h), off in zip(cams, offs):
        r64, _, _, _ = O.render(S, cam, w, h, precision="f64")
        got = served.numpy()[3 * off:3 * (off + w * h)].reshape(h, w, 3).astype(np.float64)
        assert np.sqrt(((got - O.to_image(r64, w, h)) ** 2).mean()) <= RMSE_TOL
    scene.close()
    srv.close()


def test_budget_refuses_scene_and_oversized_request(pkg, cuda, two_scenes):
    F = pkg.renderer
    rec, tree = two_scenes[1]
    srv = F.Server(hbm_budget_bytes=(1 << 20) + 4096, arena_bytes=1 << 20)
    with pytest.raises(pkg.capi.KdgrError) as e:
        srv.add_scene(tree, rec)
    assert e.value.status == 6  # KDGR_ERR_BUDGET
    srv.close()
    srv = F.Server(hbm_budget_bytes=2 << 30, arena_bytes=64 * 1024)
    slot = srv.add_scene(tree, rec)
    views, total, _ = _views(pkg, [(pkg.scenes.front_camera(256, 256), 256, 256)])
    out = torch.zeros(total * 3)  # pageable: needs arena space
    with pytest.raises(pkg.capi.KdgrError) as e:
        srv.submit(slot, views, 1, out)
    assert e.value.status == 6
    # page-locked: written by the kernel, no arena space needed
    out = torch.zeros(total * 3).pin_memory()
    assert srv.wait(srv.submit(slot, views, 1, out))[0] == 0
    assert float(out.abs().sum()) > 0
    srv.close()


def test_small_arena_defers_but_completes_everything(pkg, cuda, two_scenes):
    """The arena holds one 96x96 request at a time: later requests wait for
    space (admission), none is refused, all complete."""
    F = pkg.renderer
    rec, tree = two_scenes[0]
    srv = F.Server(hbm_budget_bytes=2 << 30, arena_bytes=12 * 96 * 96 + 4096, lanes=2)
    slot = srv.add_scene(tree, rec)
    reqs = [_request(pkg, srv, slot, pkg.scenes.sphere_cameras(1, seed=60 + i, resolutions=[(96, 96)]),
                     pinned=False) for i in range(8)]
    for t, out in reqs:
        assert srv.wait(t)[0] == 0
    assert srv.stats()["max_views_per_launch"] == 1
    srv.close()


def test_cancel_evict_and_bounded_wait(pkg, cuda, two_scenes):
    F = pkg.renderer
    rec, tree = two_scenes[1]
    # one lane and an arena for one request: the queue backs up behind it
    srv = F.Server(hbm_budget_bytes=2 << 30, arena_bytes=12 * 256 * 256 + 4096, lanes=1)
    slot = srv.add_scene(tree, rec)
    big = [(pkg.scenes.front_camera(256, 256), 256, 256)]
    subs = [_request(pkg, srv, slot, big, pinned=False) for _ in range(6)]  # keeps the host buffers alive
    tickets = [t for t, _ in subs]
    assert srv.cancel(tickets[-1]) == 0
    assert srv.wait(tickets[-1])[0] == 9  # KDGR_ERR_CANCELLED
    rc, _ = srv.wait(tickets[-2], timeout_ms=0)
    assert rc in (0, 7)  # finished already, or KDGR_ERR_TIMEOUT: the wait is bounded
    srv.remove_scene(slot)  # queued requests of the scene are cancelled
    pending = tickets[:-2] + ([tickets[-2]] if rc == 7 else [])
    statuses = [srv.wait(t, timeout_ms=60_000)[0] for t in pending]
    assert all(s in (0, 9) for s in statuses)
    del subs
    views, _, _ = _views(pkg, big)
    with pytest.raises(pkg.capi.KdgrError):  # the slot is empty now
        srv.submit(slot, views, 1, torch.zeros(256 * 256 * 3))
    srv.close()


def test_direct_and_arena_requests_mixed(pkg, cuda, two_scenes):
    """Page-locked and pageable requests of both scenes, queued behind a
    large request on a single lane so that they share launches: every frame
    equals the batch call's, and the page-locked ones complete although each
    is larger than the arena (they take no arena space)."""
    F = pkg.renderer
    sc = pkg.scenes
    srv = F.Server(hbm_budget_bytes=4 << 30, arena_bytes=12 * 200 * 150 * 4 + 4096, lanes=1)
    slots = [srv.add_scene(t, rec) for rec, t in two_scenes]
    reqs = []
    for i in range(13):
        if i == 0:  # keeps the lane busy while the others queue
            cams, pinned = sc.sphere_cameras(8, seed=299, resolutions=[(1280, 720)]), True
        else:
            cams = sc.sphere_cameras(int(1 + i % 3), seed=300 + i, resolutions=[(200, 150), (120, 90)])
            pinned = i % 2 == 0
            if pinned:
                cams = cams + sc.sphere_cameras(2, seed=400 + i, resolutions=[(320, 240)])  # > arena
        t, out = _request(pkg, srv, slots[i % 2], cams, pinned=pinned)
        reqs.append((i % 2, cams, out, t))
    for _, _, _, t in reqs:
        assert srv.wait(t, timeout_ms=60_000)[0] == 0
    assert srv.stats()["completed"] == len(reqs)
    alone = [F.Scene(t, rec) for rec, t in two_scenes]
    for k, cams, out, _ in reqs:
        views, total, _ = _views(pkg, cams)
        ref = torch.zeros(total * 3, device=cuda)
        alone[k].render_batch(views, len(cams), ref)
        torch.cuda.synchronize()
        np.testing.assert_allclose(out.numpy(), ref.cpu().numpy(), rtol=0, atol=1e-5)
        assert float(out.abs().sum()) > 0
    for a in alone:
        a.close()
    srv.close()
