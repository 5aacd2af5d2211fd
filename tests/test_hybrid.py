"""Secondary-ray hybrid path (renderKernelGaussian_Mesh_Hybrid,
cudaRenderer.cu:2217-2311): OBJ ingest, oracle invariants on the CPU, and
the kernel against the oracle bit for bit on the GPU (mirror, glass, opaque
spheres and a mirror mesh)."""
import numpy as np
import pytest


def _sph(s):
    m = s.material
    return (tuple(s.center), s.radius, m.material, m.reflectivity, m.ior, tuple(m.color))


def _mat(m):
    return (m.material, m.reflectivity, m.ior, tuple(m.color))


def _mirror_quad(F):
    """Two triangles forming a mirror square at z = -0.6 behind the scene,
    facing the camera, with the reference mesh's default mirror material."""
    a, b, c, d = (-0.9, -0.9, -0.6), (0.9, -0.9, -0.6), (0.9, 0.9, -0.6), (-0.9, 0.9, -0.6)
    tris = np.array([a + b + c, a + c + d], np.float32)
    return tris, F.mesh_material_default()


def _oscene(O, fx):
    return O.OracleScene(fx.tree.nodes, fx.tree.offsets, fx.tree.aabb, O.invert_scales(fx.rec))


def test_hybrid_without_primitives_is_the_plain_render(pkg, O, fixtures):
    """No secondary hit: one Gaussian pass with max_t = 1e8, then the pixel is
    the plain render clamped to 1."""
    fx = fixtures["dense800"]
    S = _oscene(O, fx)
    for _, cam, w, h, ci in fx.cameras():
        plain, _, _, _ = O.render(S, cam, w, h)
        hyb = O.render_hybrid(S, cam, w, h)
        np.testing.assert_array_equal(hyb, np.minimum(plain, np.float32(1.0)))


def test_opaque_sphere_in_front_shows_its_colour(pkg, O, fixtures):
    """An opaque sphere between the eye and every Gaussian: rays that hit it
    get exactly its colour (nothing to composite before it); the others see
    the plain render."""
    F = pkg.renderer
    fx = fixtures["uniform2k"]
    S = _oscene(O, fx)
    _, cam, w, h, _ = fx.cameras()[0]
    col = (0.25, 0.5, 0.75)
    sph = F.sphere((0.0, 0.0, 1.6), 0.2, F.material(F.OPAQUE, 0.0, 1.0, col))
    hyb = O.render_hybrid(S, cam, w, h, spheres=[_sph(sph)])
    plain, _, _, _ = O.render(S, cam, w, h)
    hit = np.all(hyb == np.array(col, np.float32), axis=1)
    assert 20 < hit.sum() < w * h // 2
    np.testing.assert_array_equal(hyb[~hit], np.minimum(plain[~hit], 1.0))


def test_mirror_and_glass_change_the_image(pkg, O, fixtures):
    F = pkg.renderer
    fx = fixtures["dense800"]
    S = _oscene(O, fx)
    _, cam, w, h, _ = fx.cameras()[0]
    plain = np.minimum(O.render(S, cam, w, h)[0], 1.0)
    tris, m = _mirror_quad(F)
    with_mesh = O.render_hybrid(S, cam, w, h, tris=tris, tri_material=_mat(m))
    with_demo = O.render_hybrid(S, cam, w, h, spheres=[_sph(s) for s in F.demo_spheres()])
    assert (with_mesh != plain).any(axis=1).sum() > 50
    assert (with_demo != plain).any(axis=1).sum() > 0
    assert np.isfinite(with_mesh).all() and (with_mesh <= 1.0).all() and (with_mesh >= 0.0).all()


def test_read_obj_triangulates_and_swaps_axes(pkg, tmp_path):
    p = tmp_path / "m.obj"
    p.write_text("# comment\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 2\nvt 0 0\nvn 0 0 1\n"
                 "f 1/1/1 2/1/1 3/1/1 4/1/1\nf -4//1 -3//1 -1//1\n")
    tris = pkg.renderer.read_obj(str(p))
    v = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 2]], np.float32)
    sw = np.stack([v[:, 0], -v[:, 2], v[:, 1]], 1)  # (x, y, z) -> (x, -z, y)
    want = np.array([np.concatenate([sw[0], sw[1], sw[2]]), np.concatenate([sw[0], sw[2], sw[3]]),
                     np.concatenate([sw[0], sw[1], sw[3]])], np.float32)
    np.testing.assert_array_equal(tris, want)
    (tmp_path / "bad.obj").write_text("v 0 0 0\nf 1 2 3\n")
    with pytest.raises(pkg.capi.KdgrError):
        pkg.renderer.read_obj(str(tmp_path / "bad.obj"))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["dense800", "cluster2k"])
def test_hybrid_kernel_matches_oracle_bitwise(pkg, O, cuda, fixtures, name):
    import torch
    F = pkg.renderer
    fx = fixtures[name]
    scene = F.Scene(fx.tree, fx.rec)
    S = _oscene(O, fx)
    tris, m = _mirror_quad(F)
    setups = [
        dict(spheres=F.demo_spheres()),
        dict(tris=tris, tri_material=m),
        dict(spheres=[F.sphere((0.0, 0.0, 1.6), 0.2, F.material(F.OPAQUE, 0.0, 1.0, (0.2, 0.4, 0.6))),
                      F.sphere((-0.5, 0.3, 0.9), 0.35, F.material(F.GLASS, 1.0, 1.5, (0.9, 1.0, 0.9)))],
             tris=tris, tri_material=F.material(F.MIRROR, 0.8, 1.0, (0.3, 0.3, 0.3))),
    ]
    for setup in setups:
        sec = F.Secondary(**setup)
        for _, cam, w, h, _ in fx.cameras():
            rgb = torch.zeros(w * h * 3, device=cuda)
            scene.render_hybrid(cam, w, h, sec, rgb)
            torch.cuda.synchronize()
            want = O.render_hybrid(S, cam, w, h, spheres=[_sph(s) for s in setup.get("spheres", [])],
                                   tris=setup.get("tris"),
                                   tri_material=_mat(setup["tri_material"]) if "tri_material" in setup else None)
            np.testing.assert_array_equal(rgb.cpu().numpy().reshape(h, w, 3), O.to_image(want, w, h))
        sec.close()
    assert scene.status() == 0
    scene.close()
