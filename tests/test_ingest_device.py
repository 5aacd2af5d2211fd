"""Scene ingest on the device (kdgr_read_ply_device, kdgr_scene_create_device,
kdgr_scene_create_from_files) against the host loader and host upload.

* PLY activation on the device gives the host loader's records: equal bit
  for bit except where exp/log/pow enter (opacity, scales, k_scale), which
  may differ by at most one float ulp (both round a double evaluation once;
  CUDA's double functions are within 1 ulp of double);
* a file larger than one streaming chunk, and a vertex layout whose floats
  are not 4-byte aligned;
* a scene built from the two files renders the same frames, all forms, as
  the scene created from the host loader's records and tree.
Through the C ABI."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

EXP_FIELDS = [3, 4, 5, 6, 7]  # opacity (sigmoid), scale (exp), k_scale (log, pow)


def _ulps(a, b):
    ai = a.view(np.int32).astype(np.int64)
    bi = b.view(np.int32).astype(np.int64)
    return np.abs(ai - bi)


def _compare_records(host, dev):
    assert host.shape == dev.shape
    other = [k for k in range(64) if k not in EXP_FIELDS]
    np.testing.assert_array_equal(dev[:, other].view(np.uint32), host[:, other].view(np.uint32))
    u = _ulps(host[:, EXP_FIELDS], dev[:, EXP_FIELDS])
    assert u.max() <= 1
    assert (u > 0).mean() < 1e-3  # a 1-ulp difference needs a double result at a float rounding boundary


@pytest.mark.parametrize("n", [150_000, 3_001])
def test_ply_on_device_matches_host_loader(pkg, cuda, tmp_path, n):
    """150k vertices stream through three 16 MB chunks."""
    sc = pkg.scenes
    path = str(tmp_path / "g.ply")
    sc.write_ply(path, sc.raw_gaussians(n, seed=9))
    host = pkg.kdtree.read_ply(path)
    dev = pkg.renderer.read_ply_device(path, cuda)
    torch.cuda.synchronize()
    _compare_records(host, dev.cpu().numpy())


def test_unaligned_vertex_fields(pkg, cuda, tmp_path):
    """A uchar property before x: all 62 floats of a vertex sit at odd byte
    offsets."""
    sc = pkg.scenes
    n = 777
    fields = sc.raw_gaussians(n, seed=10)
    path = str(tmp_path / "u.ply")
    # write by hand: uchar first, then the 3DGS floats
    dt = np.dtype([("flag", "u1")] + [(k, "<f4") for k in sc.PLY_FIELDS])
    data = np.zeros(n, dt)
    data["flag"] = np.arange(n) % 200
    for k in sc.PLY_FIELDS:
        data[k] = fields[k]
    head = ["ply", "format binary_little_endian 1.0", f"element vertex {n}", "property uchar flag"]
    head += [f"property float {k}" for k in sc.PLY_FIELDS] + ["end_header"]
    with open(path, "wb") as f:
        f.write(("\n".join(head) + "\n").encode())
        f.write(data.tobytes())
    host = pkg.kdtree.read_ply(path)
    dev = pkg.renderer.read_ply_device(path, cuda)
    torch.cuda.synchronize()
    _compare_records(host, dev.cpu().numpy())


def test_scene_from_files_renders_as_host_upload(pkg, O, cuda, tmp_path):
    sc = pkg.scenes
    F = pkg.renderer
    n = 20_000
    path = str(tmp_path / "s.ply")
    sc.write_ply(path, sc.raw_gaussians(n, seed=12))
    rec = pkg.kdtree.read_ply(path)
    tree = pkg.kdtree.build(rec)
    kdt = str(tmp_path / "s.kdt")
    pkg.kdtree.write_kdt(tree, kdt)
    forms = F.FORM_EXACT | F.FORM_FAST | F.FORM_PACKED
    a = F.Scene(tree, rec, forms=forms)
    b = F.Scene.from_files(path, kdt, forms=forms)
    c = F.Scene.from_device(tree, torch.from_numpy(rec).to(cuda), forms=forms)
    ia, ib = a.info(), b.info()
    assert ib["n_gaussians"] == n and ib["n_aniso"] == ia["n_aniso"] and ib["device_bytes"] == ia["device_bytes"]
    W, H = 96, 64
    cam = sc.front_camera(W, H, dist=1.6)
    outs = []
    for s in (a, b, c):
        imgs = []
        rgb = torch.zeros(W * H * 3, device=cuda)
        s.render(cam, W, H, rgb)
        imgs.append(rgb.cpu().numpy().copy())
        for prec in (0, 1):
            s.render_fast(cam, W, H, rgb, precision=prec)
            imgs.append(rgb.cpu().numpy().copy())
        torch.cuda.synchronize()
        assert s.status() == 0
        outs.append(imgs)
    assert float(np.abs(outs[0][0]).sum()) > 0
    for k in range(3):
        # device-created records equal the host records except in vanishingly
        # rare 1-ulp cases, so the frames agree to the parity tolerance
        np.testing.assert_allclose(outs[1][k], outs[0][k], rtol=0, atol=1e-5)
        np.testing.assert_array_equal(outs[2][k], outs[0][k])
    # the plain frame of the file-built scene is still the oracle's
    r32 = O.render(O.OracleScene(tree.nodes, tree.offsets, tree.aabb, O.invert_scales(rec)), cam, W, H)[0]
    np.testing.assert_allclose(outs[1][0].reshape(H, W, 3), O.to_image(r32, W, H), rtol=0, atol=1e-5)
    for s in (a, b, c):
        s.close()


def test_device_ingest_errors(pkg, cuda, tmp_path):
    """Missing files, a tree whose IDs exceed the PLY's vertices, inverted
    scales (PLY records are activated) and a buffer too small for the file
    are refused with the library's status codes; nothing is left half made."""
    sc = pkg.scenes
    F = pkg.renderer
    KdgrError = pkg.capi.KdgrError
    ply = str(tmp_path / "a.ply")
    sc.write_ply(ply, sc.raw_gaussians(500, seed=3))
    rec = pkg.kdtree.read_ply(ply)
    tree = pkg.kdtree.build(rec)
    kdt = str(tmp_path / "a.kdt")
    pkg.kdtree.write_kdt(tree, kdt)
    small = str(tmp_path / "small.ply")
    sc.write_ply(small, sc.raw_gaussians(100, seed=4))
    cases = [((str(tmp_path / "missing.ply"), kdt, F.FORM_FAST), 4),   # KDGR_ERR_IO
             ((ply, str(tmp_path / "missing.kdt"), F.FORM_FAST), 4),
             ((small, kdt, F.FORM_FAST), 5),                            # IDs >= 100: KDGR_ERR_FORMAT
             ((ply, kdt, F.FORM_FAST | F.SCALES_INVERTED), 1)]          # KDGR_ERR_INVALID_ARG
    for args, status in cases:
        with pytest.raises(KdgrError) as ei:
            F.Scene.from_files(*args)
        assert f"status {status}" in str(ei.value), (args, str(ei.value))
    # a device buffer smaller than the file: KDGR_ERR_LIMIT
    import ctypes
    buf = torch.zeros((499, 64), device=cuda)
    n = ctypes.c_uint32()
    L = pkg.capi.lib()
    rc = L.kdgr_read_ply_device(ply.encode(), ctypes.c_void_p(buf.data_ptr()), 499, ctypes.byref(n), None)
    assert rc == 10 and b"capacity" in L.kdgr_last_error()
    # the good pair still works after the failures
    s = F.Scene.from_files(ply, kdt, forms=F.FORM_FAST)
    assert s.info()["n_gaussians"] == 500
    s.close()
