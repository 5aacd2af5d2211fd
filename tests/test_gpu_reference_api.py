"""The reference-signature C++ entry points (include/kdgr_reference_api.h),
driven by a C++ program through the reference caller's own sequence
(read_kd_tree_from_file, caller-side scale inversion, initCuda,
renderGaussianWithCudaSetup, renderGaussianWithCudaFrame): the framebuffer
equals the oracle's bit for bit."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _demo(pkg, tmp_path):
    cuda_home = _cuda_home()
    exe = tmp_path / "ref_api_demo"
    libdir = os.path.dirname(pkg.capi.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(REPO, "include"),
                    "-I" + os.path.join(cuda_home, "include"), os.path.join(REPO, "tests", "cpp", "ref_api_demo.cpp"),
                    "-L" + libdir, "-l:libkdgr.so", "-Wl,-rpath," + libdir,
                    "-L" + os.path.join(cuda_home, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(cuda_home, "lib64"),
                    "-o", str(exe)], check=True)
    return exe


def _cam_args(cam, w, h):
    return [str(w), str(h)] + [repr(float(v)) for v in list(cam.pos) + list(cam.uaxis) + list(cam.vaxis) +
                               list(cam.naxis)] + [repr(cam.fovy), repr(cam.aspect), repr(cam.near_c)]


@pytest.mark.parametrize("name", ["dense800", "cluster2k"])
def test_reference_call_sequence_bit_exact(pkg, O, cuda, fixtures, tmp_path, name):
    exe = _demo(pkg, tmp_path)
    fx = fixtures[name]
    kdgs = tmp_path / "scene.kdgs"
    pkg.scenes.write_kdgs(str(kdgs), fx.rec)
    _, cam, w, h, _ = fx.cameras()[1]
    out = tmp_path / "fb.bin"
    args = [str(exe), str(kdgs), fx.kdt, str(w), str(h)] + [repr(float(v)) for v in
                                                            list(cam.pos) + list(cam.uaxis) + list(cam.vaxis) +
                                                            list(cam.naxis)] + \
           [repr(cam.fovy), repr(cam.aspect), repr(cam.near_c), str(out)]
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    fb = np.fromfile(out, dtype=np.float32).reshape(h, w, 3)
    S = O.OracleScene(fx.tree.nodes, fx.tree.offsets, fx.tree.aabb, O.invert_scales(fx.rec))
    rgb, _, _, _ = O.render(S, cam, w, h)
    np.testing.assert_array_equal(fb, O.to_image(rgb, w, h))
    assert fb.any()


def test_reference_call_sequence_from_ply(pkg, O, cuda, tmp_path):
    """loadGaussiansFromPly -> read_kd_tree_from_file -> setup -> frame, with
    the oracle fed by the restatement of the reference's PLY loader."""
    import sys
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import ply_ref
    exe = _demo(pkg, tmp_path)
    ply = tmp_path / "scene.ply"
    pkg.scenes.write_ply(str(ply), pkg.scenes.raw_gaussians(3000, seed=11))
    rec = ply_ref.load_gaussians_from_ply(str(ply))
    tree = pkg.kdtree.build(rec)
    kdt = tmp_path / "scene.kdt"
    pkg.kdtree.write_kdt(tree, str(kdt))
    cam, w, h = pkg.scenes.front_camera(64, 48), 64, 48
    out = tmp_path / "fb.bin"
    r = subprocess.run([str(exe), str(ply), str(kdt)] + _cam_args(cam, w, h) + [str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    fb = np.fromfile(out, dtype=np.float32).reshape(h, w, 3)
    S = O.OracleScene(tree.nodes, tree.offsets, tree.aabb, O.invert_scales(rec))
    rgb, _, _, _ = O.render(S, cam, w, h)
    np.testing.assert_array_equal(fb, O.to_image(rgb, w, h))
    assert fb.any()


@pytest.mark.parametrize("prim", ["sphere", "tri"])
def test_reference_secondary_ray_build(pkg, O, cuda, fixtures, tmp_path, prim):
    """The SECONDARY_RAY build's setup (with a SecondaryMesh) and frame: the
    framebuffer equals the oracle's secondary-ray transcription bit for bit,
    against the demo spheres or the mesh."""
    exe = _demo(pkg, tmp_path)
    fx = fixtures["dense800"]
    kdgs = tmp_path / "scene.kdgs"
    pkg.scenes.write_kdgs(str(kdgs), fx.rec)
    _, cam, w, h, _ = fx.cameras()[0]
    out = tmp_path / "fb.bin"
    env = dict(os.environ, KDGR_DEMO_SECONDARY=prim)
    r = subprocess.run([str(exe), str(kdgs), fx.kdt] + _cam_args(cam, w, h) + [str(out)], capture_output=True,
                       text=True, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    fb = np.fromfile(out, dtype=np.float32).reshape(h, w, 3)
    F = pkg.renderer
    S = O.OracleScene(fx.tree.nodes, fx.tree.offsets, fx.tree.aabb, O.invert_scales(fx.rec))
    if prim == "sphere":
        sph = [(tuple(x.center), x.radius, x.material.material, x.material.reflectivity, x.material.ior,
                tuple(x.material.color)) for x in F.demo_spheres()]
        want = O.render_hybrid(S, cam, w, h, spheres=sph)
    else:
        a, b, c, d = (-0.9, -0.9, -0.6), (0.9, -0.9, -0.6), (0.9, 0.9, -0.6), (-0.9, 0.9, -0.6)
        tris = np.array([a + b + c, a + c + d], np.float32)
        m = F.mesh_material_default()
        want = O.render_hybrid(S, cam, w, h, tris=tris, tri_material=(m.material, m.reflectivity, m.ior,
                                                                      tuple(m.color)))
    np.testing.assert_array_equal(fb, O.to_image(want, w, h))



def test_reference_frame_writes_debug_report(pkg, O, cuda, fixtures, tmp_path):
    """With KDGR_DEBUG_REPORT_DIR set (the HIT_AND_NODE_COUNT_DEBUG build),
    a frame writes the reference's report files; they equal the report of
    the oracle's traces, file for file."""
    exe = _demo(pkg, tmp_path)
    fx = fixtures["cluster2k"]
    kdgs = tmp_path / "scene.kdgs"
    pkg.scenes.write_kdgs(str(kdgs), fx.rec)
    _, cam, w, h, _ = fx.cameras()[1]
    out_dir = tmp_path / "report"
    out_dir.mkdir()
    env = dict(os.environ, KDGR_DEBUG_REPORT_DIR=str(out_dir))
    r = subprocess.run([str(exe), str(kdgs), fx.kdt] + _cam_args(cam, w, h) + [str(tmp_path / "fb.bin")],
                       capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    S = O.OracleScene(fx.tree.nodes, fx.tree.offsets, fx.tree.aabb, O.invert_scales(fx.rec))
    _, _, _, tr = O.render(S, cam, w, h, trace=True)
    want_dir = tmp_path / "want"
    want_dir.mkdir()
    pkg.renderer.debug_report(tr, w, h, out_dir=str(want_dir))
    names = sorted(os.listdir(want_dir))
    assert len(names) == 16 and sorted(os.listdir(out_dir)) == names
    for n in names:
        assert (out_dir / n).read_bytes() == (want_dir / n).read_bytes(), n
