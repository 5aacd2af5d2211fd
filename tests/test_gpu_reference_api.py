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


@pytest.mark.parametrize("name", ["dense800", "cluster2k"])
def test_reference_call_sequence_bit_exact(pkg, O, cuda, fixtures, tmp_path, name):
    cuda_home = _cuda_home()
    exe = tmp_path / "ref_api_demo"
    libdir = os.path.dirname(pkg.capi.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(REPO, "include"),
                    "-I" + os.path.join(cuda_home, "include"), os.path.join(REPO, "tests", "cpp", "ref_api_demo.cpp"),
                    "-L" + libdir, "-l:libkdgr.so", "-Wl,-rpath," + libdir,
                    "-L" + os.path.join(cuda_home, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(cuda_home, "lib64"),
                    "-o", str(exe)], check=True)
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
