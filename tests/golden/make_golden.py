"""Generate the committed golden fixtures (run in a tree where the reference
sources are present; machines without them only read the outputs).

For each fixture scene:
  * <name>.scene.npy  -- activated Gaussian records (n, 64) float32;
  * <name>.ref.kdt    -- the tree written by the REFERENCE builder
                          (oracle/_ref/ref_kdbuild, the reference's own
                          Kd-treeConstructor.cpp compiled by oracle/build_ref.sh)
                          with the render benchmark's flags -m 24 -f 16;
  * <name>.out.npz    -- per camera: the CameraInfo words, the FP32 oracle's
                          rgb/alpha/depth and per-ray traces, the FP64
                          oracle's rgb.

The reference has no tests or golden data of its own for this path; these
fixtures pin (a) the product tree builder to the reference builder and (b)
the oracle across machines.

Usage: python tests/golden/make_golden.py
"""
import importlib
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))
import oracle as O  # noqa: E402

sc = importlib.import_module("3dgrt_kdtree_gb300.scenes")
kd = importlib.import_module("3dgrt_kdtree_gb300.kdtree")

REF_BIN = os.path.join(REPO, "oracle", "_ref", "ref_kdbuild")

FIXTURES = {
    "uniform2k": lambda: sc.uniform_cube(2000, seed=0),
    "cluster2k": lambda: sc.cluster_shell(2000, seed=1, n_clusters=8),
    # denser: larger Gaussians so most rays composite several hits per leaf
    "dense800": lambda: sc.uniform_cube(800, seed=3, scale=0.03),
}


def cameras():
    cams = [("front", sc.front_camera(48, 40), 48, 40)]
    c, w, h = sc.sphere_cameras(1, seed=5, resolutions=[(40, 32)])[0]
    cams.append(("orbit", c, w, h))
    return cams


def caminfo_words(ci) -> np.ndarray:
    return np.array(list(ci.eye) + list(ci.u) + list(ci.v) + list(ci.start) + [ci.step_x, ci.step_y], np.float32)


def main() -> None:
    if not os.path.exists(REF_BIN):
        raise SystemExit("reference builder not built: run oracle/build_ref.sh")
    for name, gen in FIXTURES.items():
        rec = gen()
        np.save(os.path.join(HERE, f"{name}.scene.npy"), rec)
        kdgs = os.path.join(HERE, f"_{name}.kdgs")
        sc.write_kdgs(kdgs, rec)
        kdt = os.path.join(HERE, f"{name}.ref.kdt")
        subprocess.run([REF_BIN, kdgs, kdt, "-m", "24", "-f", "16"], check=True, capture_output=True)
        os.remove(kdgs)
        tree = kd.read_kdt(kdt)
        S = O.OracleScene(tree.nodes, tree.offsets, tree.aabb, O.invert_scales(rec))
        out = {}
        for cname, cam, w, h in cameras():
            ci = O.caminfo(cam, w, h)
            rgb, a, d, tr = O.render(S, ci, w, h, trace=True)
            r64, _, _, _ = O.render(S, ci, w, h, precision="f64")
            out[f"{cname}_caminfo"] = caminfo_words(ci)
            out[f"{cname}_camera"] = np.array(list(cam.pos) + list(cam.uaxis) + list(cam.vaxis) + list(cam.naxis)
                                              + [cam.fovy, cam.aspect, cam.near_c, w, h], np.float64)
            out[f"{cname}_rgb"] = rgb
            out[f"{cname}_alpha"] = a
            out[f"{cname}_depth"] = d
            out[f"{cname}_trace"] = tr
            out[f"{cname}_rgb64"] = r64
        np.savez_compressed(os.path.join(HERE, f"{name}.out.npz"), **out)
        print(name, "nodes", tree.n_nodes, "offsets", tree.offsets.size, "depth", tree.depth)


if __name__ == "__main__":
    main()
