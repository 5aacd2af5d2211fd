import importlib
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
for p in (REPO, os.path.join(REPO, "oracle"), os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box with -m gpu)")


@pytest.fixture(scope="session")
def pkg():
    lib = os.path.join(REPO, "3dgrt_kdtree_gb300", "libkdgr.so")
    if not os.path.exists(lib):
        importlib.import_module("3dgrt_kdtree_gb300.build").build()
    return importlib.import_module("3dgrt_kdtree_gb300")


@pytest.fixture(scope="session")
def O():
    import oracle
    if not os.path.exists(oracle.LIB):
        oracle.build()
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    importlib.import_module("3dgrt_kdtree_gb300.renderer").init(0)
    return torch.device("cuda:0")


class Fixture:
    def __init__(self, name, pkg):
        self.name = name
        self.rec = np.load(os.path.join(GOLDEN, f"{name}.scene.npy"))
        self.kdt = os.path.join(GOLDEN, f"{name}.ref.kdt")
        self.tree = pkg.kdtree.read_kdt(self.kdt)
        self.out = np.load(os.path.join(GOLDEN, f"{name}.out.npz"))

    def cameras(self):
        """[(name, Camera, W, H, caminfo words)]"""
        sc = importlib.import_module("3dgrt_kdtree_gb300.scenes")
        res = []
        for cname in ("front", "orbit"):
            c = self.out[f"{cname}_camera"]
            cam = sc.Camera(tuple(c[0:3]), tuple(c[3:6]), tuple(c[6:9]), tuple(c[9:12]), float(c[12]),
                            float(c[13]), float(c[14]))
            res.append((cname, cam, int(c[15]), int(c[16]), self.out[f"{cname}_caminfo"]))
        return res


FIXTURE_NAMES = ["uniform2k", "cluster2k", "dense800"]


@pytest.fixture(scope="session")
def fixtures(pkg):
    return {n: Fixture(n, pkg) for n in FIXTURE_NAMES}
