"""Known-answer scenes: hand-built trees and Gaussians whose expected render
is known analytically or structurally.  Shared by the CPU oracle tests and
the GPU parity tests."""
import importlib

import numpy as np

sc = importlib.import_module("3dgrt_kdtree_gb300.scenes")
kd = importlib.import_module("3dgrt_kdtree_gb300.kdtree")


def gaussian(pos, scale, quat=(1.0, 0.0, 0.0, 0.0), opacity=0.8, dc=(0.3, 0.5, 0.7), rest=None):
    r = np.zeros(64, np.float32)
    r[0:3] = pos
    r[3] = opacity
    r[4:7] = scale
    r[7] = 1.0
    q = np.asarray(quat, np.float64)
    r[8:12] = q / np.linalg.norm(q)
    r[12:15] = dc
    if rest is not None:
        r[15:60] = rest
    return r


def leaf(count, off):
    return [(count << 3) | 3, off]


def inner(axis, child, split):
    return [(child << 3) | axis, int(np.float32(split).view(np.uint32))]


def make_tree(nodes, offsets, aabb):
    return kd.KdTree(np.array(nodes, np.uint32).reshape(-1, 2), np.array(offsets, np.uint32),
                     np.array(aabb, np.float32))


def single(gs, aabb=(-1, -1, -1, 1, 1, 1)):
    """All Gaussians in one leaf, in list order."""
    return make_tree([leaf(len(gs), 0)], list(range(len(gs))), aabb), np.stack(gs)


def analytic_single():
    """One axis-aligned Gaussian in one leaf; camera on +z."""
    g = gaussian((0.05, -0.03, 0.0), (0.1, 0.2, 0.3), opacity=0.8)
    tree, rec = single([g])
    return tree, rec, sc.front_camera(32, 24)


def straddle():
    """Root splits x at 0; both leaves list Gaussian 0 (centred at x=0.02).
    Camera on +x: every ray crosses the plane; the Gaussian must be
    composited once."""
    g = gaussian((0.02, 0.0, 0.0), (0.05, 0.08, 0.06), opacity=0.7)
    tree = make_tree([inner(0, 1, 0.0), leaf(1, 0), leaf(1, 1)], [0, 0], (-1, -1, -1, 1, 1, 1))
    cam = sc.look_at((2.5, 0.0, 0.0), fovy=20.0, aspect=1.0)
    flat, rec = single([g])
    return tree, flat, rec, cam


def comb(levels=20):
    """A comb of `levels` z-splits: the far child of each inner node is a
    leaf holding one Gaussian inside its slab; a ray from +z pushes every
    far leaf, overflowing the 12-entry short stack and forcing restarts.
    Returns (comb tree, flat single-leaf tree, records, camera)."""
    zs = np.linspace(-0.9, 0.9, levels + 1)
    nodes = []
    offsets = []
    gs = []
    # node 0 = first inner; each inner i: children at (c, c+1) = (leaf_i, inner_{i+1})
    n_inner = levels
    nodes = [None] * (1 + 2 * n_inner)
    idx = 0
    for i in range(n_inner):
        c = 1 + 2 * i
        nodes[idx] = inner(2, c, zs[i + 1])
        zc = 0.5 * (zs[i] + zs[i + 1])
        gs.append(gaussian((0.0, 0.0, zc), (0.02, 0.02, 0.01), opacity=0.15, dc=(0.2 + 0.02 * i, 0.5, 0.4)))
        nodes[c] = leaf(1, len(offsets))
        offsets.append(i)
        idx = c + 1
    # last right child: a leaf with one more Gaussian near the top
    gs.append(gaussian((0.0, 0.0, 0.95), (0.02, 0.02, 0.01), opacity=0.15))
    nodes[idx] = leaf(1, len(offsets))
    offsets.append(len(gs) - 1)
    tree = make_tree(nodes, offsets, (-1, -1, -1, 1, 1, 1))
    flat, rec = single(gs)
    cam = sc.look_at((0.0, 0.0, 2.5), fovy=2.0, aspect=1.0)
    return tree, flat, rec, cam


def ties(n=20, order=None):
    """n identical Gaussians in one leaf; the leaf lists them in `order`
    (default 0..n-1).  Equal t: the composite order must be the leaf order."""
    g = gaussian((0.0, 0.0, 0.0), (0.1, 0.1, 0.1), opacity=0.04)
    rec = np.stack([g] * n)
    order = list(range(n)) if order is None else list(order)
    tree = make_tree([leaf(n, 0)], order, (-1, -1, -1, 1, 1, 1))
    return tree, rec, sc.front_camera(8, 8, fovy=10.0)


def big_leaf(n=100, seed=7):
    """One leaf with n Gaussians strung along the view axis (many hits per
    ray: the hit buffer takes several passes)."""
    rng = np.random.default_rng(seed)
    gs = [gaussian((rng.normal(0, 0.02), rng.normal(0, 0.02), z), (0.05, 0.05, 0.02), opacity=0.05,
                   dc=rng.normal(0.5, 0.2, 3)) for z in rng.uniform(-0.8, 0.8, n)]
    tree, rec = single(gs)
    return tree, rec, sc.front_camera(16, 16, fovy=6.0)


def mixed_aniso(n=41, seed=11):
    """Two leaves split at z = 0: the front leaf mixes n Gaussians of which
    every third is very thin (scale ratio 2000, so the precision form reads
    its FP64-precomputed factors), the back leaf holds only thin ones; odd
    counts in both, so both of the precision form's pair streams end on a
    padding entry."""
    rng = np.random.default_rng(seed)
    front, back = [], []
    for i in range(n):
        q = rng.normal(0, 1, 4)
        thin = i % 3 == 0
        s = (0.08, 0.06, 0.00004) if thin else (0.05, 0.04, 0.03)
        front.append(gaussian((rng.normal(0, 0.03), rng.normal(0, 0.03), rng.uniform(0.05, 0.7)), s, quat=q,
                              opacity=0.3, dc=rng.normal(0.5, 0.2, 3)))
    for i in range(7):
        q = rng.normal(0, 1, 4)
        back.append(gaussian((rng.normal(0, 0.03), rng.normal(0, 0.03), rng.uniform(-0.7, -0.05)),
                             (0.07, 0.05, 0.00003), quat=q, opacity=0.4, dc=rng.normal(0.5, 0.2, 3)))
    gs = front + back
    nodes = [inner(2, 1, 0.0), leaf(len(back), len(front)), leaf(len(front), 0)]
    tree = make_tree(nodes, list(range(len(gs))), (-1, -1, -1, 1, 1, 1))
    return tree, np.stack(gs), sc.front_camera(16, 16, fovy=6.0)


def empty():
    g = gaussian((0.0, 0.0, 0.0), (0.1, 0.1, 0.1))
    tree = make_tree([leaf(0, 0)], [], (-1, -1, -1, 1, 1, 1))
    return tree, np.stack([g]), sc.front_camera(8, 8)


def miss():
    """Camera looking away from the scene box."""
    tree, rec, _ = analytic_single()
    return tree, rec, sc.look_at((0.0, 0.0, 2.5), target=(0.0, 0.0, 5.0), aspect=1.0)


# ---------------------------------------------------------------- pins
# Scenes whose expected images come from mathematics written independently of
# the oracle (tests/closed_form.py): one SH basis function at a time, a row
# of Gaussians composited front to back, and opacity reaching exactly 0.99.

def sh_probe(k: int, channel: int, coef: float):
    """One isotropic Gaussian at the origin whose only colour term is SH
    basis function k (1..15) of `channel` (DC coefficients zero), seen by
    six wide-angle cameras around it, so the ray directions cover the
    sphere.  Returns (tree, rec, [(camera, W, H)])."""
    rest = np.zeros(45, np.float32)
    rest[channel * 15 + (k - 1)] = coef  # f_rest is channel-major (cudaRenderer.cu:498)
    g = gaussian((0.0, 0.0, 0.0), (0.35, 0.35, 0.35), opacity=0.9, dc=(0.0, 0.0, 0.0), rest=rest)
    tree, rec = single([g])
    eyes = [(0, 0, 1.2), (0, 0, -1.2), (1.2, 0, 0), (-1.2, 0, 0), (0.7, 0.7, 0.7), (-0.6, -0.8, 0.5)]
    cams = [(sc.look_at(e, fovy=70.0, aspect=1.0), 20, 20) for e in eyes]
    return tree, rec, cams


def row(order=(3, 0, 4, 1, 2)):
    """Five small isotropic Gaussians on the view axis at z = 0.6, 0.3, 0,
    -0.3, -0.6 (front to back from the camera at z = 2.5), listed in one
    leaf in a shuffled order: opacities 0.5, 0.7, 0.003 (alpha always below
    1/255: skipped), 1.0 (alpha capped at 0.99 near the axis), 0.6."""
    zs = [0.6, 0.3, 0.0, -0.3, -0.6]
    ops = [0.5, 0.7, 0.003, 1.0, 0.6]
    dcs = [(0.9, 0.1, 0.2), (0.2, 0.8, 0.1), (0.5, 0.5, 0.5), (0.1, 0.3, 0.9), (0.7, 0.6, 0.0)]
    gs = [gaussian((0.0, 0.0, z), (0.05, 0.05, 0.05), opacity=o, dc=c) for z, o, c in zip(zs, ops, dcs)]
    tree = make_tree([leaf(5, 0)], list(order), (-1, -1, -1, 1, 1, 1))
    return tree, np.stack(gs), sc.front_camera(32, 32, fovy=6.0)


def exact_099(split: bool):
    """Gaussian P (opacity 1, z = 0.3) in front of Q (opacity 0.5, z = -0.3).
    Near the axis P's alpha is capped at exactly 0.99, so the accumulated
    opacity reaches exactly 0.99 after P.  Inside a leaf the walk stops only
    when it exceeds 0.99, so with both in one leaf Q is still composited; at a
    leaf boundary it stops once it reaches 0.99, so with a split plane at
    z = 0 between them (split=True) Q is not."""
    gp = gaussian((0.0, 0.0, 0.3), (0.05, 0.05, 0.05), opacity=1.0, dc=(0.9, 0.2, 0.1))
    gq = gaussian((0.0, 0.0, -0.3), (0.05, 0.05, 0.05), opacity=0.5, dc=(0.1, 0.9, 0.4))
    if split:
        tree = make_tree([inner(2, 1, 0.0), leaf(1, 0), leaf(1, 1)], [1, 0], (-1, -1, -1, 1, 1, 1))
    else:
        tree = make_tree([leaf(2, 0)], [0, 1], (-1, -1, -1, 1, 1, 1))
    return tree, np.stack([gp, gq]), sc.front_camera(24, 24, fovy=4.0)
