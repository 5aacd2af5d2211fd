"""Seeded synthetic Gaussian scenes and pinhole cameras.

The reference renders trained 3D Gaussian Splatting captures loaded from
``.ply`` files (Kd-treeConverterMain.cpp:1652-1769).  No capture ships with
it, so every workload here is generated: positions, scales, rotations,
opacities and degree-3 SH coefficients drawn from fixed distributions with a
fixed seed.  Records come out *activated* exactly as the reference's PLY
loader leaves them: opacity through a sigmoid (:1729), scale through exp
(:1732-1734), the quaternion normalised in FP32 and stored w,x,y,z (:1737-1738,
fMyVecNormalize4D :1568-1577) and ``k_scale`` from calcKernelScale
(Gaussian.h:6-15, :1747).

Record layout (float32 index within a 64-float / 256-byte record, the
reference's ``Gaussian`` struct, Kd-treeConverter.h:319-335)::

    0-2 pos | 3 opacity | 4-6 scale | 7 k_scale | 8-11 rot (w,x,y,z)
    12-14 f_dc | 15-59 f_rest (channel-major: f_rest[c*15 + k]) | 60-63 pad

Workloads (the five configurations of the render benchmark):

* ``uniform``  -- 100k Gaussians uniform in the unit cube centred on the
  origin (the camera's target), log-scale ~ N(ln 0.01, 0.5) per axis.
* ``cluster``  -- cluster+shell mixture: 80% from anisotropic clusters
  (centres U[-1,1]^3, per-cluster axis scales U(0.02,0.2), random cluster
  rotation), 20% on a radius-1.5 shell; log-scale ~ N(ln 0.005, 0.7); a 5%
  heavy tail stretched to axis ratios of 10^U(2, 3.4); opacity
  sigmoid(N(0.5,1.2)).
* SH for both: DC ~ N(0.5, 0.2), the 45 higher coefficients ~ N(0, 0.05).

Generation uses numpy's PCG64 stream, so a seed gives the same scene for a
given numpy version.
"""
from __future__ import annotations

import math
import struct
from dataclasses import dataclass
from typing import Sequence

import numpy as np

REC_FLOATS = 64
F_POS, F_OPACITY, F_SCALE, F_KSCALE, F_ROT, F_DC, F_REST = 0, 3, 4, 7, 8, 12, 15

KERNEL_MIN_RESPONSE = np.float32(0.0113)


def _normalize_quat_f32(q: np.ndarray) -> np.ndarray:
    """fMyVecNormalize4D (Kd-treeConverterMain.cpp:1568-1577) in float32."""
    q = q.astype(np.float32)
    len_sq = q[:, 0] * q[:, 0] + q[:, 1] * q[:, 1]
    len_sq = len_sq + q[:, 2] * q[:, 2]
    len_sq = len_sq + q[:, 3] * q[:, 3]
    inv = np.float32(1.0) / np.sqrt(len_sq)
    ok = len_sq > np.float32(0.00001)
    out = q.copy()
    out[ok] = q[ok] * inv[ok, None]
    return out


def _kernel_scale_f32(density: np.ndarray) -> np.ndarray:
    """calcKernelScale (Gaussian.h:6-15): radius where the degree-4 kernel
    falls to the clamped minimum response.  Unused by the render path; kept
    so records match the reference's."""
    d = density.astype(np.float64)
    min_resp = np.minimum(0.0113 / d, 0.97)
    a = -4.5 / 3.0 ** 4
    return np.power(np.log(min_resp) / a, 0.25).astype(np.float32)


def _assemble(pos, log_scale, quat_raw, opacity_logit, dc, rest) -> np.ndarray:
    n = pos.shape[0]
    rec = np.zeros((n, REC_FLOATS), dtype=np.float32)
    rec[:, F_POS:F_POS + 3] = pos.astype(np.float32)
    op = (1.0 / (1.0 + np.exp(-opacity_logit.astype(np.float32)))).astype(np.float32)
    rec[:, F_OPACITY] = op
    rec[:, F_SCALE:F_SCALE + 3] = np.exp(log_scale.astype(np.float32)).astype(np.float32)
    rec[:, F_KSCALE] = _kernel_scale_f32(op)
    rec[:, F_ROT:F_ROT + 4] = _normalize_quat_f32(quat_raw)
    rec[:, F_DC:F_DC + 3] = dc.astype(np.float32)
    rec[:, F_REST:F_REST + 45] = rest.astype(np.float32)
    return rec


def _sh(rng, n):
    dc = rng.normal(0.5, 0.2, size=(n, 3))
    rest = rng.normal(0.0, 0.05, size=(n, 45))
    return dc, rest


def uniform_cube(n: int = 100_000, seed: int = 0, scale: float = 0.01) -> np.ndarray:
    """The small plain workload: uniform positions in [-0.5, 0.5]^3,
    log-scale ~ N(ln scale, 0.5)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = rng.uniform(-0.5, 0.5, size=(n, 3))
    log_scale = rng.normal(math.log(scale), 0.5, size=(n, 3))
    quat = rng.normal(0.0, 1.0, size=(n, 4))
    opacity_logit = rng.normal(0.0, 1.0, size=n)
    dc, rest = _sh(rng, n)
    return _assemble(pos, log_scale, quat, opacity_logit, dc, rest)


def _quat_to_mat(q: np.ndarray) -> np.ndarray:
    q = q / np.linalg.norm(q, axis=-1, keepdims=True)
    w, x, y, z = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
        np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
        np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1),
    ], -2)


def cluster_shell(n: int = 1_000_000, seed: int = 1, n_clusters: int = 64,
                  shell_frac: float = 0.2, tail_frac: float = 0.05) -> np.ndarray:
    """The at-scale workload: anisotropic clusters plus a spherical shell."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n_shell = int(round(n * shell_frac))
    n_cl = n - n_shell
    centres = rng.uniform(-1.0, 1.0, size=(n_clusters, 3))
    axes = rng.uniform(0.02, 0.2, size=(n_clusters, 3))
    crot = _quat_to_mat(rng.normal(0.0, 1.0, size=(n_clusters, 4)))
    cid = rng.integers(0, n_clusters, size=n_cl)
    local = rng.normal(0.0, 1.0, size=(n_cl, 3)) * axes[cid]
    pos_cl = centres[cid] + np.einsum("nij,nj->ni", crot[cid], local)
    d = rng.normal(0.0, 1.0, size=(n_shell, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    pos_sh = d * (1.5 + rng.normal(0.0, 0.01, size=(n_shell, 1)))
    pos = np.concatenate([pos_cl, pos_sh], 0)
    perm = rng.permutation(n)
    pos = pos[perm]
    log_scale = rng.normal(math.log(0.005), 0.7, size=(n, 3))
    tail = rng.random(n) < tail_frac
    ratio = 10.0 ** rng.uniform(2.0, 3.4, size=n)
    half = 0.5 * np.log(ratio)
    log_scale[tail, 0] += half[tail]
    log_scale[tail, 2] -= half[tail]
    quat = rng.normal(0.0, 1.0, size=(n, 4))
    opacity_logit = rng.normal(0.5, 1.2, size=n)
    dc, rest = _sh(rng, n)
    return _assemble(pos, log_scale, quat, opacity_logit, dc, rest)


def scale_ratio(rec: np.ndarray) -> np.ndarray:
    s = rec[:, F_SCALE:F_SCALE + 3]
    return s.max(1) / s.min(1)


# ---------------------------------------------------------------- cameras
@dataclass
class Camera:
    """The fields of the reference's ``Camera`` the renderer reads
    (OpenGLStuffs.h:21-28): position, right/up/back axes and the double
    fovy (degrees), aspect and near plane.  The camera looks along -naxis."""
    pos: tuple
    uaxis: tuple
    vaxis: tuple
    naxis: tuple
    fovy: float = 60.0
    aspect: float = 1.0
    near_c: float = 0.005   # NEAR_PLANE, DefineConst.h:21

    def pack(self) -> bytes:
        """Binary image of ``kdgr_camera`` (include/kdgr.h)."""
        f = list(self.pos) + list(self.uaxis) + list(self.vaxis) + list(self.naxis)
        return struct.pack("<12f", *f) + struct.pack("<3d", self.fovy, self.aspect, self.near_c)


def look_at(eye, target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), fovy=60.0,
            aspect=1.0) -> Camera:
    eye = np.asarray(eye, np.float64)
    n = eye - np.asarray(target, np.float64)
    n /= np.linalg.norm(n)
    up = np.asarray(up, np.float64)
    if abs(float(np.dot(up, n))) > 0.999:
        up = np.array([0.0, 0.0, 1.0])
    u = np.cross(up, n)
    u /= np.linalg.norm(u)
    v = np.cross(n, u)
    f32 = lambda a: tuple(float(np.float32(x)) for x in a)
    return Camera(f32(eye), f32(u), f32(v), f32(n), float(fovy), float(aspect))


RESOLUTIONS = [(256, 256), (640, 480), (1280, 720), (1920, 1080)]


def sphere_cameras(n: int = 64, seed: int = 11, r_lo: float = 2.0, r_hi: float = 4.0,
                   resolutions=RESOLUTIONS, fovy: float = 60.0):
    """``n`` views on spheres of radius U(r_lo, r_hi) looking at the origin,
    an equal share at each resolution.  Returns [(Camera, W, H)]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    per = max(1, n // len(resolutions))
    for i in range(n):
        w, h = resolutions[min(i // per, len(resolutions) - 1)]
        d = rng.normal(0.0, 1.0, size=3)
        d /= np.linalg.norm(d)
        r = rng.uniform(r_lo, r_hi)
        out.append((look_at(d * r, fovy=fovy, aspect=w / h), w, h))
    return out


def front_camera(w: int, h: int, dist: float = 2.5, fovy: float = 60.0) -> Camera:
    """Eye at (0, 0, dist) looking at the origin, +y up."""
    return look_at((0.0, 0.0, dist), fovy=fovy, aspect=w / h)


# ---------------------------------------------------------------- files
def write_kdgs(path: str, rec: np.ndarray) -> None:
    """KDGS scene file: 'KDGS', u32 version 1, u32 n, u32 64, records."""
    rec = np.ascontiguousarray(rec, dtype=np.float32)
    with open(path, "wb") as f:
        f.write(b"KDGS" + struct.pack("<3I", 1, rec.shape[0], REC_FLOATS))
        f.write(rec.tobytes())


def read_kdgs(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        hdr = f.read(16)
        if hdr[:4] != b"KDGS":
            raise ValueError(f"{path}: not a KDGS scene file")
        ver, n, fl = struct.unpack("<3I", hdr[4:])
        if ver != 1 or fl != REC_FLOATS:
            raise ValueError(f"{path}: unsupported KDGS version {ver}/{fl}")
        data = np.frombuffer(f.read(n * REC_FLOATS * 4), dtype=np.float32)
    return data.reshape(n, REC_FLOATS).copy()


# ------------------------------------------------------------------ .ply
PLY_FIELDS = (["x", "y", "z", "nx", "ny", "nz", "f_dc_0", "f_dc_1", "f_dc_2"]
              + [f"f_rest_{i}" for i in range(45)]
              + ["opacity", "scale_0", "scale_1", "scale_2", "rot_0", "rot_1", "rot_2", "rot_3"])


def raw_gaussians(n: int, seed: int = 0) -> dict:
    """Pre-activation Gaussian fields as a trained 3DGS capture stores them
    (position, normal, SH, opacity logit, log-scale, raw quaternion), float32,
    drawn like the uniform workload."""
    rng = np.random.default_rng(seed)
    out = {
        "x": rng.uniform(-0.5, 0.5, n), "y": rng.uniform(-0.5, 0.5, n), "z": rng.uniform(-0.5, 0.5, n),
        "nx": np.zeros(n), "ny": np.zeros(n), "nz": np.zeros(n),
        "opacity": rng.normal(0.0, 1.0, n),
    }
    for c in range(3):
        out[f"f_dc_{c}"] = rng.normal(0.5, 0.2, n)
        out[f"scale_{c}"] = rng.normal(math.log(0.01), 0.5, n)
    for i in range(45):
        out[f"f_rest_{i}"] = rng.normal(0.0, 0.05, n)
    for i in range(4):
        out[f"rot_{i}"] = rng.normal(0.0, 1.0, n)
    return {k: v.astype(np.float32) for k, v in out.items()}


def write_ply(path: str, fields: dict, order: Sequence[str] | None = None,
              extra: Sequence[tuple] = ()) -> None:
    """Binary little-endian .ply with one vertex element: float properties in
    ``order`` (default: the 3DGS layout, PLY_FIELDS) plus ``extra`` properties
    given as (ply type, name, numpy array)."""
    order = list(order or PLY_FIELDS)
    n = len(fields[order[0]])
    np_types = {"float": "<f4", "double": "<f8", "uchar": "u1", "int": "<i4", "short": "<i2"}
    cols = [(name, "float", np.asarray(fields[name], np.float32)) for name in order]
    cols += [(name, t, np.asarray(v).astype(np_types[t])) for t, name, v in extra]
    dt = np.dtype([(name, np_types[t]) for name, t, _ in cols])
    data = np.zeros(n, dt)
    for name, _, v in cols:
        data[name] = v
    head = ["ply", "format binary_little_endian 1.0", f"element vertex {n}"]
    head += [f"property {t} {name}" for name, t, _ in cols]
    head += ["end_header"]
    with open(path, "wb") as f:
        f.write(("\n".join(head) + "\n").encode("ascii"))
        f.write(data.tobytes())
