"""Expected renders from mathematics, written without the oracle.

* real_sh(l, m, d): the real spherical harmonic of degree l and order m
  (Condon-Shortley phase) at unit direction d, from the published closed
  form Y_l^m = K_l^|m| P_l^|m|(cos theta) x {sqrt2 cos(m phi), 1,
  sqrt2 sin(|m| phi)} with K_l^m = sqrt((2l+1)/(4 pi) (l-m)!/(l+m)!) and
  the associated Legendre functions from their standard three-term
  recursion.  The reference's degree-3 colour term is
  sum_k coef_k Y_k(d) + 0.5 with k = l^2 + l + m (cudaRenderer.cu:487-558,
  constants cudaRenderer.h:33-48).
* ray_dirs: the primary ray of each pixel (cudaRenderer.cu:2336-2339) in
  double precision from the camera words.
* composite: the front-to-back recurrence of cudaRenderer.cu:1608-1708 in
  double precision for Gaussians listed per leaf: per Gaussian the closest
  approach along the ray (t* = (mu - o)^T S^-1 d / d^T S^-1 d, squared
  Mahalanobis distance g of that point), accepted when g < 8 and t* lies in
  the leaf's interval; response exp(-g^2 / 18); alpha = min(0.99, opacity
  * response), skipped when the response is below 0.0113 or alpha below
  1/255; C += c alpha (1 - A), A += alpha (1 - A); inside a leaf the walk
  stops when A > 0.99, at a leaf boundary when A >= 0.99.  Also returns
  per ray the number of Gaussians accepted (hits found in visited leaves)
  and blended.
"""
from __future__ import annotations

import math

import numpy as np


def assoc_legendre(l: int, m: int, x: np.ndarray) -> np.ndarray:
    """P_l^m(x), m >= 0, with the Condon-Shortley phase, by the recursion
    P_m^m = (-1)^m (2m-1)!! (1-x^2)^(m/2), P_{m+1}^m = x (2m+1) P_m^m,
    (l-m) P_l^m = x (2l-1) P_{l-1}^m - (l+m-1) P_{l-2}^m."""
    x = np.asarray(x, np.float64)
    pmm = np.ones_like(x)
    if m > 0:
        s = np.sqrt(np.maximum(0.0, 1.0 - x * x))
        fact = 1.0
        for _ in range(m):
            pmm = -pmm * fact * s
            fact += 2.0
    if l == m:
        return pmm
    pmm1 = x * (2 * m + 1) * pmm
    if l == m + 1:
        return pmm1
    pll = pmm1
    for ll in range(m + 2, l + 1):
        pll = (x * (2 * ll - 1) * pmm1 - (ll + m - 1) * pmm) / (ll - m)
        pmm, pmm1 = pmm1, pll
    return pll


def real_sh(l: int, m: int, d: np.ndarray) -> np.ndarray:
    """Real SH Y_l^m at unit directions d (n, 3): z = cos(theta),
    (x, y) = sin(theta) (cos(phi), sin(phi))."""
    d = np.asarray(d, np.float64)
    x, y, z = d[:, 0], d[:, 1], d[:, 2]
    am = abs(m)
    k = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
    p = assoc_legendre(l, am, z)
    phi = np.arctan2(y, x)
    if m > 0:
        return math.sqrt(2.0) * k * p * np.cos(m * phi)
    if m < 0:
        return math.sqrt(2.0) * k * p * np.sin(am * phi)
    return k * p


def sh_index(k: int) -> tuple:
    """Basis index k = l^2 + l + m -> (l, m)."""
    l = int(math.isqrt(k))
    return l, k - l * l - l


def ray_dirs(ci, width: int, height: int) -> tuple:
    """(eye (3,), unit directions (H*W, 3)) in pixel order y*W + x.  The
    unnormalised direction is formed in FP32 in the reference's order
    (cudaRenderer.cu:2336-2339: ((start + u sx stepX) - v sy stepY) - eye),
    because with the near plane at 0.005 that subtraction loses about 1e-5
    of the direction's precision and every FP32 renderer sees those
    directions; the normalisation is in double."""
    f = np.float32
    eye = np.array(list(ci.eye), f)
    start = np.array(list(ci.start), f)
    u = np.array(list(ci.u), f)
    v = np.array(list(ci.v), f)
    ys, xs = np.mgrid[0:height, 0:width]
    sx = xs.reshape(-1).astype(f) + f(0.5)
    sy = ys.reshape(-1).astype(f) + f(0.5)
    a = (u[None] * sx[:, None]) * f(ci.step_x)
    b = (v[None] * sy[:, None]) * f(ci.step_y)
    d = ((start[None] + a) - b) - eye[None]
    d = d.astype(np.float64)
    return eye.astype(np.float64), d / np.linalg.norm(d, axis=1, keepdims=True)


def colour(rec: np.ndarray, d: np.ndarray) -> np.ndarray:
    """Degree-3 SH colour of one 64-float record at unit directions d:
    sum_k c_k Y_k(d) + 0.5, clamped below at 0 (channel-major f_rest)."""
    out = np.full((d.shape[0], 3), 0.5)
    for k in range(16):
        l, m = sh_index(k)
        y = real_sh(l, m, d)
        for c in range(3):
            coef = float(rec[12 + c]) if k == 0 else float(rec[15 + c * 15 + (k - 1)])
            if coef != 0.0:
                out[:, c] += coef * y
    return np.maximum(out, 0.0)


def _rot(q: np.ndarray) -> np.ndarray:
    w, x, y, z = q / np.linalg.norm(q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def closest_approach(rec: np.ndarray, eye: np.ndarray, d: np.ndarray) -> tuple:
    """(t*, g) of one Gaussian record for rays eye + t d: the maximum of the
    response along the ray and the squared Mahalanobis distance there."""
    mu = rec[0:3].astype(np.float64)
    s = rec[4:7].astype(np.float64)
    rot = _rot(rec[8:12].astype(np.float64))
    m = (rot / s[None, :]).T  # rows of diag(1/s) R^T
    ng = m @ (eye - mu)
    gd = d @ m.T
    q = (gd * gd).sum(1)
    t = -(gd @ ng) / q
    p = ng[None, :] + t[:, None] * gd
    return t, (p * p).sum(1)


def composite(rec: np.ndarray, leaves, eye: np.ndarray, d: np.ndarray, t_bounds) -> dict:
    """Front-to-back composite for rays eye + t d through `leaves`, a list
    (front to back) of (Gaussian indices, t_near, t_far) where t_near/t_far
    are per-ray arrays.  Returns rgb, alpha, depth and `g` (n_gauss, n_rays)
    so callers can avoid rays within rounding of the g < 8 cut."""
    n = d.shape[0]
    tg = [closest_approach(rec[i], eye, d) for i in range(rec.shape[0])]
    cols = [colour(rec[i], d) for i in range(rec.shape[0])]
    rgb = np.zeros((n, 3))
    a = np.zeros(n)
    dep = np.zeros(n)
    n_accept = np.zeros(n, np.int64)
    n_blend = np.zeros(n, np.int64)
    for r in range(n):
        acc = 0.0
        done = False
        for ids, tn, tf in leaves:
            if done:
                break
            hits = []
            for i in ids:
                t, g = tg[i][0][r], tg[i][1][r]
                if g < 8.0 and tn[r] <= t <= tf[r]:
                    hits.append((t, i, g))
            hits.sort(key=lambda h: h[0])
            n_accept[r] += len(hits)
            for t, i, g in hits:
                gres = math.exp(-g * g / 18.0)
                alpha = min(0.99, float(rec[i, 3]) * gres)
                if gres < 0.0113 or alpha < 1.0 / 255.0:
                    continue
                w = alpha * (1.0 - acc)
                n_blend[r] += 1
                rgb[r] += cols[i][r] * w
                dep[r] += t * w
                acc += w
                if acc > 0.99:
                    done = True
                    break
            if acc >= 0.99:
                done = True
        a[r] = acc
    return {"rgb": rgb, "alpha": a, "depth": dep, "g": np.stack([x[1] for x in tg]),
            "t": np.stack([x[0] for x in tg]), "n_accept": n_accept, "n_blend": n_blend}


def slab(aabb, eye: np.ndarray, d: np.ndarray) -> tuple:
    """Scene-box interval of each ray (cudaRenderer.cu:379-399), t_near
    starting at 1e-2."""
    lo = np.asarray(aabb[0:3], np.float64)
    hi = np.asarray(aabb[3:6], np.float64)
    with np.errstate(divide="ignore"):
        inv = 1.0 / d
    t1 = (lo[None] - eye[None]) * inv
    t2 = (hi[None] - eye[None]) * inv
    tn = np.maximum(np.minimum(t1, t2).max(1), 1e-2)
    tf = np.maximum(t1, t2).min(1)
    return tn, tf
