"""CPU restatement of the reference's PLY loader, for tests only (the oracle;
the product reads PLY files through kdgr_read_ply).

loadGaussiansFromPly (Kd-treeConverterMain.cpp:1652-1769): header lines up
to ``end_header``; each ``property <type> <name>`` advances the vertex byte
offset (float 4, double 8, uchar 1, :1682-1684); the vertex block is read as
little-endian records of that stride; per vertex (:1720-1747):

* pos    = 3 floats at the offset of ``x``                      (:1720)
* f_dc   = 3 floats at ``f_dc_0``; f_rest = 45 floats at ``f_rest_0``
  when present                                                  (:1721-1725)
* opacity = 1 / (1 + expf(-opacity)) in FP32                    (:1729)
* scale  = expf(scale_i)                                        (:1731-1734)
* rot    = fMyVecNormalize4D(rot_0..3)                          (:1737-1738, :1568-1577)
* k_scale = calcKernelScale(opacity, 0.0113) with adaptive clamping and
  degree 4                                                      (:1747, Gaussian.h:6-15)

expf and logf/powf are taken as correctly rounded: double evaluation
rounded once to float.
"""
from __future__ import annotations

import numpy as np

_SIZES = {"float": 4, "double": 8, "uchar": 1}
f32 = np.float32


def _rounded_exp(x):
    return np.exp(x.astype(np.float64)).astype(np.float32)


def load_gaussians_from_ply(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        offsets, cur, n = {}, 0, 0
        while True:
            line = f.readline().decode("ascii").rstrip("\r\n")
            if line == "end_header":
                break
            tok = line.split()
            if tok[:2] == ["element", "vertex"]:
                n = int(tok[2])
            elif tok and tok[0] == "property":
                offsets[tok[2]] = cur
                cur += _SIZES.get(tok[1], 0)
        raw = np.frombuffer(f.read(n * cur), dtype=np.uint8).reshape(n, cur)

    def fl(name, count=1):
        o = offsets[name]
        return raw[:, o:o + 4 * count].copy().view("<f4").reshape(n, count)

    rec = np.zeros((n, 64), np.float32)
    rec[:, 0:3] = fl("x", 3)
    rec[:, 12:15] = fl("f_dc_0", 3)
    if "f_rest_0" in offsets:
        rec[:, 15:60] = fl("f_rest_0", 45)
    op = f32(1.0) / (f32(1.0) + _rounded_exp(-fl("opacity")[:, 0]))
    rec[:, 3] = op
    rec[:, 4:7] = _rounded_exp(fl("scale_0", 3))
    q = fl("rot_0", 4)
    len_sq = ((q[:, 0] * q[:, 0] + q[:, 1] * q[:, 1]) + q[:, 2] * q[:, 2]) + q[:, 3] * q[:, 3]
    ok = len_sq > f32(0.00001)
    inv = f32(1.0) / np.sqrt(np.where(ok, len_sq, f32(1.0)))
    rec[:, 8:12] = np.where(ok[:, None], q * inv[:, None], q)
    min_resp = np.minimum(f32(0.0113) / op, f32(0.97))
    a = f32(-4.5) / f32(81.0)
    lg = np.log(min_resp.astype(np.float64)).astype(np.float32)
    rec[:, 7] = np.power((lg / a).astype(np.float64), 0.25).astype(np.float32)
    return rec
