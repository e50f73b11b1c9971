"""The device's folded rotation (reflect_axis in hsmc_gb300/csrc/cluster.cu)
against the reference's general rotate() expression (src/cluster_nvt.c:342-365)
evaluated in IEEE double without contraction: the same bits for every axis,
including pivots and points on the box faces and zero differences."""
import math

import numpy as np


def rotate_general(xx, yy, zz, aa, bb, cc, uu, vv, ww, theta=math.pi):
    cost, sint = math.cos(theta), math.sin(theta)
    uu2, vv2, ww2 = uu * uu, vv * vv, ww * ww
    xr = (aa * (vv2 + ww2) - uu * (bb * vv + cc * ww - uu * xx - vv * yy - ww * zz)) * (1 - cost) + xx * cost + \
        (-cc * vv + bb * ww - ww * yy + vv * zz) * sint
    yr = (bb * (uu2 + ww2) - vv * (aa * uu + cc * ww - uu * xx - vv * yy - ww * zz)) * (1 - cost) + yy * cost + \
        (cc * uu - aa * ww + ww * xx - uu * zz) * sint
    zr = (cc * (uu2 + vv2) - ww * (aa * uu + bb * vv - uu * xx - vv * yy - ww * zz)) * (1 - cost) + zz * cost + \
        (-bb * uu + aa * vv - vv * xx + uu * yy) * sint
    return xr, yr, zr


def reflect_folded(xx, yy, zz, a, axis, s=math.sin(math.pi)):
    t = [2.0 * a[0], 2.0 * a[1], 2.0 * a[2]]
    if axis == 0:
        return xx, (t[1] - yy) + (a[2] - zz) * s, (t[2] - zz) + (yy - a[1]) * s
    if axis == 1:
        return (t[0] - xx) + (zz - a[2]) * s, yy, (t[2] - zz) + (a[0] - xx) * s
    return (t[0] - xx) + (a[1] - yy) * s, (t[1] - yy) + (xx - a[0]) * s, zz


def _bits(v):
    return np.array(v, dtype=np.float64).view(np.uint64)


def test_cos_pi_is_minus_one():
    assert math.cos(math.pi) == -1.0


def test_folded_rotation_is_bit_identical():
    rng = np.random.default_rng(5)
    L = 17.23
    pts = list(rng.uniform(0, L, size=(20000, 3)))
    piv = list(rng.uniform(0, L, size=(20000, 3)))
    edge = [0.0, L, L / 2, 1e-300, 5e-324]
    for e in edge:
        pts.append(np.array([e, e, e]))
        piv.append(np.array([e, L - e if e < L else 0.0, e]))
    for k in range(len(pts)):
        pts.append(piv[k].copy())  # point on the pivot: zero differences
        piv.append(piv[k])
    for p, a in zip(pts, piv):
        for axis in range(3):
            u = [0.0, 0.0, 0.0]
            u[axis] = 1.0
            want = rotate_general(p[0], p[1], p[2], a[0], a[1], a[2], *u)
            got = reflect_folded(p[0], p[1], p[2], a, axis)
            assert np.array_equal(_bits(got), _bits(want)), (p, a, axis, got, want)
