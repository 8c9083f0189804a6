"""A second, independent restatement (pure Python on numpy float32 scalars) of
the watertight ray/triangle test the oracle uses for mesh triangles: Woop,
Benthin and Wald, "Watertight Ray/Triangle Intersection", JCGT 2(1), 2013,
both faces, t = T / det, edge functions recomputed in double when one is
exactly zero.  Test infrastructure: pins oracle/vrg_oracle.cpp's tri_test."""
import numpy as np

F = np.float32


def tri_test(tri9, o, d, tmin=F(1e-3), tmax=F(1000.0)):
    v = [np.asarray(tri9, F).reshape(3, 3)[i] for i in range(3)]
    o = np.asarray(o, F)
    d = np.asarray(d, F)
    tmin, tmax = F(tmin), F(tmax)
    a = [abs(d[0]), abs(d[1]), abs(d[2])]
    kz = 0
    if a[1] > a[0]:
        kz = 1
    if a[2] > a[kz]:
        kz = 2
    kx = (kz + 1) % 3
    ky = (kx + 1) % 3
    if d[kz] < 0:
        kx, ky = ky, kx
    sx, sy, sz = d[kx] / d[kz], d[ky] / d[kz], F(1.0) / d[kz]
    A, B, C = v[0] - o, v[1] - o, v[2] - o
    ax, ay = A[kx] - sx * A[kz], A[ky] - sy * A[kz]
    bx, by = B[kx] - sx * B[kz], B[ky] - sy * B[kz]
    cx, cy = C[kx] - sx * C[kz], C[ky] - sy * C[kz]
    u, vv, w = cx * by - cy * bx, ax * cy - ay * cx, bx * ay - by * ax
    if u == 0 or vv == 0 or w == 0:
        D = np.float64
        u = F(D(cx) * D(by) - D(cy) * D(bx))
        vv = F(D(ax) * D(cy) - D(ay) * D(cx))
        w = F(D(bx) * D(ay) - D(by) * D(ax))
    if (u < 0 or vv < 0 or w < 0) and (u > 0 or vv > 0 or w > 0):
        return None
    det = (u + vv) + w
    if det == 0:
        return None
    az, bz, cz = sz * A[kz], sz * B[kz], sz * C[kz]
    T = (u * az + vv * bz) + w * cz
    t = T / det
    if not (tmin <= t <= tmax):
        return None
    return F(t), F(vv / det), F(w / det)
