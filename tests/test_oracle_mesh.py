"""Pins the oracle's mesh path on the CPU: its watertight ray/triangle test
against an independent Python restatement (bit for bit) and against the
property the test is chosen for (no ray from inside a closed mesh escapes,
even through shared edges and vertices); a mesh's light BLAS (luminous
triangles, power = luminance * area, scene.rs:555-571) and geometry BVH
against the independent restatement of build.rs."""
import numpy as np

import py_build_ref
import py_tri_ref
from test_gpu_mesh import iso, soup, unitcube


def test_tri_test_matches_python_restatement(orc):
    rng = np.random.default_rng(5)
    n_hit = 0
    for k in range(3000):
        tri = (rng.random(9) * 4.0 - 2.0).astype(np.float32)
        o = (rng.random(3) * 8.0 - 4.0).astype(np.float32)
        if k % 3 == 0:  # aimed at a vertex or an edge midpoint of the triangle
            t3 = tri.reshape(3, 3)
            target = t3[k % 9 // 3] if k % 2 else (t3[0] + t3[1]) * np.float32(0.5)
        else:
            target = tri.reshape(3, 3).mean(axis=0) + (rng.random(3) - 0.5).astype(np.float32)
        d = (target - o).astype(np.float32)
        d = (d / np.float32(np.sqrt(np.float32((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2])))).astype(np.float32)
        a = orc.tri_test(tri, o, d)
        b = py_tri_ref.tri_test(tri, o, d)
        assert (a is None) == (b is None), k
        if a is not None:
            n_hit += 1
            assert np.array(a, np.float32).tobytes() == np.array(b, np.float32).tobytes(), k
    assert n_hit > 1000


def test_no_ray_escapes_a_closed_rotated_cube(orc):
    """Rays from the centre of the reference's unit cube, rotated and moved,
    toward every vertex, every edge midpoint and random directions: each hits
    a triangle (the shared edges and vertices of a watertight test let none
    through)."""
    m = iso(0.7, 0.45, (12.25, 30.5, -7.75))
    cube = unitcube(1)
    p = cube["position"].astype(np.float32)
    w = np.stack([((m[r, 0] * p[:, 0] + m[r, 1] * p[:, 1]) + m[r, 2] * p[:, 2]) + m[r, 3] for r in range(3)],
                 axis=1).astype(np.float32)
    tris = w.reshape(12, 9)
    centre = m[:, 3].astype(np.float32)
    targets = list(w) + [(w[i] + w[j]) * np.float32(0.5) for i in range(0, 36, 3) for j in (i + 1, i + 2)]
    rng = np.random.default_rng(9)
    targets += list(centre + rng.normal(size=(500, 3)).astype(np.float32))
    for tg in targets:
        d = (np.asarray(tg, np.float32) - centre).astype(np.float32)
        d = (d / np.float32(np.linalg.norm(d.astype(np.float64)))).astype(np.float32)
        hits = [orc.tri_test(t, centre, d, 0.0, 1000.0) for t in tris]
        assert any(h is not None for h in hits), tg


def test_mesh_light_blas_and_geometry_bvh_match_python_restatement(orc):
    mats, n = orc.terrain_materials(3)
    W = orc.World(mats, n)
    try:
        rng = np.random.default_rng(2)
        v = soup(rng, 150, 0, 22, (5.0, 6.0, 7.0), 4.0)
        W.add_mesh(7, v, (0.0, 0.0, 0.0))
        pos = v["position"].reshape(-1, 3, 3).astype(np.float32)
        slot = v["t"][0::3]
        lum = np.array([mats[int(t)].luminance for t in slot], np.float32)
        a, b, c = pos[:, 0], pos[:, 1], pos[:, 2]
        e1, e2 = (b - a).astype(np.float32), (c - a).astype(np.float32)
        cr = np.stack([e1[:, 1] * e2[:, 2] - e2[:, 1] * e1[:, 2], e1[:, 2] * e2[:, 0] - e2[:, 2] * e1[:, 0],
                       e1[:, 0] * e2[:, 1] - e2[:, 0] * e1[:, 1]], axis=1).astype(np.float32)
        area = (np.sqrt((cr[:, 0] * cr[:, 0] + cr[:, 1] * cr[:, 1]) + cr[:, 2] * cr[:, 2]) / np.float32(2.0))
        lit = np.nonzero(lum > 0)[0]
        power = (lum[lit] * area[lit].astype(np.float32)).astype(np.float32)
        pn, po = py_build_ref.build_bl_bvh(pos[lit].reshape(-1, 9), power, lit.astype(np.uint32))
        on, oo = W.chunk_bvh(7, 0)
        assert on.tobytes() == pn.tobytes() and np.array_equal(oo, po)
        gn, go = py_build_ref.build_bl_bvh(pos.reshape(-1, 9), np.zeros(len(pos), np.float32),
                                          np.arange(len(pos), dtype=np.uint32))
        on, oo = W.chunk_bvh(7, 1)
        assert on.tobytes() == gn.tobytes() and np.array_equal(oo, go)
        assert W.chunk_info(7) == dict(triangles=150, light_triangles=len(lit), surface_blocks=150)
    finally:
        W.close()
