"""Host-side logic of the library that runs without a GPU: PCG32 seeds, the
synthetic terrain generator, the material table and the orbit camera."""
import numpy as np

import vrg


def test_pcg32_known_answer(vrglib):
    # pcg32_srandom(42, 54) of the PCG reference implementation
    r = vrg.Pcg32(42, 54)
    assert [r.next() for _ in range(6)] == [0xa15c02b7, 0x7b47f409, 0xba1d3330, 0x83d2f293, 0xbfa4784b,
                                            0xcbed606e]


def test_terrain_deterministic_and_in_spec(vrglib):
    a = vrg.terrain_blocks(5, 2, 3, 0.01)
    b = vrg.terrain_blocks(5, 2, 3, 0.01)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, vrg.terrain_blocks(6, 2, 3, 0.01))
    AIR = 22
    w = a.reshape(2, 3, 32, 32, 32)  # cx, cz, x, y, z
    solid = w < AIR
    heights = solid.sum(axis=3)
    assert heights.min() >= 8 and heights.max() <= 24
    # columns are solid from y=0 up to the height (heightfield)
    for cx in range(2):
        for cz in range(3):
            col = solid[cx, cz]
            h = heights[cx, cz]
            ys = np.arange(32)[None, :, None]
            assert np.array_equal(col, ys < h[:, None, :])
    lamps = ((a >= 6) & (a < AIR)).sum()
    assert 0 < lamps < 0.03 * solid.sum()


def test_materials(vrglib):
    mats, n = vrg.terrain_materials(9)
    assert n == 6 * 22
    for t in range(22):
        m = mats[6 * t]
        assert all(0.2 <= m.reflectivity[c] <= 0.8 for c in range(3))
        if t < 6:
            assert m.luminance == 0 and all(m.emission[c] == 0 for c in range(3))
        else:
            assert all(5 <= m.emission[c] <= 20 for c in range(3)) and m.luminance > 0
        for f in range(1, 6):
            assert mats[6 * t + f].luminance == m.luminance


def test_orbit_camera_frame(vrglib):
    cam = vrg.orbit_camera(4, 4, 3, 64, 1920, 1080)
    f, r, u = (np.array(list(v)) for v in (cam.front, cam.right, cam.up))
    assert abs(np.linalg.norm(f) - 1) < 1e-6
    assert abs(f @ r) < 1e-6 and abs(f @ u) < 1e-6 and abs(r @ u) < 1e-6
    assert u[1] < 0  # up vector points down-screen: worldup = (0,-1,0) (camera.rs:100)
