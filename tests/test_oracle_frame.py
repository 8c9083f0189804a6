"""Pins the oracle's frame restatement: the golden tiny frame, the RNG and
trigonometry it shares with the kernels, and invariants of a frame."""
import ctypes as C
import math
import os

import numpy as np
import pytest

import vrg

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _cam_from(v, W, H):
    return vrg.Camera((C.c_float * 3)(*v[0:3]), (C.c_float * 3)(*v[3:6]), (C.c_float * 3)(*v[6:9]),
                      (C.c_float * 3)(*v[9:12]), W, H)


def _py_combine(h, k):  # raygen.rs:51-59
    k = (k * 0x1b873593) & 0xFFFFFFFF
    h ^= k
    h = ((h << 13) | (h >> 19)) & 0xFFFFFFFF
    return (h * 5 + 0xe6546b64) & 0xFFFFFFFF


def _py_finalize(h):  # raygen.rs:63-70
    h ^= h >> 16
    h = (h * 0x85ebca6b) & 0xFFFFFFFF
    h ^= h >> 13
    h = (h * 0xc2b2ae35) & 0xFFFFFFFF
    h ^= h >> 16
    return h


def _py_rand(h):  # floatConstruct(murmur3_finalize(h))
    m = (_py_finalize(h) & 0x007FFFFF) | 0x3F800000
    return np.float32(np.array([m], np.uint32).view(np.float32)[0] - np.float32(1.0))


def test_murmur_and_float_construct(orc):
    rng = np.random.default_rng(5)
    for h, k in rng.integers(0, 2 ** 32, size=(2000, 2), dtype=np.uint64):
        h, k = int(h), int(k)
        assert orc.lib().orc_mm_combine(h, k) == _py_combine(h, k)
        assert np.float32(orc.lib().orc_mm_rand(h)) == _py_rand(h)
    assert _py_rand(0) == np.float32(0.0) or _py_rand(0) >= 0
    # all mantissa bits set gives the largest float below 1
    assert np.float32(np.array([0x3FFFFFFF], np.uint32).view(np.float32)[0] - np.float32(1)) < 1


def test_sincos_turns_accuracy(orc):
    s, c = C.c_float(), C.c_float()
    worst = 0.0
    for x in np.linspace(0, 1, 20001, dtype=np.float32)[:-1]:
        orc.lib().orc_sincos_turns(float(x), C.byref(s), C.byref(c))
        a = 2 * math.pi * float(x)
        worst = max(worst, abs(s.value - math.sin(a)), abs(c.value - math.cos(a)))
    assert worst < 4e-7


def test_golden_tiny_frame(orc):
    g = np.load(os.path.join(GOLDEN, "frame_tiny.npz"))
    mats, n = vrg.terrain_materials(77)
    world = g["blocks"]
    W = orc.build_world(mats, n, world)
    assert W.read_tl(0).tobytes() == g["light_tl"].tobytes()
    assert W.read_tl(1).tobytes() == g["geo_tl"].tobytes()
    R = orc.Renderer(48, 32, 3)
    try:
        for f in range(2):
            cam = _cam_from(g[f"f{f}_camera"], 48, 32)
            p = vrg.RenderParams(1, 1, 4, 3, vrg.MODE_PARITY, 0, 100 + f, 200 + f, 15.0, 0, 3, 0, 0)
            R.render(W, cam, p)
            img, _ = R.image()
            assert np.array_equal(img, g[f"f{f}_image"])
            assert np.array_equal(R.readback(vrg.DBG_HIT, 3), g[f"f{f}_hit"])
            for what, key in ((vrg.DBG_RADIANCE, "radiance"), (vrg.DBG_TEMPORAL, "temporal"),
                              (vrg.DBG_FINAL, "final")):
                assert R.readback(what, 3).tobytes() == g[f"f{f}_{key}"].tobytes(), (f, key)
    finally:
        R.close()
        W.close()


def test_frame_invariants(orc):
    mats, n = vrg.terrain_materials(3)
    world = vrg.terrain_blocks(3, 1, 1, 0.02)
    W = orc.build_world(mats, n, world)
    R = orc.Renderer(64, 48, 3)
    try:
        cam = vrg.orbit_camera(1, 1, 2, 8, 64, 48)
        R.render(W, cam, vrg.RenderParams(1, 0, 3, 3, 0, 0, 5, 6, 15.0, 0, 3, 0, 0))
        hit = R.readback(vrg.DBG_HIT, 3)
        d = R.readback(vrg.DBG_DIRECTION, 3)
        pdf = R.readback(vrg.DBG_BSDF_PDF, 3)
        mis = R.readback(vrg.DBG_MIS, 3)
        # primary rays are unit length
        assert np.allclose(np.linalg.norm(d[0], axis=1), 1, atol=1e-6)
        # a miss ends the path: direction 0 in the next slice, hit marked invalid
        miss = hit[0, :, 0] == 0xFFFFFFFF
        assert np.all(d[1][miss] == 0)
        # terminated slices carry the terminal record (raytrace.rs:406-416)
        term = hit[1, :, 0] == 0xFFFFFFFE
        assert np.all(pdf[1][term] == 1.0) and np.all(mis[1][term] == 0.0)
        assert set(np.unique(mis)).issubset({0.0, np.float32(0.3)})
        # hits name an exposed face: (face | half << 8) with face < 6, half < 2
        fh = hit[0, ~miss, 3]
        assert np.all((fh & 0xFF) < 6) and np.all((fh >> 8) < 2)
        temporal = R.readback(vrg.DBG_TEMPORAL, 3)
        m = temporal[:, 18].view(np.uint32)
        assert np.all(m >= 1)
    finally:
        R.close()
        W.close()
