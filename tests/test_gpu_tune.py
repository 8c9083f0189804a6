"""Launch configuration and autotuner: the configuration changes how a frame
is scheduled, never its bits; the autotuner restores the renderer's frame
counter and reservoir history."""
import ctypes as C

import numpy as np
import pytest

import vrg
from helpers import terrain_world

pytestmark = pytest.mark.gpu

W, H = 80, 56


@pytest.fixture(scope="module")
def world(gpu_ctx):
    mats, n, blocks = terrain_world(31, 2, 2, 0.01)
    gpu_ctx.set_materials(mats, n)
    scene, objs = vrg.build_world(gpu_ctx, blocks)
    yield scene
    scene.close()
    for o in objs:
        o.release()


def _params(f):
    return vrg.RenderParams(1, 1, 3, 3, vrg.MODE_CONFIG, f, 100 + f, 200 + f, 30.0, 20, 1, 0, 0, 4)


def _frames(r, scene, n=3):
    out = []
    for f in range(n):
        cam = vrg.orbit_camera(2, 2, f, 64, W, H)
        _, rad = r.render_params(scene, cam, _params(f), want_image=False, want_radiance=True)
        assert r.last_stats.error_flags == 0
        out.append(rad.copy())
    return out


def _same(a, b):
    return all(np.array_equal(x.view(np.uint32), y.view(np.uint32)) for x, y in zip(a, b))


def test_tuning_does_not_change_frames(gpu_ctx, world):
    ref = vrg.Renderer(gpu_ctx, W, H, 3)
    base = _frames(ref, world)
    ref.close()
    for t in (vrg.Tuning(1, 1, 1, 1, 1, 64), vrg.Tuning(0, 32, 0, 0, 32, 128), vrg.Tuning(2, 4, 3, 2, 16, 0),
              vrg.Tuning(0, 0, 0, 0, 0, 0, 1), vrg.Tuning(3, 16, 0, 4, 8, 128, 2), vrg.Tuning(0, 0, 0, 0, 0, 0, 2)):
        r = vrg.Renderer(gpu_ctx, W, H, 3)
        r.set_tuning(t)
        assert _same(base, _frames(r, world)), t.as_dict()
        r.close()


def test_autotune_restores_state_and_installs_best(gpu_ctx, world):
    ref = vrg.Renderer(gpu_ctx, W, H, 3)
    base = _frames(ref, world)
    ref.close()
    r = vrg.Renderer(gpu_ctx, W, H, 3)
    cam = vrg.orbit_camera(2, 2, 0, 64, W, H)
    best, ms = r.autotune(world, cam, _params(0), frames=1)
    assert ms > 0.0
    got = r.get_tuning()
    assert got.as_dict() == best.as_dict()
    assert 1 <= best.trace_refill <= 32 and best.stream_block in (64, 128, 256)
    n = C.c_uint32()
    gpu_ctx.lib.vrg_renderer_frame_index(r.h, C.byref(n))
    assert n.value == 0
    assert _same(base, _frames(r, world))  # same frames as an untuned renderer
    r.close()


def test_tuning_rejects_out_of_range(gpu_ctx):
    r = vrg.Renderer(gpu_ctx, 8, 8, 2)
    lib = gpu_ctx.lib
    for bad in (vrg.Tuning(0, 33, 0, 0, 0, 0), vrg.Tuning(0, 0, 0, 0, 0, 100), vrg.Tuning(65, 0, 0, 0, 0, 0),
                vrg.Tuning(0, 0, 0, 0, 0, 0, 3)):
        assert lib.vrg_renderer_set_tuning(r.h, C.byref(bad)) == vrg.ERR_INVALID_ARGUMENT
    r.close()


@pytest.mark.parametrize("w,h", [(83, 45), (96, 64), (40, 8)], ids=["83x45", "96x64", "40x8"])
def test_tma_staged_spatial_pass_bit_exact(gpu_ctx, world, orc, w, h):
    """The spatial pass with each CTA's 32x8-pixel reservoir tile staged in
    shared memory by a tensor copy (spatial_staging 1) bit for bit as with
    per-thread loads (2, the default) and as the oracle, with edge tiles partly
    outside the view."""
    from helpers import compare_frame, params
    mats, n, blocks = terrain_world(31, 2, 2, 0.01)
    OW = orc.build_world(mats, n, blocks)
    try:
        a, b = vrg.Renderer(gpu_ctx, w, h, 3), vrg.Renderer(gpu_ctx, w, h, 3)
        a.set_tuning(vrg.Tuning(0, 0, 0, 0, 0, 0, 2))
        b.set_tuning(vrg.Tuning(0, 0, 0, 0, 0, 0, 1))
        orr = orc.Renderer(w, h, 3)
        for f in range(3):
            cam = vrg.orbit_camera(2, 2, f, 64, w, h)
            p = params(nee=1, view=1, spatial=3, nb=3, seeds=(f, 40 + f, 80 + f))
            ia, ra = a.render_params(world, cam, p, want_image=True, want_radiance=True)
            ib, rb = b.render_params(world, cam, p, want_image=True, want_radiance=True)
            assert b.last_stats.error_flags == 0
            assert np.array_equal(ra.view(np.uint32), rb.view(np.uint32)) and np.array_equal(ia, ib), f
            orr.render(OW, cam, p)
            diffs = compare_frame(b, orr, 3)
            assert all(v == 0 for v in diffs.values()), (f, diffs)
        assert b.get_tuning().spatial_staging == 1 and a.get_tuning().spatial_staging == 2
        a.close()
        b.close()
        orr.close()
    finally:
        OW.close()
