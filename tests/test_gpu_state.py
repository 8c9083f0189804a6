"""Cross-frame state and host-side failures.

* A renderer's state blob (reservoir history ring, frame counter, FP64
  accumulation) replays: frames rendered after a load repeat, bit for bit, the
  frames rendered after the save, and the accumulation resumes.
* Requests the device cannot hold fail with a status, and the context keeps
  rendering afterwards: extents past the 2^31-pixel index space are refused
  before any allocation, and an allocation larger than the device returns
  VRG_ERR_OUT_OF_MEMORY (no kernel runs, nothing faults)."""
import ctypes as C

import numpy as np
import pytest

import vrg
from helpers import params, terrain_world

pytestmark = pytest.mark.gpu

W, H = 64, 40


@pytest.fixture(scope="module")
def scene(gpu_ctx):
    mats, n, blocks = terrain_world(41, 2, 1, 0.01)
    gpu_ctx.set_materials(mats, n)
    sc, objs = vrg.build_world(gpu_ctx, blocks)
    yield sc
    sc.close()
    for o in objs:
        o.release()


def _frames(r, scene, f0, n):
    out = []
    for f in range(f0, f0 + n):
        cam = vrg.orbit_camera(2, 1, f, 64, W, H)
        # parity mode: a 3-slot history ring; accumulation on
        p = params(nee=1, view=1, spatial=4, nb=3, seeds=(f, 7 * f + 1, 11 * f + 2), accumulate=1, flags=0)
        _, rad = r.render_params(scene, cam, p, want_image=False, want_radiance=True)
        assert r.last_stats.error_flags == 0
        out.append(rad.copy())
    return out


def test_state_save_load_replays_frames(gpu_ctx, scene):
    r = vrg.Renderer(gpu_ctx, W, H, 3)
    _frames(r, scene, 0, 4)
    blob = r.save_state()
    first = _frames(r, scene, 4, 3)
    acc_first, n_first = r.read_accumulation()
    # a fresh renderer of the same extent takes the blob too
    r2 = vrg.Renderer(gpu_ctx, W, H, 3)
    _frames(r2, scene, 0, 1)  # allocates its ring; the load replaces it
    for target in (r, r2):
        target.load_state(blob)
        again = _frames(target, scene, 4, 3)
        for a, b in zip(first, again):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
        acc, n = target.read_accumulation()
        assert n == n_first == 7
        assert np.array_equal(acc.view(np.uint32), acc_first.view(np.uint32))
    r.close()
    r2.close()


def test_state_load_rejects_other_renderers(gpu_ctx, scene):
    r = vrg.Renderer(gpu_ctx, W, H, 3)
    _frames(r, scene, 0, 1)
    blob = r.save_state()
    other = vrg.Renderer(gpu_ctx, W + 8, H, 3)
    lib = gpu_ctx.lib
    assert lib.vrg_renderer_state_load(other.h, vrg._ptr(blob), blob.nbytes) == vrg.ERR_INVALID_ARGUMENT
    bad = blob.copy()
    bad[0] ^= 0xFF  # magic
    assert lib.vrg_renderer_state_load(r.h, vrg._ptr(bad), bad.nbytes) == vrg.ERR_INVALID_ARGUMENT
    assert lib.vrg_renderer_state_load(r.h, vrg._ptr(blob), 16) == vrg.ERR_INVALID_ARGUMENT
    other.close()
    r.close()


def test_oversize_and_out_of_memory_fail_cleanly(gpu_ctx, scene):
    lib = gpu_ctx.lib
    h = C.c_void_p()
    # beyond the 2^31-pixel index space: refused before any allocation
    assert lib.vrg_renderer_create(gpu_ctx.h, 50000, 50000, 2, C.byref(h)) == vrg.ERR_UNSUPPORTED
    ws = np.array([40000, 40000], np.uint32)
    assert lib.vrg_renderer_create_batched(gpu_ctx.h, 2, vrg._ptr(ws), vrg._ptr(ws), 2,
                                           C.byref(h)) == vrg.ERR_UNSUPPORTED
    # 1.6 G pixels of frame state (hundreds of GB): the allocation fails
    st = lib.vrg_renderer_create(gpu_ctx.h, 40000, 40000, 8, C.byref(h))
    assert st == vrg.ERR_OUT_OF_MEMORY, st
    # the context still renders
    r = vrg.Renderer(gpu_ctx, W, H, 3)
    _frames(r, scene, 0, 1)
    r.close()
