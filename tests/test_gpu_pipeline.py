"""Frames in flight: vrg_render without stats only enqueues the frame, and up
to three frames' bounces (each frame in its own array set) run beside each
other and beside the resolve and spatial passes of the frames before them.
A sequence rendered that way into device buffers, back to
back, must give the bit-identical frames of the same sequence rendered one
frame at a time (stats requested, so each frame runs alone), including across
a scene update committed in mid-sequence, a frame with stats in between, and a
second renderer interleaved on the same context."""
import ctypes as C

import numpy as np
import pytest

import vrg
from helpers import params, terrain_world

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

W, H, NB, FRAMES = 96, 64, 3, 6
MOVE_AT = 3  # frame before which chunk 1 is moved


def _world(ctx):
    mats, n, blocks = terrain_world(43, 2, 1, 0.01)
    ctx.set_materials(mats, n)
    sc, objs = vrg.build_world(ctx, blocks)
    sc.commit()  # the material table may change again once no upload is pending
    return sc, objs


def _p(f):
    return params(nee=1, view=1, spatial=4, nb=NB, seeds=(f, 7 * f + 1, 11 * f + 2), accumulate=1, flags=0)


def _cam(f):
    return vrg.orbit_camera(2, 1, f, 32, W, H)


def _move(sc, f):
    if f == MOVE_AT:
        sc.update_object(1, (32.0, 2.0, 0.0))


def test_frames_in_flight_match_frames_one_by_one(gpu_ctx):
    lib = gpu_ctx.lib
    sc_a, objs_a = _world(gpu_ctx)
    sc_b, objs_b = _world(gpu_ctx)
    # one by one: stats make every frame run alone
    ra = vrg.Renderer(gpu_ctx, W, H, NB)
    want = []
    for f in range(FRAMES):
        _move(sc_a, f)
        _, rad = ra.render_params(sc_a, _cam(f), _p(f), want_image=False, want_radiance=True)
        assert ra.last_stats.error_flags == 0
        want.append(rad.copy())
    acc_a, n_a = ra.read_accumulation()
    # in flight: device outputs, no stats, except one frame in the middle; a
    # second renderer's frames interleaved on the same stream
    rb = vrg.Renderer(gpu_ctx, W, H, NB)
    other = vrg.Renderer(gpu_ctx, W // 2, H // 2, NB)
    dev = [torch.empty(W * H * 3, dtype=torch.float32, device="cuda") for _ in range(FRAMES)]
    torch.cuda.synchronize()
    st = vrg.FrameStats()
    for f in range(FRAMES):
        _move(sc_b, f)
        out = vrg.FrameOutput(None, dev[f].data_ptr(), 0, 0)
        cam, p = _cam(f), _p(f)
        vrg.check(lib.vrg_render(rb.h, sc_b.h, C.byref(cam), C.byref(p), C.byref(out),
                                 C.byref(st) if f == 4 else None), "vrg_render")
        if f == 4:
            assert st.error_flags == 0
        if f % 2 == 1:
            ocam, op = vrg.orbit_camera(2, 1, f, 32, W // 2, H // 2), _p(100 + f)
            vrg.check(lib.vrg_render(other.h, sc_b.h, C.byref(ocam), C.byref(op), None, None), "vrg_render")
    acc_b, n_b = rb.read_accumulation()  # waits for the library stream
    assert n_a == n_b == FRAMES
    for f in range(FRAMES):
        got = dev[f].cpu().numpy().reshape(H, W, 3)
        assert np.array_equal(got.view(np.uint32), want[f].view(np.uint32)), f
    assert np.array_equal(acc_a.view(np.uint32), acc_b.view(np.uint32))
    for r in (ra, rb, other):
        r.close()
    for sc, objs in ((sc_a, objs_a), (sc_b, objs_b)):
        sc.close()
        for o in objs:
            o.release()


def test_frames_in_flight_after_resize(gpu_ctx):
    """A resize clears the renderer's buffers on the library stream; the next
    frame's early closest hit waits for that clear."""
    lib = gpu_ctx.lib
    sc, objs = _world(gpu_ctx)
    r = vrg.Renderer(gpu_ctx, W // 2, H // 2, NB)
    for f in range(2):  # frames at the old extent, left in flight
        cam, p = vrg.orbit_camera(2, 1, f, 32, W // 2, H // 2), _p(f)
        vrg.check(lib.vrg_render(r.h, sc.h, C.byref(cam), C.byref(p), None, None), "vrg_render")
    r.resize(W, H)
    dev = torch.empty(W * H * 3, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    cam, p = _cam(0), _p(0)
    out = vrg.FrameOutput(None, dev.data_ptr(), 0, 0)
    vrg.check(lib.vrg_render(r.h, sc.h, C.byref(cam), C.byref(p), C.byref(out), None), "vrg_render")
    r.read_accumulation()
    ref = vrg.Renderer(gpu_ctx, W, H, NB)
    _, want = ref.render_params(sc, _cam(0), _p(0), want_image=False, want_radiance=True)
    got = dev.cpu().numpy().reshape(H, W, 3)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    for x in (r, ref):
        x.close()
    sc.close()
    for o in objs:
        o.release()


def test_async_host_readback_with_frame_fences(gpu_ctx):
    """VRG_OUTPUT_HOST_ASYNC: each frame's image and radiance are copied into
    page-locked host buffers behind the frame, the call returns at once, and
    vrg_renderer_wait_frame fences each frame before its buffers are read.
    Two buffer sets alternate, as in an interactive loop; every frame equals
    the frame rendered one by one."""
    lib = gpu_ctx.lib
    sc_a, objs_a = _world(gpu_ctx)
    sc_b, objs_b = _world(gpu_ctx)
    ra = vrg.Renderer(gpu_ctx, W, H, NB)
    want = []
    for f in range(FRAMES):
        img, rad = ra.render_params(sc_a, _cam(f), _p(f), want_image=True, want_radiance=True)
        want.append((img.copy(), rad.copy()))
    rb = vrg.Renderer(gpu_ctx, W, H, NB)
    pinned = [(torch.empty(W * H * 4, dtype=torch.uint8, pin_memory=True),
               torch.empty(W * H * 3, dtype=torch.float32, pin_memory=True)) for _ in range(2)]
    got = []
    for f in range(FRAMES):
        img_t, rad_t = pinned[f % 2]
        out = vrg.FrameOutput(img_t.data_ptr(), rad_t.data_ptr(), vrg.OUTPUT_HOST_ASYNC, 0)
        cam, p = _cam(f), _p(f)
        vrg.check(lib.vrg_render(rb.h, sc_b.h, C.byref(cam), C.byref(p), C.byref(out), None), "vrg_render")
        if f >= 1:  # the previous frame's buffers, once its fence has passed
            rb.wait_frame(f - 1)
            pi, pr = pinned[(f - 1) % 2]
            got.append((pi.numpy().copy(), pr.numpy().copy()))
    rb.wait_frame(FRAMES - 1)
    pi, pr = pinned[(FRAMES - 1) % 2]
    got.append((pi.numpy().copy(), pr.numpy().copy()))
    for f in range(FRAMES):
        assert np.array_equal(got[f][0].reshape(H, W, 4), want[f][0]), f
        assert np.array_equal(got[f][1].reshape(H, W, 3).view(np.uint32), want[f][1].view(np.uint32)), f
    # a frame not rendered yet has no fence; an unknown output kind is refused
    assert lib.vrg_renderer_wait_frame(rb.h, FRAMES) == vrg.ERR_INVALID_ARGUMENT
    bad = vrg.FrameOutput(None, None, 3, 0)
    cam, p = _cam(0), _p(0)
    assert lib.vrg_render(rb.h, sc_b.h, C.byref(cam), C.byref(p), C.byref(bad), None) == vrg.ERR_INVALID_ARGUMENT
    gpu_ctx.synchronize()
    for r in (ra, rb):
        r.close()
    for sc, objs in ((sc_a, objs_a), (sc_b, objs_b)):
        sc.close()
        for o in objs:
            o.release()


def test_frames_in_flight_alternating_scenes(gpu_ctx):
    """Frames in flight that alternate between two committed scenes (the
    temporal reuse carries across the switch, as for frames one by one)."""
    lib = gpu_ctx.lib
    mats, n, blocks_x = terrain_world(43, 2, 1, 0.01)
    _, _, blocks_y = terrain_world(44, 1, 2, 0.02)
    gpu_ctx.set_materials(mats, n)
    sx, ox = vrg.build_world(gpu_ctx, blocks_x)
    sy, oy = vrg.build_world(gpu_ctx, blocks_y)
    vrg.commit_scenes([sx, sy])
    scenes = [sx, sy]
    ra = vrg.Renderer(gpu_ctx, W, H, NB)
    want = []
    for f in range(FRAMES):
        _, rad = ra.render_params(scenes[f % 2], _cam(f), _p(f), want_image=False, want_radiance=True)
        assert ra.last_stats.error_flags == 0
        want.append(rad.copy())
    rb = vrg.Renderer(gpu_ctx, W, H, NB)
    dev = [torch.empty(W * H * 3, dtype=torch.float32, device="cuda") for _ in range(FRAMES)]
    torch.cuda.synchronize()
    for f in range(FRAMES):
        out = vrg.FrameOutput(None, dev[f].data_ptr(), 0, 0)
        cam, p = _cam(f), _p(f)
        vrg.check(lib.vrg_render(rb.h, scenes[f % 2].h, C.byref(cam), C.byref(p), C.byref(out), None), "vrg_render")
    gpu_ctx.synchronize()
    for f in range(FRAMES):
        got = dev[f].cpu().numpy().reshape(H, W, 3)
        assert np.array_equal(got.view(np.uint32), want[f].view(np.uint32)), f
    for r in (ra, rb):
        r.close()
    for sc, objs in ((sx, ox), (sy, oy)):
        sc.close()
        for o in objs:
            o.release()


def test_cache_frames_in_flight_match(gpu_ctx):
    """Cache frames (ReSTIR over cache-terminated paths, training branch
    forked) in flight equal the same frames rendered one by one.  The cache
    learns at rate 0, so every frame sees the same cache whatever the order
    of the training atomics."""
    lib = gpu_ctx.lib
    sc, objs = _world(gpu_ctx)
    lt, gtl = sc.get_tlas()
    lo, hi = gtl[0]["min"], gtl[0]["max"]

    def cp(f):
        p = params(nee=1, view=1, spatial=3, nb=2, seeds=(f, 7 * f + 1, 11 * f + 2), accumulate=0,
                   flags=vrg.RENDER_CACHE)
        p.cache_train_bounces = 3
        return p

    want = []
    ra = vrg.Renderer(gpu_ctx, W, H, 8)
    ca = vrg.RadianceCache(gpu_ctx, lo, hi, learning_rate=0.0, seed=5)
    ra.set_cache(ca)
    for f in range(FRAMES):
        _, rad = ra.render_params(sc, _cam(f), cp(f), want_image=False, want_radiance=True)
        assert ra.last_stats.error_flags == 0
        want.append(rad.copy())
    rb = vrg.Renderer(gpu_ctx, W, H, 8)
    cb = vrg.RadianceCache(gpu_ctx, lo, hi, learning_rate=0.0, seed=5)
    rb.set_cache(cb)
    dev = [torch.empty(W * H * 3, dtype=torch.float32, device="cuda") for _ in range(FRAMES)]
    torch.cuda.synchronize()
    for f in range(FRAMES):
        out = vrg.FrameOutput(None, dev[f].data_ptr(), 0, 0)
        cam, p = _cam(f), cp(f)
        vrg.check(lib.vrg_render(rb.h, sc.h, C.byref(cam), C.byref(p), C.byref(out), None), "vrg_render")
    gpu_ctx.synchronize()
    for f in range(FRAMES):
        got = dev[f].cpu().numpy().reshape(H, W, 3)
        assert np.array_equal(got.view(np.uint32), want[f].view(np.uint32)), f
    for r in (ra, rb):
        r.set_cache(None)
        r.close()
    for c in (ca, cb):
        c.close()
    sc.close()
    for o in objs:
        o.release()
