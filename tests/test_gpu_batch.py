"""Batched views (vrg_render_batched): several scenes of uneven chunk grids and
view extents rendered by one launch sequence must give, view by view, the
bit-identical frames of single-view renderers fed the same scene, camera,
seeds and frame index — with and without the CUDA-graph replay.  This is the
parity contract of the batched path: the batch changes only how the work is
scheduled, never a pixel's arithmetic."""
import ctypes as C

import numpy as np
import pytest

import vrg

pytestmark = pytest.mark.gpu

MAT_SEED = 20240601
# (terrain seed, chunks x, chunks z, width, height): uneven grids and extents,
# including views whose pixel counts are not multiples of the 256-pixel lookup
# group and one smaller than a group
SCENES = [(11, 1, 1, 64, 48), (12, 2, 1, 97, 61), (13, 1, 2, 12, 10), (14, 1, 1, 40, 40)]
FRAMES = 3


def _params(flags=0, accumulate=0):
    return vrg.RenderParams(1, 1, 3, 2, vrg.MODE_CONFIG, 0, 0, 0, 30.0, 20, 1, accumulate, flags, 4)


def _seeds(v, f):
    return (1000 + 17 * v + 101 * f, 2000 + 31 * v + 103 * f)


@pytest.fixture(scope="module")
def world(gpu_ctx):
    mats, n = vrg.terrain_materials(MAT_SEED)
    gpu_ctx.set_materials(mats, n)
    scenes, keep, cams = [], [], []
    for seed, nx, nz, w, h in SCENES:
        blocks = vrg.terrain_blocks(seed, nx, nz, 0.01)
        sc, objs = vrg.build_world(gpu_ctx, blocks)
        scenes.append(sc)
        keep.append(objs)
        cams.append([vrg.orbit_camera(nx, nz, f, 64, w, h) for f in range(FRAMES)])
    yield scenes, cams, keep
    for sc in scenes:
        sc.close()
    for objs in keep:
        for o in objs:
            o.release()


def _single(gpu_ctx, scenes, cams, accumulate=0):
    """Each view through its own single-view renderer."""
    out, rays = [], 0
    for v, (seed, nx, nz, w, h) in enumerate(SCENES):
        r = vrg.Renderer(gpu_ctx, w, h, 2)
        frames = []
        for f in range(FRAMES):
            p = _params(accumulate=accumulate)
            p.temporal_seed, p.spatial_seed = _seeds(v, f)
            img, rad = r.render_params(scenes[v], cams[v][f], p, want_image=True, want_radiance=True)
            frames.append((img.copy(), rad.copy()))
            rays += r.last_stats.rays_closest + r.last_stats.rays_any
        acc = r.read_accumulation() if accumulate else None
        out.append((frames, acc))
        r.close()
    return out, rays


def _batched(gpu_ctx, scenes, cams, flags, accumulate=0):
    br = vrg.BatchRenderer(gpu_ctx, [(w, h) for *_, w, h in SCENES], 2)
    frames, rays = [], []
    for f in range(FRAMES):
        imgs, rads = br.render(scenes, [cams[v][f] for v in range(len(SCENES))], _params(flags, accumulate),
                               [_seeds(v, f) for v in range(len(SCENES))], want_image=True, want_radiance=True)
        frames.append([(i.copy(), r.copy()) for i, r in zip(imgs, rads)])
        rays.append(br.last_stats.rays_closest + br.last_stats.rays_any)
        assert br.last_stats.error_flags == 0
    acc = br.read_accumulation() if accumulate else None
    br.close()
    return frames, rays, acc


def _same_bits(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("flags", [0, vrg.RENDER_GRAPH], ids=["launches", "graph"])
def test_batched_views_match_single_view_renders(gpu_ctx, world, flags):
    scenes, cams, _ = world
    single, rays_single = _single(gpu_ctx, scenes, cams)
    frames, rays, _ = _batched(gpu_ctx, scenes, cams, flags)
    for f in range(FRAMES):
        for v in range(len(SCENES)):
            img_s, rad_s = single[v][0][f]
            img_b, rad_b = frames[f][v]
            assert _same_bits(rad_s, rad_b), (f, v)
            assert np.array_equal(img_s, img_b), (f, v)
    assert sum(rays) == rays_single


def test_batched_accumulation_and_offsets(gpu_ctx, world):
    scenes, cams, _ = world
    single, _ = _single(gpu_ctx, scenes, cams, accumulate=1)
    _, _, (acc, n) = _batched(gpu_ctx, scenes, cams, vrg.RENDER_GRAPH, accumulate=1)
    assert n == FRAMES
    for v in range(len(SCENES)):
        a_s, n_s = single[v][1]
        assert n_s == FRAMES
        assert _same_bits(a_s, acc[v]), v


def test_batched_rejects_mismatched_views(gpu_ctx, world):
    scenes, cams, _ = world
    br = vrg.BatchRenderer(gpu_ctx, [(w, h) for *_, w, h in SCENES], 2)
    lib = gpu_ctx.lib
    n = len(SCENES)
    views = (vrg.View * n)()
    for v in range(n):
        views[v] = vrg.View(scenes[v].h, cams[v][0], 1, 2)
    p = _params()
    assert lib.vrg_render_batched(br.h, views, n - 1, C.byref(p), None, None) == vrg.ERR_INVALID_ARGUMENT
    views[1].camera.width += 1
    assert lib.vrg_render_batched(br.h, views, n, C.byref(p), None, None) == vrg.ERR_INVALID_ARGUMENT
    views[1].camera.width -= 1
    p.flags = vrg.RENDER_CAPTURE
    assert lib.vrg_render_batched(br.h, views, n, C.byref(p), None, None) == vrg.ERR_UNSUPPORTED
    p.flags = vrg.RENDER_GRAPH | vrg.RENDER_CACHE
    assert lib.vrg_render_batched(br.h, views, n, C.byref(p), None, None) == vrg.ERR_UNSUPPORTED
    # a single-view renderer refuses the batched call and the reverse
    r = vrg.Renderer(gpu_ctx, 8, 8, 2)
    assert lib.vrg_render_batched(r.h, views, n, C.byref(_params()), None, None) == vrg.ERR_STATE
    cam = vrg.orbit_camera(1, 1, 0, 64, SCENES[0][3], SCENES[0][4])
    assert lib.vrg_render(br.h, scenes[0].h, C.byref(cam), C.byref(_params()), None, None) == vrg.ERR_STATE
    r.close()
    br.close()


def test_commit_many_matches_single_commits(gpu_ctx):
    """Scenes committed together (one top-level and one lamp SAH build for all)
    equal the same scenes committed one by one: top-level node arrays and
    rendered frames, bit for bit.  Includes a scene without lights and an
    empty scene."""
    mats, n = vrg.terrain_materials(MAT_SEED)
    gpu_ctx.set_materials(mats, n)
    specs = [(21, 2, 2, 0.01), (22, 1, 1, 0.0), (23, 3, 1, 0.02), None]

    def make():
        out = []
        for spec in specs:
            if spec is None:
                out.append((vrg.Scene(gpu_ctx), []))
            else:
                seed, nx, nz, em = spec
                out.append(vrg.build_world(gpu_ctx, vrg.terrain_blocks(seed, nx, nz, em)))
        return out

    one = make()
    for sc, _ in one:
        sc.commit()
    many = make()
    vrg.commit_scenes([sc for sc, _ in many])
    for (a, _), (b, _), spec in zip(one, many, specs):
        ta, tb = a.get_tlas(), b.get_tlas()  # already committed: reads the top levels
        for x, y in zip(ta, tb):
            assert x.tobytes() == y.tobytes()
        nx, nz = (1, 1) if spec is None else spec[1:3]
        cam = vrg.orbit_camera(nx, nz, 3, 64, 48, 32)
        imgs = []
        for sc in (a, b):  # a fresh renderer each: same frame index, empty history
            r = vrg.Renderer(gpu_ctx, 48, 32, 2)
            p = _params()
            p.temporal_seed, p.spatial_seed = 5, 6
            _, rad = r.render_params(sc, cam, p, want_image=False, want_radiance=True)
            imgs.append(rad.copy())
            assert r.last_stats.error_flags == 0
            r.close()
        assert _same_bits(imgs[0], imgs[1])
    for group in (one, many):
        for sc, objs in group:
            sc.close()
            for o in objs:
                o.release()


def test_batched_frames_in_flight_match(gpu_ctx, world):
    """Batched frames rendered without stats into device buffers are in flight
    together (two array sets, a view table per set): they must equal, bit for
    bit, the batched frames rendered one at a time with stats."""
    torch = pytest.importorskip("torch")
    scenes, cams, _ = world
    lib = gpu_ctx.lib
    n = len(SCENES)
    frames = 5

    def views_of(f):
        views = (vrg.View * n)()
        for v in range(n):
            ts, ss = _seeds(v, f)
            views[v] = vrg.View(scenes[v].h, cams[v][f % FRAMES], ts, ss)
        return views

    ref = vrg.BatchRenderer(gpu_ctx, [(w, h) for *_, w, h in SCENES], 2)
    want = []
    for f in range(frames):
        _, rads = ref.render(scenes, [cams[v][f % FRAMES] for v in range(n)], _params(),
                             [_seeds(v, f) for v in range(n)], want_image=False, want_radiance=True)
        assert ref.last_stats.error_flags == 0
        want.append([r_.copy() for r_ in rads])
    ref.close()
    br = vrg.BatchRenderer(gpu_ctx, [(w, h) for *_, w, h in SCENES], 2)
    dev = [[torch.empty(w * h * 3, dtype=torch.float32, device="cuda") for *_, w, h in SCENES]
           for _ in range(frames)]
    torch.cuda.synchronize()
    for f in range(frames):
        outs = (vrg.FrameOutput * n)()
        for v in range(n):
            outs[v] = vrg.FrameOutput(None, dev[f][v].data_ptr(), 0, 0)
        p = _params()
        vrg.check(lib.vrg_render_batched(br.h, views_of(f), n, C.byref(p), C.cast(outs, C.c_void_p), None),
                  "vrg_render_batched")
    gpu_ctx.synchronize()
    for f in range(frames):
        for v, (_, _, _, w, h) in enumerate(SCENES):
            got = dev[f][v].cpu().numpy().reshape(h, w, 3)
            assert _same_bits(got, want[f][v]), (f, v)
    br.close()


def test_batched_cache_frame_matches_single_views(gpu_ctx):
    """A batched cache frame (2 bounces into the radiance cache, 4 training
    bounces for the training paths, ReSTIR view) forks its training branch
    after its whole query bounce; a single-view cache frame traces the
    training candidates' query bounce first and forks there, beside the
    other paths' query bounce.  The batch's first frame, before any training
    step has changed the cache, equals view by view the first cache frame of
    single-view renderers, each with a fresh cache of the same seed over the
    same scene, bit for bit; a second batched frame, on the trained cache,
    runs without device error flags."""
    mats, n = vrg.terrain_materials(MAT_SEED)
    gpu_ctx.set_materials(mats, n)
    sc, objs = vrg.build_world(gpu_ctx, vrg.terrain_blocks(15, 2, 2, 0.02))
    try:
        _, gtl = sc.get_tlas()
        lo, hi = gtl[0]["min"], gtl[0]["max"]
        ext = [(64, 48), (97, 61), (40, 40)]
        cams = [vrg.orbit_camera(2, 2, 5 + 9 * v, 64, w, h) for v, (w, h) in enumerate(ext)]
        br = vrg.BatchRenderer(gpu_ctx, ext, 8)
        cache = vrg.RadianceCache(gpu_ctx, lo, hi, seed=3)
        br.set_cache(cache)
        _, rads = br.render([sc] * len(ext), cams, _params(vrg.RENDER_CACHE),
                            [_seeds(v, 0) for v in range(len(ext))], want_radiance=True)
        assert br.last_stats.error_flags == 0
        batched = [r.copy() for r in rads]
        br.render([sc] * len(ext), cams, _params(vrg.RENDER_CACHE), [_seeds(v, 1) for v in range(len(ext))])
        assert br.last_stats.error_flags == 0
        br.set_cache(None)
        cache.close()
        br.close()
        for v, (w, h) in enumerate(ext):
            r = vrg.Renderer(gpu_ctx, w, h, 8)
            c = vrg.RadianceCache(gpu_ctx, lo, hi, seed=3)
            r.set_cache(c)
            p = _params(vrg.RENDER_CACHE)
            p.temporal_seed, p.spatial_seed = _seeds(v, 0)
            _, rad = r.render_params(sc, cams[v], p, want_image=False, want_radiance=True)
            assert r.last_stats.error_flags == 0
            assert np.abs(np.nan_to_num(rad, nan=0.0, posinf=0.0, neginf=0.0)).sum() > 0, v
            assert _same_bits(rad, batched[v]), v
            r.set_cache(None)
            c.close()
            r.close()
    finally:
        sc.close()
        for o in objs:
            o.release()
