"""Full-size parity: the headline workload itself, rendered by the CUDA path
and by the oracle.  The scene is the 4x4-chunk terrain of seed 20240601 with
0.5% emissive blocks; the frame is 1920x1080, 3 bounces, ReSTIR with 3
spatial neighbours in a 30 px box, M-cap 20 and a 1-slot history, on the orbit
camera.  Every captured per-bounce array (origin, direction, normal,
emissivity, reflectivity, mis weight, bsdf pdf, nee pdf, outgoing radiance,
q, hit), both reservoirs, the final target and the packed image are compared
bit for bit over two frames, the second reusing the first's reservoirs (any
NaN equal to any NaN: at this size a few reservoirs reach the reference's
0 / -0 weight, whose NaN encoding is the platform's)."""
import numpy as np
import pytest

import vrg
from helpers import compare_frame, params, terrain_world

pytestmark = pytest.mark.gpu

SEED, NX, NZ, EMISSIVE = 20240601, 4, 4, 0.005
W, H, NB = 1920, 1080, 3


def test_headline_workload_frames_bit_exact(gpu_ctx, orc):
    mats, n, world = terrain_world(SEED, NX, NZ, EMISSIVE)
    gpu_ctx.set_materials(mats, n)
    scene, objs = vrg.build_world(gpu_ctx, world)
    OW = orc.build_world(mats, n, world)
    gr = vrg.Renderer(gpu_ctx, W, H, NB)
    orr = orc.Renderer(W, H, NB)
    try:
        for f in range(2):
            cam = vrg.orbit_camera(NX, NZ, f, 64, W, H)
            p = params(nee=1, view=1, spatial=3, nb=NB, mode=vrg.MODE_CONFIG, seeds=(f, 1000 + f, 2000 + f),
                       radius=30.0, m_cap=20, slots=1)
            img, _ = gr.render_params(scene, cam, p)
            orr.render(OW, cam, p)
            oimg, _ = orr.image()
            diffs = compare_frame(gr, orr, NB)
            assert all(v == 0 for v in diffs.values()), (f, {k: v for k, v in diffs.items() if v})
            assert np.array_equal(img.reshape(-1), oimg.reshape(-1))
            assert gr.last_stats.error_flags == 0
            assert gr.last_stats.rays_closest > W * H
    finally:
        gr.close()
        orr.close()
        OW.close()
        scene.close()
        for o in objs:
            o.release()


def test_batched_workload_views_match_single_view_renders(gpu_ctx):
    """The 64-scene batched workload (chunk grids 1x1..8x8, extents from 256^2
    to 1920x1080, 56 M pixels, 2 bounces + ReSTIR), two frames replayed from a
    CUDA graph: every view bit for bit as a single-view renderer fed the same
    scene, camera, seeds and frame index (which the test above ties to the
    oracle at the full 1080p extent)."""
    C2_SEED, C2_SCENES = 20240602, 64
    C2_RES = [(256, 256), (640, 480), (1280, 720), (1920, 1080)]
    mats, n = vrg.terrain_materials(SEED)
    gpu_ctx.set_materials(mats, n)
    rng = np.random.default_rng(C2_SEED)
    grids = rng.integers(1, 9, size=(C2_SCENES, 2))
    res = [C2_RES[i] for i in rng.integers(0, len(C2_RES), size=C2_SCENES)]
    scenes, keep = [], []
    for i in range(C2_SCENES):
        sc, objs = vrg.build_world(gpu_ctx, vrg.terrain_blocks(C2_SEED + 1 + i, int(grids[i, 0]), int(grids[i, 1]),
                                                              EMISSIVE))
        scenes.append(sc)
        keep.append(objs)

    def params(flags):
        return vrg.RenderParams(1, 1, 3, 2, vrg.MODE_CONFIG, 0, 0, 0, 30.0, 20, 1, 0, flags, 4)

    def cams(f):
        return [vrg.orbit_camera(int(grids[v, 0]), int(grids[v, 1]), f, 64, w, h) for v, (w, h) in enumerate(res)]

    def seeds(v, f):
        return (3000 + 7 * v + 11 * f, 5000 + 13 * v + 17 * f)

    br = vrg.BatchRenderer(gpu_ctx, res, 2)
    try:
        batched = []
        for f in range(2):
            imgs, rads = br.render(scenes, cams(f), params(vrg.RENDER_GRAPH), [seeds(v, f) for v in range(C2_SCENES)],
                                   want_image=True, want_radiance=True)
            assert br.last_stats.error_flags == 0
            batched.append((imgs, rads))
        for v, (w, h) in enumerate(res):
            r = vrg.Renderer(gpu_ctx, w, h, 2)
            for f in range(2):
                p = params(0)
                p.temporal_seed, p.spatial_seed = seeds(v, f)
                img, rad = r.render_params(scenes[v], cams(f)[v], p, want_image=True, want_radiance=True)
                assert np.array_equal(img.reshape(-1), batched[f][0][v].reshape(-1)), (v, f)
                assert np.array_equal(rad.view(np.uint32).reshape(-1), batched[f][1][v].view(np.uint32).reshape(-1)), (v, f)
            r.close()
    finally:
        br.close()
        for sc in scenes:
            sc.close()
        for objs in keep:
            for o in objs:
                o.release()


def test_large_scene_frame_bit_exact(gpu_ctx, orc):
    """The large workload's scene (32x32 chunks, 1.1 M surface blocks, 0.2%
    emissive) seen at its full 3840x2160 view extent: one ReSTIR frame, every
    captured array bit for bit against the oracle (the deepest BVH of the
    workloads: the traversal stack bound and the lamp walk at full scale)."""
    n4, em4, w4, h4 = 32, 0.002, 3840, 2160
    mats, n, world = terrain_world(SEED, n4, n4, em4)
    gpu_ctx.set_materials(mats, n)
    scene, objs = vrg.build_world(gpu_ctx, world)
    OW = orc.build_world(mats, n, world)
    gr = vrg.Renderer(gpu_ctx, w4, h4, NB)
    orr = orc.Renderer(w4, h4, NB)
    try:
        cam = vrg.orbit_camera(n4, n4, 0, 64, w4, h4)
        p = params(nee=1, view=1, spatial=3, nb=NB, mode=vrg.MODE_CONFIG, seeds=(5, 1005, 2005), radius=30.0,
                   m_cap=20, slots=1)
        img, _ = gr.render_params(scene, cam, p)
        orr.render(OW, cam, p)
        oimg, _ = orr.image()
        diffs = compare_frame(gr, orr, NB)
        assert all(v == 0 for v in diffs.values()), {k: v for k, v in diffs.items() if v}
        assert np.array_equal(img.reshape(-1), oimg.reshape(-1))
        assert gr.last_stats.error_flags == 0
    finally:
        gr.close()
        orr.close()
        OW.close()
        scene.close()
        for o in objs:
            o.release()
