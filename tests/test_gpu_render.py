"""Full frame parity: the wavefront CUDA path vs the oracle on identical
seeded scenes, cameras and invocation seeds.  Every per-bounce SoA slice of
the reference's frame graph (origin, direction, normal, emissivity,
reflectivity, mis weight, bsdf pdf, nee pdf, outgoing radiance, q), the hit
(instance, triangle, voxel, face|half), both reservoirs, the ReSTIR final
target and the packed image are compared bit for bit (tolerance 0 ulp)."""
import numpy as np
import pytest

import vrg
from helpers import compare_frame, params, terrain_world

pytestmark = pytest.mark.gpu


def _setup(gpu_ctx, orc, seed, nx, nz, em, W, H, nb):
    mats, n, world = terrain_world(seed, nx, nz, em)
    gpu_ctx.set_materials(mats, n)
    scene, objs = vrg.build_world(gpu_ctx, world)
    OW = orc.build_world(mats, n, world)
    gr = vrg.Renderer(gpu_ctx, W, H, nb)
    orr = orc.Renderer(W, H, nb)
    return scene, objs, OW, gr, orr


def _frame(scene, OW, gr, orr, cam, p):
    img, rad = gr.render_params(scene, cam, p, want_image=True, want_radiance=True)
    orr.render(OW, cam, p)
    oimg, orad = orr.image()
    return img, rad, oimg, orad


@pytest.mark.parametrize("nee", [0, 1, 2])
def test_c0_frame_bit_exact(gpu_ctx, orc, nee):
    """Plain method, small: one 32^3 chunk, 128x128, 2 bounces, 1% emissive."""
    scene, objs, OW, gr, orr = _setup(gpu_ctx, orc, 1, 1, 1, 0.01, 128, 128, 2)
    try:
        cam = vrg.orbit_camera(1, 1, 0, 1, 128, 128)
        p = params(nee=nee, nb=2)
        img, rad, oimg, orad = _frame(scene, OW, gr, orr, cam, p)
        diffs = compare_frame(gr, orr, 2)
        assert all(v == 0 for v in diffs.values()), diffs
        assert np.array_equal(img.reshape(-1), oimg.reshape(-1))
        assert np.array_equal(rad.view(np.uint32).reshape(-1), orad.view(np.uint32).reshape(-1))
        st = gr.last_stats
        assert st.error_flags == 0
        assert st.rays_closest > 128 * 128
        # light-hit collection counters (bounce 0 queues light-pdf jobs when
        # NEE runs at every bounce): every job fetches the lamp root; a ray
        # crosses at most two faces of a block; each pixel whose bounce-0 nee
        # pdf is non-zero crossed at least one light triangle
        nee0 = gr.readback(vrg.DBG_NEE_PDF, 2)[0]
        assert st.light_hits <= 2 * st.light_leaves_visited
        assert st.light_hits >= int((nee0 != 0).sum())
        if nee == 1:
            assert st.rays_any > 0 and st.light_nodes_visited >= st.rays_any
            assert st.light_hits > 0
        else:
            assert st.rays_any == 0 and st.light_nodes_visited == 0
    finally:
        OW.close()


@pytest.mark.parametrize("W,H", [(83, 45), (7, 3)], ids=["83x45", "7x3"])
def test_odd_extent_bit_exact(gpu_ctx, orc, W, H):
    """Extents that are not whole 8x4 tiles (bounce 0 takes a single view's
    pixels tile by tile, the edge tiles partly outside the view): every pixel
    traced once, bit for bit as the oracle."""
    scene, objs, OW, gr, orr = _setup(gpu_ctx, orc, 4, 1, 1, 0.01, W, H, 3)
    try:
        for f in range(2):
            cam = vrg.orbit_camera(1, 1, f, 16, W, H)
            p = params(nee=1, view=1, spatial=3, nb=3, seeds=(f, 300 + f, 600 + f))
            img, rad, oimg, orad = _frame(scene, OW, gr, orr, cam, p)
            diffs = compare_frame(gr, orr, 3)
            assert all(v == 0 for v in diffs.values()), (f, diffs)
            assert np.array_equal(img.reshape(-1), oimg.reshape(-1))
            assert gr.last_stats.error_flags == 0
    finally:
        OW.close()


def test_restir_multi_frame_bit_exact(gpu_ctx, orc):
    """ReSTIR over a 3-slot ring, spatial neighbours, 3 bounces, moving camera."""
    scene, objs, OW, gr, orr = _setup(gpu_ctx, orc, 2, 2, 2, 0.005, 96, 64, 3)
    try:
        for f in range(5):
            cam = vrg.orbit_camera(2, 2, f, 64, 96, 64)
            p = params(nee=1, view=1, spatial=5, nb=3, seeds=(f, 1000 + f, 2000 + f))
            img, rad, oimg, orad = _frame(scene, OW, gr, orr, cam, p)
            diffs = compare_frame(gr, orr, 3)
            assert all(v == 0 for v in diffs.values()), (f, diffs)
            assert np.array_equal(img.reshape(-1), oimg.reshape(-1))
    finally:
        OW.close()


def test_config_mode_bit_exact(gpu_ctx, orc):
    """Config mode: M-cap 20, 1-slot history, 3 neighbours in a 30 px box, accumulation."""
    scene, objs, OW, gr, orr = _setup(gpu_ctx, orc, 3, 2, 1, 0.01, 80, 48, 3)
    try:
        for f in range(4):
            cam = vrg.orbit_camera(2, 1, f, 64, 80, 48)
            p = params(nee=1, view=1, spatial=3, nb=3, mode=vrg.MODE_CONFIG, seeds=(f, 7 + f, 9 + f),
                       radius=30.0, m_cap=20, slots=1, accumulate=1)
            _frame(scene, OW, gr, orr, cam, p)
            diffs = compare_frame(gr, orr, 3)
            assert all(v == 0 for v in diffs.values()), (f, diffs)
        acc, n = gr.read_accumulation()
        oacc, on = orr.accum()
        assert n == on == 4
        np.testing.assert_allclose(acc, (oacc / on).astype(np.float32), rtol=0, atol=0)
    finally:
        OW.close()


def test_debug_views(gpu_ctx, orc):
    scene, objs, OW, gr, orr = _setup(gpu_ctx, orc, 4, 1, 1, 0.02, 64, 64, 2)
    try:
        cam = vrg.orbit_camera(1, 1, 3, 8, 64, 64)
        for view in (0, 1, 2):
            p = params(nee=1, view=view, spatial=2, nb=2, seeds=(1, 2, 3 + view))
            img, rad, oimg, orad = _frame(scene, OW, gr, orr, cam, p)
            assert np.array_equal(img.reshape(-1), oimg.reshape(-1)), view
    finally:
        OW.close()


def test_golden_tiny_frame_gpu(gpu_ctx):
    """The CUDA path reproduces the committed golden frame (2 frames, ReSTIR)."""
    import ctypes as C
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "frame_tiny.npz"))
    mats, n = vrg.terrain_materials(77)
    gpu_ctx.set_materials(mats, n)
    scene, objs = vrg.build_world(gpu_ctx, g["blocks"])
    lt, gt = scene.get_tlas()
    assert lt.tobytes() == g["light_tl"].tobytes() and gt.tobytes() == g["geo_tl"].tobytes()
    r = vrg.Renderer(gpu_ctx, 48, 32, 3)
    for f in range(2):
        v = g[f"f{f}_camera"]
        cam = vrg.Camera((C.c_float * 3)(*v[0:3]), (C.c_float * 3)(*v[3:6]), (C.c_float * 3)(*v[6:9]),
                         (C.c_float * 3)(*v[9:12]), 48, 32)
        p = vrg.RenderParams(1, 1, 4, 3, vrg.MODE_PARITY, 0, 100 + f, 200 + f, 15.0, 0, 3, 0, vrg.RENDER_CAPTURE)
        img, _ = r.render_params(scene, cam, p)
        assert np.array_equal(img, g[f"f{f}_image"])
        assert np.array_equal(r.readback(vrg.DBG_HIT, 3), g[f"f{f}_hit"])
        for what, key in ((vrg.DBG_RADIANCE, "radiance"), (vrg.DBG_TEMPORAL, "temporal"), (vrg.DBG_FINAL, "final")):
            assert r.readback(what, 3).tobytes() == g[f"f{f}_{key}"].tobytes(), (f, key)


@pytest.mark.parametrize("scale", [2, 3])
def test_supersampled_frame_bit_exact(gpu_ctx, orc, scale):
    """Renderer.scale: traced at scale x the output extent, each output pixel
    the mean of its scale x scale samples (postprocess.rs:39-88) — against the
    oracle frame at the traced extent, postprocessed by the oracle."""
    OWd, OHd = 40, 24
    mats, n, world = terrain_world(4, 1, 2, 0.01)
    gpu_ctx.set_materials(mats, n)
    scene, objs = vrg.build_world(gpu_ctx, world)
    OW = orc.build_world(mats, n, world)
    try:
        gr = vrg.Renderer(gpu_ctx, OWd, OHd, 3, scale=scale)
        orr = orc.Renderer(OWd * scale, OHd * scale, 3)
        for f in range(2):
            cam = vrg.orbit_camera(1, 2, f, 64, OWd, OHd)
            ocam = vrg.orbit_camera(1, 2, f, 64, OWd * scale, OHd * scale)
            p = params(nee=1, view=1, spatial=3, nb=3, seeds=(f, 10 + f, 20 + f))
            img, rad = gr.render_params(scene, cam, p, want_image=True, want_radiance=True)
            orr.render(OW, ocam, p)
            _, oview = orr.image()
            oimg, orad = orc.postprocess_scaled(oview, scale)
            assert img.shape == (OHd, OWd, 4) and rad.shape == (OHd, OWd, 3)
            assert np.array_equal(img, oimg), f
            assert np.array_equal(rad.view(np.uint32), orad.view(np.uint32)), f
            assert gr.last_stats.error_flags == 0
        gr.close()
        orr.close()
    finally:
        OW.close()


def _atlas(rng, mats, n_types, size=16):
    """Random RGBA8 maps per slot; block type 0 is a mirror (metallicity 1),
    type 1 glass (alpha 0.3, translucent); emissive types keep emissive maps."""
    n = 6 * n_types
    a = np.zeros((n, 3, size, size, 4), np.uint8)
    a[:, 0, :, :, :3] = rng.integers(40, 220, size=(n, size, size, 3))
    a[:, 0, :, :, 3] = 255
    for t in range(n):
        if mats[t].emission[0] > 0:
            a[t, 1, :, :, :3] = rng.integers(30, 90, size=(size, size, 3))
    a[:, 1, :, :, 3] = 255
    a[:, 2, :, :, 3] = 255
    a[0:6, 2, :, :, 0] = 255          # mirror
    a[6:12, 0, :, :, 3] = 77          # glass
    return a


def test_texture_atlas_mirror_glass_bit_exact(gpu_ctx, orc):
    """Texture-atlas materials (three sRGB maps per slot sampled at the hit's
    gen_mesh uv, raytrace.rs:457-480), with mirror and glass blocks exercising
    the specular and transmissive branches (raytrace.rs:481-494)."""
    rng = np.random.default_rng(77)
    mats, n, world = terrain_world(6, 2, 2, 0.02)
    world[world == 2] = 0  # more mirror blocks
    world[(world == 3)] = 1  # and glass
    mats[6].flags = vrg.MAT_TRANSLUCENT  # block type 1 (slots 6..11) is glass
    atlas = _atlas(rng, mats, n // 6)
    gpu_ctx.set_materials(mats, n)
    gpu_ctx.set_atlas(atlas)
    scene, objs = vrg.build_world(gpu_ctx, world)
    OW = orc.World(mats, n)
    OW.set_atlas(atlas)
    floor = np.zeros(vrg.CHUNK_BLOCKS, dtype=np.uint8)
    for cx in range(2):
        for cz in range(2):
            OW.add_chunk(cx * 2 + cz, world[cx, cz], vrg.chunk_neighbours(world, cx, cz, floor), (32 * cx, 0, 32 * cz))
    OW.commit()
    try:
        W, H = 72, 48
        gr = vrg.Renderer(gpu_ctx, W, H, 3)
        orr = orc.Renderer(W, H, 3)
        for f in range(3):
            cam = vrg.orbit_camera(2, 2, 3 * f, 64, W, H)
            p = params(nee=1, view=1, spatial=3, nb=3, seeds=(f, 40 + f, 80 + f))
            img, rad, oimg, orad = _frame(scene, OW, gr, orr, cam, p)
            diffs = compare_frame(gr, orr, 3)
            assert all(v == 0 for v in diffs.values()), (f, diffs)
            assert np.array_equal(img.reshape(-1), oimg.reshape(-1))
            # the specular / transmissive branches (bsdf pdf 1 at a hit) were taken
            pdf = gr.readback(vrg.DBG_BSDF_PDF, 3)
            hit = gr.readback(vrg.DBG_HIT, 3)
            assert ((pdf == 1.0) & (hit[..., 0] != 0xFFFFFFFF)).sum() > 0
        gr.close()
        orr.close()
        lt, _ = scene.get_tlas()  # light TL over atlas luminances
        assert lt.tobytes() == OW.read_tl(0).tobytes()
    finally:
        gpu_ctx.set_atlas(None)
        OW.close()


@pytest.mark.parametrize("nb", [2, 3])
def test_plain_frames_equal_captured_frames(gpu_ctx, nb):
    """Frames rendered without VRG_RENDER_CAPTURE (the fast path: no per-bounce
    arrays kept, and the last vertex's continuation skipped because only its
    emission reaches the image) equal, bit for bit, the captured frames that
    the other tests compare with the oracle."""
    mats, n, world = terrain_world(6, 2, 1, 0.01)
    gpu_ctx.set_materials(mats, n)
    scene, objs = vrg.build_world(gpu_ctx, world)
    W, H = 88, 52
    outs = []
    for flags in (vrg.RENDER_CAPTURE, 0):
        r = vrg.Renderer(gpu_ctx, W, H, nb)
        frames = []
        for f in range(3):
            cam = vrg.orbit_camera(2, 1, f, 16, W, H)
            p = params(nee=1, view=1, spatial=3, nb=nb, seeds=(f, 40 + f, 80 + f), flags=flags)
            img, rad = r.render_params(scene, cam, p, want_image=True, want_radiance=True)
            assert r.last_stats.error_flags == 0
            frames.append((img.copy(), rad.copy()))
        outs.append(frames)
        r.close()
    for (ia, ra), (ib, rb) in zip(*outs):
        assert np.array_equal(ia, ib)
        assert np.array_equal(ra.view(np.uint32), rb.view(np.uint32))
    scene.close()
    for o in objs:
        o.release()


def test_axis_parallel_rays_bit_exact(gpu_ctx, orc):
    """Cameras looking exactly along -z and +x: the middle row and column of
    pixels get directions with a component of exactly 0 (parallel to the
    block planes of that axis).  Bit for bit as
    the oracle; and their primary rays walk about as many nodes as those of a
    camera tilted off the axes (a zero component culls on its axis like any
    other, instead of keeping every box that the other two axes cross)."""
    from test_gpu_mesh import look_at
    W, H = 64, 48  # even: row 24 has v = 0 and column 32 has u = 0 exactly
    scene, objs, OW, gr, orr = _setup(gpu_ctx, orc, 31, 2, 2, 0.02, W, H, 3)
    try:
        # eye heights above the highest block (its top is at y = 23): the
        # middle row's rays run level over the whole terrain without a hit
        for f, (eye, target) in enumerate([((21.0, 26.0, 70.0), (21.0, 26.0, 0.0)),
                                           ((-6.0, 26.5, 37.0), (60.0, 26.5, 37.0))]):
            cam = look_at(eye, target, W, H)
            p = params(nee=1, view=1, spatial=3, nb=3, seeds=(f, 50 + f, 90 + f))
            img, rad, oimg, orad = _frame(scene, OW, gr, orr, cam, p)
            diffs = compare_frame(gr, orr, 3)
            assert all(v == 0 for v in diffs.values()), (f, diffs)
            assert np.array_equal(img.reshape(-1), oimg.reshape(-1))
            dirs = gr.readback(vrg.DBG_DIRECTION, 3)[0].reshape(H, W, 3)
            assert (dirs[H // 2, :, 1] == 0).all() and (dirs[:, W // 2, 0 if f == 0 else 2] == 0).all()
            assert gr.last_stats.error_flags == 0
            # nodes per closest-hit ray against the same view tilted off the
            # axes (a renderer of its own: the frame counter of gr stays in
            # step with the oracle's)
            per_ray = []
            rs = vrg.Renderer(gpu_ctx, W, H, 2)
            for tgt in (target, (target[0] + 0.37, target[1] + 0.41, target[2] + 0.29)):
                rs.render_params(scene, look_at(eye, tgt, W, H), params(nee=1, nb=2, flags=vrg.RENDER_PLAIN_ONLY),
                                 want_image=False, want_radiance=True)
                st = rs.last_stats
                assert st.error_flags == 0 and st.rays_closest >= W * H
                per_ray.append(st.nodes_visited / st.rays_closest)
            rs.close()
            assert per_ray[0] < 1.25 * per_ray[1], per_ray
    finally:
        OW.close()
