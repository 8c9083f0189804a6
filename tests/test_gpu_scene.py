"""GPU chunk extraction (gen_mesh order + upload_object light prims) and the
batched BLAS / top-level builds vs the oracle: counts, node arrays and prim
order bit-exact."""
import numpy as np
import pytest

import vrg
from helpers import first_node_diff, nodes_equal, terrain_world

pytestmark = pytest.mark.gpu


def _worlds(gpu_ctx, orc, seed, nx, nz, emissive):
    mats, n, world = terrain_world(seed, nx, nz, emissive)
    gpu_ctx.set_materials(mats, n)
    scene, objs = vrg.build_world(gpu_ctx, world)
    W = orc.build_world(mats, n, world)
    return scene, objs, W


@pytest.mark.parametrize("seed,nx,nz,em", [(1, 1, 1, 0.01), (2, 2, 3, 0.005), (5, 4, 4, 0.02)])
def test_chunk_blas_bit_exact(gpu_ctx, orc, seed, nx, nz, em):
    scene, objs, W = _worlds(gpu_ctx, orc, seed, nx, nz, em)
    try:
        for key, o in enumerate(objs):
            gi = o.info()
            oi = W.chunk_info(key)
            assert gi["triangles"] == oi["triangles"]
            assert gi["light_triangles"] == oi["light_triangles"]
            assert gi["surface_blocks"] == oi["surface_blocks"]
            for which in (0, 1):
                gn, go = o.read_bvh(which)
                on, oo = W.chunk_bvh(key, which)
                assert nodes_equal(gn, on), (key, which, first_node_diff(gn, on))
                assert np.array_equal(go, oo)
        lt, gt = scene.get_tlas()
        assert nodes_equal(lt, W.read_tl(0)), first_node_diff(lt, W.read_tl(0))
        assert nodes_equal(gt, W.read_tl(1)), first_node_diff(gt, W.read_tl(1))
    finally:
        W.close()


def test_no_lights_dummy_tl(gpu_ctx, orc):
    scene, objs, W = _worlds(gpu_ctx, orc, 9, 2, 1, 0.0)
    try:
        lt, gt = scene.get_tlas()
        assert len(lt) == 1 and lt[0]["left"] == 0xFFFFFFFF and lt[0]["right"] == 0xFFFFFFFF
        assert nodes_equal(gt, W.read_tl(1))
    finally:
        W.close()


def test_air_chunk_is_empty_object(gpu_ctx, vrglib):
    mats, n = vrg.terrain_materials(1)
    gpu_ctx.set_materials(mats, n)
    up = vrg.SceneUploader(gpu_ctx)
    o = up.upload_chunk(np.full(vrg.CHUNK_BLOCKS, 22, np.uint8))
    assert o.info() == dict(faces=0, triangles=0, light_triangles=0, surface_blocks=0)
    sc = vrg.Scene(gpu_ctx)
    sc.add_object(1, o)
    lt, gt = sc.get_tlas()
    assert len(gt) == 0 and len(lt) == 1


def test_update_missing_key_is_error(gpu_ctx):
    sc = vrg.Scene(gpu_ctx)
    with pytest.raises(vrg.VrgError) as e:
        sc.update_object(12345, (0, 0, 0))
    assert e.value.status == vrg.ERR_NOT_FOUND


def test_transform_update_matches_oracle(gpu_ctx, orc):
    """Scene::update_object (scene.rs:205): moving a chunk keeps its BLAS and
    rebuilds the top levels and world-space layouts; the committed top levels
    and a rendered frame equal the oracle's world built with the chunk at its
    new place."""
    from helpers import compare_frame, params
    mats, n, world = terrain_world(12, 3, 2, 0.02)
    gpu_ctx.set_materials(mats, n)
    scene, objs = vrg.build_world(gpu_ctx, world)
    scene.commit()
    moved = {1: (0, 24, 32), 4: (64, -8, 32)}  # key = cx * nz + cz
    for key, t in moved.items():
        scene.update_object(key, t)
    lt, gt = scene.get_tlas()
    floor = np.zeros(vrg.CHUNK_BLOCKS, dtype=np.uint8)
    OW = orc.World(mats, n)
    try:
        for cx in range(3):
            for cz in range(2):
                key = cx * 2 + cz
                t = moved.get(key, (32 * cx, 0, 32 * cz))
                OW.add_chunk(key, world[cx, cz], vrg.chunk_neighbours(world, cx, cz, floor), t)
        OW.commit()
        assert nodes_equal(lt, OW.read_tl(0)), first_node_diff(lt, OW.read_tl(0))
        assert nodes_equal(gt, OW.read_tl(1)), first_node_diff(gt, OW.read_tl(1))
        W, H = 64, 48
        gr = vrg.Renderer(gpu_ctx, W, H, 3)
        orr = orc.Renderer(W, H, 3)
        cam = vrg.orbit_camera(3, 2, 5, 64, W, H)
        p = params(nee=1, view=1, spatial=3, nb=3, seeds=(1, 2, 3))
        img, rad = gr.render_params(scene, cam, p, want_image=True, want_radiance=True)
        orr.render(OW, cam, p)
        oimg, orad = orr.image()
        diffs = compare_frame(gr, orr, 3)
        assert all(v == 0 for v in diffs.values()), diffs
        assert np.array_equal(img.reshape(-1), oimg.reshape(-1))
        gr.close()
        orr.close()
    finally:
        OW.close()


def test_concurrent_uploads_match_serial(gpu_ctx):
    """SceneUploader is Clone and called from the chunk workers' pool
    (chunk_manager.rs:234-248): chunks uploaded from 8 threads at once give
    the same committed scene (top levels and every chunk's BLAS) as serial
    uploads."""
    from concurrent.futures import ThreadPoolExecutor
    mats, n, world = terrain_world(17, 4, 4, 0.01)
    gpu_ctx.set_materials(mats, n)
    floor = np.zeros(vrg.CHUNK_BLOCKS, dtype=np.uint8)
    up = vrg.SceneUploader(gpu_ctx)
    keys = [(cx, cz) for cx in range(4) for cz in range(4)]

    def upload(k):
        cx, cz = k
        return up.upload_chunk(world[cx, cz], vrg.chunk_neighbours(world, cx, cz, floor))

    with ThreadPoolExecutor(max_workers=8) as ex:
        objs = list(ex.map(upload, keys))
    par = vrg.Scene(gpu_ctx)
    for (cx, cz), o in zip(keys, objs):
        par.add_object(cx * 4 + cz, o, (32 * cx, 0, 32 * cz))
    ser, ser_objs = vrg.build_world(gpu_ctx, world)
    tp, ts = par.get_tlas(), ser.get_tlas()
    for a, b in zip(tp, ts):
        assert nodes_equal(a, b)
    for (cx, cz), o, so in zip(keys, objs, ser_objs):
        for which in (0, 1):
            na, pa = o.read_bvh(which)
            nb_, pb = so.read_bvh(which)
            assert nodes_equal(na, nb_) and np.array_equal(pa, pb), (cx, cz, which)
    for sc in (par, ser):
        sc.close()
    for o in objs + ser_objs:
        o.release()
