"""Triangle meshes and rotated instances at the boundary: the reference's
SceneUploader::upload_object of an arbitrary Vec<Vertex3D> (scene.rs:547-725)
placed by a full isometry (scene.rs:150-216, scene_manager.rs:23-35), as its
own ego entity is: utils::unitcube() (utils.rs:81-176) added at main.rs:86-101.

Checked bit for bit (tolerance 0 ulp, any NaN equal to any NaN) against the
oracle on the same scenes: the meshes' light BLAS and geometry BVH, the light
top level over rotated instances, and every per-bounce array, hit, reservoir
and image of frames that see the rotated cube, lit by it when it is emissive
(the light descent, light sampling and light-pdf walk through a rotated
instance's transform)."""
import ctypes as C
import math

import numpy as np
import pytest

import vrg
from helpers import compare_frame, nodes_equal, params, terrain_world

pytestmark = pytest.mark.gpu


def cuboid(loc, dims, block):
    """utils.rs:81-170: 36 vertices, faces left, right, down, up, back, front;
    texture index t = 6 * block + face; each face's uvs as the reference
    lists them (the reference's unit cube uses block 1)."""
    fx, fy, fz = (loc[i] - 0.5 * dims[i] for i in range(3))
    dx, dy, dz = dims

    def v(a, b, c):
        return (fx + a * dx, fy + b * dy, fz + c * dz)

    faces = [
        [(v(0, 0, 1), (0, 1)), (v(0, 1, 0), (1, 0)), (v(0, 0, 0), (1, 1)),
         (v(0, 1, 1), (0, 0)), (v(0, 1, 0), (1, 0)), (v(0, 0, 1), (0, 1))],
        [(v(1, 1, 0), (0, 0)), (v(1, 0, 1), (1, 1)), (v(1, 0, 0), (0, 1)),
         (v(1, 1, 0), (0, 0)), (v(1, 1, 1), (1, 0)), (v(1, 0, 1), (1, 1))],
        [(v(0, 0, 0), (0, 0)), (v(1, 0, 0), (1, 0)), (v(0, 0, 1), (0, 1)),
         (v(1, 0, 0), (1, 0)), (v(1, 0, 1), (1, 1)), (v(0, 0, 1), (0, 1))],
        [(v(0, 1, 1), (1, 1)), (v(1, 1, 0), (0, 0)), (v(0, 1, 0), (1, 0)),
         (v(0, 1, 1), (1, 1)), (v(1, 1, 1), (0, 1)), (v(1, 1, 0), (0, 0))],
        [(v(0, 1, 0), (0, 0)), (v(1, 0, 0), (1, 1)), (v(0, 0, 0), (0, 1)),
         (v(0, 1, 0), (0, 0)), (v(1, 1, 0), (1, 0)), (v(1, 0, 0), (1, 1))],
        [(v(0, 0, 1), (1, 1)), (v(1, 0, 1), (0, 1)), (v(0, 1, 1), (1, 0)),
         (v(1, 0, 1), (0, 1)), (v(1, 1, 1), (0, 0)), (v(0, 1, 1), (1, 0))],
    ]
    out = np.zeros(36, vrg.VERTEX_DTYPE)
    k = 0
    for f, verts in enumerate(faces):
        for p, uv in verts:
            out[k] = (np.float32(p), 6 * block + f, np.float32(uv))
            k += 1
    return out


def unitcube(block=1):
    return cuboid((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), block)


def iso(yaw, pitch, t):
    """The matrix of an isometry: rotation about y by yaw, then about x by pitch, then translation t."""
    cy, sy, cp, sp = math.cos(yaw), math.sin(yaw), math.cos(pitch), math.sin(pitch)
    ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    rx = np.array([[1, 0, 0], [0, cp, -sp], [0, sp, cp]])
    m = np.zeros((3, 4), np.float32)
    m[:, :3] = (rx @ ry).astype(np.float32)
    m[:, 3] = np.float32(t)
    return m


def look_at(eye, target, W, H):
    """A camera at eye looking at target (right = front x (0,-1,0), up = right x front, tan 0.55)."""
    e = np.array(eye, np.float64)
    f = np.array(target, np.float64) - e
    f /= np.linalg.norm(f)
    r = np.cross(f, [0.0, -1.0, 0.0])
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    cam = vrg.Camera()
    cam.eye[:] = [float(x) for x in e.astype(np.float32)]
    cam.front[:] = [float(x) for x in f.astype(np.float32)]
    cam.right[:] = [float(x) for x in (0.55 * r).astype(np.float32)]
    cam.up[:] = [float(x) for x in (0.55 * u).astype(np.float32)]
    cam.width, cam.height = W, H
    return cam


def soup(rng, n, block_lo, block_hi, centre, radius):
    """n random triangles around centre (edges up to 2), slots of blocks in [block_lo, block_hi)."""
    c = rng.random((n, 1, 3)) * 2 * radius - radius + np.array(centre)
    tri = (c + rng.random((n, 3, 3)) * 2.0 - 1.0).astype(np.float32).reshape(-1, 3)
    v = np.zeros(3 * n, vrg.VERTEX_DTYPE)
    v["position"] = tri
    blocks = rng.integers(block_lo, block_hi, n)
    faces = rng.integers(0, 6, n)
    v["t"] = np.repeat(6 * blocks + faces, 3)
    v["uv"] = rng.random((3 * n, 2)).astype(np.float32)
    return v


def _world(gpu_ctx, orc, seed=5, nx=2, nz=2, em=0.01):
    mats, n, world = terrain_world(seed, nx, nz, em)
    gpu_ctx.set_materials(mats, n)
    scene, objs = vrg.build_world(gpu_ctx, world)
    OW = orc.build_world(mats, n, world)
    return mats, n, scene, objs, OW


def _add_mesh(gpu_ctx, scene, OW, key, verts, m):
    obj = vrg.SceneUploader(gpu_ctx).upload_object(verts)
    scene.add_object(key, obj, m)
    OW.add_mesh(key, verts, m)
    return obj


def _render_compare(gpu_ctx, scene, OW, orc, cam, nb, frames, W, H, view=1, spatial=3):
    gr = vrg.Renderer(gpu_ctx, W, H, nb)
    orr = orc.Renderer(W, H, nb)
    try:
        for f in range(frames):
            p = params(nee=1, view=view, spatial=spatial, nb=nb, seeds=(f, 100 + f, 200 + f))
            img, rad = gr.render_params(scene, cam, p, want_image=True, want_radiance=True)
            orr.render(OW, cam, p)
            oimg, orad = orr.image()
            diffs = compare_frame(gr, orr, nb)
            assert all(v == 0 for v in diffs.values()), (f, diffs)
            assert np.array_equal(img.reshape(-1), oimg.reshape(-1)), f
            assert gr.last_stats.error_flags == 0
        return gr.readback(vrg.DBG_HIT, nb)
    finally:
        gr.close()
        orr.close()


def test_mesh_bvhs_bit_exact(gpu_ctx, orc):
    """The light BLAS (build_bl_bvh over the luminous triangles, power =
    luminance * area) and the geometry BVH of meshes, and the light top
    level over translated and rotated instances."""
    rng = np.random.default_rng(3)
    mats, n, scene, objs, OW = _world(gpu_ctx, orc)
    try:
        meshes = [(1000, unitcube(6), iso(0.5, 0.0, (20.0, 30.0, 22.0))),  # emissive, rotated
                  (1001, soup(rng, 700, 0, 22, (40.0, 28.0, 40.0), 6.0), iso(1.1, 0.4, (3.0, -2.0, 1.5))),
                  (1002, unitcube(1), (30.0, 27.0, 30.0))]  # translated only
        keep = [_add_mesh(gpu_ctx, scene, OW, k, v, m) for k, v, m in meshes]
        lt, gt = scene.get_tlas()
        OW.commit()
        for (key, v, _), obj in zip(meshes, keep):
            for which in (0, 1):
                g_nodes, g_order = obj.read_bvh(which)
                o_nodes, o_order = OW.chunk_bvh(key, which)
                assert nodes_equal(g_nodes, o_nodes), (key, which)
                assert np.array_equal(g_order, o_order), (key, which)
        assert keep[0].info()["light_triangles"] == 12
        assert nodes_equal(lt, OW.read_tl(0)), "light TL"
        assert nodes_equal(gt, OW.read_tl(1)), "geometry TL"
    finally:
        OW.close()


@pytest.mark.parametrize("block,yaw,pitch", [(1, 0.6, 0.0), (6, 0.6, 0.35), (9, -1.2, 0.8)],
                         ids=["cube-y", "emissive-cube-yx", "emissive-cube-tilted"])
def test_rotated_ego_cube_frames_bit_exact(gpu_ctx, orc, block, yaw, pitch):
    """The reference's ego cube (utils::unitcube), rotated, above voxel
    terrain; two frames with ReSTIR (temporal + 3 spatial neighbours) and
    3 bounces.  With an emissive block's slots the cube is a light of its
    own: the descent, the sampled light point and the light-pdf walk go
    through its rotation."""
    mats, n, scene, objs, OW = _world(gpu_ctx, orc)
    try:
        centre = (32.0, 30.0, 32.0)
        cube = _add_mesh(gpu_ctx, scene, OW, 1000, unitcube(block), iso(yaw, pitch, centre))
        scene.get_tlas()
        OW.commit()
        W, H = 96, 64
        cam = look_at((35.5, 32.0, 35.0), (32.0, 29.5, 32.0), W, H)
        hit = _render_compare(gpu_ctx, scene, OW, orc, cam, 3, 2, W, H)
        inst = len([o for o in objs if o.info()["triangles"]])
        assert (hit[0, :, 0] == inst).sum() > 200, "the cube covers part of the image"
        assert (hit[0, :, 2] == 0xFFFFFFFF).sum() >= (hit[0, :, 0] == inst).sum()
        if block >= 6:
            assert cube.info()["light_triangles"] == 12
    finally:
        OW.close()


def test_mesh_soup_and_transform_update_bit_exact(gpu_ctx, orc):
    """A 1500-triangle soup of mixed slots (Lambertian and emissive, so both
    its geometry BVH and its light triangles are walked), rotated and tilted;
    then the same object moved by vrg_scene_update (no re-upload)."""
    rng = np.random.default_rng(11)
    mats, n, scene, objs, OW = _world(gpu_ctx, orc)
    try:
        v = soup(rng, 1500, 0, 22, (0.0, 0.0, 0.0), 7.0)
        m0 = iso(0.3, -0.2, (32.0, 34.0, 32.0))
        _add_mesh(gpu_ctx, scene, OW, 1000, v, m0)
        _add_mesh(gpu_ctx, scene, OW, 1001, unitcube(7), iso(2.0, 0.5, (27.0, 29.0, 37.0)))
        scene.get_tlas()
        OW.commit()
        W, H = 80, 60
        cam = look_at((44.0, 40.0, 46.0), (32.0, 30.0, 32.0), W, H)
        hit = _render_compare(gpu_ctx, scene, OW, orc, cam, 3, 2, W, H)
        assert (hit[0, :, 2] == 0xFFFFFFFF).sum() > 300, "the soup covers part of the image"
        m1 = iso(1.4, 0.6, (30.0, 35.0, 31.0))
        scene.update_object(1000, m1)
        scene.get_tlas()
        OW.add_mesh(1000, v, m1)
        OW.commit()
        _render_compare(gpu_ctx, scene, OW, orc, cam, 3, 1, W, H)
    finally:
        OW.close()


def test_batched_view_of_a_mesh_scene(gpu_ctx, orc):
    """A batched frame whose views include a scene with a rotated emissive
    mesh renders each view as the single-view renderer does."""
    mats, n, scene, objs, OW = _world(gpu_ctx, orc)
    OW.close()
    _add_mesh_gpu = vrg.SceneUploader(gpu_ctx).upload_object(unitcube(8))
    scene.add_object(1000, _add_mesh_gpu, iso(0.9, 0.3, (32.0, 30.0, 32.0)))
    scene.get_tlas()
    ext = [(64, 48), (40, 40)]
    cams = [look_at((35.5, 32.0, 35.0), (32.0, 29.5, 32.0), 64, 48), vrg.orbit_camera(2, 2, 3, 16, 40, 40)]
    br = vrg.BatchRenderer(gpu_ctx, ext, 2)
    p = params(nee=1, view=1, spatial=3, nb=2, mode=vrg.MODE_CONFIG, radius=30.0, m_cap=20, slots=1, flags=0)
    seeds = [(7, 8), (9, 10)]
    _, rads = br.render([scene, scene], cams, p, seeds, want_radiance=True)
    assert br.last_stats.error_flags == 0
    for v, (w, h) in enumerate(ext):
        r = vrg.Renderer(gpu_ctx, w, h, 2)
        pv = params(nee=1, view=1, spatial=3, nb=2, mode=vrg.MODE_CONFIG, radius=30.0, m_cap=20, slots=1,
                    seeds=(0, seeds[v][0], seeds[v][1]), flags=0)
        _, rad = r.render_params(scene, cams[v], pv, want_image=False, want_radiance=True)
        a, b = rad.reshape(-1).view(np.uint32), rads[v].reshape(-1).view(np.uint32)
        assert np.array_equal(a, b), v
        r.close()
    br.close()


def test_transform_validation(gpu_ctx):
    """A chunk takes a whole-block translation only; a mesh takes a
    rotation-like R and |t| <= 4096; mesh uploads check their slots."""
    mats, n = vrg.terrain_materials(1)
    gpu_ctx.set_materials(mats, n)
    blocks = vrg.terrain_blocks(1, 1, 1, 0.01)[0, 0]
    up = vrg.SceneUploader(gpu_ctx)
    chunk = up.upload_chunk(blocks)
    cube = up.upload_object(unitcube(1))
    sc = vrg.Scene(gpu_ctx)
    with pytest.raises(vrg.VrgError) as e:
        sc.add_object(1, chunk, iso(0.5, 0.0, (0.0, 0.0, 0.0)))
    assert e.value.status == vrg.ERR_UNSUPPORTED
    with pytest.raises(vrg.VrgError):
        sc.add_object(1, chunk, (0.5, 0.0, 0.0))
    sc.add_object(2, cube, iso(0.5, 0.2, (1.0, 2.0, 3.0)))
    with pytest.raises(vrg.VrgError):
        sc.update_object(2, iso(0.5, 0.2, (5000.0, 0.0, 0.0)))
    scaled = np.eye(3, 4, dtype=np.float32) * 2.0
    with pytest.raises(vrg.VrgError):
        sc.update_object(2, scaled)
    bad = unitcube(1)
    bad["t"][0] = n  # past the material table
    with pytest.raises(vrg.VrgError) as e:
        up.upload_object(bad)
    assert e.value.status == vrg.ERR_INVALID_ARGUMENT
    with pytest.raises(vrg.VrgError):
        up.upload_object(unitcube(1)[:35])
    empty = up.upload_object(np.zeros(0, vrg.VERTEX_DTYPE))
    assert empty.info()["triangles"] == 0
    sc.add_object(3, empty)
    sc.get_tlas()
    sc.close()
