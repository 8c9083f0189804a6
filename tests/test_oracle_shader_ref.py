"""Pins the oracle's frame against a second restatement of the reference's
shaders (tests/py_shader_ref.py, written from the GLSL, not from the oracle):
on a two-chunk terrain world, four frames through the reservoir ring (the
fourth reuses the first frame's slot), every
captured slice (per-bounce origin, direction, normal, emissivity,
reflectivity, MIS weight, BSDF pdf, NEE pdf, outgoing radiance, sampling pdf;
the temporal and spatial reservoirs; the ReSTIR target; the packed image)
bit for bit.  The chunk meshes, light BLASes and light TL of the restatement
are checked against the oracle's first."""
import numpy as np
import pytest

import py_shader_ref as ref
import vrg
from helpers import params
from test_gpu_mesh import look_at

pytestmark = pytest.mark.filterwarnings("ignore::RuntimeWarning")  # the reference's 0/0 NaNs

W, H, NB = 28, 18, 3


def _bits_equal(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    same = a.view(np.uint32) == b.view(np.uint32)
    same |= np.isnan(a) & np.isnan(b)
    return int((~same).sum())


@pytest.fixture(scope="module")
def worlds(orc):
    mats, n = orc.terrain_materials(17)
    blocks = orc.terrain_blocks(17, 2, 1, 0.15)
    OW = orc.build_world(mats, n, blocks)
    floor = np.zeros(vrg.CHUNK_BLOCKS, np.uint8)
    chunks = []
    for cx in range(2):
        c = ref.Chunk(blocks[cx, 0], vrg.chunk_neighbours(blocks, cx, 0, floor), mats, n)
        chunks.append((c, (32 * cx, 0, 0)))
    PW = ref.World(chunks, mats)
    yield OW, PW
    OW.close()


def test_meshes_and_light_trees_match(worlds):
    OW, PW = worlds
    n_light = 0
    for key, (c, _) in enumerate(PW.inst):
        info = OW.chunk_info(key)
        assert info["triangles"] == len(c.tris) and info["light_triangles"] == c.n_light
        nodes, _ = OW.chunk_bvh(key, 0)
        if c.n_light:
            assert nodes.tobytes() == c.light_nodes.tobytes(), key
        n_light += c.n_light
    assert n_light >= 200  # lamps enough for deep descents and many NEE hits
    assert OW.read_tl(0).tobytes() == PW.light_tl.tobytes()


def test_frames_match_the_shader_restatement(orc, worlds):
    OW, PW = worlds
    orr = orc.Renderer(W, H, NB)
    history = ref.empty_history(W * H)
    n_nee = n_lamp_dirs = n_merged = 0
    try:
        for f, (nee, view) in enumerate([(1, 1), (2, 0), (1, 2), (1, 1)]):
            cam = look_at((10.0 + 14 * f, 34.0, -14.0), (30.0 + 2 * f, 16.0, 18.0), W, H)
            p = params(nee=nee, view=view, spatial=5, nb=NB, seeds=(f, 40 + 7 * f, 90 + 3 * f))
            orr.render(OW, cam, p)
            hit = orr.readback(vrg.DBG_HIT, NB)
            hits = [[None if hit[b, q, 0] >= 0xFFFFFFFE else (int(hit[b, q, 0]), int(hit[b, q, 1]))
                     for q in range(W * H)] for b in range(NB)]
            out = ref.render(PW, cam, p, hits, f, history)
            diffs = {}
            for what, key in [(vrg.DBG_ORIGIN, "origin"), (vrg.DBG_DIRECTION, "direction"),
                              (vrg.DBG_NORMAL, "normal"), (vrg.DBG_EMISSIVITY, "emissivity"),
                              (vrg.DBG_REFLECTIVITY, "reflectivity"), (vrg.DBG_MIS, "mis"),
                              (vrg.DBG_BSDF_PDF, "bsdf_pdf"), (vrg.DBG_NEE_PDF, "nee_pdf"),
                              (vrg.DBG_RADIANCE, "radiance"), (vrg.DBG_Q, "q")]:
                diffs[key] = _bits_equal(orr.readback(what, NB), np.array(out[key], np.float32))
            for what, key in [(vrg.DBG_TEMPORAL, "temporal"), (vrg.DBG_SPATIAL, "spatial")]:
                diffs[key] = _bits_equal(orr.readback(what, NB), np.stack([ref.reservoir_row(r) for r in out[key]]))
            diffs["final"] = _bits_equal(orr.readback(vrg.DBG_FINAL, NB), np.array(out["final"], np.float32))
            img, _ = orr.image()
            diffs["image"] = int((img != out["image"]).sum())
            assert all(v == 0 for v in diffs.values()), f"frame {f}: {diffs}"
            mis = np.array(out["mis"], np.float32)
            n_lamp_dirs += int((mis > 0).sum())
            n_nee += int((np.array(out["nee_pdf"], np.float32) > 0).sum())
            n_merged += sum(s["m"] > t["m"] for s, t in zip(out["spatial"], out["temporal"]))
        # the frames exercise the light descent, the reverse walk and the spatial merges
        assert n_lamp_dirs > 1000 and n_nee > 300 and n_merged > 50, (n_lamp_dirs, n_nee, n_merged)
    finally:
        orr.close()


def test_meshes_and_isometries_match_the_shader_restatement(orc):
    """Two terrain chunks, the reference's unit cube with an emissive block's
    slots turned and lifted above them, and two triangle soups of mixed slots
    (one translated, one rotated): the light BLASes and the light TL over
    transformed light AABBs, then three frames through the ring, every slice
    bit for bit against the restatement (the mesh hits' barycentrics from the
    watertight test, the isometries in their matrix form)."""
    from test_gpu_mesh import iso, soup, unitcube
    mats, n = orc.terrain_materials(17)
    blocks = orc.terrain_blocks(17, 2, 1, 0.05)
    floor = np.zeros(vrg.CHUNK_BLOCKS, np.uint8)
    rng = np.random.default_rng(23)
    meshes = [(1000, unitcube(6), iso(0.5, 0.3, (20.25, 27.5, 14.75))),
              (1001, soup(rng, 60, 0, 22, (40.0, 24.0, 10.0), 6.0), (1.5, 0.0, -2.0)),
              (1002, soup(rng, 40, 0, 22, (0.0, 0.0, 0.0), 4.0), iso(1.1, -0.4, (30.0, 26.0, 5.0)))]
    OW = orc.World(mats, n)
    try:
        insts = []
        for cx in range(2):
            nb_ = vrg.chunk_neighbours(blocks, cx, 0, floor)
            OW.add_chunk(cx, blocks[cx, 0], nb_, (32 * cx, 0, 0))
            insts.append((ref.Chunk(blocks[cx, 0], nb_, mats, n), (32 * cx, 0, 0)))
        for key, verts, m in meshes:
            OW.add_mesh(key, verts, m)
            mm = np.asarray(m, np.float32)
            X = ref.xform(translation=tuple(mm)) if mm.size == 3 else ref.xform(m=mm.reshape(-1))
            insts.append((ref.Mesh(verts, mats), X))
        OW.commit()
        PW = ref.World(insts, mats)
        for key, (c, _) in enumerate(PW.inst):
            if c.n_light:
                okey = key if key < 2 else meshes[key - 2][0]
                nodes, _ = OW.chunk_bvh(okey, 0)
                assert nodes.tobytes() == c.light_nodes.tobytes(), key
        assert sum(c.n_light for c, _ in PW.inst if c.mesh) >= 12  # the cube and the soups' lamps
        assert OW.read_tl(0).tobytes() == PW.light_tl.tobytes()
        W_, H_ = 24, 16
        orr = orc.Renderer(W_, H_, NB)
        history = ref.empty_history(W_ * H_)
        mesh_hits = 0
        for f in range(3):
            cam = look_at((8.0 + 6 * f, 33.0, -6.0), (24.0 + 4 * f, 22.0, 14.0), W_, H_)
            p = params(nee=1, view=1, spatial=4, nb=NB, seeds=(f, 60 + f, 70 + f))
            orr.render(OW, cam, p)
            hit = orr.readback(vrg.DBG_HIT, NB)
            hits = [[None if hit[b, q, 0] >= 0xFFFFFFFE else (int(hit[b, q, 0]), int(hit[b, q, 1]))
                     for q in range(W_ * H_)] for b in range(NB)]
            mesh_hits += int(((hit[:, :, 0] >= 2) & (hit[:, :, 0] < 0xFFFFFFFE)).sum())
            out = ref.render(PW, cam, p, hits, f, history)
            diffs = {}
            for what, key in [(vrg.DBG_ORIGIN, "origin"), (vrg.DBG_DIRECTION, "direction"),
                              (vrg.DBG_NORMAL, "normal"), (vrg.DBG_EMISSIVITY, "emissivity"),
                              (vrg.DBG_REFLECTIVITY, "reflectivity"), (vrg.DBG_MIS, "mis"),
                              (vrg.DBG_BSDF_PDF, "bsdf_pdf"), (vrg.DBG_NEE_PDF, "nee_pdf"),
                              (vrg.DBG_RADIANCE, "radiance"), (vrg.DBG_Q, "q")]:
                diffs[key] = _bits_equal(orr.readback(what, NB), np.array(out[key], np.float32))
            for what, key in [(vrg.DBG_TEMPORAL, "temporal"), (vrg.DBG_SPATIAL, "spatial")]:
                diffs[key] = _bits_equal(orr.readback(what, NB), np.stack([ref.reservoir_row(r) for r in out[key]]))
            diffs["final"] = _bits_equal(orr.readback(vrg.DBG_FINAL, NB), np.array(out["final"], np.float32))
            img, _ = orr.image()
            diffs["image"] = int((img != out["image"]).sum())
            assert all(v == 0 for v in diffs.values()), f"frame {f}: {diffs}"
        assert mesh_hits >= 20, mesh_hits
        orr.close()
    finally:
        OW.close()


def test_mirror_and_glass_blocks_match_the_shader_restatement(orc):
    """The same two chunks with three block types made metallic (0.7, 0.4) and
    translucent (alpha 0.45, flagged see-through, so the faces behind them are
    meshed): the mirror and transmission branches of raytrace.rs:482-499, two
    frames bit for bit against the restatement."""
    mats, n = orc.terrain_materials(17)
    for b, metal, alpha, see in ((1, 0.7, 1.0, 0), (2, 0.4, 1.0, 0), (3, 0.0, 0.45, 1)):
        for f in range(6):
            mats[6 * b + f].metallic = metal
            mats[6 * b + f].alpha = alpha
            mats[6 * b + f].flags = (mats[6 * b + f].flags & ~1) | see
    blocks = orc.terrain_blocks(17, 2, 1, 0.15)
    OW = orc.build_world(mats, n, blocks)
    floor = np.zeros(vrg.CHUNK_BLOCKS, np.uint8)
    try:
        PW = ref.World([(ref.Chunk(blocks[cx, 0], vrg.chunk_neighbours(blocks, cx, 0, floor), mats, n),
                         (32 * cx, 0, 0)) for cx in range(2)], mats)
        orr = orc.Renderer(W, H, NB)
        history = ref.empty_history(W * H)
        specular = 0
        for f in range(2):
            cam = look_at((10.0 + 9 * f, 34.0, -14.0), (30.0 + 2 * f, 16.0, 18.0), W, H)
            p = params(nee=1, view=1, spatial=4, nb=NB, seeds=(f, 20 + f, 30 + f))
            orr.render(OW, cam, p)
            hit = orr.readback(vrg.DBG_HIT, NB)
            hits = [[None if hit[b, q, 0] >= 0xFFFFFFFE else (int(hit[b, q, 0]), int(hit[b, q, 1]))
                     for q in range(W * H)] for b in range(NB)]
            out = ref.render(PW, cam, p, hits, f, history)
            diffs = {}
            for what, key in [(vrg.DBG_ORIGIN, "origin"), (vrg.DBG_DIRECTION, "direction"),
                              (vrg.DBG_EMISSIVITY, "emissivity"), (vrg.DBG_REFLECTIVITY, "reflectivity"),
                              (vrg.DBG_MIS, "mis"), (vrg.DBG_BSDF_PDF, "bsdf_pdf"), (vrg.DBG_NEE_PDF, "nee_pdf"),
                              (vrg.DBG_RADIANCE, "radiance"), (vrg.DBG_Q, "q")]:
                diffs[key] = _bits_equal(orr.readback(what, NB), np.array(out[key], np.float32))
            for what, key in [(vrg.DBG_TEMPORAL, "temporal"), (vrg.DBG_SPATIAL, "spatial")]:
                diffs[key] = _bits_equal(orr.readback(what, NB), np.stack([ref.reservoir_row(r) for r in out[key]]))
            diffs["final"] = _bits_equal(orr.readback(vrg.DBG_FINAL, NB), np.array(out["final"], np.float32))
            assert all(v == 0 for v in diffs.values()), f"frame {f}: {diffs}"
            # hits taken by the mirror or the transmission branch: bsdf pdf 1 at a hit
            pdf = orr.readback(vrg.DBG_BSDF_PDF, NB)
            specular += int(((hit[:, :, 0] < 0xFFFFFFFE) & (pdf == 1.0)).sum())
        assert specular >= 20, specular
        orr.close()
    finally:
        OW.close()


def test_texture_atlas_matches_the_shader_restatement(orc):
    """Texture-atlas materials: three sRGB maps per slot sampled at the hit's
    uv (raytrace.rs:457-480), emission 1000 x the emissivity map, the light
    powers from the maps' luminances (get_texture_luminances, utils.rs:223-235),
    a mirror block type and a glass one.  Two frames bit for bit against the
    restatement."""
    import copy
    from test_gpu_render import _atlas
    rng = np.random.default_rng(77)
    mats, n = orc.terrain_materials(6)
    blocks = orc.terrain_blocks(6, 2, 1, 0.05)
    blocks[blocks == 2] = 0  # more mirror blocks
    blocks[blocks == 3] = 1  # and glass
    mats[6].flags = vrg.MAT_TRANSLUCENT  # block type 1 (slots 6..11) is glass
    atlas = _atlas(rng, mats, n // 6)
    floor = np.zeros(vrg.CHUNK_BLOCKS, np.uint8)
    OW = orc.World(mats, n)
    OW.set_atlas(atlas)
    for cx in range(2):
        OW.add_chunk(cx, blocks[cx, 0], vrg.chunk_neighbours(blocks, cx, 0, floor), (32 * cx, 0, 0))
    OW.commit()
    try:
        pm = copy.deepcopy(mats)  # the restatement's materials with the atlas luminances
        for t, L in enumerate(ref.atlas_luminances(atlas)):
            pm[t].luminance = float(L)
        PW = ref.World([(ref.Chunk(blocks[cx, 0], vrg.chunk_neighbours(blocks, cx, 0, floor), pm, n),
                         (32 * cx, 0, 0)) for cx in range(2)], pm, atlas=atlas)
        assert OW.read_tl(0).tobytes() == PW.light_tl.tobytes()
        orr = orc.Renderer(W, H, NB)
        history = ref.empty_history(W * H)
        for f in range(2):
            cam = look_at((10.0 + 9 * f, 34.0, -14.0), (30.0 + 2 * f, 16.0, 18.0), W, H)
            p = params(nee=1, view=1, spatial=4, nb=NB, seeds=(f, 20 + f, 30 + f))
            orr.render(OW, cam, p)
            hit = orr.readback(vrg.DBG_HIT, NB)
            hits = [[None if hit[b, q, 0] >= 0xFFFFFFFE else (int(hit[b, q, 0]), int(hit[b, q, 1]))
                     for q in range(W * H)] for b in range(NB)]
            out = ref.render(PW, cam, p, hits, f, history)
            diffs = {}
            for what, key in [(vrg.DBG_ORIGIN, "origin"), (vrg.DBG_DIRECTION, "direction"),
                              (vrg.DBG_EMISSIVITY, "emissivity"), (vrg.DBG_REFLECTIVITY, "reflectivity"),
                              (vrg.DBG_MIS, "mis"), (vrg.DBG_BSDF_PDF, "bsdf_pdf"), (vrg.DBG_NEE_PDF, "nee_pdf"),
                              (vrg.DBG_RADIANCE, "radiance"), (vrg.DBG_Q, "q")]:
                diffs[key] = _bits_equal(orr.readback(what, NB), np.array(out[key], np.float32))
            for what, key in [(vrg.DBG_TEMPORAL, "temporal"), (vrg.DBG_SPATIAL, "spatial")]:
                diffs[key] = _bits_equal(orr.readback(what, NB), np.stack([ref.reservoir_row(r) for r in out[key]]))
            diffs["final"] = _bits_equal(orr.readback(vrg.DBG_FINAL, NB), np.array(out["final"], np.float32))
            img, _ = orr.image()
            diffs["image"] = int((img != out["image"]).sum())
            assert all(v == 0 for v in diffs.values()), f"frame {f}: {diffs}"
        orr.close()
    finally:
        OW.close()


@pytest.mark.parametrize("scale", [2, 3])
def test_supersampled_postprocess_matches_the_restatement(orc, scale):
    """postprocess.rs:39-88 at srcscale 2 and 3 on random view colours (values
    outside 0..1, zeros and a NaN among them), bit for bit."""
    rng = np.random.default_rng(scale)
    view = (rng.random((6 * scale, 8 * scale, 3)) * 1.6 - 0.3).astype(np.float32)
    view[0, 0] = 0.0
    view[1, 2, 1] = np.nan
    img, out = orc.postprocess_scaled(view, scale)
    rimg, rout = ref.postprocess_scaled(view, scale)
    assert np.array_equal(img, rimg)
    assert _bits_equal(out, rout) == 0


def test_config_mode_matches_the_shader_restatement(orc, worlds):
    """The benchmark's CONFIG-mode parameters (a one-slot reservoir ring,
    spatial radius 30) with the history capped at m = 2 so that the cap
    applies within the frames: five frames at one camera, bit for bit."""
    OW, PW = worlds
    orr = orc.Renderer(W, H, NB)
    history = ref.empty_history(W * H, 1)
    capped = 0
    try:
        cam = look_at((10.0, 34.0, -14.0), (30.0, 16.0, 18.0), W, H)
        for f in range(5):
            p = params(nee=1, view=1, spatial=3, nb=NB, mode=vrg.MODE_CONFIG, seeds=(f, 50 + f, 60 + f),
                       radius=30.0, m_cap=2, slots=1)
            orr.render(OW, cam, p)
            hit = orr.readback(vrg.DBG_HIT, NB)
            hits = [[None if hit[b, q, 0] >= 0xFFFFFFFE else (int(hit[b, q, 0]), int(hit[b, q, 1]))
                     for q in range(W * H)] for b in range(NB)]
            out = ref.render(PW, cam, p, hits, f, history)
            diffs = {}
            for what, key in [(vrg.DBG_TEMPORAL, "temporal"), (vrg.DBG_SPATIAL, "spatial")]:
                diffs[key] = _bits_equal(orr.readback(what, NB), np.stack([ref.reservoir_row(r) for r in out[key]]))
            diffs["final"] = _bits_equal(orr.readback(vrg.DBG_FINAL, NB), np.array(out["final"], np.float32))
            diffs["radiance"] = _bits_equal(orr.readback(vrg.DBG_RADIANCE, NB), np.array(out["radiance"], np.float32))
            assert all(v == 0 for v in diffs.values()), f"frame {f}: {diffs}"
            capped += sum(1 for t in out["temporal"] if t["m"] == 3)  # capped at 2, then this frame's sample
        assert capped > 50, capped
    finally:
        orr.close()
