"""ctypes binding of the oracle (test infrastructure only).

The oracle is the CPU restatement of the reference path in vrg_oracle.cpp;
tests, the smoke check and the benchmark's CPU baseline leg call it as the
checker.  The product library never loads it.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "vulkan-voxel-restir-gi_gb300"))
import vrg  # noqa: E402  (struct layouts only)

LIB = os.path.join(HERE, "_build", "liboracle.so")
_lib = None
_P = C.c_void_p


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            from build import build  # noqa
            build()
        L = C.CDLL(LIB)
        sig = [
            ("orc_build_tl_bvh", C.c_int, [C.c_uint32, _P, _P, _P, _P, _P, _P]),
            ("orc_build_bl_bvh", C.c_int, [C.c_uint32, _P, _P, _P, _P, _P, _P, _P]),
            ("orc_sincos_turns", None, [C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
            ("orc_tri_test", C.c_int, [_P, _P, _P, C.c_float, C.c_float, _P]),
            ("orc_mm_combine", C.c_uint32, [C.c_uint32, C.c_uint32]),
            ("orc_mm_rand", C.c_float, [C.c_uint32]),
            ("orc_world_create", _P, [C.POINTER(vrg.Material), C.c_uint32]),
            ("orc_world_destroy", None, [_P]),
            ("orc_chunk_build", _P, [_P, _P, C.POINTER(_P)]),
            ("orc_chunk_destroy", None, [_P]),
            ("orc_chunk_info", None, [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
            ("orc_chunk_read_bvh", C.c_int, [_P, C.c_uint32, _P, _P]),
            ("orc_world_add", None, [_P, C.c_uint64, _P, C.c_float, C.c_float, C.c_float]),
            ("orc_world_add_xform", None, [_P, C.c_uint64, _P, _P]),
            ("orc_mesh_build", _P, [_P, _P, C.c_uint64]),
            ("orc_world_remove", None, [_P, C.c_uint64]),
            ("orc_world_commit", None, [_P]),
            ("orc_world_read_tl", C.c_uint32, [_P, C.c_uint32, _P, C.c_uint32]),
            ("orc_world_instance_tl_idx", C.c_uint32, [_P, C.c_uint32]),
            ("orc_renderer_create", _P, [C.c_uint32, C.c_uint32, C.c_uint32]),
            ("orc_renderer_destroy", None, [_P]),
            ("orc_render", C.c_int, [_P, _P, C.POINTER(vrg.Camera), C.POINTER(vrg.RenderParams), C.c_int64,
                                     C.c_int64]),
            ("orc_readback", C.c_int, [_P, C.c_uint32, _P, C.c_uint64]),
            ("orc_read_image", C.c_int, [_P, _P, _P]),
            ("orc_postprocess_scaled", C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_uint32, _P, _P]),
            ("orc_world_set_atlas", C.c_int, [_P, _P, C.c_uint32, C.c_uint32, C.c_uint32]),
            ("orc_read_accum", C.c_uint32, [_P, _P]),
            ("orc_ray_counts", None, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
            ("orc_terrain_materials", C.c_int32, [C.c_uint64, C.POINTER(vrg.Material), C.c_uint32,
                                                  C.POINTER(C.c_uint32)]),
            ("orc_terrain_generate", C.c_int32, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_float, _P]),
            ("orc_orbit_camera", C.c_int32, [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                             C.c_uint32, C.POINTER(vrg.Camera)]),
        ]
        for name, res, args in sig:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# The synthetic inputs (the library's generator compiled into the oracle), so
# that CPU-only callers build the same scenes without the CUDA library.
def terrain_materials(seed):
    mats = (vrg.Material * (6 * 22))()
    n = C.c_uint32()
    assert lib().orc_terrain_materials(seed, mats, len(mats), C.byref(n)) == 0
    return mats, n.value


def terrain_blocks(seed, nx, nz, emissive):
    out = np.empty(nx * nz * vrg.CHUNK_BLOCKS, dtype=np.uint8)
    assert lib().orc_terrain_generate(seed, nx, nz, emissive, _p(out)) == 0
    return out.reshape(nx, nz, vrg.CHUNK_BLOCKS)


def orbit_camera(nx, nz, frame, n_frames, width, height):
    cam = vrg.Camera()
    assert lib().orc_orbit_camera(nx, nz, frame, n_frames, width, height, C.byref(cam)) == 0
    return cam


def build_tl_bvh(aabbs, power, ids, translations=None):
    """build_tl_bvh (build.rs:374-480). aabbs (n,6) float32 [min, max]."""
    aabbs = np.ascontiguousarray(aabbs, np.float32)
    n = aabbs.shape[0]
    power = np.ascontiguousarray(power, np.float32)
    ids = np.ascontiguousarray(ids, np.uint32)
    tr = None if translations is None else np.ascontiguousarray(translations, np.float32)
    nodes = np.zeros(2 * n - 1, dtype=vrg.NODE_DTYPE)
    order = np.zeros(n, dtype=np.uint32)
    assert lib().orc_build_tl_bvh(n, _p(tr), _p(aabbs), _p(power), _p(ids), _p(nodes), _p(order)) == 0
    return nodes, order


def tri_test(tri9, o, d, tmin=1e-3, tmax=1000.0):
    """The oracle's watertight ray/triangle test: (t, b1, b2) or None."""
    t = np.ascontiguousarray(tri9, np.float32).reshape(9)
    oo = np.ascontiguousarray(o, np.float32).reshape(3)
    dd = np.ascontiguousarray(d, np.float32).reshape(3)
    out = np.zeros(3, np.float32)
    if lib().orc_tri_test(_p(t), _p(oo), _p(dd), tmin, tmax, _p(out)):
        return tuple(out)
    return None


def build_bl_bvh(tris, lum, ids):
    """build_bl_bvh (build.rs:249-372). tris (n,9) float32."""
    tris = np.ascontiguousarray(tris, np.float32)
    n = tris.shape[0]
    lum = np.ascontiguousarray(lum, np.float32)
    ids = np.ascontiguousarray(ids, np.uint32)
    nodes = np.zeros(2 * n - 1, dtype=vrg.NODE_DTYPE)
    order = np.zeros(n, dtype=np.uint32)
    root = np.zeros(6, np.float32)
    pw = np.zeros(1, np.float32)
    assert lib().orc_build_bl_bvh(n, _p(lum), _p(tris), _p(ids), _p(nodes), _p(order), _p(root), _p(pw)) == 0
    return nodes, order, root, float(pw[0])


class World:
    """Oracle scene: chunks with explicit neighbours, objects in key order."""

    def __init__(self, mats, n=None):
        n = len(mats) if n is None else n
        self.h = lib().orc_world_create(mats, n)
        assert self.h
        self.chunks = {}

    def set_atlas(self, rgba):
        """rgba: (slots, 3, h, w, 4) uint8 — before adding chunks."""
        rgba = np.ascontiguousarray(rgba, np.uint8)
        n, _, h, w, _ = rgba.shape
        assert lib().orc_world_set_atlas(self.h, _p(rgba), n, w, h) == 0

    def add_chunk(self, key, blocks, neighbours, translation):
        blocks = np.ascontiguousarray(blocks, np.uint8).reshape(-1)
        keep = [None if x is None else np.ascontiguousarray(x, np.uint8).reshape(-1) for x in neighbours]
        arr = (C.c_void_p * 6)(*[None if x is None else x.ctypes.data for x in keep])
        c = lib().orc_chunk_build(self.h, _p(blocks), arr)
        lib().orc_world_add(self.h, key, c, *[float(t) for t in translation])
        self.chunks[key] = c
        return c

    def add_mesh(self, key, vertexes, transform):
        """upload_object of a triangle mesh, added with a 3x4 / 4x4 transform (or a translation)."""
        v = vrg.as_vertices(vertexes)
        c = lib().orc_mesh_build(self.h, _p(v) if len(v) else None, len(v))
        assert c, "oracle mesh build failed"
        m = np.ascontiguousarray(np.frombuffer(bytes(vrg._xform(transform)), np.float32))
        lib().orc_world_add_xform(self.h, key, c, _p(m))
        self.chunks[key] = c
        return c

    def chunk_info(self, key):
        v = [C.c_uint32() for _ in range(3)]
        lib().orc_chunk_info(self.chunks[key], *[C.byref(x) for x in v])
        return dict(triangles=v[0].value, light_triangles=v[1].value, surface_blocks=v[2].value)

    def chunk_bvh(self, key, which):
        info = self.chunk_info(key)
        n = info["surface_blocks"] if which else info["light_triangles"]
        nodes = np.zeros(max(2 * n - 1, 0), dtype=vrg.NODE_DTYPE)
        order = np.zeros(n, dtype=np.uint32)
        if n:
            assert lib().orc_chunk_read_bvh(self.chunks[key], which, _p(nodes), _p(order)) == 0
        return nodes, order

    def commit(self):
        lib().orc_world_commit(self.h)

    def read_tl(self, which):
        n = lib().orc_world_read_tl(self.h, which, None, 0)
        nodes = np.zeros(n, dtype=vrg.NODE_DTYPE)
        if n:
            lib().orc_world_read_tl(self.h, which, _p(nodes), n)
        return nodes

    def close(self):
        for c in self.chunks.values():
            lib().orc_chunk_destroy(c)
        self.chunks = {}
        if self.h:
            lib().orc_world_destroy(self.h)
            self.h = None


def postprocess_scaled(view, scale):
    """postprocess.rs:39-88 with srcscale = scale: (H, W, 3) float view colours of
    the traced frame -> ((H/s, W/s, 4) BGRA8, (H/s, W/s, 3) float mean)."""
    view = np.ascontiguousarray(view, np.float32)
    H, W = view.shape[:2]
    img = np.zeros((H // scale, W // scale, 4), np.uint8)
    out = np.zeros((H // scale, W // scale, 3), np.float32)
    assert lib().orc_postprocess_scaled(_p(view), W, H, scale, _p(img), _p(out)) == 0
    return img, out


def build_world(mats, n, world):
    nx, nz = world.shape[:2]
    floor = np.zeros(vrg.CHUNK_BLOCKS, dtype=np.uint8)
    W = World(mats, n)
    for cx in range(nx):
        for cz in range(nz):
            W.add_chunk(cx * nz + cz, world[cx, cz], vrg.chunk_neighbours(world, cx, cz, floor),
                        (32 * cx, 0, 32 * cz))
    W.commit()
    return W


class Renderer:
    def __init__(self, w, h, nb):
        self.w, self.h_, self.nb = w, h, nb
        self.h = lib().orc_renderer_create(w, h, nb)

    def render(self, world, cam, params, pix_range=None):
        P = self.w * self.h_
        b, e = (0, P) if pix_range is None else pix_range
        assert lib().orc_render(self.h, world.h, C.byref(cam), C.byref(params), b, e) == 0

    def readback(self, what, nb):
        P = self.w * self.h_
        shapes = {vrg.DBG_ORIGIN: (nb + 1, P, 3), vrg.DBG_DIRECTION: (nb + 1, P, 3), vrg.DBG_NORMAL: (nb, P, 3),
                  vrg.DBG_EMISSIVITY: (nb, P, 3), vrg.DBG_REFLECTIVITY: (nb, P, 3), vrg.DBG_MIS: (nb, P),
                  vrg.DBG_BSDF_PDF: (nb, P), vrg.DBG_NEE_PDF: (nb, P), vrg.DBG_RADIANCE: (nb, P, 3),
                  vrg.DBG_Q: (nb, P), vrg.DBG_HIT: (nb, P, 4), vrg.DBG_TEMPORAL: (P, 20),
                  vrg.DBG_SPATIAL: (P, 20), vrg.DBG_FINAL: (P, 3)}
        dt = np.uint32 if what == vrg.DBG_HIT else np.float32
        a = np.zeros(shapes[what], dtype=dt)
        assert lib().orc_readback(self.h, what, _p(a), a.nbytes) == 0
        return a

    def image(self):
        P = self.w * self.h_
        img = np.zeros(P * 4, np.uint8)
        view = np.zeros(P * 3, np.float32)
        lib().orc_read_image(self.h, _p(img), _p(view))
        return img.reshape(self.h_, self.w, 4), view.reshape(self.h_, self.w, 3)

    def accum(self):
        P = self.w * self.h_
        a = np.zeros(P * 3, np.float64)
        n = lib().orc_read_accum(self.h, _p(a))
        return a.reshape(self.h_, self.w, 3), n

    def ray_counts(self):
        a, b = C.c_uint64(), C.c_uint64()
        lib().orc_ray_counts(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def close(self):
        if self.h:
            lib().orc_renderer_destroy(self.h)
            self.h = None
