"""Python binding of libvrg.so (ctypes), mirroring the reference's render-system
interface of pimpale/vulkan-voxel-restir-gi:

    SceneUploader.upload_object   src/render_system/scene.rs:547  -> SceneUploader.upload_chunk
    Scene.add_object / update_object / remove_object / get_tlas /
          dispose_old_objects     src/render_system/scene.rs:150-234
    Renderer.render(scene, eye, front, right, up, prefs)
                                  src/render_system/interactive_rendering.rs:952
    RenderingPreferences          src/camera.rs:38-56

Every call goes to the CUDA library; there is no CPU path.  Loading fails
loudly when libvrg.so has not been built.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# VRG_LIBRARY names another build of the library (for A/B runs of builds)
LIB_PATH = os.environ.get("VRG_LIBRARY") or os.path.join(HERE, "libvrg.so")

CHUNK = 32
CHUNK_BLOCKS = 32 * 32 * 32

# status codes (include/vrg.h)
OK, ERR_INVALID_ARGUMENT, ERR_NOT_FOUND, ERR_OUT_OF_MEMORY, ERR_CUDA, ERR_UNSUPPORTED, \
    ERR_OVERFLOW, ERR_STATE, ERR_NO_DEVICE = range(9)

MODE_PARITY, MODE_CONFIG = 0, 1
MAT_TRANSLUCENT = 1
RENDER_CAPTURE, RENDER_NO_PACK, RENDER_CACHE, RENDER_PLAIN_ONLY, RENDER_GRAPH = 1, 2, 4, 8, 16
NRC_WEIGHTS, NRC_WEIGHT_GRADS, NRC_TABLE, NRC_TABLE_GRADS, NRC_ZERO_GRADS, NRC_TRAIN_PREDICTIONS = range(6)
(DBG_ORIGIN, DBG_DIRECTION, DBG_NORMAL, DBG_EMISSIVITY, DBG_REFLECTIVITY, DBG_MIS, DBG_BSDF_PDF,
 DBG_NEE_PDF, DBG_RADIANCE, DBG_Q, DBG_HIT, DBG_TEMPORAL, DBG_SPATIAL, DBG_FINAL, DBG_CACHE_TARGET) = range(15)


class BvhNode(C.Structure):
    """40-byte BvhNode (src/render_system/bvh/mod.rs:8-25)."""
    _fields_ = [("left_node_idx", C.c_uint32), ("right_node_idx_or_prim_idx", C.c_uint32),
                ("min", C.c_float * 3), ("power", C.c_float), ("max", C.c_float * 3),
                ("parent_idx", C.c_uint32)]


NODE_DTYPE = np.dtype([("left", "<u4"), ("right", "<u4"), ("min", "<f4", 3), ("power", "<f4"),
                       ("max", "<f4", 3), ("parent", "<u4")])
assert NODE_DTYPE.itemsize == C.sizeof(BvhNode) == 40


class Material(C.Structure):
    _fields_ = [("reflectivity", C.c_float * 3), ("alpha", C.c_float), ("emission", C.c_float * 3),
                ("metallic", C.c_float), ("luminance", C.c_float), ("flags", C.c_uint32),
                ("reserved", C.c_uint32 * 2)]


class Vertex3D(C.Structure):
    """Vertex3D (vertex.rs:4-14): position, texture index t, uv (24 bytes)."""
    _fields_ = [("position", C.c_float * 3), ("t", C.c_uint32), ("uv", C.c_float * 2)]


VERTEX_DTYPE = np.dtype([("position", np.float32, 3), ("t", np.uint32), ("uv", np.float32, 2)])


class ContextDesc(C.Structure):
    _fields_ = [("device", C.c_int32), ("flags", C.c_uint32)]


class Camera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("front", C.c_float * 3), ("right", C.c_float * 3),
                ("up", C.c_float * 3), ("width", C.c_uint32), ("height", C.c_uint32)]


class RenderParams(C.Structure):
    _fields_ = [("nee_type", C.c_uint32), ("debug_view", C.c_uint32), ("spatial_iterations", C.c_uint32),
                ("num_bounces", C.c_uint32), ("mode", C.c_uint32), ("raygen_seed", C.c_uint32),
                ("temporal_seed", C.c_uint32), ("spatial_seed", C.c_uint32), ("spatial_radius", C.c_float),
                ("m_cap", C.c_uint32), ("history_slots", C.c_uint32), ("accumulate", C.c_uint32),
                ("flags", C.c_uint32), ("cache_train_bounces", C.c_uint32), ("reserved", C.c_uint32 * 2)]


class NrcDesc(C.Structure):
    _fields_ = [("levels", C.c_uint32), ("log2_table", C.c_uint32), ("features", C.c_uint32),
                ("base_resolution", C.c_uint32), ("max_resolution", C.c_uint32), ("batch", C.c_uint32),
                ("learning_rate", C.c_float), ("seed", C.c_uint32), ("scene_min", C.c_float * 3),
                ("scene_max", C.c_float * 3), ("flags", C.c_uint32), ("reserved", C.c_uint32)]


NRC_TRAIN_WARP_MMA = 1


class Tuning(C.Structure):
    """Launch configuration (scheduling only); 0 fields mean the default."""
    _fields_ = [("trace_blocks_per_sm", C.c_uint32), ("trace_refill", C.c_uint32),
                ("shade_blocks_per_sm", C.c_uint32), ("anyhit_blocks_per_sm", C.c_uint32),
                ("anyhit_refill", C.c_uint32), ("stream_block", C.c_uint32), ("spatial_staging", C.c_uint32),
                ("reserved", C.c_uint32 * 1)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class View(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("camera", Camera), ("temporal_seed", C.c_uint32),
                ("spatial_seed", C.c_uint32)]


OUTPUT_DEVICE, OUTPUT_HOST, OUTPUT_HOST_ASYNC = 0, 1, 2


class FrameOutput(C.Structure):
    _fields_ = [("bgra8", C.c_void_p), ("radiance", C.c_void_p), ("host", C.c_uint32),
                ("reserved", C.c_uint32)]


class FrameStats(C.Structure):
    _fields_ = [("ms_total", C.c_float), ("ms_bounce", C.c_float * 8), ("ms_resolve", C.c_float),
                ("ms_spatial", C.c_float), ("rays_closest", C.c_uint64), ("rays_any", C.c_uint64),
                ("error_flags", C.c_uint32), ("reserved", C.c_uint32), ("ms_trace", C.c_float * 8),
                ("ms_shade", C.c_float * 8), ("ms_anyhit", C.c_float * 8), ("nodes_visited", C.c_uint64),
                ("leaves_visited", C.c_uint64), ("light_nodes_visited", C.c_uint64),
                ("light_leaves_visited", C.c_uint64), ("light_hits", C.c_uint64)]


_lib = None

# (name, restype, argtypes) of every exported symbol of include/vrg.h
_P = C.c_void_p
SIGNATURES = [
    ("vrg_context_create", C.c_int32, [C.POINTER(ContextDesc), C.POINTER(_P)]),
    ("vrg_context_destroy", C.c_int32, [_P]),
    ("vrg_context_stream", C.c_int32, [_P, C.POINTER(C.c_void_p)]),
    ("vrg_context_synchronize", C.c_int32, [_P]),
    ("vrg_renderer_wait_frame", C.c_int32, [_P, C.c_uint32]),
    ("vrg_status_string", C.c_char_p, [C.c_int32]),
    ("vrg_last_error", C.c_char_p, []),
    ("vrg_material_table_set", C.c_int32, [_P, C.POINTER(Material), C.c_uint32]),
    ("vrg_texture_atlas_set", C.c_int32, [_P, _P, C.c_uint32, C.c_uint32, C.c_uint32]),
    ("vrg_upload_chunk", C.c_int32, [_P, _P, C.POINTER(_P), C.POINTER(_P)]),
    ("vrg_upload_mesh", C.c_int32, [_P, _P, C.c_uint64, C.POINTER(_P)]),
    ("vrg_flush_uploads", C.c_int32, [_P]),
    ("vrg_object_release", C.c_int32, [_P]),
    ("vrg_object_info", C.c_int32, [_P] + [C.POINTER(C.c_uint32)] * 4),
    ("vrg_object_read_bvh", C.c_int32, [_P, C.c_uint32, _P, C.c_uint32, C.POINTER(C.c_uint32), _P, C.c_uint32,
                                        C.POINTER(C.c_uint32)]),
    ("vrg_scene_create", C.c_int32, [_P, C.POINTER(_P)]),
    ("vrg_scene_destroy", C.c_int32, [_P]),
    ("vrg_scene_add", C.c_int32, [_P, C.c_uint64, _P, C.POINTER(C.c_float)]),
    ("vrg_scene_update", C.c_int32, [_P, C.c_uint64, C.POINTER(C.c_float)]),
    ("vrg_scene_remove", C.c_int32, [_P, C.c_uint64]),
    ("vrg_scene_commit", C.c_int32, [_P]),
    ("vrg_scene_commit_many", C.c_int32, [_P, C.c_uint32]),
    ("vrg_scene_read_tl", C.c_int32, [_P, C.c_uint32, _P, C.c_uint32, C.POINTER(C.c_uint32)]),
    ("vrg_renderer_create", C.c_int32, [_P, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(_P)]),
    ("vrg_renderer_destroy", C.c_int32, [_P]),
    ("vrg_renderer_resize", C.c_int32, [_P, C.c_uint32, C.c_uint32]),
    ("vrg_render", C.c_int32, [_P, _P, C.POINTER(Camera), C.POINTER(RenderParams), C.POINTER(FrameOutput),
                               C.POINTER(FrameStats)]),
    ("vrg_renderer_frame_index", C.c_int32, [_P, C.POINTER(C.c_uint32)]),
    ("vrg_renderer_reset_accumulation", C.c_int32, [_P]),
    ("vrg_renderer_read_accumulation", C.c_int32, [_P, _P, C.POINTER(C.c_uint32)]),
    ("vrg_debug_readback", C.c_int32, [_P, C.c_uint32, _P, C.c_uint64]),
    ("vrg_build_tl_bvh_batched", C.c_int32, [_P, C.c_uint32, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    ("vrg_measure_l2_bandwidth", C.c_int32, [_P, C.c_uint64, C.c_uint32, C.POINTER(C.c_float)]),
    ("vrg_build_bl_bvh_batched", C.c_int32, [_P, C.c_uint32, _P, _P, _P, _P, _P, _P, _P, _P]),
    ("vrg_terrain_materials", C.c_int32, [C.c_uint64, C.POINTER(Material), C.c_uint32, C.POINTER(C.c_uint32)]),
    ("vrg_terrain_generate", C.c_int32, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_float, _P]),
    ("vrg_orbit_camera", C.c_int32, [C.c_uint32] * 6 + [C.POINTER(Camera)]),
    ("vrg_pcg32_next", C.c_uint32, [C.POINTER(C.c_uint64), C.c_uint64]),
    ("vrg_nrc_create", C.c_int32, [_P, C.POINTER(NrcDesc), C.POINTER(_P)]),
    ("vrg_nrc_destroy", C.c_int32, [_P]),
    ("vrg_nrc_query", C.c_int32, [_P, C.c_uint32, _P, _P, _P, _P]),
    ("vrg_nrc_train", C.c_int32, [_P, C.c_uint32, _P, _P, _P, _P, C.c_uint32, C.POINTER(C.c_float)]),
    ("vrg_nrc_read", C.c_int32, [_P, C.c_uint32, _P, C.c_uint64]),
    ("vrg_nrc_write", C.c_int32, [_P, C.c_uint32, _P, C.c_uint64]),
    ("vrg_nrc_layout", C.c_int32, [_P, C.POINTER(C.c_uint32), _P, _P, _P]),
    ("vrg_renderer_set_cache", C.c_int32, [_P, _P]),
    ("vrg_renderer_set_scale", C.c_int32, [_P, C.c_uint32]),
    ("vrg_image_write_ppm", C.c_int32, [C.c_char_p, _P, C.c_uint32, C.c_uint32]),
    ("vrg_image_write_png", C.c_int32, [C.c_char_p, _P, C.c_uint32, C.c_uint32]),
    ("vrg_image_write_pfm", C.c_int32, [C.c_char_p, _P, C.c_uint32, C.c_uint32]),
    ("vrg_renderer_state_size", C.c_int32, [_P, C.POINTER(C.c_uint64)]),
    ("vrg_renderer_state_save", C.c_int32, [_P, _P, C.c_uint64]),
    ("vrg_renderer_state_load", C.c_int32, [_P, _P, C.c_uint64]),
    ("vrg_renderer_set_tuning", C.c_int32, [_P, C.POINTER(Tuning)]),
    ("vrg_renderer_get_tuning", C.c_int32, [_P, C.POINTER(Tuning)]),
    ("vrg_renderer_autotune", C.c_int32, [_P, _P, C.POINTER(Camera), C.POINTER(RenderParams), C.c_uint32,
                                          C.POINTER(Tuning), C.POINTER(C.c_float)]),
    ("vrg_renderer_create_batched", C.c_int32, [_P, C.c_uint32, _P, _P, C.c_uint32, C.POINTER(_P)]),
    ("vrg_renderer_view_offset", C.c_int32, [_P, C.c_uint32, C.POINTER(C.c_uint64)]),
    ("vrg_render_batched", C.c_int32, [_P, C.POINTER(View), C.c_uint32, C.POINTER(RenderParams), _P,
                                       C.POINTER(FrameStats)]),
]


def load_library(path: str = LIB_PATH):
    """Loads libvrg.so; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is not None and path == LIB_PATH:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libvrg.so not found at {path}: build it with __graft_entry__.build() "
                           f"or python vulkan-voxel-restir-gi_gb300/build.py")
    lib = C.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path == LIB_PATH:
        _lib = lib
    return lib


class VrgError(RuntimeError):
    def __init__(self, status, what):
        lib = load_library()
        msg = lib.vrg_last_error().decode(errors="replace")
        super().__init__(f"{what}: {lib.vrg_status_string(status).decode()} ({status}) {msg}")
        self.status = status


def check(status, what=""):
    if status != OK:
        raise VrgError(status, what)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


@dataclass
class RenderingPreferences:
    """src/camera.rs:38-56."""
    nee_type: int = 0
    debug_view: int = 0
    restir_spatial_iterations: int = 0


def terrain_materials(seed: int):
    lib = load_library()
    mats = (Material * (6 * 22))()
    n = C.c_uint32()
    check(lib.vrg_terrain_materials(seed, mats, len(mats), C.byref(n)), "vrg_terrain_materials")
    return mats, n.value


def terrain_blocks(seed: int, nx: int, nz: int, emissive: float) -> np.ndarray:
    lib = load_library()
    out = np.empty(nx * nz * CHUNK_BLOCKS, dtype=np.uint8)
    check(lib.vrg_terrain_generate(seed, nx, nz, emissive, _ptr(out)), "vrg_terrain_generate")
    return out.reshape(nx, nz, CHUNK_BLOCKS)


def chunk_neighbours(world: np.ndarray, cx: int, cz: int, solid_floor: np.ndarray):
    """Six neighbour arrays (left, right, down, up, back, front) of chunk (cx, cz)
    in a one-chunk-tall world; outside the world is air (None), below is solid."""
    nx, nz = world.shape[:2]
    left = world[cx - 1, cz] if cx > 0 else None
    right = world[cx + 1, cz] if cx + 1 < nx else None
    back = world[cx, cz - 1] if cz > 0 else None
    front = world[cx, cz + 1] if cz + 1 < nz else None
    return [left, right, solid_floor, None, back, front]


def orbit_camera(nx, nz, frame, n_frames, width, height) -> Camera:
    lib = load_library()
    cam = Camera()
    check(lib.vrg_orbit_camera(nx, nz, frame, n_frames, width, height, C.byref(cam)), "vrg_orbit_camera")
    return cam


class Pcg32:
    """Host PCG32 stream for invocation seeds (replaces rand::rng())."""

    def __init__(self, seed: int, stream: int = 54):
        self.state = C.c_uint64(0)
        self.inc = (stream << 1) | 1
        self.next()
        self.state.value = (self.state.value + seed) & (2 ** 64 - 1)
        self.next()

    def next(self) -> int:
        return load_library().vrg_pcg32_next(C.byref(self.state), self.inc)


class Context:
    def __init__(self, device: int = 0):
        self.lib = load_library()
        self.h = C.c_void_p()
        desc = ContextDesc(device, 0)
        check(self.lib.vrg_context_create(C.byref(desc), C.byref(self.h)), "vrg_context_create")
        # handles made from this context; closed before it, whatever the
        # order in which Python collects them
        self._children = weakref.WeakSet()

    def adopt(self, obj):
        self._children.add(obj)
        return obj

    def synchronize(self):
        check(self.lib.vrg_context_synchronize(self.h), "vrg_context_synchronize")

    def stream(self) -> int:
        """The cudaStream_t the library submits on, as an integer handle."""
        p = C.c_void_p()
        check(self.lib.vrg_context_stream(self.h, C.byref(p)), "vrg_context_stream")
        return p.value or 0

    def set_materials(self, mats, n=None):
        n = len(mats) if n is None else n
        check(self.lib.vrg_material_table_set(self.h, mats, n), "vrg_material_table_set")

    def set_atlas(self, rgba):
        """Texture atlas, (slots, 3, h, w, 4) uint8 sRGB maps per material slot
        (reflectivity+alpha, emissivity, metallicity); None removes it."""
        if rgba is None:
            check(self.lib.vrg_texture_atlas_set(self.h, None, 0, 0, 0), "vrg_texture_atlas_set")
            return
        rgba = np.ascontiguousarray(rgba, np.uint8)
        n, maps, h, w, c = rgba.shape
        assert maps == 3 and c == 4
        check(self.lib.vrg_texture_atlas_set(self.h, _ptr(rgba), n, w, h), "vrg_texture_atlas_set")

    def l2_read_gbs(self, mib=32, reps=64):
        """The device's L2 read bandwidth in GB/s (vrg_measure_l2_bandwidth)."""
        g = C.c_float()
        check(self.lib.vrg_measure_l2_bandwidth(self.h, mib << 20, reps, C.byref(g)), "vrg_measure_l2_bandwidth")
        return float(g.value)

    def flush(self):
        check(self.lib.vrg_flush_uploads(self.h), "vrg_flush_uploads")

    def close(self):
        if self.h:
            for c in list(self._children):
                c.close()
            self.lib.vrg_context_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class UploadedObject:
    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self.h = handle
        ctx.adopt(self)

    def info(self):
        v = [C.c_uint32() for _ in range(4)]
        check(self.ctx.lib.vrg_object_info(self.h, *[C.byref(x) for x in v]), "vrg_object_info")
        return dict(faces=v[0].value, triangles=v[1].value, light_triangles=v[2].value,
                    surface_blocks=v[3].value)

    def read_bvh(self, which: int):
        """which 0 = light BLAS (build_bl_bvh), 1 = geometry BLAS over block AABBs."""
        nn, np_ = C.c_uint32(), C.c_uint32()
        check(self.ctx.lib.vrg_object_read_bvh(self.h, which, None, 0, C.byref(nn), None, 0, C.byref(np_)),
              "vrg_object_read_bvh")
        nodes = np.zeros(nn.value, dtype=NODE_DTYPE)
        order = np.zeros(np_.value, dtype=np.uint32)
        if nn.value:
            check(self.ctx.lib.vrg_object_read_bvh(self.h, which, _ptr(nodes), nn.value, C.byref(nn),
                                                   _ptr(order), np_.value, C.byref(np_)), "vrg_object_read_bvh")
        return nodes, order

    def release(self):
        if self.h:
            self.ctx.lib.vrg_object_release(self.h)
            self.h = None

    close = release

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class SceneUploader:
    """SceneUploader (scene.rs:534-725): voxel chunks in, GPU-built BLAS out."""

    def __init__(self, ctx: Context):
        self.ctx = ctx

    def upload_chunk(self, blocks: np.ndarray, neighbours=(None,) * 6) -> UploadedObject:
        blocks = np.ascontiguousarray(blocks, dtype=np.uint8).reshape(-1)
        assert blocks.size == CHUNK_BLOCKS
        keep = [None if n is None else np.ascontiguousarray(n, dtype=np.uint8).reshape(-1) for n in neighbours]
        arr = (C.c_void_p * 6)(*[None if n is None else n.ctypes.data for n in keep])
        h = C.c_void_p()
        check(self.ctx.lib.vrg_upload_chunk(self.ctx.h, _ptr(blocks), arr, C.byref(h)), "vrg_upload_chunk")
        return UploadedObject(self.ctx, h)

    def upload_object(self, vertexes) -> UploadedObject:
        """upload_object (scene.rs:547-725) of a triangle mesh: a VERTEX_DTYPE
        array (or (n, 6) floats: position, t, u, v), three vertices per triangle."""
        v = as_vertices(vertexes)
        h = C.c_void_p()
        check(self.ctx.lib.vrg_upload_mesh(self.ctx.h, _ptr(v) if len(v) else None, len(v), C.byref(h)),
              "vrg_upload_mesh")
        return UploadedObject(self.ctx, h)


def as_vertices(vertexes) -> np.ndarray:
    """A contiguous VERTEX_DTYPE array from structured or (n, 6) [x, y, z, t, u, v] input."""
    a = np.asarray(vertexes)
    if a.dtype == VERTEX_DTYPE:
        return np.ascontiguousarray(a)
    a = np.asarray(a, np.float64).reshape(-1, 6)
    v = np.zeros(len(a), VERTEX_DTYPE)
    v["position"] = a[:, :3]
    v["t"] = a[:, 3].astype(np.uint32)
    v["uv"] = a[:, 4:6]
    return v


def _xform(t):
    """A transform for vrg_scene_add / update: a translation (3 values) or a
    3x4 / 4x4 matrix [R|t] (the matrix of an Isometry3)."""
    m = np.asarray(t, np.float32)
    if m.size == 3:
        m = np.array([[1, 0, 0, m[0]], [0, 1, 0, m[1]], [0, 0, 1, m[2]]], np.float32)
    m = m.reshape(-1, 4)[:3]
    return (C.c_float * 12)(*[float(x) for x in m.reshape(-1)])


class Scene:
    """Scene<K> (scene.rs:86-497) with u64 keys."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.h = C.c_void_p()
        check(ctx.lib.vrg_scene_create(ctx.h, C.byref(self.h)), "vrg_scene_create")
        self._objs = {}
        ctx.adopt(self)

    def add_object(self, key: int, obj: UploadedObject, isometry=(0, 0, 0)):
        """add_object (scene.rs:150): isometry is a translation or a 3x4 / 4x4 matrix."""
        check(self.ctx.lib.vrg_scene_add(self.h, key, obj.h, _xform(isometry)), "vrg_scene_add")
        self._objs[key] = obj

    def update_object(self, key: int, isometry):
        """update_object (scene.rs:205): VrgError(ERR_NOT_FOUND) where the reference panics."""
        check(self.ctx.lib.vrg_scene_update(self.h, key, _xform(isometry)), "vrg_scene_update")

    def remove_object(self, key: int):
        check(self.ctx.lib.vrg_scene_remove(self.h, key), "vrg_scene_remove")
        self._objs.pop(key, None)

    def get_tlas(self):
        """Commits the scene (top-level builds); returns (light TL, geometry TL) node arrays."""
        check(self.ctx.lib.vrg_scene_commit(self.h), "vrg_scene_commit")
        out = []
        for which in (0, 1):
            n = C.c_uint32()
            check(self.ctx.lib.vrg_scene_read_tl(self.h, which, None, 0, C.byref(n)), "vrg_scene_read_tl")
            nodes = np.zeros(n.value, dtype=NODE_DTYPE)
            if n.value:
                check(self.ctx.lib.vrg_scene_read_tl(self.h, which, _ptr(nodes), n.value, C.byref(n)),
                      "vrg_scene_read_tl")
            out.append(nodes)
        return tuple(out)

    commit = get_tlas

    def dispose_old_objects(self):
        """Retired objects are freed stream-ordered at the next commit."""

    def close(self):
        if self.h:
            self.ctx.lib.vrg_scene_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def commit_scenes(scenes):
    """Commits several scenes together (one top-level and one lamp SAH build for all)."""
    if not scenes:
        return
    ctx = scenes[0].ctx
    arr = (C.c_void_p * len(scenes))(*[s.h.value for s in scenes])
    check(ctx.lib.vrg_scene_commit_many(arr, len(scenes)), "vrg_scene_commit_many")


def write_image(path: str, img: np.ndarray):
    """Writes a frame: BGRA8 (h, w, 4) as .ppm or .png, float RGB (h, w, 3) as .pfm."""
    lib = load_library()
    img = np.ascontiguousarray(img)
    h, w = img.shape[:2]
    ext = os.path.splitext(path)[1].lower()
    if ext == ".pfm":
        fn, want = lib.vrg_image_write_pfm, np.float32
    elif ext == ".png":
        fn, want = lib.vrg_image_write_png, np.uint8
    else:
        fn, want = lib.vrg_image_write_ppm, np.uint8
    img = np.ascontiguousarray(img, dtype=want)
    check(fn(path.encode(), _ptr(img), w, h), "vrg_image_write")


class Renderer:
    """Renderer (interactive_rendering.rs:328-1669), headless.  scale > 1
    traces scale x the extent and averages scale x scale samples per output
    pixel (Renderer.scale)."""

    def __init__(self, ctx: Context, width: int, height: int, num_bounces: int = 3, scale: int = 1):
        self.ctx = ctx
        self.width, self.height, self.num_bounces = width, height, num_bounces
        self.scale = scale
        self.h = C.c_void_p()
        check(ctx.lib.vrg_renderer_create(ctx.h, width, height, num_bounces, C.byref(self.h)),
              "vrg_renderer_create")
        ctx.adopt(self)
        if scale != 1:
            check(ctx.lib.vrg_renderer_set_scale(self.h, scale), "vrg_renderer_set_scale")
        self.seeds = Pcg32(0x5eed)
        self.last_stats = FrameStats()

    def params(self, prefs: RenderingPreferences, num_bounces=None, mode=MODE_PARITY, seeds=None,
               spatial_radius=15.0, m_cap=0, history_slots=3, accumulate=0, flags=0,
               cache_train_bounces=4) -> RenderParams:
        if seeds is None:
            seeds = (self.seeds.next(), self.seeds.next(), self.seeds.next())
        return RenderParams(prefs.nee_type, prefs.debug_view, prefs.restir_spatial_iterations,
                            self.num_bounces if num_bounces is None else num_bounces, mode, seeds[0], seeds[1],
                            seeds[2], spatial_radius, m_cap, history_slots, accumulate, flags, cache_train_bounces)

    def set_cache(self, cache):
        check(self.ctx.lib.vrg_renderer_set_cache(self.h, None if cache is None else cache.h),
              "vrg_renderer_set_cache")

    def save_state(self) -> np.ndarray:
        """Reservoir history, frame counter and accumulation as a byte array."""
        n = C.c_uint64()
        check(self.ctx.lib.vrg_renderer_state_size(self.h, C.byref(n)), "vrg_renderer_state_size")
        blob = np.empty(n.value, np.uint8)
        check(self.ctx.lib.vrg_renderer_state_save(self.h, _ptr(blob), blob.nbytes), "vrg_renderer_state_save")
        return blob

    def load_state(self, blob: np.ndarray):
        blob = np.ascontiguousarray(blob, np.uint8)
        check(self.ctx.lib.vrg_renderer_state_load(self.h, _ptr(blob), blob.nbytes), "vrg_renderer_state_load")

    def set_tuning(self, tuning: "Tuning"):
        check(self.ctx.lib.vrg_renderer_set_tuning(self.h, C.byref(tuning)), "vrg_renderer_set_tuning")

    def get_tuning(self) -> "Tuning":
        t = Tuning()
        check(self.ctx.lib.vrg_renderer_get_tuning(self.h, C.byref(t)), "vrg_renderer_get_tuning")
        return t

    def autotune(self, scene: "Scene", cam: "Camera", params: "RenderParams", frames: int = 3):
        """Times candidate launch configurations on these frames and installs
        the fastest; returns (Tuning, ms per frame)."""
        t, ms = Tuning(), C.c_float()
        check(self.ctx.lib.vrg_renderer_autotune(self.h, scene.h, C.byref(cam), C.byref(params), frames,
                                                 C.byref(t), C.byref(ms)), "vrg_renderer_autotune")
        return t, ms.value

    def render_params(self, scene: Scene, cam: Camera, params: RenderParams, want_image=True,
                      want_radiance=False):
        P = self.width * self.height
        img = np.empty(P * 4, dtype=np.uint8) if want_image else None
        rad = np.empty(P * 3, dtype=np.float32) if want_radiance else None
        out = FrameOutput(None if img is None else img.ctypes.data, None if rad is None else rad.ctypes.data, 1, 0)
        check(self.ctx.lib.vrg_render(self.h, scene.h, C.byref(cam), C.byref(params), C.byref(out),
                                      C.byref(self.last_stats)), "vrg_render")
        return (None if img is None else img.reshape(self.height, self.width, 4),
                None if rad is None else rad.reshape(self.height, self.width, 3))

    def render(self, scene: Scene, eye, front, right, up, prefs: RenderingPreferences, **kw):
        """Renderer::render(scene, eye, front, right, up, prefs); returns the BGRA8 frame."""
        cam = Camera((C.c_float * 3)(*eye), (C.c_float * 3)(*front), (C.c_float * 3)(*right),
                     (C.c_float * 3)(*up), self.width, self.height)
        img, _ = self.render_params(scene, cam, self.params(prefs, **kw))
        return img

    def readback(self, what: int, nb: int):
        P = self.width * self.height * self.scale * self.scale
        shapes = {DBG_ORIGIN: (nb + 1, P, 3), DBG_DIRECTION: (nb + 1, P, 3), DBG_NORMAL: (nb, P, 3),
                  DBG_EMISSIVITY: (nb, P, 3), DBG_REFLECTIVITY: (nb, P, 3), DBG_MIS: (nb, P),
                  DBG_BSDF_PDF: (nb, P), DBG_NEE_PDF: (nb, P), DBG_RADIANCE: (nb, P, 3), DBG_Q: (nb, P),
                  DBG_HIT: (nb, P, 4), DBG_TEMPORAL: (P, 20), DBG_SPATIAL: (P, 20), DBG_FINAL: (P, 3),
                  DBG_CACHE_TARGET: (P, 4)}
        dt = np.uint32 if what == DBG_HIT else np.float32
        a = np.zeros(shapes[what], dtype=dt)
        check(self.ctx.lib.vrg_debug_readback(self.h, what, _ptr(a), a.nbytes), "vrg_debug_readback")
        return a

    def frame_index(self) -> int:
        """The index the next frame will have."""
        n = C.c_uint32()
        check(self.ctx.lib.vrg_renderer_frame_index(self.h, C.byref(n)), "vrg_renderer_frame_index")
        return n.value

    def wait_frame(self, frame_index: int):
        """Blocks until that frame (and its copies out) is done."""
        check(self.ctx.lib.vrg_renderer_wait_frame(self.h, frame_index), "vrg_renderer_wait_frame")

    def resize(self, width: int, height: int):
        """Renderer::rebuild(extent) (interactive_rendering.rs:818): new frame
        buffers, frame counter and history reset."""
        check(self.ctx.lib.vrg_renderer_resize(self.h, width, height), "vrg_renderer_resize")
        self.width, self.height = width, height

    def read_accumulation(self):
        n = C.c_uint32()
        w, h = self.width * self.scale, self.height * self.scale
        a = np.zeros(w * h * 3, dtype=np.float32)
        check(self.ctx.lib.vrg_renderer_read_accumulation(self.h, _ptr(a), C.byref(n)),
              "vrg_renderer_read_accumulation")
        return a.reshape(h, w, 3), n.value

    def reset_accumulation(self):
        check(self.ctx.lib.vrg_renderer_reset_accumulation(self.h), "vrg_renderer_reset_accumulation")

    def close(self):
        if self.h:
            self.ctx.lib.vrg_renderer_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchRenderer:
    """Many views of independent scenes and extents rendered by one launch
    sequence (vrg_render_batched); no reference counterpart."""

    def __init__(self, ctx: Context, extents, num_bounces: int = 2):
        self.ctx = ctx
        self.extents = [(int(w), int(h)) for w, h in extents]
        self.num_bounces = num_bounces
        n = len(self.extents)
        ws = np.array([w for w, _ in self.extents], np.uint32)
        hs = np.array([h for _, h in self.extents], np.uint32)
        self.h = C.c_void_p()
        check(ctx.lib.vrg_renderer_create_batched(ctx.h, n, _ptr(ws), _ptr(hs), num_bounces, C.byref(self.h)),
              "vrg_renderer_create_batched")
        ctx.adopt(self)
        self.offsets = []
        for v in range(n):
            o = C.c_uint64()
            check(ctx.lib.vrg_renderer_view_offset(self.h, v, C.byref(o)), "vrg_renderer_view_offset")
            self.offsets.append(o.value)
        self.pixels = sum(w * h for w, h in self.extents)
        self.last_stats = FrameStats()

    def render(self, scenes, cameras, params: RenderParams, seeds, want_image=False, want_radiance=False):
        """scenes/cameras/seeds: one per view (seeds = (temporal, spatial)).
        Returns per-view lists of images / radiance (None when not asked for)."""
        n = len(self.extents)
        views = (View * n)()
        for v in range(n):
            views[v] = View(scenes[v].h, cameras[v], seeds[v][0], seeds[v][1])
        imgs, rads = [], []
        outs = (FrameOutput * n)()
        for v, (w, h) in enumerate(self.extents):
            img = np.empty((h, w, 4), np.uint8) if want_image else None
            rad = np.empty((h, w, 3), np.float32) if want_radiance else None
            outs[v] = FrameOutput(None if img is None else img.ctypes.data, None if rad is None else rad.ctypes.data,
                                  1, 0)
            imgs.append(img)
            rads.append(rad)
        check(self.ctx.lib.vrg_render_batched(self.h, views, n, C.byref(params),
                                              C.cast(outs, C.c_void_p) if (want_image or want_radiance) else None,
                                              C.byref(self.last_stats)), "vrg_render_batched")
        return imgs, rads

    def set_cache(self, cache):
        check(self.ctx.lib.vrg_renderer_set_cache(self.h, None if cache is None else cache.h),
              "vrg_renderer_set_cache")

    def set_tuning(self, tuning: "Tuning"):
        check(self.ctx.lib.vrg_renderer_set_tuning(self.h, C.byref(tuning)), "vrg_renderer_set_tuning")

    save_state = Renderer.save_state
    load_state = Renderer.load_state

    def reset_accumulation(self):
        check(self.ctx.lib.vrg_renderer_reset_accumulation(self.h), "vrg_renderer_reset_accumulation")

    def read_accumulation(self):
        n = C.c_uint32()
        a = np.zeros(self.pixels * 3, dtype=np.float32)
        check(self.ctx.lib.vrg_renderer_read_accumulation(self.h, _ptr(a), C.byref(n)),
              "vrg_renderer_read_accumulation")
        out = []
        for (w, h), o in zip(self.extents, self.offsets):
            out.append(a[3 * o:3 * (o + w * h)].reshape(h, w, 3))
        return out, n.value

    def close(self):
        if self.h:
            self.ctx.lib.vrg_renderer_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


NRC_MASTER = 5 * 64 * 64 + 16 * 64


class RadianceCache:
    """Neural radiance cache (no reference counterpart): hash grid + 5x64 MLP."""

    def __init__(self, ctx: Context, scene_min, scene_max, levels=16, log2_table=19, base_resolution=16,
                 max_resolution=2048, batch=65536, learning_rate=1e-2, seed=1, flags=0):
        self.ctx = ctx
        self.levels, self.log2_table = levels, log2_table
        d = NrcDesc(levels, log2_table, 2, base_resolution, max_resolution, batch, learning_rate, seed,
                    (C.c_float * 3)(*scene_min), (C.c_float * 3)(*scene_max), flags, 0)
        self.h = C.c_void_p()
        check(ctx.lib.vrg_nrc_create(ctx.h, C.byref(d), C.byref(self.h)), "vrg_nrc_create")
        ctx.adopt(self)

    def query(self, pos, normal, direction):
        pos, normal, direction = (np.ascontiguousarray(a, np.float32) for a in (pos, normal, direction))
        out = np.zeros((len(pos), 3), np.float32)
        check(self.ctx.lib.vrg_nrc_query(self.h, len(pos), _ptr(pos), _ptr(normal), _ptr(direction), _ptr(out)),
              "vrg_nrc_query")
        return out

    def train(self, pos, normal, direction, target, update=True):
        pos, normal, direction, target = (np.ascontiguousarray(a, np.float32)
                                          for a in (pos, normal, direction, target))
        loss = C.c_float()
        check(self.ctx.lib.vrg_nrc_train(self.h, len(pos), _ptr(pos), _ptr(normal), _ptr(direction), _ptr(target),
                                         1 if update else 0, C.byref(loss)), "vrg_nrc_train")
        self._last_train_n = len(pos)
        return loss.value

    def train_predictions(self):
        """The last train() batch's outputs from the training pass's own forward pass (n x 3)."""
        out = np.zeros((self._last_train_n, 3), np.float32)
        check(self.ctx.lib.vrg_nrc_read(self.h, NRC_TRAIN_PREDICTIONS, _ptr(out), out.nbytes), "vrg_nrc_read")
        return out

    def read(self, what):
        n = NRC_MASTER if what in (NRC_WEIGHTS, NRC_WEIGHT_GRADS) else self.levels * (1 << self.log2_table) * 2
        a = np.zeros(n, np.float32)
        check(self.ctx.lib.vrg_nrc_read(self.h, what, _ptr(a), a.nbytes), "vrg_nrc_read")
        return a

    def write(self, what, a=None):
        if a is None:
            check(self.ctx.lib.vrg_nrc_write(self.h, what, None, 0), "vrg_nrc_write")
        else:
            a = np.ascontiguousarray(a, np.float32)
            check(self.ctx.lib.vrg_nrc_write(self.h, what, _ptr(a), a.nbytes), "vrg_nrc_write")

    def layout(self):
        lv = C.c_uint32()
        sc = np.zeros(16, np.float32)
        dn = np.zeros(16, np.uint32)
        r1 = np.zeros(16, np.uint32)
        check(self.ctx.lib.vrg_nrc_layout(self.h, C.byref(lv), _ptr(sc), _ptr(dn), _ptr(r1)), "vrg_nrc_layout")
        n = lv.value
        return sc[:n], dn[:n], r1[:n]

    def close(self):
        if self.h:
            self.ctx.lib.vrg_nrc_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def build_world(ctx: Context, world: np.ndarray):
    """Uploads every chunk of a (nx, nz, 32768) world into a new Scene; key =
    cx*nz + cz, translation (32cx, 0, 32cz).  Returns (scene, objects)."""
    nx, nz = world.shape[:2]
    floor = np.zeros(CHUNK_BLOCKS, dtype=np.uint8)  # solid ground below the world
    up = SceneUploader(ctx)
    scene = Scene(ctx)
    objs = []
    for cx in range(nx):
        for cz in range(nz):
            o = up.upload_chunk(world[cx, cz], chunk_neighbours(world, cx, cz, floor))
            scene.add_object(cx * nz + cz, o, (32 * cx, 0, 32 * cz))
            objs.append(o)
    return scene, objs
