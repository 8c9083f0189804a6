/*
 * vrg.h — C ABI of the GB300-native voxel path tracer (binned-SAH BVH build,
 * wavefront trace/shade with light-BVH next-event estimation, ReSTIR temporal
 * and spatial resampling, finalize and pack).
 *
 * Every entry point returns a vrg_status (0 == VRG_OK).  Handles are opaque.
 * Host arrays passed in are copied; device memory is owned by the library.
 * Upload entry points (vrg_upload_chunk) are thread-safe; scene and render
 * calls on one scene/renderer must be externally synchronised, as the
 * reference's Rc<RefCell<Scene>> / &mut Renderer are.
 *
 * Reference interfaces replaced (paths inside pimpale/vulkan-voxel-restir-gi):
 *   SceneUploader::upload_object        src/render_system/scene.rs:547
 *   Scene::new / add_object / update_object / remove_object /
 *         dispose_old_objects / get_tlas src/render_system/scene.rs:112,150,205,218,227,234
 *   Renderer::new / render / rebuild    src/render_system/interactive_rendering.rs:447,952,818
 *   bvh::build::build_bl_bvh / build_tl_bvh  src/render_system/bvh/build.rs:249,374
 *   BvhNode                             src/render_system/bvh/mod.rs:8-25
 *   gen_mesh face order                 src/game_system/chunk.rs:158-292
 */
#ifndef VRG_H
#define VRG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define VRG_API __declspec(dllexport)
#else
#define VRG_API __attribute__((visibility("default")))
#endif

typedef int32_t vrg_status;
enum {
    VRG_OK = 0,
    VRG_ERR_INVALID_ARGUMENT = 1,
    VRG_ERR_NOT_FOUND = 2,        /* reference panics instead (scene.rs:214) */
    VRG_ERR_OUT_OF_MEMORY = 3,
    VRG_ERR_CUDA = 4,
    VRG_ERR_UNSUPPORTED = 5,
    VRG_ERR_OVERFLOW = 6,         /* a bounded device structure overflowed */
    VRG_ERR_STATE = 7,            /* call made in the wrong order */
    VRG_ERR_NO_DEVICE = 8
};

/* Chunk geometry, as the reference's game_system/chunk.rs:14-20. */
#define VRG_CHUNK_DIM 32
#define VRG_CHUNK_BLOCKS (32 * 32 * 32) /* index = x*1024 + y*32 + z */

/* Block faces in gen_mesh emission order (block.rs:9-17, chunk.rs:225-285). */
enum { VRG_FACE_LEFT = 0, VRG_FACE_RIGHT, VRG_FACE_DOWN, VRG_FACE_UP, VRG_FACE_BACK, VRG_FACE_FRONT };

/* 40-byte BVH node, the reference's wire format (bvh/mod.rs:8-25).
 * left_node_idx == 0xFFFFFFFF marks a leaf; both indices 0xFFFFFFFF marks
 * the dummy node of an empty light BVH. */
typedef struct vrg_bvh_node {
    uint32_t left_node_idx;
    uint32_t right_node_idx_or_prim_idx;
    float min[3];
    float power;
    float max[3];
    uint32_t parent_idx;
} vrg_bvh_node;

/* One material per (block type, face): index t = 6*block + face, as the
 * reference's texture index (block.rs:116-119).  The three texture maps of
 * the reference become constants:
 *   reflectivity/alpha = tex0.rgba, emission = 1000*tex1.rgb,
 *   metallic = tex2.r (raytrace.rs:465-478);
 *   luminance = the light power weight of the face, the reference's
 *   get_texture_luminances value, mean(r8+g8+b8) of the emissivity texture
 *   (utils.rs:223-235).  A face is a light iff luminance > 0 (scene.rs:560).
 * flags bit 0 (VRG_MAT_TRANSLUCENT) on face 0 of a block type marks the block
 * translucent for face culling (block.rs:125-127). */
#define VRG_MAT_TRANSLUCENT 1u
typedef struct vrg_material {
    float reflectivity[3];
    float alpha;
    float emission[3];
    float metallic;
    float luminance;
    uint32_t flags;
    uint32_t reserved[2];
} vrg_material;

/* One vertex of an uploaded triangle mesh, the reference's Vertex3D
 * (vertex.rs:4-14, 24 bytes): position, texture index t (a material-table
 * slot; a triangle's slot is its first vertex's t, raytrace.rs:455 and
 * scene.rs:559) and texture coordinate (interpolated for the atlas). */
typedef struct vrg_vertex3d {
    float position[3];
    uint32_t t;
    float uv[2];
} vrg_vertex3d;

typedef struct vrg_context_desc {
    int32_t device;          /* CUDA device ordinal */
    uint32_t flags;          /* reserved, 0 */
} vrg_context_desc;

/* eye/front/right/up as Renderer::render takes them (interactive_rendering.rs:952). */
typedef struct vrg_camera {
    float eye[3];
    float front[3];
    float right[3];
    float up[3];
    uint32_t width;
    uint32_t height;
} vrg_camera;

/* Render modes.  PARITY reproduces the reference's constants and quirks;
 * CONFIG enables the extensions that have no reference counterpart
 * (M-cap, 1-frame history ring, accumulation). */
enum { VRG_MODE_PARITY = 0, VRG_MODE_CONFIG = 1 };

/* Per-frame parameters: RenderingPreferences (camera.rs:38-56) plus the
 * compile-time constants and the invocation seeds the reference draws from
 * ThreadRng (interactive_rendering.rs:1044,1448,1491). */
typedef struct vrg_render_params {
    uint32_t nee_type;            /* 0 none, 1 light-BVH NEE, 2 NEE at bounce 1 only */
    uint32_t debug_view;          /* 0 plain path, 1 ReSTIR, 2 debug (W/10) */
    uint32_t spatial_iterations;  /* ReSTIR spatial neighbours, 0..20 */
    uint32_t num_bounces;         /* >= 2 when ReSTIR is read (view 1) */
    uint32_t mode;                /* VRG_MODE_* */
    uint32_t raygen_seed;         /* unused by the math (jitter is x0.00), kept for the API */
    uint32_t temporal_seed;
    uint32_t spatial_seed;
    float spatial_radius;         /* reference: 15 (restir_spatial_resampling.rs:314) */
    uint32_t m_cap;               /* 0 = none (reference) */
    uint32_t history_slots;       /* reservoir ring length; reference: 3 (frame % 3) */
    uint32_t accumulate;          /* 1 = add this frame's radiance to the accumulator */
    uint32_t flags;               /* VRG_RENDER_* */
    uint32_t cache_train_bounces; /* extra bounces of the cache's training paths (4) */
    uint32_t reserved[2];
} vrg_render_params;

#define VRG_RENDER_CAPTURE 1u      /* keep the full per-bounce SoA for vrg_debug_readback */
#define VRG_RENDER_NO_PACK 2u      /* skip the u8 pack (radiance output only) */
#define VRG_RENDER_CACHE 4u        /* terminate paths into the attached radiance cache after
                                      num_bounces-1 bounces; 1/16 of the paths trace
                                      cache_train_bounces more bounces and train the cache; ReSTIR
                                      then resamples the cache-terminated samples */
#define VRG_RENDER_PLAIN_ONLY 8u   /* skip the ReSTIR stages (plain path tracer, view 0) */
#define VRG_RENDER_GRAPH 16u       /* batched frames: record the frame's launch sequence once
                                      in a CUDA graph and replay it (see vrg_render_batched) */

/* Where the frame goes.  Pointers may be NULL (not written).
 *   host == VRG_OUTPUT_DEVICE: device pointers, written on the library's stream;
 *   host == VRG_OUTPUT_HOST: host memory, copied back before the call returns;
 *   host == VRG_OUTPUT_HOST_ASYNC: host memory (page-locked for the copy to
 *     overlap), copied on the library's stream after the frame; the call returns
 *     at once and the buffer holds the frame once vrg_renderer_wait_frame says
 *     that frame is done.  This is the readback of the reference's frames in
 *     flight, each fenced (interactive_rendering.rs:1633-1660). */
#define VRG_OUTPUT_DEVICE 0u
#define VRG_OUTPUT_HOST 1u
#define VRG_OUTPUT_HOST_ASYNC 2u
typedef struct vrg_frame_output {
    uint8_t *bgra8;        /* W*H*4 bytes, B,G,R,255 (postprocess.rs:78) */
    float *radiance;       /* W*H*3 floats: the view selected by debug_view */
    uint32_t host;         /* VRG_OUTPUT_* */
    uint32_t reserved;
} vrg_frame_output;

typedef struct vrg_frame_stats {
    float ms_total;            /* device time of the whole frame (CUDA events) */
    float ms_bounce[8];        /* per bounce: closest hit + shading (the light-pdf walk of
                                  bounce b runs on its own stream beside bounce b+1) */
    float ms_resolve;          /* outgoing radiance + temporal (+ cache inference/training) */
    float ms_spatial;          /* spatial + finalize + pack */
    uint64_t rays_closest;     /* closest-hit queries issued */
    uint64_t rays_any;         /* light any-hit queries issued */
    uint32_t error_flags;      /* device-side error word (stack overflow etc.) */
    uint32_t reserved;
    float ms_trace[8];         /* per bounce: k_trace alone */
    float ms_shade[8];         /* per bounce: k_shade alone */
    float ms_anyhit[8];        /* per bounce: the light-pdf walk (k_anyhit, k_hit_eval,
                                  k_hit_sum) on its stream */
    uint64_t nodes_visited;    /* closest-hit traversal: 4-wide inner nodes fetched (128 B each) */
    uint64_t leaves_visited;   /* closest-hit traversal: surface-block records tested (16 B each) */
    uint64_t light_nodes_visited;   /* light-hit collection: 4-wide lamp nodes fetched (112 B each) */
    uint64_t light_leaves_visited;  /* light-hit collection: lamp-block records tested (16 B each) */
    uint64_t light_hits;            /* light-hit collection: light triangles crossed */
} vrg_frame_stats;

typedef struct vrg_context vrg_context;
typedef struct vrg_object vrg_object;
typedef struct vrg_scene vrg_scene;
typedef struct vrg_renderer vrg_renderer;

/* ---- context ---------------------------------------------------------- */
VRG_API vrg_status vrg_context_create(const vrg_context_desc *desc, vrg_context **out);
/* Drops the handle.  Objects, scenes, renderers and caches made from the
 * context each hold a reference to it (as the reference's Arc-shared queue and
 * allocators, scene.rs:112): the context, its stream and its buffers are freed
 * when the last of them is destroyed, so handles may be destroyed in any
 * order, and a child keeps working after the context handle is gone. */
VRG_API vrg_status vrg_context_destroy(vrg_context *ctx);
/* The cudaStream_t the context submits on (the queue the reference's Scene
 * and Renderer submit to, scene.rs:112, interactive_rendering.rs:447).  A
 * caller orders its own work after a frame, or times frames with CUDA events,
 * on this stream. */
VRG_API vrg_status vrg_context_stream(vrg_context *ctx, void **stream);
/* Waits until everything submitted on the context's stream is done. */
VRG_API vrg_status vrg_context_synchronize(vrg_context *ctx);
VRG_API const char *vrg_status_string(vrg_status s);
VRG_API const char *vrg_last_error(void);

/* Replaces the texture atlas + texture_luminances given to Renderer::new /
 * Scene::new (interactive_rendering.rs:379-444, scene.rs:112).  n must be a
 * multiple of 6; air is block id n/6 (block.rs:106-107,121-123). */
VRG_API vrg_status vrg_material_table_set(vrg_context *ctx, const vrg_material *mats, uint32_t n);
/* The texture atlas itself (interactive_rendering.rs:379-444,736-760;
 * block.rs:70-119): per material slot t = 6*block + face (the slots of the
 * material table), three RGBA8 sRGB maps of width x height texels —
 * reflectivity + alpha, emissivity, metallicity (.r) — laid out
 * [slot][map][row][column][rgba], row 0 first.  With an atlas, shading samples
 * the three maps at the hit's interpolated gen_mesh uv (nearest texel, clamped
 * to the edge, sRGB decoded; raytrace.rs:457-480) in place of the slot's
 * constant colours, and the emission is 1000 * emissivity.rgb; each slot's
 * luminance becomes the mean of r8+g8+b8 over its emissivity map
 * (get_texture_luminances, utils.rs:223-235).  Set it after the material
 * table (n_slots = its length) and before uploading chunks, as the reference
 * fixes the luminances at Scene::new.  rgba8 == NULL removes the atlas. */
VRG_API vrg_status vrg_texture_atlas_set(vrg_context *ctx, const uint8_t *rgba8, uint32_t n_slots, uint32_t width,
                                         uint32_t height);

/* ---- objects (SceneUploader::upload_object, scene.rs:547) -------------- */
/* One 32^3 chunk of u8 block ids plus its six neighbours (L,R,D,U,B,F as
 * gen_mesh's NeighboringChunkData, chunk.rs:149-156); a NULL neighbour is air.
 * Extraction of exposed faces, light triangles and both BVHs runs on the GPU,
 * batched with the other pending uploads at the next vrg_scene_commit or
 * vrg_flush_uploads.  An all-air chunk yields an empty object (the
 * reference's SceneUploadedObjectHandle::Empty).  Thread-safe. */
VRG_API vrg_status vrg_upload_chunk(vrg_context *ctx, const uint8_t *blocks,
                                    const uint8_t *const neighbours[6], vrg_object **out);
/* SceneUploader::upload_object (scene.rs:547-725) for arbitrary triangles:
 * nverts vertices, three per triangle (a multiple of 3, as the reference
 * asserts).  A triangle is a light iff the luminance of its slot is > 0; its
 * power is luminance * area (scene.rs:555-571).  Before the call returns,
 * the GPU builds the light BLAS over the light triangles (build_bl_bvh, leaf
 * prim ids = triangle indices) and a geometry BVH over all triangles (the
 * same builder) that replaces the driver BLAS.  nverts == 0 yields an empty
 * object.  Every t must be a slot of the material table.  Thread-safe. */
VRG_API vrg_status vrg_upload_mesh(vrg_context *ctx, const vrg_vertex3d *v, uint64_t nverts, vrg_object **out);
/* Runs every pending upload now (one batched launch sequence). */
VRG_API vrg_status vrg_flush_uploads(vrg_context *ctx);
VRG_API vrg_status vrg_object_release(vrg_object *obj);
/* Counts of an uploaded object (after a flush): exposed faces, triangles,
 * light triangles, geometry prims (surface blocks). */
VRG_API vrg_status vrg_object_info(vrg_object *obj, uint32_t *n_faces, uint32_t *n_triangles,
                                   uint32_t *n_light_triangles, uint32_t *n_surface_blocks);
/* Copies the object's light BLAS (build_bl_bvh output, chunk-local) and its
 * geometry BLAS (build_tl_bvh semantics over per-block AABBs) into host
 * arrays of 2n-1 nodes; prim_order receives the final primitive permutation. */
VRG_API vrg_status vrg_object_read_bvh(vrg_object *obj, uint32_t which /*0 light, 1 geometry*/,
                                       vrg_bvh_node *nodes, uint32_t cap_nodes, uint32_t *n_nodes,
                                       uint32_t *prim_order, uint32_t cap_prims, uint32_t *n_prims);

/* ---- scene (Scene, scene.rs:86-497) ----------------------------------- */
VRG_API vrg_status vrg_scene_create(vrg_context *ctx, vrg_scene **out);
VRG_API vrg_status vrg_scene_destroy(vrg_scene *scene);
/* xform3x4 is the instance transform as a row-major 3x4 matrix [R|t] (the
 * matrix of the reference's Isometry3, InstanceData.transform, scene.rs:407-416;
 * NULL = identity).  Mesh objects take any finite matrix (the reference passes
 * isometries, e.g. its ego cube, main.rs:86-101, scene_manager.rs:23-35).
 * Chunk objects take identity R and an integral translation within +-16384
 * (the reference only translates chunks, chunk_manager.rs:234-248);
 * anything else returns VRG_ERR_UNSUPPORTED. */
VRG_API vrg_status vrg_scene_add(vrg_scene *scene, uint64_t key, vrg_object *obj, const float xform3x4[12]);
VRG_API vrg_status vrg_scene_update(vrg_scene *scene, uint64_t key, const float xform3x4[12]);
VRG_API vrg_status vrg_scene_remove(vrg_scene *scene, uint64_t key);
/* = get_tlas: rebuilds the top levels (light TL BVH, geometry TL BVH) and
 * the traversal layouts when something changed; frees retired objects. */
VRG_API vrg_status vrg_scene_commit(vrg_scene *scene);
/* Commits several scenes of one context at once (no reference counterpart):
 * the same result per scene as vrg_scene_commit, with all their top-level
 * trees built by one SAH build and all their lamp-block trees by another. */
VRG_API vrg_status vrg_scene_commit_many(vrg_scene *const *scenes, uint32_t n);
/* Copies the top-level BVHs (which: 0 light TL, 1 geometry TL). */
VRG_API vrg_status vrg_scene_read_tl(vrg_scene *scene, uint32_t which, vrg_bvh_node *nodes,
                                     uint32_t cap, uint32_t *n_nodes);

/* ---- renderer (Renderer, interactive_rendering.rs:328-1669) ----------- */
VRG_API vrg_status vrg_renderer_create(vrg_context *ctx, uint32_t width, uint32_t height,
                                       uint32_t max_bounces, vrg_renderer **out);
VRG_API vrg_status vrg_renderer_destroy(vrg_renderer *r);
/* Renderer::rebuild: new extent, all per-pixel state reset. */
VRG_API vrg_status vrg_renderer_resize(vrg_renderer *r, uint32_t width, uint32_t height);
/* Renderer.scale (interactive_rendering.rs:329,1010; postprocess.rs:39-88):
 * frames are traced at scale x the output extent, and each output pixel (BGRA8
 * and radiance) is the mean of its scale x scale traced pixels.  Cameras keep
 * the output extent; accumulation and debug readback are at the traced
 * resolution.  1..8 (1 = the reference's default); reallocates like
 * vrg_renderer_resize.  Single-view renderers. */
VRG_API vrg_status vrg_renderer_set_scale(vrg_renderer *r, uint32_t scale);

/* Image files of a frame (replacing the swapchain copy,
 * interactive_rendering.rs:1625-1629): BGRA8 as binary PPM (P6) or PNG
 * (8-bit RGB, stored deflate blocks), float RGB as PFM (little-endian,
 * bottom row first as the format requires).  Host buffers, row 0 = top. */
VRG_API vrg_status vrg_image_write_ppm(const char *path, const uint8_t *bgra8, uint32_t width, uint32_t height);
VRG_API vrg_status vrg_image_write_png(const char *path, const uint8_t *bgra8, uint32_t width, uint32_t height);
VRG_API vrg_status vrg_image_write_pfm(const char *path, const float *rgb, uint32_t width, uint32_t height);
/* Renderer::render.  frame_index = the renderer's frame counter, advanced by
 * one per call (interactive_rendering.rs:1668); the raytrace invocation seed
 * is frame_index*num_bounces + bounce (:1189).
 * With stats == NULL and device, asynchronous host or no outputs the call
 * only enqueues the frame and returns; the frame is complete when the
 * library's stream has passed it (or vrg_renderer_wait_frame returns).  Such
 * frames are in flight together, as the reference's frames in flight are: a
 * frame's first bounce starts beside the previous frame's resolve and spatial
 * passes (it reads only the committed scene, the camera and the materials, and
 * fills its own set of path records).  The images are those of frames
 * rendered one by one.  With stats the frame runs alone and is timed stage by
 * stage. */
VRG_API vrg_status vrg_render(vrg_renderer *r, vrg_scene *scene, const vrg_camera *cam,
                              const vrg_render_params *params, const vrg_frame_output *out,
                              vrg_frame_stats *stats);
VRG_API vrg_status vrg_renderer_frame_index(vrg_renderer *r, uint32_t *frame_index);
/* Blocks until frame frame_index of this renderer (and its copies out) is
 * done: the fence of a frame in flight (the reference signals a fence per
 * frame slot, interactive_rendering.rs:1652, and waits on it before reusing
 * the slot, :1634-1642).  A frame index not yet rendered is an error. */
VRG_API vrg_status vrg_renderer_wait_frame(vrg_renderer *r, uint32_t frame_index);
VRG_API vrg_status vrg_renderer_reset_accumulation(vrg_renderer *r);
/* Accumulated mean radiance (W*H*3 floats, host) after n frames with accumulate=1. */
VRG_API vrg_status vrg_renderer_read_accumulation(vrg_renderer *r, float *rgb, uint32_t *n_frames);

/* Debug / parity readback of the last frame rendered with VRG_RENDER_CAPTURE.
 * what selects an array; the layout is W*H*comps floats per bounce slice:
 *   VRG_DBG_ORIGIN (nb+1 slices, 3), VRG_DBG_DIRECTION (nb+1, 3),
 *   VRG_DBG_NORMAL (nb, 3), VRG_DBG_EMISSIVITY (nb, 3), VRG_DBG_REFLECTIVITY (nb, 3),
 *   VRG_DBG_MIS (nb, 1), VRG_DBG_BSDF_PDF (nb, 1), VRG_DBG_NEE_PDF (nb, 1),
 *   VRG_DBG_RADIANCE (nb, 3), VRG_DBG_Q (nb, 1),
 *   VRG_DBG_HIT (nb, 4 u32: instance, triangle, block index, face|half<<8),
 *   VRG_DBG_TEMPORAL / VRG_DBG_SPATIAL (1, 20: x_v,n_v,x_s,n_s,l_o_hat,p_omega,
 *       seed,ucw,m,w_sum as floats with seed/m bit-cast u32),
 *   VRG_DBG_FINAL (1, 3). */
enum {
    VRG_DBG_ORIGIN = 0, VRG_DBG_DIRECTION, VRG_DBG_NORMAL, VRG_DBG_EMISSIVITY,
    VRG_DBG_REFLECTIVITY, VRG_DBG_MIS, VRG_DBG_BSDF_PDF, VRG_DBG_NEE_PDF,
    VRG_DBG_RADIANCE, VRG_DBG_Q, VRG_DBG_HIT, VRG_DBG_TEMPORAL, VRG_DBG_SPATIAL,
    VRG_DBG_FINAL,
    VRG_DBG_CACHE_TARGET,  /* (1, 4): the radiance cache's training target per pixel (rgb, 0) as
                              left by the last cache frame (no capture needed) */
    VRG_DBG_COUNT
};
VRG_API vrg_status vrg_debug_readback(vrg_renderer *r, uint32_t what, void *dst, uint64_t bytes);

/* ---- cross-frame state (no reference counterpart) ------------------------
 * Everything a renderer carries from one frame to the next — the reservoir
 * history ring (5 x 16 bytes per pixel and slot), the frame counter (which
 * seeds the per-pixel streams) and the FP64 accumulation with its frame count
 * — as one host blob, for checkpoints and deterministic replay: frames
 * rendered after a load repeat, bit for bit, the frames rendered after the
 * save.  A blob loads only into a renderer of the same pixel count and ring
 * length.  The radiance cache is saved apart (vrg_nrc_read / vrg_nrc_write). */
VRG_API vrg_status vrg_renderer_state_size(vrg_renderer *r, uint64_t *bytes);
VRG_API vrg_status vrg_renderer_state_save(vrg_renderer *r, void *dst, uint64_t bytes);
VRG_API vrg_status vrg_renderer_state_load(vrg_renderer *r, const void *src, uint64_t bytes);

/* ---- launch configuration and autotuner (no reference counterpart) -----
 * Every field changes only how the frame's work is scheduled, never a result
 * (the tests render the same bits under any configuration).  0 = default. */
typedef struct vrg_tuning {
    uint32_t trace_blocks_per_sm;   /* persistent closest-hit grid: CTAs of 128 threads per SM
                                       (default and maximum: full occupancy) */
    uint32_t trace_refill;          /* idle lanes of a warp that trigger its ray refill, 1..32 (8) */
    uint32_t shade_blocks_per_sm;   /* shading / light-pdf evaluation grids */
    uint32_t anyhit_blocks_per_sm;  /* light-hit collection grid */
    uint32_t anyhit_refill;         /* as trace_refill, for the light-hit collection (8) */
    uint32_t stream_block;          /* threads per CTA of the per-pixel kernels: 64, 128 or 256 (256) */
    uint32_t spatial_staging;       /* how the spatial pass reads reservoirs: 1 each CTA's 32x8-pixel tile
                                       staged in shared memory by one tensor copy (TMA; single-view
                                       renderers of at least 32x8 pixels, else 2), 2 per-thread loads;
                                       0 = 2.  The autotuner keeps the value it is given: staged tiles
                                       speed up the spatial pass alone but slow frames in flight, whose
                                       walks beside it lose L1 to the tile's shared memory */
    uint32_t reserved[1];
} vrg_tuning;

VRG_API vrg_status vrg_renderer_set_tuning(vrg_renderer *r, const vrg_tuning *t);
/* The configuration in effect, defaults resolved to their values. */
VRG_API vrg_status vrg_renderer_get_tuning(vrg_renderer *r, vrg_tuning *t);
/* Autotuner: renders frames of (scene, cam, params) under candidate launch
 * configurations, one field at a time over its candidate values (coordinate
 * descent, two passes).  Each candidate is timed as frames are rendered in
 * use: `frames` frames enqueued back to back (frames in flight), bracketed by
 * CUDA events on the library stream, after one untimed frame; the median of
 * three such runs, per frame.  A candidate that times faster than the current
 * choice is timed again, beside the current choice, and taken only if it is
 * still faster.  Installs the result and returns it with its time per frame.  The tuning frames do not count: the frame counter,
 * reservoir history and accumulation are restored afterwards.  Single-view
 * renderers; params must not carry VRG_RENDER_CACHE / CAPTURE / GRAPH (the
 * result applies to those frames as well). */
VRG_API vrg_status vrg_renderer_autotune(vrg_renderer *r, vrg_scene *scene, const vrg_camera *cam,
                                         const vrg_render_params *params, uint32_t frames, vrg_tuning *best,
                                         float *best_ms);

/* ---- batched views (no reference counterpart: the reference renders one
 * swapchain view per Renderer::render) ------------------------------------
 * A batched renderer owns n_views views of independent extents; one
 * vrg_render_batched call renders every view, each of its own scene and
 * camera, through ONE wavefront launch sequence: the views' pixels are
 * numbered view after view (view v starts at pixel_offset(v)), every kernel
 * looks up its pixel's view, and the queues are shared, so small views do
 * not leave the GPU idle.  A view renders exactly the image that a
 * single-view renderer of its extent renders with the same scene, camera,
 * seeds and frame index.  Per-view data (scene BVHs, cameras, seeds, frame
 * index) lives in a device table refreshed at the start of every call, so
 * with VRG_RENDER_GRAPH the launch sequence is recorded once in a CUDA graph
 * (one per history-ring slot and parameter set; a change of num_bounces,
 * flags or the other parameters records a new one) and replayed.
 * VRG_RENDER_GRAPH cannot be combined with VRG_RENDER_CACHE or
 * VRG_RENDER_CAPTURE (VRG_ERR_UNSUPPORTED); the stats of a graph frame carry
 * ms_total and the counters, not the per-kernel times.  Without stats, graph
 * or cache, two batched frames are in flight together, as vrg_render's frames
 * are (each in its own array set, with its own view table). */
typedef struct vrg_view {
    vrg_scene *scene;          /* committed by the call if dirty (all views' scenes
                                  are committed before any view renders) */
    vrg_camera camera;         /* width/height must equal the view's extent */
    uint32_t temporal_seed;    /* this view's ReSTIR seeds (the params' seeds are unused) */
    uint32_t spatial_seed;
} vrg_view;

VRG_API vrg_status vrg_renderer_create_batched(vrg_context *ctx, uint32_t n_views, const uint32_t *widths,
                                               const uint32_t *heights, uint32_t max_bounces,
                                               vrg_renderer **out);
/* Pixel offset of a view in the batch's pixel numbering (0 for a single-view renderer). */
VRG_API vrg_status vrg_renderer_view_offset(vrg_renderer *r, uint32_t view, uint64_t *pixel_offset);
/* Renders all views.  outs: NULL or n_views entries (per view, like
 * vrg_render's out; host or device pointers).  vrg_renderer_read_accumulation
 * and vrg_debug_readback of a batched renderer cover all views' pixels in
 * batch order. */
VRG_API vrg_status vrg_render_batched(vrg_renderer *r, const vrg_view *views, uint32_t n_views,
                                      const vrg_render_params *params, const vrg_frame_output *outs,
                                      vrg_frame_stats *stats);

/* ---- standalone SAH builds (build.rs:249,374), batched, device-side --- */
/* Builds `count` independent trees in one launch sequence.  Tree i owns
 * prims [prim_offset[i], prim_offset[i]+n[i]) of the input arrays and writes
 * 2n-1 nodes at node_offset[i].  All pointers are HOST arrays; the library
 * stages them to the device, builds on the GPU and copies the nodes back.
 *   tl variant: aabbs (6 floats: min, max) + translation (3 floats)
 *   bl variant: triangles (9 floats) */
VRG_API vrg_status vrg_build_tl_bvh_batched(vrg_context *ctx, uint32_t count, const uint32_t *n,
                                            const uint32_t *prim_offset, const uint32_t *node_offset,
                                            const float *translations, const float *aabbs,
                                            const float *power, const uint32_t *ids,
                                            vrg_bvh_node *nodes_out, uint32_t *prim_order_out);
VRG_API vrg_status vrg_build_bl_bvh_batched(vrg_context *ctx, uint32_t count, const uint32_t *n,
                                            const uint32_t *prim_offset, const uint32_t *node_offset,
                                            const float *luminance, const float *triangles,
                                            const uint32_t *ids, vrg_bvh_node *nodes_out,
                                            uint32_t *prim_order_out);

/* Builds one tree with build_tl_bvh semantics (identity isometries) without
 * allocating any memory.  No counterpart in the reference.  It is meant for
 * callers that may not allocate device memory while they run: an engine
 * that owns the whole device-memory budget, or a streaming worker building
 * next to a frame in flight, where cudaMalloc/cudaFree can synchronize the
 * device.  All pointers are device pointers owned by the caller: aabbs n x 6
 * floats (min, max), power n floats, ids n u32; nodes receives 2n-1 nodes,
 * prim_order n u32.  stream is a cudaStream_t (NULL = legacy default).
 * n must be 1..32768; larger n returns VRG_ERR_INVALID_ARGUMENT.
 * Scratch is one fixed device array of about 2.4 MiB inside the library,
 * held by every GPU that loads it until the process exits.  Each call looks
 * up that array's device address in the current context
 * (cudaGetSymbolAddress, which allocates nothing).  Every call shares the
 * array: calls that overlap on the GPU (other threads or streams) race and
 * must be serialized by the caller.  The call copies small host values to
 * the device, synchronizes `stream` once per BVH level (it reads each
 * level's work count back to the host) and returns after the build has
 * finished on `stream`; an error return also synchronizes `stream` first. */
VRG_API vrg_status vrg_build_tl_bvh_noalloc(const float *aabbs, const float *power, const uint32_t *ids,
                                            uint32_t n, vrg_bvh_node *nodes, uint32_t *prim_order, void *stream);

/* ---- roofline denominator (no reference counterpart) ------------------
 * Measures the device's L2 read bandwidth: a library kernel sweeps a buffer
 * of `bytes` (1..96 MiB, small enough to stay in L2) `reps` times with
 * 16-byte loads that bypass L1, on the context's stream; *gbs = bytes * reps
 * / the CUDA-event time of that launch.  The BVH walks are held against it
 * (their node fetches are L1/L2 traffic).  Synchronizes the stream. */
VRG_API vrg_status vrg_measure_l2_bandwidth(vrg_context *ctx, uint64_t bytes, uint32_t reps, float *gbs);

/* ---- neural radiance cache (no reference counterpart) ----------------
 * Multiresolution hash-grid encoding of the position (levels x 2 features,
 * 2^log2_table entries per level, resolutions base..max geometric) plus
 * octahedral normal and view direction, 5 hidden ReLU layers of width 64 and
 * a linear RGB output; BF16 weights/activations on the tensor cores with
 * FP32 accumulation; relative L2 loss; Adam (beta1 0.9, beta2 0.99). */
typedef struct vrg_nrc vrg_nrc;
typedef struct vrg_nrc_desc {
    uint32_t levels;           /* 16 */
    uint32_t log2_table;       /* 19 */
    uint32_t features;         /* 2 */
    uint32_t base_resolution;  /* 16 */
    uint32_t max_resolution;   /* 2048 */
    uint32_t batch;            /* training samples per frame, 65536 */
    float learning_rate;       /* 1e-2 */
    uint32_t seed;
    float scene_min[3];        /* box mapped to the unit cube */
    float scene_max[3];
    uint32_t flags;            /* VRG_NRC_* below */
    uint32_t reserved;
} vrg_nrc_desc;
/* Training runs on the 5th-generation tensor cores (tcgen05: 128-sample tiles,
 * tensor-memory accumulators) unless VRG_NRC_TRAIN_WARP_MMA selects the
 * warp-level mma.sync training kernel (32-sample tiles). */
#define VRG_NRC_TRAIN_WARP_MMA 1u
/* vrg_nrc_read / vrg_nrc_write selectors.  VRG_NRC_TRAIN_PREDICTIONS (read
 * only): the network's outputs for the last vrg_nrc_train batch, n x 3 floats,
 * from the training pass's own forward pass (the tensor-core path of the
 * training kernel, next to vrg_nrc_query's). */
enum { VRG_NRC_WEIGHTS = 0, VRG_NRC_WEIGHT_GRADS, VRG_NRC_TABLE, VRG_NRC_TABLE_GRADS, VRG_NRC_ZERO_GRADS,
       VRG_NRC_TRAIN_PREDICTIONS };
VRG_API vrg_status vrg_nrc_create(vrg_context *ctx, const vrg_nrc_desc *desc, vrg_nrc **out);
VRG_API vrg_status vrg_nrc_destroy(vrg_nrc *nrc);
/* Host arrays: pos/normal/dir n x 3 floats (dir = the incoming ray direction;
 * the network sees -dir), rgb n x 3 out. */
VRG_API vrg_status vrg_nrc_query(vrg_nrc *nrc, uint32_t n, const float *pos, const float *normal, const float *dir,
                                 float *rgb);
/* One training batch: gradients accumulate; update != 0 applies an Adam step
 * (and clears the gradients). *loss = mean relative L2 loss of the batch. */
VRG_API vrg_status vrg_nrc_train(vrg_nrc *nrc, uint32_t n, const float *pos, const float *normal, const float *dir,
                                 const float *target, uint32_t update, float *loss);
/* Parameter / gradient access (fp32): weights = 5 x 64x64 then 16x64
 * (rows 0..2 used), [out][in]; table = levels x 2^log2_table x 2. */
VRG_API vrg_status vrg_nrc_read(vrg_nrc *nrc, uint32_t what, void *dst, uint64_t bytes);
VRG_API vrg_status vrg_nrc_write(vrg_nrc *nrc, uint32_t what, const void *src, uint64_t bytes);
VRG_API vrg_status vrg_nrc_layout(vrg_nrc *nrc, uint32_t *levels, float *scales, uint32_t *dense, uint32_t *res1);
/* Attaches a cache to a renderer for VRG_RENDER_CACHE frames (NULL detaches).
 * A cache frame computes its training step's gradients; their Adam step runs
 * when the cache is next used (the next cache frame, beside its bounces, or
 * first thing in any vrg_nrc_* call), so every use sees the cache as if the
 * step had ended the frame. */
VRG_API vrg_status vrg_renderer_set_cache(vrg_renderer *r, vrg_nrc *nrc);

/* ---- synthetic scenes (no reference counterpart; the reference uses
 *      OpenSimplex worldgen, chunk.rs:56-109) -------------------------- */
/* Fills mats (capacity >= 6*(6+16)) with 6 opaque Lambertian block types
 * (albedo U[0.2,0.8]^3) and 16 emissive types (radiance U[5,20]^3); returns
 * the count in *n.  Air is block id (*n)/6. */
VRG_API vrg_status vrg_terrain_materials(uint64_t seed, vrg_material *mats, uint32_t cap, uint32_t *n);
/* World of nx*nz chunks (one chunk tall): 2-octave value-noise heightfield,
 * heights 8..24, solid blocks uniform over the 6 Lambertian types, a fraction
 * `emissive` of surface blocks emissive.  blocks: nx*nz*32768 bytes, chunk
 * (cx,cz) at offset (cx*nz+cz)*32768, chunk-local index x*1024+y*32+z. */
VRG_API vrg_status vrg_terrain_generate(uint64_t seed, uint32_t nx, uint32_t nz, float emissive,
                                        uint8_t *blocks);
/* Orbit camera of the benchmark path: frame f of n around the world centre. */
VRG_API vrg_status vrg_orbit_camera(uint32_t nx, uint32_t nz, uint32_t frame, uint32_t n_frames,
                                    uint32_t width, uint32_t height, vrg_camera *cam);
/* PCG32 host stream for invocation seeds (replaces rand::rng()). */
VRG_API uint32_t vrg_pcg32_next(uint64_t *state, uint64_t inc);

#ifdef __cplusplus
}
#endif
#endif /* VRG_H */
