// Host-side internals shared by the library's translation units.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <array>
#include <atomic>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/vrg.h"
#include "vrg_device.cuh"
#include "vrg_frame.cuh"

namespace vrg {

void set_error(const char *fmt, ...);

#define VRG_CUDA_TRY(expr)                                                              \
    do {                                                                                \
        cudaError_t _e = (expr);                                                        \
        if (_e != cudaSuccess) {                                                        \
            ::vrg::set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), __FILE__, \
                             __LINE__);                                                 \
            return VRG_ERR_CUDA;                                                        \
        }                                                                               \
    } while (0)

#define VRG_TRY(expr)                   \
    do {                                \
        vrg_status _s = (expr);         \
        if (_s != VRG_OK) return _s;    \
    } while (0)

// Stream-ordered device allocation owned by a shared_ptr: freed with
// cudaFreeAsync on the owning stream, so a buffer retired while frames that
// read it are still queued is released only after them (the reference keeps
// retired objects alive in old_data for the same reason, scene.rs:58-70).
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    cudaStream_t stream = nullptr;
    ~DevBuf();
};
using DevBufPtr = std::shared_ptr<DevBuf>;
vrg_status dev_alloc(cudaStream_t s, size_t bytes, DevBufPtr &out);

// ---- SAH builder ------------------------------------------------------
struct SahTree {
    uint32_t n;          // prims
    uint32_t prim_off;   // into the prim arrays
    uint32_t node_off;   // into the node array (2n-1 nodes)
    uint32_t pad;
};
struct SahInputs {
    const float4 *lo;    // prim AABB min (xyz)
    const float4 *hi;    // prim AABB max (xyz)
    const float4 *cen;   // centroid (xyz), w = power
    const uint32_t *id;  // prim index id written into leaves
};
struct SahOutputs {
    vrg_bvh_node *nodes;
    uint32_t *perm;       // local prim order per tree (prim_off-relative)
    uint32_t *leaf_prim;  // per node: local prim index of a leaf, INVALID for internal nodes
};
// Builds every tree; trees with n == 0 are skipped.  *levels receives the
// number of level passes (an upper bound on depth - 2).
vrg_status sah_build(cudaStream_t s, const std::vector<SahTree> &trees, uint32_t total_prims,
                     uint32_t total_nodes, const SahInputs &in, const SahOutputs &out, uint32_t *levels);

// ---- chunk extraction ---------------------------------------------------
struct ChunkSummary {      // per chunk, copied to the host after a flush
    uint32_t n_faces, n_tris, n_light, n_geo;
    float light_lo[3], light_hi[3];
    float light_power;
    float geo_lo[3], geo_hi[3];
    uint32_t pad;
};

struct Context;

struct Object {
    Context *ctx = nullptr;
    std::vector<uint8_t> blocks;          // pending until flushed
    std::vector<uint8_t> slabs;           // 6 x 1024 neighbour boundary planes
    uint32_t slab_present = 0;            // bit i: neighbour i given
    bool flushed = false;
    ChunkSummary sum{};
    DevBufPtr batch;                      // device arrays of the flush batch
    // pointers into the batch (device)
    const int2 *geo_local = nullptr;      // per geometry prim: (blk | mask<<15 | id<<21, first_tri)
    const vrg_bvh_node *geo_nodes = nullptr;
    const uint32_t *geo_perm = nullptr;
    const uint32_t *geo_leaf = nullptr;
    const vrg_bvh_node *light_nodes = nullptr;
    const uint32_t *light_perm = nullptr;
    const uint32_t *light_leaf = nullptr;
    const uint32_t *light_tri = nullptr;  // per light prim: lx|ly<<5|lz<<10|face<<15|half<<18
    const uint32_t *light_leaf_tri = nullptr;  // per light node (leaf payload, same packing)
    uint32_t levels = 0;                  // SAH level passes of the batch (depth bound)
    // an uploaded triangle mesh (vrg_upload_mesh) instead of a chunk: its
    // object-space triangles (3 float4: v0 | material slot bits, v1, v2) and
    // vertex uvs (6 floats per triangle); geo_* is the BVH over the triangles
    // (leaf prim = triangle), light_tri / light_leaf_tri hold triangle indices
    bool mesh = false;
    const float4 *mesh_tri = nullptr;
    const float *mesh_uv = nullptr;
    std::atomic<int> refs{1};
    virtual ~Object();  // frees its buffers, then drops its reference to the context
};

struct Context {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<vrg_material> mats;
    DevBufPtr d_mats;
    DevBufPtr d_atlas;                   // texture atlas (RGBA8) + sRGB table, or empty
    uint32_t atlas_w = 0, atlas_h = 0;
    const float *d_srgb = nullptr;
    uint32_t n_types = 0;
    std::mutex mu;                       // guards pending + stream use from upload threads
    std::vector<Object *> pending;
    int num_sms = 0;
    // references: the handle, and every object, scene, renderer and cache made
    // from it (as the reference's Arc-shared queues and allocators): the
    // context, its stream and its buffers are freed when the last one is
    // dropped, whatever the order in which the handles are destroyed
    std::atomic<int> refs{1};
};
void ctx_retain(Context *c);
void ctx_release(Context *c);

vrg_status extract_and_build(Context *ctx, std::vector<Object *> &batch);
// upload_object of a triangle mesh: validates, builds the light BLAS and the
// geometry BVH on the GPU and fills the object (mesh.cu)
vrg_status mesh_upload(Context *ctx, const vrg_vertex3d *v, uint64_t nverts, Object *o);

// ---- scene -------------------------------------------------------------
struct SceneEntry {
    Object *obj;
    float off[3];       // the translation
    float m[12];        // the transform, row-major [R|t]
    bool tonly;         // R is exactly the identity: points move by p + off
};

struct Scene {
    Context *ctx = nullptr;
    std::map<uint64_t, SceneEntry> objects;
    bool dirty = true;
    // committed state
    std::vector<Object *> inst_objs;      // instance order (key order, non-empty)
    std::vector<std::array<float, 3>> inst_off;
    std::vector<std::array<float, 12>> inst_xf;
    std::vector<uint8_t> inst_tonly;
    DevBufPtr d_buf;                      // wide layouts, records, TLs, instance table
    DevBufPtr lamp_buf;                   // lamp-block any-hit layout
    DevScene dev{};
    std::vector<vrg_bvh_node> h_light_tl, h_geo_tl;
    uint32_t depth_bound = 0;
    std::vector<Object *> retired;        // released when the next commit completes
};
vrg_status scene_commit(Scene *sc);
// the scene's device description with the context's current material table
// and texture atlas
DevScene frame_scene(const Scene *sc);
// Commits every dirty scene of scs (one context); their top-level and lamp
// trees are built by one SAH build each.
vrg_status scene_commit_many(Scene *const *scs, uint32_t n);
// Standalone batched builds of the C ABI: tri == false -> build_tl_bvh over
// (aabb[6], translation[3]) prims, tri == true -> build_bl_bvh over triangles.
vrg_status standalone_sah(Context *ctx, bool tri, uint32_t count, const uint32_t *n, const uint32_t *prim_offset,
                          const uint32_t *node_offset, const float *prims, const float *translations,
                          const float *power, const uint32_t *ids, vrg_bvh_node *nodes_out, uint32_t *order_out);

// ---- neural radiance cache (nrc.cu) ---------------------------------------
struct Nrc;
vrg_status nrc_create(Context *ctx, const vrg_nrc_desc *d, Nrc **out);
void nrc_destroy(Nrc *N);
vrg_status nrc_set_bounds(Nrc *N, const float lo[3], const float hi[3]);
// err: the device error word the kernels flag (NULL: the cache's own word,
// checked by the host-array entry points)
vrg_status nrc_infer(Nrc *N, cudaStream_t s, uint32_t n, const uint32_t *n_dev, const uint32_t *list,
                     const float4 *pos, const float4 *dir, const float4 *nrm, float4 *out, uint32_t *err);
// pred (optional): the forward pass's prediction of each sample
vrg_status nrc_train(Nrc *N, cudaStream_t s, uint32_t n, const uint32_t *n_dev, const uint32_t *list,
                     const float4 *pos, const float4 *dir, const float4 *nrm, const float4 *target, bool update,
                     uint32_t *err, float4 *pred = nullptr);
vrg_status nrc_update(Nrc *N, cudaStream_t s);
vrg_status nrc_flush(Nrc *N, cudaStream_t s);
bool nrc_pending(const Nrc *N);
void nrc_defer_update(Nrc *N);
uint32_t nrc_batch(const Nrc *N);
vrg_status nrc_query_host(Nrc *N, uint32_t n, const float *pos, const float *nrm, const float *dir, float *rgb);
vrg_status nrc_train_host(Nrc *N, uint32_t n, const float *pos, const float *nrm, const float *dir, const float *target,
                          uint32_t update, float *loss_out);
vrg_status nrc_read(Nrc *N, uint32_t what, void *dst, uint64_t bytes);
vrg_status nrc_write(Nrc *N, uint32_t what, const void *src, uint64_t bytes);
void nrc_layout(uint32_t *levels, float *scales, uint32_t *dense, uint32_t *res1, const Nrc *N);

// ---- renderer ------------------------------------------------------------
struct Renderer {
    Context *ctx = nullptr;
    uint32_t W = 0, H = 0, nb_max = 0;
    uint64_t P = 0;                       // pixels of a frame (all views of a batched renderer)
    uint32_t scale = 1;                   // supersampling: W x H = out_w*scale x out_h*scale traced pixels
    uint32_t out_w = 0, out_h = 0;        // output extent (the camera's)
    DevBufPtr out_buf;                    // output-resolution radiance when scale > 1
    float *radiance_out = nullptr;
    // batched views (n_views == 0: single-view renderer)
    uint32_t n_views = 0;
    std::vector<uint32_t> vw, vh;         // view extents
    std::vector<uint64_t> voff;           // first pixel of each view
    DevBufPtr view_buf;                   // a ViewDev[n_views] table per array set + vtab
    ViewDev *d_views[3] = {};
    uint16_t *d_vtab = nullptr;
    ViewDev *h_views = nullptr;           // pinned staging, 2 x n_views
    cudaEvent_t ev_stage[2] = {};         // after the copy out of each staging half
    uint32_t stage = 0;
    struct GraphEntry {
        std::vector<uint8_t> key;         // the frame's FrameArgs bytes
        cudaGraphExec_t exec;
    };
    std::vector<GraphEntry> graphs;
    uint32_t frame = 0;
    uint32_t ring_slots = 0;
    uint32_t last_nb = 0;
    uint32_t last_ring = 0;
    bool captured = false;
    DevBufPtr buf;
    // Device arrays (P = W*H).  The arrays of a frame's bounces come in SETS
    // sets (one for batched renderers), taken in turn by frame index: up to
    // SETS frames' bounces may be in flight at once, each in its own set; the
    // arrays after the sets are read and written only by the frames' resolve
    // and spatial passes, which run one frame after the other on the library
    // stream.
    struct FrameSet {
        float4 *ray_o = nullptr, *ray_d = nullptr;
        uint32_t *queue[2] = {nullptr, nullptr};
        uint32_t *counters = nullptr;          // CNT_* words of vrg_frame.cuh
        uint32_t *aqueue[2] = {nullptr, nullptr};  // light-pdf jobs by bounce parity
        float4 *ajob[2] = {nullptr, nullptr};      // their ray copies (2 float4 per job)
        int4 *hits = nullptr;                  // closest hit per pixel
        uint4 *hitbuf = nullptr;               // light hits of the any-hit pass
        float *hitval = nullptr;
        uint2 *jmeta = nullptr;
        uint8_t *nlive = nullptr;
        float4 *rec = nullptr;                 // [nb][2][P]
        float4 *xv = nullptr, *nv = nullptr, *xs = nullptr, *ns = nullptr;
    };
    static constexpr int SETS = 3;        // frames whose bounces may be in flight at once (at most)
    uint32_t n_sets = SETS;               // this renderer's sets (a batched renderer: 2)
                                          // (2 -> 3: 1.264 -> 1.247 ms per 1080p frame)
    FrameSet fs[SETS];
    float4 *plain = nullptr;              // L[0] per pixel
    float4 *res = nullptr;                // [ring][5][P] temporal reservoirs
    DevBufPtr res_buf;
    float4 *spatial = nullptr;            // [5][P] spatial reservoirs (capture)
    float4 *final_t = nullptr;            // restir final target (capture)
    uint8_t *bgra = nullptr;
    float *radiance = nullptr;            // [P*3]
    double *accum = nullptr;              // [P*3]
    uint32_t accum_n = 0;
    // capture arrays
    DevBufPtr cap;
    float *c_origin = nullptr, *c_dir = nullptr, *c_normal = nullptr, *c_emis = nullptr, *c_refl = nullptr;
    float *c_mis = nullptr, *c_pdf = nullptr, *c_nee = nullptr, *c_L = nullptr, *c_q = nullptr;
    uint32_t *c_hit = nullptr;
    // host staging
    uint8_t *h_pinned = nullptr;
    size_t h_pinned_bytes = 0;
    cudaStream_t aux = nullptr;           // second stream: a cache frame's training paths and step
    cudaStream_t aux_lp = nullptr;        // the training bounces' light-pdf walks, beside the next bounce
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_start = nullptr, ev_updated = nullptr;
    // Per set: the bounce stream of frames in flight and the light-pdf stream
    // (bounce b's walk beside bounce b + 1), the dependency events per bounce,
    // the end of the set's bounces and the end of its frame (after the
    // resolve and spatial passes on the library stream).
    cudaStream_t bs[SETS] = {}, lps[SETS] = {};
    cudaEvent_t ev_shaded[SETS][8] = {}, ev_lpdone[SETS][8] = {};
    cudaEvent_t ev_bounced[SETS] = {}, ev_done[SETS] = {};
    // per-frame fences (frame index % FENCES): recorded after the frame and its
    // copies out; vrg_renderer_wait_frame waits on them
    static constexpr uint32_t FENCES = 8;
    cudaEvent_t ev_fence[FENCES] = {};
    cudaEvent_t ev_lp[2][8] = {};         // timing: light-pdf passes of bounce b begin / end
    cudaEvent_t ev[16] = {};
    cudaEvent_t ev_k[2][8] = {};          // after k_trace / after k_shade, per bounce
    Nrc *cache = nullptr;                 // attached radiance cache (not owned)
    DevBufPtr cache_buf;                  // per-pixel cache queries / predictions / targets
    uint32_t cache_cap = 0;               // training paths cache_buf was sized for
    // a cache frame's arrays, one set per array set: cache queries,
    // predictions and targets per pixel, the query and training lists, and
    // the training branch's light-pdf jobs and hits (its walks run beside the
    // main walk of the query bounce), sized for the training paths
    struct CacheSet {
        float4 *q_pos = nullptr, *q_dir = nullptr, *pred = nullptr, *target = nullptr;
        uint32_t *infer_list = nullptr, *train_list = nullptr;
        uint8_t *qflag = nullptr;
        uint32_t *t_aqueue[2] = {};
        float4 *t_ajob[2] = {};
        // a single-view frame's training candidates for the query bounce, and
        // the training bounces' ray queues (the branch forks before the main
        // paths' query bounce has read its own queue)
        uint32_t *tq = nullptr;
        uint32_t *t_queue[2] = {};
        uint4 *t_hitbuf = nullptr;
        float *t_hitval = nullptr;
        uint2 *t_jmeta = nullptr;
    };
    CacheSet cs[SETS];
    int last_cache_set = -1;              // the set of the last cache frame (its targets)
    vrg_tuning tune{};                    // launch configuration (0 fields = defaults)
    // per reservoir-ring slot: a 3-D tensor map (4*W floats x H rows x 5
    // planes) for the TMA-staged spatial pass of a single view
    CUtensorMap res_map[8];
    bool res_map_ok = false;
};

}  // namespace vrg
