// C ABI of the path tracer: context, materials, chunk uploads, scene,
// renderer orchestration (the frame graph of Renderer::render,
// interactive_rendering.rs:952-1669, as one CUDA stream), debug readback and
// the standalone batched SAH builds.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "vrg_frame.cuh"
#include "vrg_internal.h"

namespace vrg {

vrg_status upload_frames(cudaStream_t s);
vrg_status launch_trace_shade(cudaStream_t s, const FrameArgs &a, uint32_t b, cudaEvent_t ev_trace, uint32_t max_rays);
vrg_status launch_light_pdf(cudaStream_t s, const FrameArgs &a, uint32_t b, uint32_t max_rays);
vrg_status launch_resolve(cudaStream_t s, const FrameArgs &a);
vrg_status launch_spatial(cudaStream_t s, const FrameArgs &a, const CUtensorMap *res_map);
vrg_status launch_train_targets(cudaStream_t s, const FrameArgs &a);
void bounce_occupancy(bool batch, int occ[3], int *sms);

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

DevBuf::~DevBuf() {
    if (ptr) cudaFreeAsync(ptr, stream);
}

vrg_status dev_alloc(cudaStream_t s, size_t bytes, DevBufPtr &out) {
    auto b = std::make_shared<DevBuf>();
    b->stream = s;
    b->bytes = bytes;
    cudaError_t e = cudaMallocAsync(&b->ptr, bytes ? bytes : 16, s);
    if (e != cudaSuccess) {
        cudaGetLastError();  // a failed allocation is reported here, not by the next launch check
        b->ptr = nullptr;
        set_error("cudaMallocAsync(%zu) failed: %s", bytes, cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? VRG_ERR_OUT_OF_MEMORY : VRG_ERR_CUDA;
    }
    out = b;
    return VRG_OK;
}

static void release_object(Object *o) {
    if (o && --o->refs == 0) delete o;
}

}  // namespace vrg

using namespace vrg;

struct vrg_context : Context {};

namespace vrg {

void ctx_retain(Context *c) { c->refs++; }

void ctx_release(Context *c) {
    if (--c->refs) return;
    for (Object *o : c->pending) release_object(o);
    c->pending.clear();
    c->d_mats.reset();
    c->d_atlas.reset();
    cudaStreamSynchronize(c->stream);
    cudaStreamDestroy(c->stream);
    delete static_cast<vrg_context *>(c);
}

Object::~Object() {
    batch.reset();  // stream-ordered free on the context's stream, before the context may go
    if (ctx) ctx_release(ctx);
}

}  // namespace vrg
struct vrg_object : Object {};
struct vrg_scene : Scene {};
struct vrg_renderer : Renderer {};

extern "C" {

VRG_API const char *vrg_status_string(vrg_status s) {
    switch (s) {
    case VRG_OK: return "ok";
    case VRG_ERR_INVALID_ARGUMENT: return "invalid argument";
    case VRG_ERR_NOT_FOUND: return "not found";
    case VRG_ERR_OUT_OF_MEMORY: return "out of memory";
    case VRG_ERR_CUDA: return "cuda error";
    case VRG_ERR_UNSUPPORTED: return "unsupported";
    case VRG_ERR_OVERFLOW: return "device structure overflow";
    case VRG_ERR_STATE: return "invalid state";
    case VRG_ERR_NO_DEVICE: return "no cuda device";
    default: return "unknown status";
    }
}

VRG_API const char *vrg_last_error(void) { return g_err; }

VRG_API vrg_status vrg_context_create(const vrg_context_desc *desc, vrg_context **out) {
    if (!out) return VRG_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        set_error("no CUDA device visible");
        return VRG_ERR_NO_DEVICE;
    }
    int dev = desc ? desc->device : 0;
    if (dev < 0 || dev >= n) {
        set_error("device %d out of range (%d devices)", dev, n);
        return VRG_ERR_INVALID_ARGUMENT;
    }
    VRG_CUDA_TRY(cudaSetDevice(dev));
    vrg_context *c = new vrg_context();
    c->device = dev;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        set_error("cudaStreamCreate: %s", cudaGetErrorString(e));
        return VRG_ERR_CUDA;
    }
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, dev);
    vrg_status st = upload_frames(c->stream);
    if (st != VRG_OK) {
        cudaStreamDestroy(c->stream);
        delete c;
        return st;
    }
    *out = c;
    return VRG_OK;
}

VRG_API vrg_status vrg_context_stream(vrg_context *ctx, void **stream) {
    if (!ctx || !stream) return VRG_ERR_INVALID_ARGUMENT;
    *stream = (void *)ctx->stream;
    return VRG_OK;
}

VRG_API vrg_status vrg_context_synchronize(vrg_context *ctx) {
    if (!ctx) return VRG_ERR_INVALID_ARGUMENT;
    VRG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return VRG_OK;
}

VRG_API vrg_status vrg_context_destroy(vrg_context *ctx) {
    if (!ctx) return VRG_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        for (Object *o : ctx->pending) release_object(o);  // the pending list's references
        ctx->pending.clear();
    }
    ctx_release(ctx);  // the handle's reference; children still alive keep the context
    return VRG_OK;
}

VRG_API vrg_status vrg_material_table_set(vrg_context *ctx, const vrg_material *mats, uint32_t n) {
    if (!ctx || !mats || n == 0 || n % 6 || n / 6 > 255) {
        set_error("material table needs a multiple of 6 entries, at most 6*255");
        return VRG_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (!ctx->pending.empty()) {
        set_error("material table changed with uploads pending");
        return VRG_ERR_STATE;
    }
    ctx->mats.assign(mats, mats + n);
    ctx->n_types = n / 6;
    ctx->d_atlas.reset();  // an atlas belongs to one table: set it again after a new table
    ctx->atlas_w = ctx->atlas_h = 0;
    ctx->d_srgb = nullptr;
    DevBufPtr b;
    VRG_TRY(dev_alloc(ctx->stream, n * sizeof(vrg_material), b));
    VRG_CUDA_TRY(cudaMemcpyAsync(b->ptr, mats, n * sizeof(vrg_material), cudaMemcpyHostToDevice, ctx->stream));
    VRG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    ctx->d_mats = b;
    return VRG_OK;
}

VRG_API vrg_status vrg_texture_atlas_set(vrg_context *ctx, const uint8_t *rgba8, uint32_t n_slots, uint32_t width,
                                         uint32_t height) {
    if (!ctx) return VRG_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (!ctx->pending.empty()) {
        set_error("texture atlas changed with uploads pending");
        return VRG_ERR_STATE;
    }
    if (!rgba8) {
        ctx->d_atlas.reset();
        ctx->atlas_w = ctx->atlas_h = 0;
        ctx->d_srgb = nullptr;
        return VRG_OK;
    }
    if (ctx->mats.empty() || n_slots != ctx->mats.size() || width == 0 || height == 0 || width > 4096 ||
        height > 4096) {
        set_error("atlas needs one slot per material-table entry (%zu) and 1..4096 texels a side", ctx->mats.size());
        return VRG_ERR_INVALID_ARGUMENT;
    }
    const size_t map = (size_t)width * height;
    // get_texture_luminances (utils.rs:223-235): mean of r8+g8+b8 over the emissivity map
    std::vector<vrg_material> mats = ctx->mats;
    for (uint32_t t = 0; t < n_slots; t++) {
        const uint8_t *e = rgba8 + ((size_t)t * 3 + 1) * map * 4;
        float L = 0.0f;
        for (size_t i = 0; i < map; i++) L += ((float)e[4 * i] + (float)e[4 * i + 1]) + (float)e[4 * i + 2];
        mats[t].luminance = L / (float)(width * height);
    }
    // sRGB decode of the R8G8B8A8_SRGB maps (the EOTF, evaluated in double)
    float lut[256];
    for (int i = 0; i < 256; i++) {
        const double c = (double)i / 255.0;
        lut[i] = (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
    }
    const size_t atlas_bytes = (size_t)n_slots * 3 * map * 4, lut_off = (atlas_bytes + 255) & ~(size_t)255;
    DevBufPtr ab, mb;
    VRG_TRY(dev_alloc(ctx->stream, lut_off + sizeof(lut), ab));
    VRG_TRY(dev_alloc(ctx->stream, mats.size() * sizeof(vrg_material), mb));
    VRG_CUDA_TRY(cudaMemcpyAsync(ab->ptr, rgba8, atlas_bytes, cudaMemcpyHostToDevice, ctx->stream));
    VRG_CUDA_TRY(cudaMemcpyAsync((uint8_t *)ab->ptr + lut_off, lut, sizeof(lut), cudaMemcpyHostToDevice, ctx->stream));
    VRG_CUDA_TRY(cudaMemcpyAsync(mb->ptr, mats.data(), mats.size() * sizeof(vrg_material), cudaMemcpyHostToDevice,
                                 ctx->stream));
    VRG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    ctx->mats = mats;
    ctx->d_mats = mb;
    ctx->d_atlas = ab;
    ctx->atlas_w = width;
    ctx->atlas_h = height;
    ctx->d_srgb = (const float *)((const uint8_t *)ab->ptr + lut_off);
    return VRG_OK;
}

VRG_API vrg_status vrg_upload_chunk(vrg_context *ctx, const uint8_t *blocks, const uint8_t *const neighbours[6],
                                    vrg_object **out) {
    if (!ctx || !blocks || !out) return VRG_ERR_INVALID_ARGUMENT;
    if (ctx->n_types == 0) {
        set_error("material table not set");
        return VRG_ERR_STATE;
    }
    const uint32_t air = ctx->n_types;
    for (uint32_t i = 0; i < VRG_CHUNK_BLOCKS; i++)
        if (blocks[i] > air) {
            set_error("block id %u at %u exceeds air id %u", blocks[i], i, air);
            return VRG_ERR_INVALID_ARGUMENT;
        }
    vrg_object *o = new vrg_object();
    o->ctx = ctx;
    ctx_retain(ctx);
    o->blocks.assign(blocks, blocks + VRG_CHUNK_BLOCKS);
    o->slabs.assign(6 * 1024, (uint8_t)air);
    for (int f = 0; f < 6; f++) {
        const uint8_t *nb = neighbours ? neighbours[f] : nullptr;
        if (!nb) continue;
        o->slab_present |= 1u << f;
        uint8_t *s = o->slabs.data() + f * 1024;
        for (int a = 0; a < 32; a++)
            for (int b = 0; b < 32; b++) {
                uint32_t idx;
                switch (f) {  // the neighbour's boundary plane facing this chunk
                case 0: idx = 31 * 1024 + a * 32 + b; break;  // left: x=31, (y,z)
                case 1: idx = 0 * 1024 + a * 32 + b; break;   // right: x=0
                case 2: idx = a * 1024 + 31 * 32 + b; break;  // down: y=31, (x,z)
                case 3: idx = a * 1024 + 0 * 32 + b; break;   // up: y=0
                case 4: idx = a * 1024 + b * 32 + 31; break;  // back: z=31, (x,y)
                default: idx = a * 1024 + b * 32 + 0; break;  // front: z=0
                }
                uint8_t v = nb[idx];
                if (v > air) {
                    delete o;
                    set_error("neighbour %d block id %u exceeds air id %u", f, v, air);
                    return VRG_ERR_INVALID_ARGUMENT;
                }
                s[a * 32 + b] = v;
            }
    }
    o->refs = 2;  // caller + pending list
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        ctx->pending.push_back(o);
    }
    *out = o;
    return VRG_OK;
}

VRG_API vrg_status vrg_upload_mesh(vrg_context *ctx, const vrg_vertex3d *v, uint64_t nverts, vrg_object **out) {
    if (!ctx || !out || (nverts && !v)) return VRG_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (ctx->n_types == 0) {
        set_error("material table not set");
        return VRG_ERR_STATE;
    }
    vrg_object *o = new vrg_object();
    o->ctx = ctx;
    ctx_retain(ctx);
    vrg_status st;
    {  // one upload at a time on the context's stream (the builder synchronizes it)
        std::lock_guard<std::mutex> lk(ctx->mu);
        st = mesh_upload(ctx, v, nverts, o);
    }
    if (st != VRG_OK) {
        release_object(o);
        return st;
    }
    *out = o;
    return VRG_OK;
}

VRG_API vrg_status vrg_flush_uploads(vrg_context *ctx) {
    if (!ctx) return VRG_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(ctx->mu);
    std::vector<Object *> pend;
    pend.swap(ctx->pending);
    vrg_status st = extract_and_build(ctx, pend);
    if (st != VRG_OK) {
        ctx->pending.insert(ctx->pending.end(), pend.begin(), pend.end());
        return st;
    }
    for (Object *o : pend) release_object(o);
    return VRG_OK;
}

VRG_API vrg_status vrg_object_release(vrg_object *obj) {
    if (!obj) return VRG_ERR_INVALID_ARGUMENT;
    release_object(obj);
    return VRG_OK;
}

static vrg_status ensure_flushed(Object *o) {
    if (o->flushed) return VRG_OK;
    return vrg_flush_uploads(static_cast<vrg_context *>(o->ctx));
}

VRG_API vrg_status vrg_object_info(vrg_object *obj, uint32_t *n_faces, uint32_t *n_triangles,
                                   uint32_t *n_light_triangles, uint32_t *n_surface_blocks) {
    if (!obj) return VRG_ERR_INVALID_ARGUMENT;
    VRG_TRY(ensure_flushed(obj));
    if (n_faces) *n_faces = obj->sum.n_faces;
    if (n_triangles) *n_triangles = obj->sum.n_tris;
    if (n_light_triangles) *n_light_triangles = obj->sum.n_light;
    if (n_surface_blocks) *n_surface_blocks = obj->sum.n_geo;
    return VRG_OK;
}

VRG_API vrg_status vrg_object_read_bvh(vrg_object *obj, uint32_t which, vrg_bvh_node *nodes, uint32_t cap_nodes,
                                       uint32_t *n_nodes, uint32_t *prim_order, uint32_t cap_prims,
                                       uint32_t *n_prims) {
    if (!obj || which > 1) return VRG_ERR_INVALID_ARGUMENT;
    VRG_TRY(ensure_flushed(obj));
    uint32_t np = which ? obj->sum.n_geo : obj->sum.n_light;
    uint32_t nn = np ? 2 * np - 1 : 0;
    if (n_nodes) *n_nodes = nn;
    if (n_prims) *n_prims = np;
    if (np == 0) return VRG_OK;
    cudaStream_t s = obj->ctx->stream;
    if (nodes) {
        if (cap_nodes < nn) return VRG_ERR_INVALID_ARGUMENT;
        VRG_CUDA_TRY(cudaMemcpyAsync(nodes, which ? obj->geo_nodes : obj->light_nodes, nn * sizeof(vrg_bvh_node),
                                     cudaMemcpyDeviceToHost, s));
    }
    if (prim_order) {
        if (cap_prims < np) return VRG_ERR_INVALID_ARGUMENT;
        VRG_CUDA_TRY(cudaMemcpyAsync(prim_order, which ? obj->geo_perm : obj->light_perm, np * 4,
                                     cudaMemcpyDeviceToHost, s));
    }
    VRG_CUDA_TRY(cudaStreamSynchronize(s));
    return VRG_OK;
}

VRG_API vrg_status vrg_scene_create(vrg_context *ctx, vrg_scene **out) {
    if (!ctx || !out) return VRG_ERR_INVALID_ARGUMENT;
    vrg_scene *s = new vrg_scene();
    s->ctx = ctx;
    ctx_retain(ctx);
    *out = s;
    return VRG_OK;
}

VRG_API vrg_status vrg_scene_destroy(vrg_scene *scene) {
    if (!scene) return VRG_ERR_INVALID_ARGUMENT;
    cudaStreamSynchronize(scene->ctx->stream);
    for (auto &kv : scene->objects) release_object(kv.second.obj);
    for (Object *o : scene->retired) release_object(o);
    Context *c = scene->ctx;
    delete scene;
    ctx_release(c);
    return VRG_OK;
}

// The instance transform of add_object / update_object (scene.rs:150,205),
// as a row-major [R|t].  A chunk takes a translation by whole blocks (its
// voxel records hold integer world coordinates); a mesh takes a rotation-like
// R (entries within +-1, as an isometry's) and |t| <= 4096, which keeps the
// rounding of its transformed vertices inside the traversal boxes' margin.
static vrg_status parse_xform(const Object *obj, const float *x, SceneEntry &e) {
    static const float I12[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    const float *m = x ? x : I12;
    bool tonly = true, ok = true;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 4; c++) {
            const float v = m[4 * r + c];
            if (c < 3) {
                tonly = tonly && v == (r == c ? 1.0f : 0.0f);
                ok = ok && fabsf(v) <= 1.0f;
            } else {
                ok = ok && fabsf(v) <= (obj->mesh ? 4096.0f : 16384.0f);
            }
        }
    if (!obj->mesh) {
        if (!tonly) {
            set_error("a chunk takes a translation only (chunks are translated, chunk_manager.rs:234-248)");
            return VRG_ERR_UNSUPPORTED;
        }
        for (int r = 0; r < 3; r++)
            if (m[4 * r + 3] != floorf(m[4 * r + 3]) || !ok) {
                set_error("a chunk translation must be integral and within +-16384");
                return VRG_ERR_UNSUPPORTED;
            }
    } else if (!ok) {
        set_error("a mesh transform needs finite R entries within +-1 and |t| <= 4096");
        return VRG_ERR_UNSUPPORTED;
    }
    memcpy(e.m, m, sizeof(e.m));
    e.off[0] = m[3];
    e.off[1] = m[7];
    e.off[2] = m[11];
    e.tonly = tonly;
    return VRG_OK;
}

VRG_API vrg_status vrg_scene_add(vrg_scene *scene, uint64_t key, vrg_object *obj, const float xform3x4[12]) {
    if (!scene || !obj) return VRG_ERR_INVALID_ARGUMENT;
    SceneEntry e{};
    e.obj = obj;
    VRG_TRY(parse_xform(obj, xform3x4, e));
    obj->refs++;
    auto it = scene->objects.find(key);
    if (it != scene->objects.end()) scene->retired.push_back(it->second.obj);
    scene->objects[key] = e;
    scene->dirty = true;
    return VRG_OK;
}

VRG_API vrg_status vrg_scene_update(vrg_scene *scene, uint64_t key, const float xform3x4[12]) {
    if (!scene) return VRG_ERR_INVALID_ARGUMENT;
    auto it = scene->objects.find(key);
    if (it == scene->objects.end()) {
        set_error("object with key %llu does not exist", (unsigned long long)key);
        return VRG_ERR_NOT_FOUND;  // reference panics (scene.rs:214)
    }
    SceneEntry e = it->second;
    VRG_TRY(parse_xform(e.obj, xform3x4, e));
    it->second = e;
    scene->dirty = true;
    return VRG_OK;
}

VRG_API vrg_status vrg_scene_remove(vrg_scene *scene, uint64_t key) {
    if (!scene) return VRG_ERR_INVALID_ARGUMENT;
    auto it = scene->objects.find(key);
    if (it == scene->objects.end()) return VRG_OK;  // reference: removing a missing key is a no-op
    scene->retired.push_back(it->second.obj);
    scene->objects.erase(it);
    scene->dirty = true;
    return VRG_OK;
}

VRG_API vrg_status vrg_scene_commit(vrg_scene *scene) {
    if (!scene) return VRG_ERR_INVALID_ARGUMENT;
    return scene_commit(scene);
}

VRG_API vrg_status vrg_scene_commit_many(vrg_scene *const *scenes, uint32_t n) {
    if (!scenes && n) return VRG_ERR_INVALID_ARGUMENT;
    std::vector<Scene *> scs(n);
    for (uint32_t i = 0; i < n; i++) {
        if (!scenes[i]) return VRG_ERR_INVALID_ARGUMENT;
        scs[i] = scenes[i];
    }
    return scene_commit_many(scs.data(), n);
}

VRG_API vrg_status vrg_scene_read_tl(vrg_scene *scene, uint32_t which, vrg_bvh_node *nodes, uint32_t cap,
                                     uint32_t *n_nodes) {
    if (!scene || which > 1) return VRG_ERR_INVALID_ARGUMENT;
    if (scene->dirty) {
        set_error("scene not committed");
        return VRG_ERR_STATE;
    }
    const auto &v = which ? scene->h_geo_tl : scene->h_light_tl;
    if (n_nodes) *n_nodes = (uint32_t)v.size();
    if (nodes) {
        if (cap < v.size()) return VRG_ERR_INVALID_ARGUMENT;
        memcpy(nodes, v.data(), v.size() * sizeof(vrg_bvh_node));
    }
    return VRG_OK;
}

// ---- renderer -------------------------------------------------------------

static void drop_graphs(vrg_renderer *r) {
    for (auto &g : r->graphs) cudaGraphExecDestroy(g.exec);
    r->graphs.clear();
}

static vrg_status renderer_alloc(vrg_renderer *r) {
    const size_t P = (size_t)r->P;
    const uint32_t nb = r->nb_max;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    size_t o = 0;
    // the arrays of a frame's bounces, one set per frame in flight
    struct SetOff {
        size_t ro, rd, q0, q1, cnt, aq0, aq1, aj0, aj1, hit, hb, hv, jm, nl, rec, xv, nv, xs, ns;
    } so[Renderer::SETS];
    const int sets = (int)r->n_sets;
    for (int k = 0; k < sets; k++) {
        SetOff &q = so[k];
        q.ro = o; o += al(P * 16);
        q.rd = o; o += al(P * 16);
        q.q0 = o; o += al(P * 4);
        q.q1 = o; o += al(P * 4);
        q.cnt = o; o += al(CNT_WORDS * 4);
        q.aq0 = o; o += al(P * 4);
        q.aq1 = o; o += al(P * 4);
        q.aj0 = o; o += al(P * 32);
        q.aj1 = o; o += al(P * 32);
        q.hit = o; o += al(P * 16);
        q.hb = o; o += al(P * 2 * 32);
        q.hv = o; o += al(P * 2 * 4);
        q.jm = o; o += al(P * 8);
        q.nl = o; o += al(P);
        q.rec = o; o += al(P * 32 * nb);
        q.xv = o; o += al(P * 16);
        q.nv = o; o += al(P * 16);
        q.xs = o; o += al(P * 16);
        q.ns = o; o += al(P * 16);
    }
    size_t o_pl = o; o += al(P * 16);
    size_t o_sp = o; o += al(P * 80);
    size_t o_ft = o; o += al(P * 16);
    size_t o_bg = o; o += al(P * 4);
    size_t o_rad = o; o += al(P * 12);
    size_t o_acc = o; o += al(P * 24);
    DevBufPtr b;
    VRG_TRY(dev_alloc(r->ctx->stream, o, b));
    uint8_t *B = (uint8_t *)b->ptr;
    for (int k = 0; k < Renderer::SETS; k++) {
        const SetOff &q = so[k < sets ? k : 0];
        Renderer::FrameSet &F = r->fs[k];
        F.ray_o = (float4 *)(B + q.ro);
        F.ray_d = (float4 *)(B + q.rd);
        F.queue[0] = (uint32_t *)(B + q.q0);
        F.queue[1] = (uint32_t *)(B + q.q1);
        F.counters = (uint32_t *)(B + q.cnt);
        F.aqueue[0] = (uint32_t *)(B + q.aq0);
        F.aqueue[1] = (uint32_t *)(B + q.aq1);
        F.ajob[0] = (float4 *)(B + q.aj0);
        F.ajob[1] = (float4 *)(B + q.aj1);
        F.hits = (int4 *)(B + q.hit);
        F.hitbuf = (uint4 *)(B + q.hb);
        F.hitval = (float *)(B + q.hv);
        F.jmeta = (uint2 *)(B + q.jm);
        F.nlive = B + q.nl;
        F.rec = (float4 *)(B + q.rec);
        F.xv = (float4 *)(B + q.xv);
        F.nv = (float4 *)(B + q.nv);
        F.xs = (float4 *)(B + q.xs);
        F.ns = (float4 *)(B + q.ns);
    }
    r->plain = (float4 *)(B + o_pl);
    r->spatial = (float4 *)(B + o_sp);
    r->final_t = (float4 *)(B + o_ft);
    r->bgra = B + o_bg;
    r->radiance = (float *)(B + o_rad);
    r->accum = (double *)(B + o_acc);
    VRG_CUDA_TRY(cudaMemsetAsync(B, 0, o, r->ctx->stream));
    // frames in flight start their bounces after this clear
    for (cudaEvent_t e : r->ev_done)
        if (e) VRG_CUDA_TRY(cudaEventRecord(e, r->ctx->stream));
    r->out_buf.reset();
    r->radiance_out = nullptr;
    if (r->scale > 1) {
        DevBufPtr ob;
        VRG_TRY(dev_alloc(r->ctx->stream, (size_t)r->out_w * r->out_h * 12, ob));
        r->out_buf = ob;
        r->radiance_out = (float *)ob->ptr;
    }
    drop_graphs(r);
    r->buf = b;
    r->res = nullptr;
    r->res_buf.reset();
    r->ring_slots = 0;
    r->frame = 0;
    r->accum_n = 0;
    r->cap.reset();
    r->cache_buf.reset();
    r->cache_cap = 0;
    for (auto &q : r->cs) q = Renderer::CacheSet{};
    r->last_cache_set = -1;
    r->captured = false;
    return VRG_OK;
}

static vrg_status renderer_events(vrg_renderer *r) {
    // the training branch of a cache frame is the frame's critical path: it
    // runs on a higher-priority stream, so its few blocks are placed first
    int lo_prio = 0, hi_prio = 0;
    VRG_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio));
    VRG_CUDA_TRY(cudaStreamCreateWithPriority(&r->aux, cudaStreamNonBlocking, hi_prio));
    VRG_CUDA_TRY(cudaStreamCreateWithPriority(&r->aux_lp, cudaStreamNonBlocking, hi_prio));
    for (int k = 0; k < Renderer::SETS; k++) {
        VRG_CUDA_TRY(cudaStreamCreateWithFlags(&r->bs[k], cudaStreamNonBlocking));
        VRG_CUDA_TRY(cudaStreamCreateWithFlags(&r->lps[k], cudaStreamNonBlocking));
        for (auto &e : r->ev_shaded[k]) VRG_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        for (auto &e : r->ev_lpdone[k]) VRG_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        VRG_CUDA_TRY(cudaEventCreateWithFlags(&r->ev_bounced[k], cudaEventDisableTiming));
        VRG_CUDA_TRY(cudaEventCreateWithFlags(&r->ev_done[k], cudaEventDisableTiming));
        VRG_CUDA_TRY(cudaEventRecord(r->ev_done[k], r->ctx->stream));  // after the buffers' clear
    }
    for (auto &row : r->ev_lp)
        for (auto &e : row) VRG_CUDA_TRY(cudaEventCreate(&e));
    VRG_CUDA_TRY(cudaEventCreateWithFlags(&r->ev_fork, cudaEventDisableTiming));
    VRG_CUDA_TRY(cudaEventCreateWithFlags(&r->ev_join, cudaEventDisableTiming));
    VRG_CUDA_TRY(cudaEventCreateWithFlags(&r->ev_start, cudaEventDisableTiming));
    VRG_CUDA_TRY(cudaEventCreateWithFlags(&r->ev_updated, cudaEventDisableTiming));
    for (auto &e : r->ev) VRG_CUDA_TRY(cudaEventCreate(&e));
    for (auto &row : r->ev_k)
        for (auto &e : row) VRG_CUDA_TRY(cudaEventCreate(&e));
    for (auto &e : r->ev_fence) VRG_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    // the kernels' occupancy grids, queried once here (never inside a stream capture)
    int occ[3], sms = 1;
    bounce_occupancy(false, occ, &sms);
    return VRG_OK;
}

VRG_API vrg_status vrg_renderer_create(vrg_context *ctx, uint32_t width, uint32_t height, uint32_t max_bounces,
                                       vrg_renderer **out) {
    if (!ctx || !out || width == 0 || height == 0 || max_bounces == 0 || max_bounces > MAX_BOUNCES)
        return VRG_ERR_INVALID_ARGUMENT;
    if ((uint64_t)width * height >= (1ull << 31)) return VRG_ERR_UNSUPPORTED;
    vrg_renderer *r = new vrg_renderer();
    r->ctx = ctx;
    ctx_retain(ctx);
    r->W = r->out_w = width;
    r->H = r->out_h = height;
    r->P = (uint64_t)width * height;
    r->nb_max = max_bounces;
    vrg_status st = renderer_alloc(r);
    if (st == VRG_OK) st = renderer_events(r);
    if (st != VRG_OK) {
        vrg_renderer_destroy(r);
        return st;
    }
    *out = r;
    return VRG_OK;
}

VRG_API vrg_status vrg_renderer_create_batched(vrg_context *ctx, uint32_t n_views, const uint32_t *widths,
                                               const uint32_t *heights, uint32_t max_bounces,
                                               vrg_renderer **out) {
    if (!ctx || !out || !widths || !heights || n_views == 0 || n_views > 65535 || max_bounces == 0 ||
        max_bounces > MAX_BOUNCES)
        return VRG_ERR_INVALID_ARGUMENT;
    uint64_t P = 0;
    std::vector<uint64_t> off(n_views);
    for (uint32_t v = 0; v < n_views; v++) {
        if (widths[v] == 0 || heights[v] == 0) return VRG_ERR_INVALID_ARGUMENT;
        off[v] = P;
        P += (uint64_t)widths[v] * heights[v];
    }
    if (P >= (1ull << 31)) {
        set_error("a batch holds fewer than 2^31 pixels (asked for %llu)", (unsigned long long)P);
        return VRG_ERR_UNSUPPORTED;
    }
    vrg_renderer *r = new vrg_renderer();
    r->ctx = ctx;
    ctx_retain(ctx);
    r->W = r->out_w = widths[0];
    r->H = r->out_h = heights[0];
    r->P = P;
    r->nb_max = max_bounces;
    r->n_views = n_views;
    r->vw.assign(widths, widths + n_views);
    r->vh.assign(heights, heights + n_views);
    r->voff = off;
    r->n_sets = 2;  // two frames' bounces in flight (a set is large: all views' pixels)
    auto fail = [&](vrg_status st) {
        vrg_renderer_destroy(r);
        return st;
    };
    vrg_status st = renderer_alloc(r);
    if (st == VRG_OK) st = renderer_events(r);
    if (st != VRG_OK) return fail(st);
    // view table + pixel-group lookup (the view of each group's first pixel)
    const size_t n_groups = (size_t)((P + (1u << VIEW_SHIFT) - 1) >> VIEW_SHIFT);
    const size_t view_tab = ((size_t)n_views * sizeof(ViewDev) + 255) & ~(size_t)255;
    const size_t tab_off = view_tab * r->n_sets;
    DevBufPtr vb;
    st = dev_alloc(ctx->stream, tab_off + n_groups * 2, vb);
    if (st != VRG_OK) return fail(st);
    r->view_buf = vb;
    for (uint32_t k = 0; k < r->n_sets; k++) r->d_views[k] = (ViewDev *)((uint8_t *)vb->ptr + k * view_tab);
    r->d_vtab = (uint16_t *)((uint8_t *)vb->ptr + tab_off);
    std::vector<uint16_t> vtab(n_groups);
    uint32_t v = 0;
    for (size_t g = 0; g < n_groups; g++) {
        const uint64_t p = (uint64_t)g << VIEW_SHIFT;
        while (v + 1 < n_views && p >= off[v + 1]) v++;
        vtab[g] = (uint16_t)v;
    }
    if (cudaMemcpyAsync(r->d_vtab, vtab.data(), n_groups * 2, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess ||
        cudaHostAlloc((void **)&r->h_views, 2 * (size_t)n_views * sizeof(ViewDev), cudaHostAllocDefault) !=
            cudaSuccess) {
        set_error("batched renderer set-up failed");
        return fail(VRG_ERR_CUDA);
    }
    memset(r->h_views, 0, 2 * (size_t)n_views * sizeof(ViewDev));
    for (auto &e : r->ev_stage)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return fail(VRG_ERR_CUDA);
    *out = r;
    return VRG_OK;
}

VRG_API vrg_status vrg_renderer_view_offset(vrg_renderer *r, uint32_t view, uint64_t *pixel_offset) {
    if (!r || !pixel_offset) return VRG_ERR_INVALID_ARGUMENT;
    if (r->n_views == 0) {
        if (view != 0) return VRG_ERR_INVALID_ARGUMENT;
        *pixel_offset = 0;
        return VRG_OK;
    }
    if (view >= r->n_views) return VRG_ERR_INVALID_ARGUMENT;
    *pixel_offset = r->voff[view];
    return VRG_OK;
}

VRG_API vrg_status vrg_renderer_destroy(vrg_renderer *r) {
    if (!r) return VRG_ERR_INVALID_ARGUMENT;
    cudaStreamSynchronize(r->ctx->stream);
    drop_graphs(r);
    for (auto &e : r->ev)
        if (e) cudaEventDestroy(e);
    for (auto &row : r->ev_k)
        for (auto &e : row)
            if (e) cudaEventDestroy(e);
    for (auto &e : r->ev_stage)
        if (e) cudaEventDestroy(e);
    for (int k = 0; k < Renderer::SETS; k++) {
        for (cudaStream_t q : {r->bs[k], r->lps[k]})
            if (q) {
                cudaStreamSynchronize(q);
                cudaStreamDestroy(q);
            }
        for (auto &e : r->ev_shaded[k])
            if (e) cudaEventDestroy(e);
        for (auto &e : r->ev_lpdone[k])
            if (e) cudaEventDestroy(e);
        if (r->ev_bounced[k]) cudaEventDestroy(r->ev_bounced[k]);
        if (r->ev_done[k]) cudaEventDestroy(r->ev_done[k]);
    }
    for (auto &row : r->ev_lp)
        for (auto &e : row)
            if (e) cudaEventDestroy(e);
    for (auto &e : r->ev_fence)
        if (e) cudaEventDestroy(e);
    if (r->ev_fork) cudaEventDestroy(r->ev_fork);
    if (r->ev_join) cudaEventDestroy(r->ev_join);
    if (r->ev_start) cudaEventDestroy(r->ev_start);
    if (r->ev_updated) cudaEventDestroy(r->ev_updated);
    for (cudaStream_t q : {r->aux, r->aux_lp})
        if (q) {
            cudaStreamSynchronize(q);
            cudaStreamDestroy(q);
        }
    if (r->h_pinned) cudaFreeHost(r->h_pinned);
    if (r->h_views) cudaFreeHost(r->h_views);
    r->res_buf.reset();
    Context *c = r->ctx;
    delete r;  // its buffers are freed on the context's stream, before the context may go
    ctx_release(c);
    return VRG_OK;
}

VRG_API vrg_status vrg_renderer_resize(vrg_renderer *r, uint32_t width, uint32_t height) {
    if (!r || width == 0 || height == 0) return VRG_ERR_INVALID_ARGUMENT;
    if (r->n_views) {
        set_error("a batched renderer has fixed view extents");
        return VRG_ERR_STATE;
    }
    if ((uint64_t)width * height * r->scale * r->scale >= (1ull << 31)) return VRG_ERR_UNSUPPORTED;
    cudaStreamSynchronize(r->ctx->stream);
    r->out_w = width;
    r->out_h = height;
    r->W = width * r->scale;
    r->H = height * r->scale;
    r->P = (uint64_t)r->W * r->H;
    return renderer_alloc(r);
}

VRG_API vrg_status vrg_renderer_set_scale(vrg_renderer *r, uint32_t scale) {
    if (!r || scale == 0 || scale > 8) return VRG_ERR_INVALID_ARGUMENT;
    if (r->n_views) {
        set_error("a batched renderer renders at scale 1");
        return VRG_ERR_STATE;
    }
    if (scale == r->scale) return VRG_OK;
    if ((uint64_t)r->out_w * r->out_h * scale * scale >= (1ull << 31)) return VRG_ERR_UNSUPPORTED;
    cudaStreamSynchronize(r->ctx->stream);
    r->scale = scale;
    r->W = r->out_w * scale;
    r->H = r->out_h * scale;
    r->P = (uint64_t)r->W * r->H;
    return renderer_alloc(r);
}

VRG_API vrg_status vrg_renderer_frame_index(vrg_renderer *r, uint32_t *frame_index) {
    if (!r || !frame_index) return VRG_ERR_INVALID_ARGUMENT;
    *frame_index = r->frame;
    return VRG_OK;
}

VRG_API vrg_status vrg_renderer_reset_accumulation(vrg_renderer *r) {
    if (!r) return VRG_ERR_INVALID_ARGUMENT;
    VRG_CUDA_TRY(cudaMemsetAsync(r->accum, 0, (size_t)r->P * 24, r->ctx->stream));
    r->accum_n = 0;
    return VRG_OK;
}

VRG_API vrg_status vrg_renderer_read_accumulation(vrg_renderer *r, float *rgb, uint32_t *n_frames) {
    if (!r) return VRG_ERR_INVALID_ARGUMENT;
    if (n_frames) *n_frames = r->accum_n;
    if (!rgb) return VRG_OK;
    const size_t P = (size_t)r->P;
    std::vector<double> h(P * 3);
    VRG_CUDA_TRY(cudaMemcpyAsync(h.data(), r->accum, P * 24, cudaMemcpyDeviceToHost, r->ctx->stream));
    VRG_CUDA_TRY(cudaStreamSynchronize(r->ctx->stream));
    double inv = r->accum_n ? 1.0 / (double)r->accum_n : 0.0;
    for (size_t i = 0; i < P * 3; i++) rgb[i] = (float)(h[i] * inv);
    return VRG_OK;
}

static vrg_status ensure_capture(vrg_renderer *r) {
    if (r->cap) return VRG_OK;
    const size_t P = (size_t)r->P, nb = r->nb_max;
    size_t floats = (nb + 1) * P * 3 * 2 + nb * P * 3 * 4 + nb * P * 4 + nb * P * 4;
    DevBufPtr b;
    VRG_TRY(dev_alloc(r->ctx->stream, floats * 4, b));
    float *f = (float *)b->ptr;
    r->c_origin = f; f += (nb + 1) * P * 3;
    r->c_dir = f; f += (nb + 1) * P * 3;
    r->c_normal = f; f += nb * P * 3;
    r->c_emis = f; f += nb * P * 3;
    r->c_refl = f; f += nb * P * 3;
    r->c_L = f; f += nb * P * 3;
    r->c_mis = f; f += nb * P;
    r->c_pdf = f; f += nb * P;
    r->c_nee = f; f += nb * P;
    r->c_q = f; f += nb * P;
    r->c_hit = (uint32_t *)f;
    VRG_CUDA_TRY(cudaMemsetAsync(b->ptr, 0, floats * 4, r->ctx->stream));
    r->cap = b;
    return VRG_OK;
}

// cuTensorMapEncodeTiled, from the driver through the runtime (the library
// links no driver API); null when the driver does not offer it
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
        else
            cudaGetLastError();
    });
    return fn;
}

// Tensor maps of the ring slots for the TMA-staged spatial pass: a single
// view's slot [5 planes][H rows][W pixels x 4 floats], boxes of 32 pixels x 8
// rows x 5 planes (the 16-byte aligned inner coordinate is 4 x the pixel)
static void make_res_maps(vrg_renderer *r) {
    r->res_map_ok = false;
    EncodeTiledFn enc = encode_tiled();
    if (!enc || r->n_views != 0 || r->W < 32 || r->H < 8 || r->ring_slots > 8) return;
    const cuuint64_t P = (cuuint64_t)r->P;
    const cuuint64_t dims[3] = {4 * (cuuint64_t)r->W, r->H, 5};
    const cuuint64_t strides[2] = {16 * (cuuint64_t)r->W, 16 * P};
    const cuuint32_t box[3] = {4 * 32, 8, 5}, estr[3] = {1, 1, 1};
    for (uint32_t k = 0; k < r->ring_slots; k++)
        if (enc(&r->res_map[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void *)(r->res + (size_t)k * 5 * P), dims,
                strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return;
    r->res_map_ok = true;
}

static vrg_status ensure_ring(vrg_renderer *r, uint32_t slots) {
    if (slots == r->ring_slots) return VRG_OK;
    const size_t P = (size_t)r->P;
    cudaStream_t s = r->ctx->stream;
    DevBufPtr b;
    VRG_TRY(dev_alloc(s, (size_t)slots * 5 * P * 16, b));
    VRG_CUDA_TRY(cudaMemsetAsync(b->ptr, 0, (size_t)slots * 5 * P * 16, s));
    drop_graphs(r);
    r->res_buf = b;
    r->res = (float4 *)b->ptr;
    r->ring_slots = slots;
    make_res_maps(r);
    return VRG_OK;
}

// the renderer's launch configuration with defaults resolved
static vrg_tuning effective_tuning(const vrg_renderer *r) {
    int occ[3], sms = 1;
    bounce_occupancy(r->n_views != 0, occ, &sms);
    const vrg_tuning &t = r->tune;
    vrg_tuning e{};
    e.trace_blocks_per_sm = t.trace_blocks_per_sm ? std::min<uint32_t>(t.trace_blocks_per_sm, occ[0]) : occ[0];
    e.shade_blocks_per_sm = t.shade_blocks_per_sm ? std::min<uint32_t>(t.shade_blocks_per_sm, occ[1]) : occ[1];
    e.anyhit_blocks_per_sm = t.anyhit_blocks_per_sm ? std::min<uint32_t>(t.anyhit_blocks_per_sm, occ[2]) : occ[2];
    e.trace_refill = t.trace_refill ? t.trace_refill : 8;
    e.anyhit_refill = t.anyhit_refill ? t.anyhit_refill : 8;
    e.stream_block = t.stream_block ? t.stream_block : 256;
    // Per-thread loads unless TMA-staged tiles are asked for.  Staged tiles
    // make the spatial pass itself faster (0.113 against 0.117-0.119 ms per
    // 1080p frame), but the frame in flight slower (1.110-1.126 against
    // 1.078-1.091 ms): their 20.5 KB of shared memory per CTA takes L1 from
    // the closest-hit and light-hit walks of the next frames beside them.
    e.spatial_staging = (t.spatial_staging == 1 && r->n_views == 0 && r->W >= 32 && r->H >= 8) ? 1u : 2u;
    return e;
}

static void apply_tuning(const vrg_renderer *r, FrameArgs &a) {
    int occ[3], sms = 1;
    bounce_occupancy(r->n_views != 0, occ, &sms);
    const vrg_tuning e = effective_tuning(r);
    a.refill_trace = e.trace_refill;
    a.refill_any = e.anyhit_refill;
    a.grid_trace = (uint32_t)sms * e.trace_blocks_per_sm;
    a.grid_shade = (uint32_t)sms * e.shade_blocks_per_sm;
    a.grid_any = (uint32_t)sms * e.anyhit_blocks_per_sm;
    a.stream_block = e.stream_block;
}

// Frame set-up shared by vrg_render and vrg_render_batched: parameter checks,
// the reservoir ring, capture and cache buffers, and every FrameArgs field but
// the view ones.
// the array set of the frame about to be rendered (frame index mod SETS; batched
// renderers have one)
static uint32_t frame_set(const vrg_renderer *r) { return r->frame % r->n_sets; }

static vrg_status frame_setup(vrg_renderer *r, const vrg_render_params *pr, bool want_radiance, FrameArgs &a) {
    if (pr->num_bounces == 0 || pr->spatial_iterations > 64 || pr->nee_type > 2 || pr->mode > 1) {
        set_error("invalid render parameters");
        return VRG_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t s = r->ctx->stream;
    const size_t P = (size_t)r->P;
    const uint32_t slots = pr->history_slots ? pr->history_slots : 3;
    if (slots > 8) return VRG_ERR_INVALID_ARGUMENT;
    VRG_TRY(ensure_ring(r, slots));
    const bool capture = (pr->flags & VRG_RENDER_CAPTURE) != 0;
    if (capture) VRG_TRY(ensure_capture(r));
    const bool cache = (pr->flags & VRG_RENDER_CACHE) != 0;
    const uint32_t nb_total = cache ? pr->num_bounces + pr->cache_train_bounces : pr->num_bounces;
    if (cache) {
        if (!r->cache) {
            set_error("VRG_RENDER_CACHE without an attached radiance cache");
            return VRG_ERR_STATE;
        }
        if (pr->num_bounces < 2 || nb_total > r->nb_max) {
            set_error("cache mode needs num_bounces >= 2 and num_bounces + cache_train_bounces <= %u", r->nb_max);
            return VRG_ERR_INVALID_ARGUMENT;
        }
        const uint32_t cap = nrc_batch(r->cache);
        if (!r->cache_buf || r->cache_cap < cap) {  // (a later cache may train larger batches)
            auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
            struct Off {
                size_t qp, qd, pr, tg, il, tl, qf, taq0, taq1, taj0, taj1, thb, thv, tjm, tq, tq0, tq1;
            } off[Renderer::SETS];
            size_t o = 0;
            for (uint32_t k = 0; k < r->n_sets; k++) {
                Off &q = off[k];
                q.qp = o; o += al(P * 16);
                q.qd = o; o += al(P * 16);
                q.pr = o; o += al(P * 16);
                q.tg = o; o += al(P * 16);
                q.il = o; o += al(P * 4);
                q.tl = o; o += al((size_t)cap * 4);
                q.qf = o; o += al(P);
                q.taq0 = o; o += al((size_t)cap * 4);
                q.taq1 = o; o += al((size_t)cap * 4);
                q.taj0 = o; o += al((size_t)cap * 32);
                q.taj1 = o; o += al((size_t)cap * 32);
                q.thb = o; o += al((size_t)cap * 2 * 32);
                q.thv = o; o += al((size_t)cap * 2 * 4);
                q.tjm = o; o += al((size_t)cap * 8);
                q.tq = o; o += al(P * 4);
                q.tq0 = o; o += al((size_t)cap * 4);
                q.tq1 = o; o += al((size_t)cap * 4);
            }
            DevBufPtr b;
            VRG_TRY(dev_alloc(s, o, b));
            VRG_CUDA_TRY(cudaMemsetAsync(b->ptr, 0, o, s));
            uint8_t *B = (uint8_t *)b->ptr;
            for (uint32_t k = 0; k < r->n_sets; k++) {
                const Off &q = off[k];
                Renderer::CacheSet &Q = r->cs[k];
                Q.q_pos = (float4 *)(B + q.qp);
                Q.q_dir = (float4 *)(B + q.qd);
                Q.pred = (float4 *)(B + q.pr);
                Q.target = (float4 *)(B + q.tg);
                Q.infer_list = (uint32_t *)(B + q.il);
                Q.train_list = (uint32_t *)(B + q.tl);
                Q.qflag = B + q.qf;
                Q.t_aqueue[0] = (uint32_t *)(B + q.taq0);
                Q.t_aqueue[1] = (uint32_t *)(B + q.taq1);
                Q.t_ajob[0] = (float4 *)(B + q.taj0);
                Q.t_ajob[1] = (float4 *)(B + q.taj1);
                Q.t_hitbuf = (uint4 *)(B + q.thb);
                Q.t_hitval = (float *)(B + q.thv);
                Q.t_jmeta = (uint2 *)(B + q.tjm);
                Q.tq = (uint32_t *)(B + q.tq);
                Q.t_queue[0] = (uint32_t *)(B + q.tq0);
                Q.t_queue[1] = (uint32_t *)(B + q.tq1);
            }
            r->cache_buf = b;
            r->cache_cap = cap;
        }
    } else if (nb_total > r->nb_max) {
        return VRG_ERR_INVALID_ARGUMENT;
    }
    const uint32_t ring = r->frame % slots;
    memset(&a, 0, sizeof(a));
    a.P = (uint32_t)P;
    a.tiles_x = (r->W + 7) / 8;
    a.n0 = r->n_views ? (uint32_t)P : a.tiles_x * ((r->H + 3) / 4) * 32u;
    a.nb = nb_total;
    a.nb_render = pr->num_bounces;
    a.cache = cache ? 1u : 0u;
    a.train_cap = cache ? nrc_batch(r->cache) : 0u;
    a.restir = (pr->flags & VRG_RENDER_PLAIN_ONLY) ? 0u : 1u;
    {
        const Renderer::CacheSet &Q = r->cs[frame_set(r)];
        a.q_pos = Q.q_pos;
        a.q_dir = Q.q_dir;
        a.pred = Q.pred;
        a.target = Q.target;
        a.infer_list = Q.infer_list;
        a.train_list = Q.train_list;
        a.qflag = Q.qflag;
        a.tq = Q.tq;
    }
    // single-view cache frames that fork their training branch: the query
    // bounce in two launches, the training candidates first (a batched
    // frame's query bounce is long enough to hide its branch: four 3840x2160
    // views took 15.14-15.23 ms per frame one at a time split, 14.85 whole)
    a.tq_split = (cache && !capture && !r->n_views) ? 1u : 0u;
    a.nee_type = pr->nee_type;
    a.mode = pr->mode;
    a.spatial_iters = pr->spatial_iterations;
    a.spatial_radius = pr->spatial_radius;
    a.m_cap = pr->m_cap;
    a.debug_view = pr->debug_view;
    a.accumulate = pr->accumulate;
    a.pack = (pr->flags & VRG_RENDER_NO_PACK) ? 0u : 1u;
    const Renderer::FrameSet &F = r->fs[frame_set(r)];
    a.ray_o = F.ray_o;
    a.ray_d = F.ray_d;
    a.queue[0] = F.queue[0];
    a.queue[1] = F.queue[1];
    a.aqueue[0] = F.aqueue[0];
    a.aqueue[1] = F.aqueue[1];
    a.ajob[0] = F.ajob[0];
    a.ajob[1] = F.ajob[1];
    a.hits = F.hits;
    a.hitbuf = F.hitbuf;
    a.hitval = F.hitval;
    a.jmeta = F.jmeta;
    a.hit_cap = (uint32_t)std::min<size_t>(2 * P, 0xFFFFFFF0u);
    a.counters = F.counters;
    a.hit_count = a.counters + CNT_HITS;
    a.nlive = F.nlive;
    a.rec = F.rec;
    a.xv = F.xv;
    a.nv = F.nv;
    a.xs = F.xs;
    a.ns = F.ns;
    a.plain = r->plain;
    a.res = r->res + (size_t)ring * 5 * P;
    a.spatial = r->spatial;
    a.final_t = r->final_t;
    a.bgra = r->bgra;
    a.radiance = (want_radiance || r->scale > 1) ? r->radiance : nullptr;
    a.scale = r->scale;
    a.out_w = r->out_w;
    a.out_h = r->out_h;
    a.out_bgra = r->bgra;
    a.out_radiance = (want_radiance && r->scale > 1) ? r->radiance_out : nullptr;
    a.accum = r->accum;
    a.capture = capture ? 1u : 0u;
    a.c_origin = r->c_origin;
    a.c_dir = r->c_dir;
    a.c_normal = r->c_normal;
    a.c_emis = r->c_emis;
    a.c_refl = r->c_refl;
    a.c_mis = r->c_mis;
    a.c_pdf = r->c_pdf;
    a.c_nee = r->c_nee;
    a.c_L = r->c_L;
    a.c_q = r->c_q;
    a.c_hit = r->c_hit;
    apply_tuning(r, a);
    r->last_ring = ring;
    return VRG_OK;
}

// The frame's launch sequence on the context stream.  timed: CUDA events
// around every stage (r->ev: frame start, after each bounce, after resolve,
// after spatial; r->ev_k: after k_trace / k_shade of each bounce); a graph
// recording passes false.
//
// A cache frame forks once the training paths' query vertices are shaded,
// while that bounce's light-pdf walk still runs: the training paths' extra
// bounces (with light-pdf job and hit buffers of their own) and the cache's
// training step run on the renderer's second stream while the main stream
// infers the cache for the rendered paths and runs resolve (after the walk)
// and spatial.  A single-view frame traces its query bounce in two launches,
// the training candidates (whose pixels the shading before queued apart)
// first, and forks between them, before the other paths' query bounce; the
// training bounces then take ray queues of their own.  A batched frame forks
// after its whole query bounce.
// Neither branch reads what the other writes, except the cache itself: the
// training branch computes its gradients beside the queries, and their Adam
// step, which rewrites the weights and the table the queries read, is left to
// the next user of the cache; the next cache frame runs it on its training
// stream beside its own bounces, before its queries and its own training
// (the frames see the same cache as with the step at the end of each frame).
// With capture the frame stays on one stream.
// Frames in flight (pipelined: frames without stats or capture).
// A frame's bounces (closest hit, shading, light-pdf walks) read the committed
// scene, the camera and the material table, and write only the arrays of the
// frame's set, its cache arrays included (sets are taken in turn by frame
// index).  So they run on the set's own bounce stream as soon as the set's
// previous frame, n_sets frames back, has finished (ev_done), beside the
// previous frames' bounces, resolve and spatial passes and cache work.  The
// library stream waits for the bounces (ev_bounced) and then runs the frame's
// cache queries, resolve and spatial passes in frame order (a cache frame's
// training branch forks from there), so the frame is complete when the
// library stream has passed it.  Scene commits and
// material / atlas changes synchronize the library stream before they return,
// so a scene's device data is final before any frame reads it; a resize
// clears the arrays on the library stream and re-records ev_done.
// Other frames run their bounces on the library stream itself.
static vrg_status frame_launch(vrg_renderer *r, const FrameArgs &a, bool timed, bool pipelined = false,
                               bool in_graph = false) {
    cudaStream_t s = r->ctx->stream;
    const uint32_t k = frame_set(r);
    const bool fork = a.cache && !a.capture;
    const uint32_t nb_main = fork ? a.nb_render : a.nb;
    const bool own = pipelined && !a.capture && !timed && !in_graph;
    cudaStream_t bs = own ? r->bs[k] : s;  // stream of the bounces
    cudaStream_t lp = r->lps[k];
    if (own) VRG_CUDA_TRY(cudaStreamWaitEvent(bs, r->ev_done[k], 0));
    // A cache frame in flight starts its bounces once the previous cache
    // frame's training branch is done: that branch is a chain of small
    // latency-bound launches which persistent bounce kernels beside it would
    // hold off the SMs (ReSTIR over the cache, frames in flight: 1080p on 8x8
    // chunks 1.76 ms per frame with the wait, 1.80-1.85 without; four
    // 3840x2160 views of the 32x32-chunk scene 15.06-15.09 ms with the wait,
    // 17.0-17.6 without).
    if (own && fork) VRG_CUDA_TRY(cudaStreamWaitEvent(bs, r->ev_join, 0));
    // a cache frame runs the previous cache frame's Adam step on the training
    // stream beside its own bounces (after all earlier work on the library
    // stream); its cache queries wait for it
    bool updated = false;
    if (fork && nrc_pending(r->cache)) {
        VRG_CUDA_TRY(cudaEventRecord(r->ev_start, s));
        VRG_CUDA_TRY(cudaStreamWaitEvent(r->aux, r->ev_start, 0));
        VRG_TRY(nrc_flush(r->cache, r->aux));
        VRG_CUDA_TRY(cudaEventRecord(r->ev_updated, r->aux));
        updated = true;
    }
    VRG_CUDA_TRY(cudaMemsetAsync(a.counters, 0, CNT_WORDS * 4, bs));
    if (timed) VRG_CUDA_TRY(cudaEventRecord(r->ev[0], s));
    // Bounce b's light-pdf walk runs on the light-pdf stream beside bounce
    // b + 1's closest hit and shading.  Ordering: the walk of b waits for the
    // shading of b; the shading of b + 2 (which refills the job buffers of
    // parity b & 1) waits for the walk of b; resolve waits for every walk.
    int last_lp = -1;
    auto walk = [&](uint32_t b) -> vrg_status {
        VRG_CUDA_TRY(cudaEventRecord(r->ev_shaded[k][b], bs));
        VRG_CUDA_TRY(cudaStreamWaitEvent(lp, r->ev_shaded[k][b], 0));
        if (timed) VRG_CUDA_TRY(cudaEventRecord(r->ev_lp[0][b], lp));
        VRG_TRY(launch_light_pdf(lp, a, b, 0));
        if (timed) VRG_CUDA_TRY(cudaEventRecord(r->ev_lp[1][b], lp));
        VRG_CUDA_TRY(cudaEventRecord(r->ev_lpdone[k][b], lp));
        last_lp = (int)b;
        return VRG_OK;
    };
    // The training branch: the training paths' extra bounces (with light-pdf
    // job and hit buffers of their own) and the cache's training step, on
    // the renderer's second stream, forked from `from` once the training
    // paths' query vertices are shaded.
    cudaStream_t st = s;  // stream of the training branch
    const Renderer::CacheSet &Q = r->cs[k];
    auto branch = [&](cudaStream_t from, bool own_queues) -> vrg_status {
        st = r->aux;
        VRG_CUDA_TRY(cudaEventRecord(r->ev_fork, from));
        VRG_CUDA_TRY(cudaStreamWaitEvent(st, r->ev_fork, 0));
        // The training bounces' light-pdf jobs and hits go to buffers of their
        // own, so they need not wait for the main walks still running (which
        // read the main job buffers and write their own bounces' records);
        // forked before the main paths' query bounce, their ray queues too.
        FrameArgs at = a;
        for (int q = 0; q < 2; q++) {
            at.aqueue[q] = Q.t_aqueue[q];
            at.ajob[q] = Q.t_ajob[q];
        }
        if (own_queues) {  // training bounce nb_main reads queue[(nb_main + 1) & 1]
            at.queue[(nb_main + 1) & 1] = Q.t_queue[0];
            at.queue[nb_main & 1] = Q.t_queue[1];
        }
        at.qsel = 0;
        at.hitbuf = Q.t_hitbuf;
        at.hitval = Q.t_hitval;
        at.jmeta = Q.t_jmeta;
        at.hit_cap = 2 * a.train_cap;
        at.hit_count = a.counters + CNT_HITS_TRAIN;
        // As on the main path, training bounce b's light-pdf walk runs on a
        // stream of its own beside bounce b + 1; bounce b + 2, which refills
        // the job buffers of parity b & 1, waits for it.
        int last_tw = -1;
        for (uint32_t b = nb_main; b < a.nb; b++) {
            if (b >= nb_main + 2 && (int)b - 2 <= last_tw)
                VRG_CUDA_TRY(cudaStreamWaitEvent(st, r->ev_lpdone[k][b - 2], 0));
            VRG_TRY(launch_trace_shade(st, at, b, timed ? r->ev_k[0][b] : nullptr, a.train_cap));
            if (timed) VRG_CUDA_TRY(cudaEventRecord(r->ev_k[1][b], st));
            if (b + 1 < a.nb) {
                VRG_CUDA_TRY(cudaEventRecord(r->ev_shaded[k][b], st));
                VRG_CUDA_TRY(cudaStreamWaitEvent(r->aux_lp, r->ev_shaded[k][b], 0));
                VRG_TRY(launch_light_pdf(r->aux_lp, at, b, a.train_cap));
                VRG_CUDA_TRY(cudaEventRecord(r->ev_lpdone[k][b], r->aux_lp));
                last_tw = (int)b;
            }
            if (timed) VRG_CUDA_TRY(cudaEventRecord(r->ev[b + 1], st));
        }
        if (last_tw >= 0) VRG_CUDA_TRY(cudaStreamWaitEvent(st, r->ev_lpdone[k][last_tw], 0));
        // the targets' recurrence starts at the query vertex, whose record the
        // main walk of that bounce completes
        VRG_CUDA_TRY(cudaStreamWaitEvent(st, r->ev_lpdone[k][last_lp], 0));
        VRG_TRY(launch_train_targets(st, at));
        VRG_TRY(nrc_train(r->cache, st, a.train_cap, a.counters + CNT_TRAIN, a.train_list, a.q_pos, a.q_dir,
                          nullptr, a.target, false, a.counters + CNT_ERROR));
        return VRG_OK;
    };
    const bool early = fork && a.tq_split;
    for (uint32_t b = 0; b < nb_main; b++) {
        if (b >= 2 && (int)b - 2 <= last_lp) VRG_CUDA_TRY(cudaStreamWaitEvent(bs, r->ev_lpdone[k][b - 2], 0));
        if (early && b + 1 == nb_main) {
            // The query bounce of a single-view cache frame, first for the
            // training candidates that the previous shading queued apart: it
            // grants the training slots and queues the training paths' next
            // rays and light-pdf jobs, so the training branch and the query
            // bounce's walk start here, beside the other paths' query bounce.
            // (max_rays = P: the plain mapping in the shading, no routed
            // batches for this short queue.)
            FrameArgs aT = a;
            aT.qsel = 1;
            aT.queue[b & 1] = Q.t_queue[0];  // its continuing rays: the first training bounce's queue
            aT.queue[(b + 1) & 1] = Q.t_queue[1];
            VRG_TRY(launch_trace_shade(bs, aT, b, nullptr, a.P));
            if (b + 1 < a.nb) VRG_TRY(walk(b));
            VRG_TRY(branch(bs, true));
        }
        VRG_TRY(launch_trace_shade(bs, a, b, timed ? r->ev_k[0][b] : nullptr, 0));
        if (timed) {  // (timed frames run their bounces on the library stream)
            VRG_CUDA_TRY(cudaEventRecord(r->ev_k[1][b], s));
            VRG_CUDA_TRY(cudaEventRecord(r->ev[b + 1], s));
        }
        if (b + 1 < a.nb && !(early && b + 1 == nb_main)) VRG_TRY(walk(b));
    }
    // a cache frame's training branch and cache queries start before the last
    // main walk ends: only resolve reads what that walk writes
    if (last_lp >= 0 && !fork) VRG_CUDA_TRY(cudaStreamWaitEvent(bs, r->ev_lpdone[k][last_lp], 0));
    if (own) {
        VRG_CUDA_TRY(cudaEventRecord(r->ev_bounced[k], bs));
        VRG_CUDA_TRY(cudaStreamWaitEvent(s, r->ev_bounced[k], 0));
    }
    if (fork && !early) VRG_TRY(branch(s, false));
    if (a.cache) {  // radiance-cache queries of every path that ends into the cache
        if (updated) VRG_CUDA_TRY(cudaStreamWaitEvent(s, r->ev_updated, 0));
        if (!fork) VRG_TRY(nrc_flush(r->cache, s));
        VRG_TRY(nrc_infer(r->cache, s, a.P, a.counters + CNT_INFER, a.infer_list, a.q_pos, a.q_dir, nullptr,
                          a.pred, a.counters + CNT_ERROR));
    }
    if (fork) {
        // This frame's Adam step would rewrite the weights and table that its
        // queries read: it waits for the next user of the cache (the next
        // cache frame runs it beside its bounces; any other use runs it first).
        nrc_defer_update(r->cache);
        VRG_CUDA_TRY(cudaEventRecord(r->ev_join, st));
        VRG_CUDA_TRY(cudaStreamWaitEvent(s, r->ev_lpdone[k][last_lp], 0));
    }
    VRG_TRY(launch_resolve(s, a));
    if (a.cache && !fork) {  // one training step on this frame's long paths
        VRG_TRY(launch_train_targets(s, a));
        VRG_TRY(nrc_train(r->cache, s, a.train_cap, a.counters + CNT_TRAIN, a.train_list, a.q_pos, a.q_dir,
                          nullptr, a.target, true, a.counters + CNT_ERROR));
    }
    if (timed) VRG_CUDA_TRY(cudaEventRecord(r->ev[a.nb + 1], s));
    // the TMA-staged spatial pass when the tuning asks for it and the ring
    // slot has its tensor map
    const CUtensorMap *res_map = nullptr;
    if (effective_tuning(r).spatial_staging == 1 && r->res_map_ok && !in_graph && r->ring_slots) {
        const size_t slot = (size_t)(a.res - r->res) / (5 * (size_t)r->P);
        if (slot < r->ring_slots) res_map = &r->res_map[slot];
    }
    VRG_TRY(launch_spatial(s, a, res_map));
    if (fork) VRG_CUDA_TRY(cudaStreamWaitEvent(s, r->ev_join, 0));
    // the set is free for the frame n_sets ahead (recorded after the graph
    // launch when the frame is recorded in a graph)
    if (!in_graph) VRG_CUDA_TRY(cudaEventRecord(r->ev_done[k], s));
    if (timed) VRG_CUDA_TRY(cudaEventRecord(r->ev[a.nb + 2], s));
    return VRG_OK;
}

// Stats of the frame just launched (synchronizes).  per_kernel: the frame was
// launched with timed == true; otherwise ev[0]/ev[1] bracket a graph launch.
static vrg_status frame_stats(vrg_renderer *r, const FrameArgs &a, bool per_kernel, vrg_frame_stats *stats) {
    VRG_CUDA_TRY(cudaStreamSynchronize(r->ctx->stream));
    memset(stats, 0, sizeof(*stats));
    float ms = 0.0f;
    if (per_kernel) {
        cudaEventElapsedTime(&ms, r->ev[0], r->ev[a.nb + 2]);
        stats->ms_total = ms;
        // main-stream bounces: closest hit + shading; their light-pdf walks
        // run beside the next bounce and are timed on their own stream
        const uint32_t nb_main = (a.cache && !a.capture) ? a.nb_render : a.nb;
        for (uint32_t b = 0; b < a.nb && b < 8; b++) {
            cudaEventElapsedTime(&ms, r->ev[b], r->ev[b + 1]);
            stats->ms_bounce[b] = ms;
            cudaEventElapsedTime(&ms, r->ev[b], r->ev_k[0][b]);
            stats->ms_trace[b] = ms;
            cudaEventElapsedTime(&ms, r->ev_k[0][b], r->ev_k[1][b]);
            stats->ms_shade[b] = ms;
            if (b < nb_main) {
                if (b + 1 < a.nb) {
                    cudaEventElapsedTime(&ms, r->ev_lp[0][b], r->ev_lp[1][b]);
                    stats->ms_anyhit[b] = ms;
                }
            } else {
                cudaEventElapsedTime(&ms, r->ev_k[1][b], r->ev[b + 1]);
                stats->ms_anyhit[b] = ms;
            }
        }
        // a forked cache frame's resolve stage starts at the fork (it runs beside the training branch)
        cudaEventElapsedTime(&ms, r->ev[(a.cache && !a.capture) ? a.nb_render : a.nb], r->ev[a.nb + 1]);
        stats->ms_resolve = ms;
        cudaEventElapsedTime(&ms, r->ev[a.nb + 1], r->ev[a.nb + 2]);
        stats->ms_spatial = ms;
    } else {
        cudaEventElapsedTime(&ms, r->ev[0], r->ev[1]);
        stats->ms_total = ms;
    }
    uint32_t cnt[CNT_WORDS];
    VRG_CUDA_TRY(cudaMemcpy(cnt, a.counters, sizeof(cnt), cudaMemcpyDeviceToHost));
    uint64_t rays, any, nn, nlv;
    memcpy(&rays, cnt + CNT_RAYS, 8);
    memcpy(&any, cnt + CNT_ANY, 8);
    memcpy(&nn, cnt + CNT_NODES, 8);
    memcpy(&nlv, cnt + CNT_LEAVES, 8);
    stats->rays_closest = rays;
    stats->rays_any = any;
    stats->nodes_visited = nn;
    stats->leaves_visited = nlv;
    memcpy(&stats->light_nodes_visited, cnt + CNT_ANODES, 8);
    memcpy(&stats->light_leaves_visited, cnt + CNT_ALEAVES, 8);
    memcpy(&stats->light_hits, cnt + CNT_AHITS, 8);
    stats->error_flags = cnt[CNT_ERROR];
    if (cnt[CNT_ERROR]) {
        set_error("device error flags 0x%x", cnt[CNT_ERROR]);
        return VRG_ERR_OVERFLOW;
    }
    return VRG_OK;
}

// after the frame's launches and copies out: its fence, then the counters
static vrg_status frame_done(vrg_renderer *r, const FrameArgs &a, const vrg_render_params *pr) {
    VRG_CUDA_TRY(cudaEventRecord(r->ev_fence[r->frame % Renderer::FENCES], r->ctx->stream));
    if (a.cache) r->last_cache_set = (int)frame_set(r);
    r->last_nb = a.nb;
    r->captured = a.capture != 0;
    if (pr->accumulate) r->accum_n++;
    r->frame++;
    return VRG_OK;
}

VRG_API vrg_status vrg_render(vrg_renderer *r, vrg_scene *scene, const vrg_camera *cam,
                              const vrg_render_params *pr, const vrg_frame_output *out, vrg_frame_stats *stats) {
    if (!r || !scene || !cam || !pr) return VRG_ERR_INVALID_ARGUMENT;
    if (r->n_views) {
        set_error("a batched renderer renders with vrg_render_batched");
        return VRG_ERR_STATE;
    }
    if (cam->width != r->out_w || cam->height != r->out_h) {
        set_error("camera extent %ux%u differs from the renderer's %ux%u (call vrg_renderer_resize)", cam->width,
                  cam->height, r->out_w, r->out_h);
        return VRG_ERR_INVALID_ARGUMENT;
    }
    if (pr->flags & VRG_RENDER_GRAPH) {
        set_error("VRG_RENDER_GRAPH is a flag of vrg_render_batched");
        return VRG_ERR_UNSUPPORTED;
    }
    if (scene->ctx != r->ctx) return VRG_ERR_INVALID_ARGUMENT;
    if (out && out->host > VRG_OUTPUT_HOST_ASYNC) return VRG_ERR_INVALID_ARGUMENT;
    cudaStream_t s = r->ctx->stream;
    // Renderer::render starts with scene.get_tlas() (interactive_rendering.rs:961)
    VRG_TRY(scene_commit(scene));
    const size_t P = (size_t)r->P;
    FrameArgs a;
    VRG_TRY(frame_setup(r, pr, out && out->radiance, a));
    if (a.cache && !scene->h_geo_tl.empty())
        nrc_set_bounds(r->cache, scene->h_geo_tl[0].min, scene->h_geo_tl[0].max);
    a.v0.sc = frame_scene(scene);
    a.mesh = a.v0.sc.n_tri_rec ? 1u : 0u;
    a.v0.eye = f3{cam->eye[0], cam->eye[1], cam->eye[2]};
    a.v0.front = f3{cam->front[0], cam->front[1], cam->front[2]};
    a.v0.right = f3{cam->right[0], cam->right[1], cam->right[2]};
    a.v0.up = f3{cam->up[0], cam->up[1], cam->up[2]};
    a.v0.W = r->W;
    a.v0.H = r->H;
    a.v0.pix_off = 0;
    a.v0.pix_end = (uint32_t)P;
    a.v0.frame = r->frame;
    a.v0.temporal_seed = pr->temporal_seed;
    a.v0.spatial_seed = pr->spatial_seed;
    if (out && !out->host) {  // device outputs are written in place
        if (r->scale > 1) {
            if (out->radiance) a.out_radiance = out->radiance;
            if (out->bgra8) a.out_bgra = out->bgra8;
        } else {
            if (out->radiance) a.radiance = out->radiance;
            if (out->bgra8) a.bgra = out->bgra8;
        }
    }
    // without stats the frame is not timed and may start beside the previous one
    VRG_TRY(frame_launch(r, a, stats != nullptr, stats == nullptr));
    if (out && out->host) {
        const size_t Po = (size_t)r->out_w * r->out_h;
        if (out->bgra8 && a.pack)
            VRG_CUDA_TRY(cudaMemcpyAsync(out->bgra8, r->scale > 1 ? a.out_bgra : a.bgra, Po * 4,
                                         cudaMemcpyDeviceToHost, s));
        if (out->radiance)
            VRG_CUDA_TRY(cudaMemcpyAsync(out->radiance, r->scale > 1 ? a.out_radiance : a.radiance, Po * 12,
                                         cudaMemcpyDeviceToHost, s));
    }
    VRG_TRY(frame_done(r, a, pr));
    if (stats) return frame_stats(r, a, true, stats);
    if (out && out->host == VRG_OUTPUT_HOST) VRG_CUDA_TRY(cudaStreamSynchronize(s));
    return VRG_OK;
}

VRG_API vrg_status vrg_renderer_wait_frame(vrg_renderer *r, uint32_t frame_index) {
    if (!r) return VRG_ERR_INVALID_ARGUMENT;
    if (frame_index >= r->frame) {
        set_error("frame %u has not been rendered (next frame index %u)", frame_index, r->frame);
        return VRG_ERR_INVALID_ARGUMENT;
    }
    // the slot holds this frame's fence or a later frame's (stream order: that
    // one completes after this one)
    VRG_CUDA_TRY(cudaEventSynchronize(r->ev_fence[frame_index % Renderer::FENCES]));
    return VRG_OK;
}

VRG_API vrg_status vrg_render_batched(vrg_renderer *r, const vrg_view *views, uint32_t n_views,
                                      const vrg_render_params *pr, const vrg_frame_output *outs,
                                      vrg_frame_stats *stats) {
    if (!r || !views || !pr) return VRG_ERR_INVALID_ARGUMENT;
    if (r->n_views == 0) {
        set_error("vrg_render_batched needs a renderer made by vrg_renderer_create_batched");
        return VRG_ERR_STATE;
    }
    if (n_views != r->n_views) {
        set_error("%u views given, the renderer has %u", n_views, r->n_views);
        return VRG_ERR_INVALID_ARGUMENT;
    }
    const bool graph = (pr->flags & VRG_RENDER_GRAPH) != 0;
    if ((pr->flags & VRG_RENDER_CAPTURE) || (graph && (pr->flags & VRG_RENDER_CACHE))) {
        set_error("batched frames take neither VRG_RENDER_CAPTURE nor VRG_RENDER_GRAPH with VRG_RENDER_CACHE");
        return VRG_ERR_UNSUPPORTED;
    }
    for (uint32_t v = 0; v < n_views; v++) {
        const vrg_view &w = views[v];
        if (!w.scene || w.scene->ctx != r->ctx) return VRG_ERR_INVALID_ARGUMENT;
        if (w.camera.width != r->vw[v] || w.camera.height != r->vh[v]) {
            set_error("view %u: camera extent %ux%u differs from the view's %ux%u", v, w.camera.width,
                      w.camera.height, r->vw[v], r->vh[v]);
            return VRG_ERR_INVALID_ARGUMENT;
        }
        if (outs && outs[v].host > VRG_OUTPUT_HOST_ASYNC) return VRG_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t s = r->ctx->stream;
    {
        std::vector<Scene *> scs(n_views);
        for (uint32_t v = 0; v < n_views; v++) scs[v] = views[v].scene;
        VRG_TRY(scene_commit_many(scs.data(), n_views));
    }
    bool want_rad = false;
    if (outs)
        for (uint32_t v = 0; v < n_views; v++) want_rad |= outs[v].radiance != nullptr;
    FrameArgs a;
    VRG_TRY(frame_setup(r, pr, want_rad, a));
    if (a.cache) {  // the cache spans every view's scene
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (uint32_t v = 0; v < n_views; v++) {
            const auto &tl = views[v].scene->h_geo_tl;
            if (tl.empty()) continue;
            for (int k = 0; k < 3; k++) {
                lo[k] = std::min(lo[k], tl[0].min[k]);
                hi[k] = std::max(hi[k], tl[0].max[k]);
            }
        }
        if (lo[0] <= hi[0]) nrc_set_bounds(r->cache, lo, hi);
    }
    // per-view table: staged in pinned memory (two halves, so that the next
    // call does not overwrite a half whose copy has not run yet)
    ViewDev *hv = r->h_views + (size_t)r->stage * n_views;
    VRG_CUDA_TRY(cudaEventSynchronize(r->ev_stage[r->stage]));
    for (uint32_t v = 0; v < n_views; v++) {
        const vrg_view &w = views[v];
        ViewDev &d = hv[v];
        memset(&d, 0, sizeof(d));
        d.sc = frame_scene(w.scene);
        if (d.sc.n_tri_rec) a.mesh = 1u;
        d.eye = f3{w.camera.eye[0], w.camera.eye[1], w.camera.eye[2]};
        d.front = f3{w.camera.front[0], w.camera.front[1], w.camera.front[2]};
        d.right = f3{w.camera.right[0], w.camera.right[1], w.camera.right[2]};
        d.up = f3{w.camera.up[0], w.camera.up[1], w.camera.up[2]};
        d.W = r->vw[v];
        d.H = r->vh[v];
        d.pix_off = (uint32_t)r->voff[v];
        d.pix_end = (uint32_t)(r->voff[v] + (uint64_t)r->vw[v] * r->vh[v]);
        d.frame = r->frame;
        d.temporal_seed = w.temporal_seed;
        d.spatial_seed = w.spatial_seed;
    }
    // The set's view table: a frame in flight fills it on its set's bounce
    // stream once the set's previous frame is done; any other frame on the
    // library stream.
    const uint32_t set = frame_set(r);
    const bool in_flight = !graph && !stats;
    cudaStream_t cs = in_flight ? r->bs[set] : s;
    if (in_flight) VRG_CUDA_TRY(cudaStreamWaitEvent(cs, r->ev_done[set], 0));
    VRG_CUDA_TRY(
        cudaMemcpyAsync(r->d_views[set], hv, (size_t)n_views * sizeof(ViewDev), cudaMemcpyHostToDevice, cs));
    VRG_CUDA_TRY(cudaEventRecord(r->ev_stage[r->stage], cs));
    r->stage ^= 1u;
    a.views = r->d_views[set];
    a.vtab = r->d_vtab;
    a.n_views = n_views;
    if (graph) {
        // the FrameArgs bytes name the recording: buffers, ring slot and parameters
        std::vector<uint8_t> key((const uint8_t *)&a, (const uint8_t *)&a + sizeof(a));
        Renderer::GraphEntry *ge = nullptr;
        for (auto &g : r->graphs)
            if (g.key == key) ge = &g;
        if (!ge) {
            if (r->graphs.size() >= 8) drop_graphs(r);
            cudaGraph_t g = nullptr;
            VRG_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            vrg_status st = frame_launch(r, a, false, false, true);
            cudaError_t ce = cudaStreamEndCapture(s, &g);
            if (st != VRG_OK) {
                if (g) cudaGraphDestroy(g);
                return st;
            }
            VRG_CUDA_TRY(ce);
            cudaGraphExec_t ex = nullptr;
            ce = cudaGraphInstantiate(&ex, g, 0);
            cudaGraphDestroy(g);
            VRG_CUDA_TRY(ce);
            r->graphs.push_back(Renderer::GraphEntry{key, ex});
            ge = &r->graphs.back();
        }
        VRG_CUDA_TRY(cudaEventRecord(r->ev[0], s));
        VRG_CUDA_TRY(cudaGraphLaunch(ge->exec, s));
        VRG_CUDA_TRY(cudaEventRecord(r->ev[1], s));
        VRG_CUDA_TRY(cudaEventRecord(r->ev_done[set], s));
    } else {
        // without stats the frame is not timed and may run beside the previous one
        VRG_TRY(frame_launch(r, a, stats != nullptr, stats == nullptr));
    }
    bool host_out = false;
    if (outs) {
        for (uint32_t v = 0; v < n_views; v++) {
            const vrg_frame_output &o = outs[v];
            const size_t off = (size_t)r->voff[v], n = (size_t)r->vw[v] * r->vh[v];
            const cudaMemcpyKind k = o.host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
            if (o.bgra8 && a.pack) VRG_CUDA_TRY(cudaMemcpyAsync(o.bgra8, r->bgra + 4 * off, n * 4, k, s));
            if (o.radiance) VRG_CUDA_TRY(cudaMemcpyAsync(o.radiance, r->radiance + 3 * off, n * 12, k, s));
            host_out |= o.host == VRG_OUTPUT_HOST && (o.bgra8 || o.radiance);
        }
    }
    VRG_TRY(frame_done(r, a, pr));
    if (stats) return frame_stats(r, a, !graph, stats);
    if (host_out) VRG_CUDA_TRY(cudaStreamSynchronize(s));
    return VRG_OK;
}

// ---- cross-frame state -------------------------------------------------------

struct StateHeader {
    uint32_t magic;     // 'VRGS'
    uint32_t version;
    uint64_t pixels;
    uint32_t ring_slots;
    uint32_t frame;
    uint32_t accum_n;
    uint32_t pad;
};
static constexpr uint32_t STATE_MAGIC = 0x53475256u;

static uint64_t state_bytes(const vrg_renderer *r) {
    return sizeof(StateHeader) + (uint64_t)r->ring_slots * 5 * r->P * 16 + r->P * 24;
}

VRG_API vrg_status vrg_renderer_state_size(vrg_renderer *r, uint64_t *bytes) {
    if (!r || !bytes) return VRG_ERR_INVALID_ARGUMENT;
    *bytes = state_bytes(r);
    return VRG_OK;
}

VRG_API vrg_status vrg_renderer_state_save(vrg_renderer *r, void *dst, uint64_t bytes) {
    if (!r || !dst || bytes < state_bytes(r)) return VRG_ERR_INVALID_ARGUMENT;
    cudaStream_t s = r->ctx->stream;
    StateHeader h{STATE_MAGIC, 1u, r->P, r->ring_slots, r->frame, r->accum_n, 0u};
    uint8_t *d = (uint8_t *)dst;
    memcpy(d, &h, sizeof(h));
    d += sizeof(h);
    const size_t ring = (size_t)r->ring_slots * 5 * r->P * 16;
    if (ring) VRG_CUDA_TRY(cudaMemcpyAsync(d, r->res, ring, cudaMemcpyDeviceToHost, s));
    VRG_CUDA_TRY(cudaMemcpyAsync(d + ring, r->accum, (size_t)r->P * 24, cudaMemcpyDeviceToHost, s));
    VRG_CUDA_TRY(cudaStreamSynchronize(s));
    return VRG_OK;
}

VRG_API vrg_status vrg_renderer_state_load(vrg_renderer *r, const void *src, uint64_t bytes) {
    if (!r || !src || bytes < sizeof(StateHeader)) return VRG_ERR_INVALID_ARGUMENT;
    StateHeader h;
    memcpy(&h, src, sizeof(h));
    if (h.magic != STATE_MAGIC || h.version != 1u || h.pixels != r->P || h.ring_slots > 8) {
        set_error("state blob does not fit this renderer (%llu pixels, ring %u)", (unsigned long long)h.pixels,
                  h.ring_slots);
        return VRG_ERR_INVALID_ARGUMENT;
    }
    const size_t ring = (size_t)h.ring_slots * 5 * r->P * 16;
    if (bytes < sizeof(h) + ring + r->P * 24) return VRG_ERR_INVALID_ARGUMENT;
    if (h.ring_slots) VRG_TRY(ensure_ring(r, h.ring_slots));
    cudaStream_t s = r->ctx->stream;
    const uint8_t *p = (const uint8_t *)src + sizeof(h);
    if (ring) VRG_CUDA_TRY(cudaMemcpyAsync(r->res, p, ring, cudaMemcpyHostToDevice, s));
    VRG_CUDA_TRY(cudaMemcpyAsync(r->accum, p + ring, (size_t)r->P * 24, cudaMemcpyHostToDevice, s));
    VRG_CUDA_TRY(cudaStreamSynchronize(s));
    r->frame = h.frame;
    r->accum_n = h.accum_n;
    return VRG_OK;
}

VRG_API vrg_status vrg_renderer_set_tuning(vrg_renderer *r, const vrg_tuning *t) {
    if (!r || !t) return VRG_ERR_INVALID_ARGUMENT;
    if (t->trace_refill > 32 || t->anyhit_refill > 32 || t->trace_blocks_per_sm > 64 ||
        t->shade_blocks_per_sm > 64 || t->anyhit_blocks_per_sm > 64 ||
        (t->stream_block != 0 && t->stream_block != 64 && t->stream_block != 128 && t->stream_block != 256) ||
        t->spatial_staging > 2) {
        set_error("tuning out of range (refills 0..32, CTAs per SM 0..64, stream_block 0/64/128/256, "
                  "spatial_staging 0/1/2)");
        return VRG_ERR_INVALID_ARGUMENT;
    }
    r->tune = *t;
    memset(r->tune.reserved, 0, sizeof(r->tune.reserved));
    return VRG_OK;
}

VRG_API vrg_status vrg_renderer_get_tuning(vrg_renderer *r, vrg_tuning *t) {
    if (!r || !t) return VRG_ERR_INVALID_ARGUMENT;
    *t = effective_tuning(r);
    return VRG_OK;
}

VRG_API vrg_status vrg_renderer_autotune(vrg_renderer *r, vrg_scene *scene, const vrg_camera *cam,
                                         const vrg_render_params *params, uint32_t frames, vrg_tuning *best,
                                         float *best_ms) {
    if (!r || !scene || !cam || !params) return VRG_ERR_INVALID_ARGUMENT;
    if (r->n_views) {
        set_error("the autotuner renders single-view frames (tune one view, then vrg_renderer_set_tuning)");
        return VRG_ERR_STATE;
    }
    if (params->flags & (VRG_RENDER_CACHE | VRG_RENDER_CAPTURE | VRG_RENDER_GRAPH)) {
        set_error("the autotuner takes no cache, capture or graph frames");
        return VRG_ERR_UNSUPPORTED;
    }
    frames = std::max(1u, std::min(frames, 64u));
    cudaStream_t s = r->ctx->stream;
    const uint32_t slots = params->history_slots ? params->history_slots : 3;
    if (slots > 8) return VRG_ERR_INVALID_ARGUMENT;
    VRG_TRY(scene_commit(scene));
    VRG_TRY(ensure_ring(r, slots));
    // state the tuning frames change: frame counter and reservoir history
    const size_t ring_bytes = (size_t)slots * 5 * (size_t)r->P * 16;
    DevBufPtr saved;
    VRG_TRY(dev_alloc(s, ring_bytes, saved));
    VRG_CUDA_TRY(cudaMemcpyAsync(saved->ptr, r->res, ring_bytes, cudaMemcpyDeviceToDevice, s));
    const uint32_t frame0 = r->frame, accum0 = r->accum_n, last_nb0 = r->last_nb, last_ring0 = r->last_ring;
    const bool captured0 = r->captured;
    const vrg_tuning user = r->tune;
    vrg_render_params p = *params;
    p.accumulate = 0;
    // per frame, as frames run in use: back to back, in flight
    auto measure = [&](const vrg_tuning &t, float *ms_out) -> vrg_status {
        r->tune = t;
        VRG_TRY(vrg_render(r, scene, cam, &p, nullptr, nullptr));
        float reps[3];
        for (float &rep : reps) {
            VRG_CUDA_TRY(cudaEventRecord(r->ev[0], s));
            for (uint32_t f = 0; f < frames; f++) VRG_TRY(vrg_render(r, scene, cam, &p, nullptr, nullptr));
            VRG_CUDA_TRY(cudaEventRecord(r->ev[1], s));
            VRG_CUDA_TRY(cudaEventSynchronize(r->ev[1]));
            VRG_CUDA_TRY(cudaEventElapsedTime(&rep, r->ev[0], r->ev[1]));
            rep /= (float)frames;
        }
        std::sort(reps, reps + 3);
        *ms_out = reps[1];
        return VRG_OK;
    };
    int occ[3], sms = 1;
    bounce_occupancy(false, occ, &sms);
    auto bpsm_candidates = [](int o) {
        std::vector<uint32_t> c;
        for (int k : {1, 2, 3, 4, 6, 8, 12, 16})
            if (k < o) c.push_back((uint32_t)k);
        c.push_back((uint32_t)o);
        return c;
    };
    const std::vector<uint32_t> refills = {1, 2, 4, 8, 12, 16, 24, 32};
    struct Field {
        uint32_t vrg_tuning::*m;
        std::vector<uint32_t> cand;
    };
    const std::vector<Field> fields = {
        {&vrg_tuning::trace_refill, refills},
        {&vrg_tuning::trace_blocks_per_sm, bpsm_candidates(occ[0])},
        {&vrg_tuning::shade_blocks_per_sm, bpsm_candidates(occ[1])},
        {&vrg_tuning::anyhit_refill, refills},
        {&vrg_tuning::anyhit_blocks_per_sm, bpsm_candidates(occ[2])},
        {&vrg_tuning::stream_block, {64, 128, 256}},
    };
    vrg_tuning cur = effective_tuning(r);
    float cur_ms = 0.0f;
    vrg_status st = measure(cur, &cur_ms);
    for (int pass = 0; pass < 2 && st == VRG_OK; pass++) {
        for (const Field &fd : fields) {
            for (uint32_t v : fd.cand) {
                if (cur.*(fd.m) == v) continue;
                vrg_tuning t = cur;
                t.*(fd.m) = v;
                float ms = 0.0f;
                st = measure(t, &ms);
                if (st != VRG_OK) break;
                if (ms < cur_ms) {
                    // A candidate that timed faster is timed again beside the
                    // current choice before it is taken: out of dozens of
                    // noisy timings some come out low by chance, and such a
                    // configuration (often fewer closest-hit CTAs per SM)
                    // then runs slower in use.
                    float ms2 = 0.0f, cur2 = 0.0f;
                    st = measure(t, &ms2);
                    if (st == VRG_OK) st = measure(cur, &cur2);
                    if (st != VRG_OK) break;
                    if (ms2 < cur2) {
                        cur = t;
                        cur_ms = ms2;
                    } else {
                        cur_ms = cur2;
                    }
                }
            }
            if (st != VRG_OK) break;
        }
    }
    // restore the state the tuning frames changed
    VRG_CUDA_TRY(cudaMemcpyAsync(r->res, saved->ptr, ring_bytes, cudaMemcpyDeviceToDevice, s));
    VRG_CUDA_TRY(cudaStreamSynchronize(s));
    r->frame = frame0;
    r->accum_n = accum0;
    r->last_nb = last_nb0;
    r->last_ring = last_ring0;
    r->captured = captured0;
    if (st != VRG_OK) {
        r->tune = user;
        return st;
    }
    r->tune = cur;
    if (best) *best = cur;
    if (best_ms) *best_ms = cur_ms;
    return VRG_OK;
}

VRG_API vrg_status vrg_debug_readback(vrg_renderer *r, uint32_t what, void *dst, uint64_t bytes) {
    if (!r || !dst || what >= VRG_DBG_COUNT) return VRG_ERR_INVALID_ARGUMENT;
    if (what == VRG_DBG_CACHE_TARGET) {
        const size_t n = (size_t)r->P * 16;
        if (r->last_cache_set < 0 || !r->cs[r->last_cache_set].target) {
            set_error("no cache frame rendered");
            return VRG_ERR_STATE;
        }
        if (bytes < n) return VRG_ERR_INVALID_ARGUMENT;
        VRG_CUDA_TRY(cudaMemcpyAsync(dst, r->cs[r->last_cache_set].target, n, cudaMemcpyDeviceToHost,
                                     r->ctx->stream));
        VRG_CUDA_TRY(cudaStreamSynchronize(r->ctx->stream));
        return VRG_OK;
    }
    if (!r->captured) {
        set_error("last frame was not rendered with VRG_RENDER_CAPTURE");
        return VRG_ERR_STATE;
    }
    cudaStream_t s = r->ctx->stream;
    const size_t P = (size_t)r->P, nb = r->last_nb;
    auto copy = [&](const void *src, size_t n) -> vrg_status {
        if (bytes < n) return VRG_ERR_INVALID_ARGUMENT;
        VRG_CUDA_TRY(cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToHost, s));
        VRG_CUDA_TRY(cudaStreamSynchronize(s));
        return VRG_OK;
    };
    auto copy_res = [&](const float4 *planes) -> vrg_status {
        if (bytes < P * 80) return VRG_ERR_INVALID_ARGUMENT;
        std::vector<float4> h(5 * P);
        VRG_CUDA_TRY(cudaMemcpyAsync(h.data(), planes, 5 * P * 16, cudaMemcpyDeviceToHost, s));
        VRG_CUDA_TRY(cudaStreamSynchronize(s));
        float *o = (float *)dst;
        for (size_t p = 0; p < P; p++) {
            float *d = o + 20 * p;
            const float4 &a = h[p], &b = h[P + p], &c = h[2 * P + p], &e = h[3 * P + p], &l = h[4 * P + p];
            d[0] = a.x; d[1] = a.y; d[2] = a.z;
            d[3] = b.x; d[4] = b.y; d[5] = b.z;
            d[6] = c.x; d[7] = c.y; d[8] = c.z;
            d[9] = e.x; d[10] = e.y; d[11] = e.z;
            d[12] = l.x; d[13] = l.y; d[14] = l.z;
            d[15] = e.w;
            d[16] = l.w;
            d[17] = a.w;
            d[18] = c.w;
            d[19] = b.w;
        }
        return VRG_OK;
    };
    switch (what) {
    case VRG_DBG_ORIGIN: return copy(r->c_origin, (nb + 1) * P * 12);
    case VRG_DBG_DIRECTION: return copy(r->c_dir, (nb + 1) * P * 12);
    case VRG_DBG_NORMAL: return copy(r->c_normal, nb * P * 12);
    case VRG_DBG_EMISSIVITY: return copy(r->c_emis, nb * P * 12);
    case VRG_DBG_REFLECTIVITY: return copy(r->c_refl, nb * P * 12);
    case VRG_DBG_MIS: return copy(r->c_mis, nb * P * 4);
    case VRG_DBG_BSDF_PDF: return copy(r->c_pdf, nb * P * 4);
    case VRG_DBG_NEE_PDF: return copy(r->c_nee, nb * P * 4);
    case VRG_DBG_RADIANCE: return copy(r->c_L, nb * P * 12);
    case VRG_DBG_Q: return copy(r->c_q, nb * P * 4);
    case VRG_DBG_HIT: return copy(r->c_hit, nb * P * 16);
    case VRG_DBG_TEMPORAL: return copy_res(r->res + (size_t)r->last_ring * 5 * P);
    case VRG_DBG_SPATIAL: return copy_res(r->spatial);
    case VRG_DBG_FINAL: {
        if (bytes < P * 12) return VRG_ERR_INVALID_ARGUMENT;
        std::vector<float4> h(P);
        VRG_CUDA_TRY(cudaMemcpyAsync(h.data(), r->final_t, P * 16, cudaMemcpyDeviceToHost, s));
        VRG_CUDA_TRY(cudaStreamSynchronize(s));
        float *o = (float *)dst;
        for (size_t p = 0; p < P; p++) { o[3 * p] = h[p].x; o[3 * p + 1] = h[p].y; o[3 * p + 2] = h[p].z; }
        return VRG_OK;
    }
    default: return VRG_ERR_INVALID_ARGUMENT;
    }
}

// ---- standalone batched builds --------------------------------------------

VRG_API vrg_status vrg_build_tl_bvh_batched(vrg_context *ctx, uint32_t count, const uint32_t *n,
                                            const uint32_t *prim_offset, const uint32_t *node_offset,
                                            const float *translations, const float *aabbs, const float *power,
                                            const uint32_t *ids, vrg_bvh_node *nodes_out,
                                            uint32_t *prim_order_out) {
    if (!ctx || !n || !prim_offset || !node_offset || !aabbs || !power || !ids) return VRG_ERR_INVALID_ARGUMENT;
    return standalone_sah(ctx, false, count, n, prim_offset, node_offset, aabbs, translations, power, ids,
                          nodes_out, prim_order_out);
}

VRG_API vrg_status vrg_build_bl_bvh_batched(vrg_context *ctx, uint32_t count, const uint32_t *n,
                                            const uint32_t *prim_offset, const uint32_t *node_offset,
                                            const float *luminance, const float *triangles, const uint32_t *ids,
                                            vrg_bvh_node *nodes_out, uint32_t *prim_order_out) {
    if (!ctx || !n || !prim_offset || !node_offset || !luminance || !triangles || !ids)
        return VRG_ERR_INVALID_ARGUMENT;
    return standalone_sah(ctx, true, count, n, prim_offset, node_offset, triangles, nullptr, luminance, ids,
                          nodes_out, prim_order_out);
}

// ---- neural radiance cache ------------------------------------------------

static Nrc *NR(vrg_nrc *p) { return reinterpret_cast<Nrc *>(p); }

VRG_API vrg_status vrg_nrc_create(vrg_context *ctx, const vrg_nrc_desc *desc, vrg_nrc **out) {
    if (!ctx || !desc || !out) return VRG_ERR_INVALID_ARGUMENT;
    Nrc *n = nullptr;
    VRG_TRY(nrc_create(ctx, desc, &n));
    *out = reinterpret_cast<vrg_nrc *>(n);
    return VRG_OK;
}
VRG_API vrg_status vrg_nrc_destroy(vrg_nrc *nrc) {
    if (!nrc) return VRG_ERR_INVALID_ARGUMENT;
    nrc_destroy(NR(nrc));
    return VRG_OK;
}
VRG_API vrg_status vrg_nrc_query(vrg_nrc *nrc, uint32_t n, const float *pos, const float *normal, const float *dir,
                                 float *rgb) {
    if (!nrc || !pos || !normal || !dir || !rgb) return VRG_ERR_INVALID_ARGUMENT;
    if (n == 0) return VRG_OK;
    return nrc_query_host(NR(nrc), n, pos, normal, dir, rgb);
}
VRG_API vrg_status vrg_nrc_train(vrg_nrc *nrc, uint32_t n, const float *pos, const float *normal, const float *dir,
                                 const float *target, uint32_t update, float *loss) {
    if (!nrc || !pos || !normal || !dir || !target) return VRG_ERR_INVALID_ARGUMENT;
    if (n == 0) return VRG_OK;
    return nrc_train_host(NR(nrc), n, pos, normal, dir, target, update, loss);
}
VRG_API vrg_status vrg_nrc_read(vrg_nrc *nrc, uint32_t what, void *dst, uint64_t bytes) {
    if (!nrc || !dst) return VRG_ERR_INVALID_ARGUMENT;
    return nrc_read(NR(nrc), what, dst, bytes);
}
VRG_API vrg_status vrg_nrc_write(vrg_nrc *nrc, uint32_t what, const void *src, uint64_t bytes) {
    if (!nrc || (!src && what != VRG_NRC_ZERO_GRADS)) return VRG_ERR_INVALID_ARGUMENT;
    return nrc_write(NR(nrc), what, src, bytes);
}
VRG_API vrg_status vrg_nrc_layout(vrg_nrc *nrc, uint32_t *levels, float *scales, uint32_t *dense, uint32_t *res1) {
    if (!nrc || !levels || !scales || !dense || !res1) return VRG_ERR_INVALID_ARGUMENT;
    nrc_layout(levels, scales, dense, res1, NR(nrc));
    return VRG_OK;
}
VRG_API vrg_status vrg_renderer_set_cache(vrg_renderer *r, vrg_nrc *nrc) {
    if (!r) return VRG_ERR_INVALID_ARGUMENT;
    r->cache = NR(nrc);
    return VRG_OK;
}

}  // extern "C"
