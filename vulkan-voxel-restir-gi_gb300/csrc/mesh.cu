// Triangle-mesh objects: SceneUploader::upload_object (scene.rs:547-725) for
// arbitrary Vec<Vertex3D>, the path the reference takes for every object it
// renders (chunks are meshed on the CPU and uploaded the same way; its ego
// entity is a unit cube, main.rs:86-101).
//
// The light primitives are the luminous triangles (the luminance of the
// triangle's texture slot t, taken from its first vertex, is > 0), each with
// power = luminance * area (scene.rs:555-571); the light BLAS over them is
// build_bl_bvh with the triangle indices as leaf prim ids (build.rs:249-372).
// The driver BLAS over all triangles (scene.rs:164-171) is replaced by the
// same SAH builder over the triangles (build_bl_bvh inputs), whose leaves the
// closest-hit walk tests with a watertight ray/triangle test.  Both trees are
// built by one batched launch sequence on the GPU; the per-triangle inputs
// are prepared on the host, where the reference prepares them too.
#include <algorithm>
#include <cstring>

#include "vrg_internal.h"

namespace vrg {

static float bits_as_float(uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
}

vrg_status mesh_upload(Context *ctx, const vrg_vertex3d *v, uint64_t nverts, Object *o) {
    if (nverts % 3) {
        set_error("vrg_upload_mesh: %llu vertices is not a multiple of 3", (unsigned long long)nverts);
        return VRG_ERR_INVALID_ARGUMENT;
    }
    if (nverts / 3 > (1u << 24)) {
        set_error("vrg_upload_mesh: more than 2^24 triangles");
        return VRG_ERR_UNSUPPORTED;
    }
    const uint32_t n = (uint32_t)(nverts / 3);
    const uint32_t n_slots = (uint32_t)ctx->mats.size();
    o->mesh = true;
    memset(&o->sum, 0, sizeof(o->sum));
    if (n == 0) {  // SceneUploadedObjectHandle::Empty
        o->flushed = true;
        return VRG_OK;
    }
    // per triangle: object-space vertices with the slot, uvs; light prims
    std::vector<float4> tri(3 * (size_t)n);
    std::vector<float> uv(6 * (size_t)n);
    std::vector<uint32_t> light_tri;
    std::vector<float> light_power;
    for (uint32_t i = 0; i < n; i++) {
        const vrg_vertex3d *x = v + 3 * (size_t)i;
        const uint32_t t = x[0].t;
        if (t >= n_slots) {
            set_error("vrg_upload_mesh: triangle %u uses texture slot %u of %u", i, t, n_slots);
            return VRG_ERR_INVALID_ARGUMENT;
        }
        for (int j = 0; j < 3; j++) {
            for (int a = 0; a < 3; a++)
                if (!(fabsf(x[j].position[a]) <= 1024.0f)) {
                    set_error("vrg_upload_mesh: vertex coordinates must be finite and within +-1024");
                    return VRG_ERR_UNSUPPORTED;
                }
            tri[3 * (size_t)i + j] = make_float4(x[j].position[0], x[j].position[1], x[j].position[2],
                                                 j == 0 ? bits_as_float(t) : 0.0f);
            uv[6 * (size_t)i + 2 * j] = x[j].uv[0];
            uv[6 * (size_t)i + 2 * j + 1] = x[j].uv[1];
        }
        const float L = ctx->mats[t].luminance;
        if (L > 0.0f) {  // scene.rs:559-571: power = luminance * |(b - a) x (c - a)| / 2
            const f3 a = f3{x[0].position[0], x[0].position[1], x[0].position[2]};
            const f3 b = f3{x[1].position[0], x[1].position[1], x[1].position[2]};
            const f3 c = f3{x[2].position[0], x[2].position[1], x[2].position[2]};
            const float area = len3(cross3(sub3(b, a), sub3(c, a))) / 2.0f;
            light_tri.push_back(i);
            light_power.push_back(L * area);
        }
    }
    const uint32_t nl = (uint32_t)light_tri.size();
    // builder inputs: geometry prims [0, n), light prims [n, n + nl); AABB of
    // the three points, centroid (v0 + v1 + v2) / 3, w = power (build.rs:262-270)
    const uint32_t np = n + nl;
    std::vector<float4> lo(np), hi(np), cen(np);
    std::vector<uint32_t> ids(np);
    auto prim = [&](uint32_t k, uint32_t t, float power) {
        const float4 *q = &tri[3 * (size_t)t];
        float l[3], h[3], s[3];
        for (int a = 0; a < 3; a++) {
            const float c0 = a == 0 ? q[0].x : (a == 1 ? q[0].y : q[0].z);
            const float c1 = a == 0 ? q[1].x : (a == 1 ? q[1].y : q[1].z);
            const float c2 = a == 0 ? q[2].x : (a == 1 ? q[2].y : q[2].z);
            l[a] = fminf(fminf(fminf(c0, c0), c1), c2);
            h[a] = fmaxf(fmaxf(fmaxf(c0, c0), c1), c2);
            s[a] = (c0 + c1) + c2;
        }
        lo[k] = make_float4(l[0], l[1], l[2], 0.0f);
        hi[k] = make_float4(h[0], h[1], h[2], 0.0f);
        cen[k] = make_float4(s[0] / 3.0f, s[1] / 3.0f, s[2] / 3.0f, power);
        ids[k] = t;
    };
    for (uint32_t i = 0; i < n; i++) prim(i, i, 0.0f);
    for (uint32_t k = 0; k < nl; k++) prim(n + k, light_tri[k], light_power[k]);
    // persistent arrays of the object, then the builder's inputs
    const uint32_t n_geo_nodes = 2 * n - 1, n_light_nodes = nl ? 2 * nl - 1 : 0;
    const uint32_t n_nodes = n_geo_nodes + n_light_nodes;
    auto al = [](uint64_t x) { return (x + 255) & ~255ull; };
    uint64_t off = 0;
    const uint64_t o_tri = off; off += al((uint64_t)n * 48);
    const uint64_t o_uv = off; off += al((uint64_t)n * 24);
    const uint64_t o_ltri = off; off += al((uint64_t)nl * 4 + 4);
    const uint64_t o_nodes = off; off += al((uint64_t)n_nodes * sizeof(vrg_bvh_node));
    const uint64_t o_perm = off; off += al((uint64_t)np * 4);
    const uint64_t o_leaf = off; off += al((uint64_t)n_nodes * 4);
    const uint64_t o_payload = off; off += al((uint64_t)n_light_nodes * 4 + 4);
    const uint64_t o_lo = off; off += al((uint64_t)np * 16);
    const uint64_t o_hi = off; off += al((uint64_t)np * 16);
    const uint64_t o_cen = off; off += al((uint64_t)np * 16);
    const uint64_t o_id = off; off += al((uint64_t)np * 4);
    cudaStream_t s = ctx->stream;
    DevBufPtr buf;
    VRG_TRY(dev_alloc(s, off, buf));
    uint8_t *B = (uint8_t *)buf->ptr;
    VRG_CUDA_TRY(cudaMemcpyAsync(B + o_tri, tri.data(), (size_t)n * 48, cudaMemcpyHostToDevice, s));
    VRG_CUDA_TRY(cudaMemcpyAsync(B + o_uv, uv.data(), (size_t)n * 24, cudaMemcpyHostToDevice, s));
    if (nl) VRG_CUDA_TRY(cudaMemcpyAsync(B + o_ltri, light_tri.data(), (size_t)nl * 4, cudaMemcpyHostToDevice, s));
    VRG_CUDA_TRY(cudaMemcpyAsync(B + o_lo, lo.data(), (size_t)np * 16, cudaMemcpyHostToDevice, s));
    VRG_CUDA_TRY(cudaMemcpyAsync(B + o_hi, hi.data(), (size_t)np * 16, cudaMemcpyHostToDevice, s));
    VRG_CUDA_TRY(cudaMemcpyAsync(B + o_cen, cen.data(), (size_t)np * 16, cudaMemcpyHostToDevice, s));
    VRG_CUDA_TRY(cudaMemcpyAsync(B + o_id, ids.data(), (size_t)np * 4, cudaMemcpyHostToDevice, s));
    std::vector<SahTree> trees{SahTree{n, 0, 0, 0}};
    if (nl) trees.push_back(SahTree{nl, n, n_geo_nodes, 0});
    SahInputs in{(const float4 *)(B + o_lo), (const float4 *)(B + o_hi), (const float4 *)(B + o_cen),
                 (const uint32_t *)(B + o_id)};
    vrg_bvh_node *nodes = (vrg_bvh_node *)(B + o_nodes);
    uint32_t *leaf = (uint32_t *)(B + o_leaf);
    SahOutputs out{nodes, (uint32_t *)(B + o_perm), leaf};
    uint32_t levels = 0;
    VRG_TRY(sah_build(s, trees, np, n_nodes, in, out, &levels));
    // roots (build_bl_bvh's returned AABB and power, build.rs:359-371: a leaf
    // root holds its prim's unpadded AABB and power) and the light leaf payload
    // (node -> triangle index)
    std::vector<vrg_bvh_node> root(2);
    std::vector<uint32_t> lleaf(n_light_nodes);
    VRG_CUDA_TRY(cudaMemcpyAsync(&root[0], nodes, sizeof(vrg_bvh_node), cudaMemcpyDeviceToHost, s));
    if (nl) {
        VRG_CUDA_TRY(cudaMemcpyAsync(&root[1], nodes + n_geo_nodes, sizeof(vrg_bvh_node), cudaMemcpyDeviceToHost, s));
        VRG_CUDA_TRY(cudaMemcpyAsync(lleaf.data(), leaf + n_geo_nodes, (size_t)n_light_nodes * 4,
                                     cudaMemcpyDeviceToHost, s));
    }
    VRG_CUDA_TRY(cudaStreamSynchronize(s));
    if (nl) {
        std::vector<uint32_t> payload(n_light_nodes);
        for (uint32_t j = 0; j < n_light_nodes; j++) payload[j] = lleaf[j] == INVALID ? INVALID : light_tri[lleaf[j]];
        VRG_CUDA_TRY(cudaMemcpyAsync(B + o_payload, payload.data(), (size_t)n_light_nodes * 4,
                                     cudaMemcpyHostToDevice, s));
        VRG_CUDA_TRY(cudaStreamSynchronize(s));
    }
    ChunkSummary &cs = o->sum;
    cs.n_faces = n;
    cs.n_tris = n;
    cs.n_light = nl;
    cs.n_geo = n;
    for (int a = 0; a < 3; a++) {
        cs.geo_lo[a] = root[0].min[a];
        cs.geo_hi[a] = root[0].max[a];
    }
    if (nl) {
        for (int a = 0; a < 3; a++) {
            cs.light_lo[a] = root[1].min[a];
            cs.light_hi[a] = root[1].max[a];
        }
        cs.light_power = root[1].power;
    }
    o->batch = buf;
    o->mesh_tri = (const float4 *)(B + o_tri);
    o->mesh_uv = (const float *)(B + o_uv);
    o->geo_local = nullptr;
    o->geo_nodes = nodes;
    o->geo_perm = (const uint32_t *)(B + o_perm);
    o->geo_leaf = leaf;
    if (nl) {
        o->light_nodes = nodes + n_geo_nodes;
        o->light_perm = (const uint32_t *)(B + o_perm) + n;
        o->light_leaf = leaf + n_geo_nodes;
        o->light_tri = (const uint32_t *)(B + o_ltri);
        o->light_leaf_tri = (const uint32_t *)(B + o_payload);
    }
    o->levels = levels;
    o->flushed = true;
    return VRG_OK;
}

}  // namespace vrg
