// GPU chunk meshing and light-primitive extraction, batched over chunks.
//
// Replaces, per chunk, the reference's CPU pipeline chunk::gen_mesh
// (chunk.rs:158-292) -> SceneUploader::upload_object (scene.rs:547-725) ->
// build_bl_bvh (build.rs:249-372): a face of a non-air block is exposed when
// the neighbouring block (inside the chunk or in the neighbour chunk's
// boundary plane) is air or translucent; exposed faces become two triangles
// each, numbered in gen_mesh's scan order (x, y, z, then faces left, right,
// down, up, back, front); a triangle is a light when its face material has
// luminance > 0, with power luminance * area.  The geometry primitives are
// the surface blocks (>= 1 exposed face) with AABB [x, x+1]^3.
//
// One CTA of 1024 threads per chunk; thread t owns the 32 consecutive block
// indices 32t..32t+31 (x = t/32, y = t%32, z = 0..31), so a CTA-wide
// exclusive scan of per-thread counts gives gen_mesh's numbering directly.
#include "vrg_internal.h"

namespace vrg {

namespace {

constexpr int CHUNK_BYTES = VRG_CHUNK_BLOCKS + 6 * 1024;  // blocks + 6 neighbour planes

struct ExtractArgs {
    const uint8_t *in;           // [n_chunks][CHUNK_BYTES]
    uint8_t *masks;              // [n_chunks][32768]
    uint32_t *counts;            // [n_chunks][4]: faces, light faces, surface blocks, pad
    const vrg_material *mats;
    uint32_t air;
};

__device__ __forceinline__ bool translucent(const vrg_material *mats, uint32_t air, uint32_t b) {
    if (b == air) return true;
    return (mats[6u * b].flags & VRG_MAT_TRANSLUCENT) != 0u;
}

// neighbour block id across face f of block (x,y,z) (chunk.rs:170-205)
__device__ __forceinline__ uint32_t neighbour(const uint8_t *blk, const uint8_t *slabs, int x, int y, int z, int f) {
    switch (f) {
    case 0: return x == 0 ? slabs[0 * 1024 + y * 32 + z] : blk[(x - 1) * 1024 + y * 32 + z];
    case 1: return x == 31 ? slabs[1 * 1024 + y * 32 + z] : blk[(x + 1) * 1024 + y * 32 + z];
    case 2: return y == 0 ? slabs[2 * 1024 + x * 32 + z] : blk[x * 1024 + (y - 1) * 32 + z];
    case 3: return y == 31 ? slabs[3 * 1024 + x * 32 + z] : blk[x * 1024 + (y + 1) * 32 + z];
    case 4: return z == 0 ? slabs[4 * 1024 + x * 32 + y] : blk[x * 1024 + y * 32 + z - 1];
    default: return z == 31 ? slabs[5 * 1024 + x * 32 + y] : blk[x * 1024 + y * 32 + z + 1];
    }
}

__device__ __forceinline__ uint32_t block_reduce_add(uint32_t v, uint32_t *sh) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    uint32_t r = 0;
    if (w == 0) {
        r = sh[lane];
        for (int o = 16; o; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
        if (lane == 0) sh[32] = r;
    }
    __syncthreads();
    r = sh[32];
    __syncthreads();
    return r;
}

// exclusive scan over the 1024 threads of the CTA
__device__ __forceinline__ uint32_t block_exscan(uint32_t v, uint32_t *sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) sh[w] = inc;
    __syncthreads();
    if (w == 0) {
        uint32_t s = sh[lane];
        uint32_t si = s;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, si, o);
            if (lane >= o) si += t;
        }
        sh[lane] = si - s;  // exclusive warp offsets
    }
    __syncthreads();
    uint32_t r = sh[w] + inc - v;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(1024) k_extract_masks(ExtractArgs a) {
    __shared__ uint32_t sh[33];
    const uint8_t *in = a.in + (size_t)blockIdx.x * CHUNK_BYTES;
    const uint8_t *slabs = in + VRG_CHUNK_BLOCKS;
    uint8_t *masks = a.masks + (size_t)blockIdx.x * VRG_CHUNK_BLOCKS;
    const int t = threadIdx.x, x = t >> 5, y = t & 31;
    uint32_t faces = 0, lfaces = 0, surf = 0;
    for (int z = 0; z < 32; z++) {
        uint32_t bi = (uint32_t)(t * 32 + z);
        uint32_t b = in[bi];
        uint32_t m = 0;
        if (b != a.air) {
            for (int f = 0; f < 6; f++) {
                if (translucent(a.mats, a.air, neighbour(in, slabs, x, y, z, f))) {
                    m |= 1u << f;
                    if (a.mats[6u * b + (uint32_t)f].luminance > 0.0f) lfaces++;
                }
            }
        }
        faces += __popc(m);
        surf += m ? 1u : 0u;
        masks[bi] = (uint8_t)m;
    }
    uint32_t F = block_reduce_add(faces, sh);
    uint32_t Lf = block_reduce_add(lfaces, sh);
    uint32_t S = block_reduce_add(surf, sh);
    if (t == 0) {
        a.counts[4 * blockIdx.x + 0] = F;
        a.counts[4 * blockIdx.x + 1] = Lf;
        a.counts[4 * blockIdx.x + 2] = S;
        a.counts[4 * blockIdx.x + 3] = 0;
    }
}

struct WriteArgs {
    const uint8_t *in;
    const uint8_t *masks;
    const vrg_material *mats;
    uint32_t air;
    const uint32_t *geo_off;     // [n_chunks] prim offset of the chunk's geometry prims
    const uint32_t *light_off;   // [n_chunks] prim offset of the chunk's light prims
    const uint32_t *loc_off;     // [n_chunks] offset into geo_local / light_tri
    const uint32_t *lloc_off;
    // builder inputs
    float4 *lo, *hi, *cen;
    uint32_t *id;
    // persistent per-object outputs
    int2 *geo_local;
    uint32_t *light_tri;
};

__global__ void __launch_bounds__(1024) k_extract_write(WriteArgs a) {
    __shared__ uint32_t sh[33];
    const uint32_t c = blockIdx.x;
    const uint8_t *in = a.in + (size_t)c * CHUNK_BYTES;
    const uint8_t *masks = a.masks + (size_t)c * VRG_CHUNK_BLOCKS;
    const int t = threadIdx.x;
    uint32_t faces = 0, lfaces = 0, surf = 0;
    for (int z = 0; z < 32; z++) {
        uint32_t bi = (uint32_t)(t * 32 + z);
        uint32_t m = masks[bi];
        if (!m) continue;
        uint32_t b = in[bi];
        faces += __popc(m);
        surf++;
        for (int f = 0; f < 6; f++)
            if ((m >> f) & 1u)
                if (a.mats[6u * b + (uint32_t)f].luminance > 0.0f) lfaces++;
    }
    uint32_t face_base = block_exscan(faces, sh);
    uint32_t lface_base = block_exscan(lfaces, sh);
    uint32_t surf_base = block_exscan(surf, sh);
    const int x = t >> 5, y = t & 31;
    const uint32_t goff = a.geo_off[c], loff = a.light_off[c], gl = a.loc_off[c], ll = a.lloc_off[c];
    for (int z = 0; z < 32; z++) {
        uint32_t bi = (uint32_t)(t * 32 + z);
        uint32_t m = masks[bi];
        if (!m) continue;
        uint32_t b = in[bi];
        uint32_t first_tri = 2u * face_base;
        // geometry prim: block AABB, centroid (min+max)/2 (build.rs:391-400)
        {
            uint32_t g = goff + surf_base;
            float lx = (float)x, ly = (float)y, lz = (float)z;
            float hx = (float)(x + 1), hy = (float)(y + 1), hz = (float)(z + 1);
            a.lo[g] = make_float4(lx, ly, lz, 0.0f);
            a.hi[g] = make_float4(hx, hy, hz, 0.0f);
            a.cen[g] = make_float4((lx + hx) / 2.0f, (ly + hy) / 2.0f, (lz + hz) / 2.0f, 0.0f);
            a.id[g] = bi;
            a.geo_local[gl + surf_base] = make_int2((int)(bi | (m << 15) | (b << 21)), (int)first_tri);
        }
        uint32_t rank = 0;
        for (int f = 0; f < 6; f++) {
            if (!((m >> f) & 1u)) continue;
            float L = a.mats[6u * b + (uint32_t)f].luminance;
            if (L > 0.0f) {
                for (int h = 0; h < 2; h++) {
                    uint32_t lp = 2u * lface_base + (uint32_t)h;
                    uint32_t g = loff + lp;
                    f3 v0 = corner_pos(x, y, z, face_corner(f, h, 0));
                    f3 v1 = corner_pos(x, y, z, face_corner(f, h, 1));
                    f3 v2 = corner_pos(x, y, z, face_corner(f, h, 2));
                    // Aabb::from_points (aabb.rs:10-22)
                    float mnx = fminf(fminf(fminf(v0.x, v0.x), v1.x), v2.x);
                    float mny = fminf(fminf(fminf(v0.y, v0.y), v1.y), v2.y);
                    float mnz = fminf(fminf(fminf(v0.z, v0.z), v1.z), v2.z);
                    float mxx = fmaxf(fmaxf(fmaxf(v0.x, v0.x), v1.x), v2.x);
                    float mxy = fmaxf(fmaxf(fmaxf(v0.y, v0.y), v1.y), v2.y);
                    float mxz = fmaxf(fmaxf(fmaxf(v0.z, v0.z), v1.z), v2.z);
                    // centroid (v0+v1+v2)/3 (build.rs:267-270); power = lum*area (scene.rs:560-571)
                    f3 s = add3(add3(v0, v1), v2);
                    float area = len3(cross3(sub3(v1, v0), sub3(v2, v0))) / 2.0f;
                    a.lo[g] = make_float4(mnx, mny, mnz, 0.0f);
                    a.hi[g] = make_float4(mxx, mxy, mxz, 0.0f);
                    a.cen[g] = make_float4(s.x / 3.0f, s.y / 3.0f, s.z / 3.0f, L * area);
                    a.id[g] = first_tri + 2u * rank + (uint32_t)h;
                    a.light_tri[ll + lp] = (uint32_t)x | ((uint32_t)y << 5) | ((uint32_t)z << 10) |
                                           ((uint32_t)f << 15) | ((uint32_t)h << 18);
                }
                lface_base++;
            }
            rank++;
        }
        face_base += __popc(m);
        surf_base++;
    }
}

// per light node: leaf payload (the triangle of the leaf's prim)
__global__ void k_light_leaf_payload(const uint32_t *leaf_prim, const uint32_t *light_tri, uint32_t *payload,
                                     uint32_t n_nodes) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_nodes) return;
    uint32_t p = leaf_prim[i];
    payload[i] = (p == INVALID) ? INVALID : light_tri[p];
}

}  // namespace

vrg_status extract_and_build(Context *ctx, std::vector<Object *> &batch) {
    if (batch.empty()) return VRG_OK;
    cudaStream_t s = ctx->stream;
    const uint32_t nc = (uint32_t)batch.size();
    if (nc > 65535) {
        set_error("too many chunks in one flush (%u)", nc);
        return VRG_ERR_UNSUPPORTED;
    }
    // stage blocks + neighbour planes
    size_t in_bytes = (size_t)nc * CHUNK_BYTES;
    uint8_t *h_in = nullptr;
    VRG_CUDA_TRY(cudaMallocHost(&h_in, in_bytes + 16 * (size_t)nc));
    std::unique_ptr<uint8_t, void (*)(uint8_t *)> h_guard(h_in, [](uint8_t *x) { cudaFreeHost(x); });
    for (uint32_t c = 0; c < nc; c++) {
        memcpy(h_in + (size_t)c * CHUNK_BYTES, batch[c]->blocks.data(), VRG_CHUNK_BLOCKS);
        memcpy(h_in + (size_t)c * CHUNK_BYTES + VRG_CHUNK_BLOCKS, batch[c]->slabs.data(), 6 * 1024);
    }
    DevBufPtr tmp;
    VRG_TRY(dev_alloc(s, in_bytes + (size_t)nc * VRG_CHUNK_BLOCKS + 16 * (size_t)nc, tmp));
    uint8_t *d_in = (uint8_t *)tmp->ptr;
    uint8_t *d_masks = d_in + in_bytes;
    uint32_t *d_counts = (uint32_t *)(d_masks + (size_t)nc * VRG_CHUNK_BLOCKS);
    VRG_CUDA_TRY(cudaMemcpyAsync(d_in, h_in, in_bytes, cudaMemcpyHostToDevice, s));
    ExtractArgs ea{d_in, d_masks, d_counts, (const vrg_material *)ctx->d_mats->ptr, ctx->n_types};
    k_extract_masks<<<nc, 1024, 0, s>>>(ea);
    VRG_CUDA_TRY(cudaGetLastError());
    uint32_t *h_counts = (uint32_t *)(h_in + in_bytes);
    VRG_CUDA_TRY(cudaMemcpyAsync(h_counts, d_counts, 16 * (size_t)nc, cudaMemcpyDeviceToHost, s));
    VRG_CUDA_TRY(cudaStreamSynchronize(s));

    // layout of the batch: persistent arrays per object + builder inputs (temp)
    uint64_t tot_geo = 0, tot_light = 0, tot_geo_nodes = 0, tot_light_nodes = 0;
    std::vector<uint32_t> geo_off(nc), light_off(nc);
    for (uint32_t c = 0; c < nc; c++) {
        uint32_t F = h_counts[4 * c], Lf = h_counts[4 * c + 1], S = h_counts[4 * c + 2];
        ChunkSummary &cs = batch[c]->sum;
        memset(&cs, 0, sizeof(cs));
        cs.n_faces = F;
        cs.n_tris = 2 * F;
        cs.n_light = 2 * Lf;
        cs.n_geo = S;
        geo_off[c] = (uint32_t)tot_geo;
        light_off[c] = (uint32_t)tot_light;
        tot_geo += S;
        tot_light += 2 * Lf;
        if (S) tot_geo_nodes += 2 * (uint64_t)S - 1;
        if (Lf) tot_light_nodes += 4 * (uint64_t)Lf - 1;
    }
    if (tot_geo + tot_light > 0x7FFFFFFFull) {
        set_error("flush too large");
        return VRG_ERR_UNSUPPORTED;
    }
    const uint64_t n_prims = tot_geo + tot_light;
    const uint64_t n_nodes = tot_geo_nodes + tot_light_nodes;
    auto al = [](uint64_t x) { return (x + 255) & ~255ull; };
    uint64_t o = 0;
    uint64_t o_geo_local = o; o += al(tot_geo * 8);
    uint64_t o_light_tri = o; o += al(tot_light * 4);
    uint64_t o_nodes = o; o += al(n_nodes * sizeof(vrg_bvh_node));
    uint64_t o_perm = o; o += al(n_prims * 4);
    uint64_t o_leaf = o; o += al(n_nodes * 4);
    uint64_t o_payload = o; o += al(tot_light_nodes * 4);
    uint64_t persist_bytes = o;
    DevBufPtr batch_buf;
    VRG_TRY(dev_alloc(s, std::max<uint64_t>(persist_bytes, 256), batch_buf));
    uint8_t *B = (uint8_t *)batch_buf->ptr;
    DevBufPtr bin;
    uint64_t ob = 0;
    uint64_t o_lo = ob; ob += al(n_prims * 16);
    uint64_t o_hi = ob; ob += al(n_prims * 16);
    uint64_t o_cen = ob; ob += al(n_prims * 16);
    uint64_t o_id = ob; ob += al(n_prims * 4);
    uint64_t o_offs = ob; ob += al(4 * (uint64_t)nc * 4);
    VRG_TRY(dev_alloc(s, std::max<uint64_t>(ob, 256), bin));
    uint8_t *I = (uint8_t *)bin->ptr;
    // prim index space: geometry prims first, then light prims
    std::vector<uint32_t> offs(4 * (size_t)nc);
    for (uint32_t c = 0; c < nc; c++) {
        offs[c] = geo_off[c];
        offs[nc + c] = (uint32_t)tot_geo + light_off[c];
        offs[2 * nc + c] = geo_off[c];
        offs[3 * nc + c] = light_off[c];
    }
    uint32_t *d_offs = (uint32_t *)(I + o_offs);
    VRG_CUDA_TRY(cudaMemcpyAsync(d_offs, offs.data(), offs.size() * 4, cudaMemcpyHostToDevice, s));
    WriteArgs wa;
    wa.in = d_in;
    wa.masks = d_masks;
    wa.mats = (const vrg_material *)ctx->d_mats->ptr;
    wa.air = ctx->n_types;
    wa.geo_off = d_offs;
    wa.light_off = d_offs + nc;
    wa.loc_off = d_offs + 2 * nc;
    wa.lloc_off = d_offs + 3 * nc;
    wa.lo = (float4 *)(I + o_lo);
    wa.hi = (float4 *)(I + o_hi);
    wa.cen = (float4 *)(I + o_cen);
    wa.id = (uint32_t *)(I + o_id);
    wa.geo_local = (int2 *)(B + o_geo_local);
    wa.light_tri = (uint32_t *)(B + o_light_tri);
    k_extract_write<<<nc, 1024, 0, s>>>(wa);
    VRG_CUDA_TRY(cudaGetLastError());

    // one batched SAH build: geometry trees (build_tl_bvh semantics over block
    // AABBs) and light trees (build_bl_bvh over light triangles)
    std::vector<SahTree> trees;
    std::vector<uint32_t> tree_node_off(2 * (size_t)nc, INVALID);
    uint64_t node_cursor = 0;
    for (uint32_t c = 0; c < nc; c++) {
        const ChunkSummary &cs = batch[c]->sum;
        if (cs.n_geo) {
            tree_node_off[2 * c] = (uint32_t)node_cursor;
            trees.push_back(SahTree{cs.n_geo, geo_off[c], (uint32_t)node_cursor, 0});
            node_cursor += 2 * (uint64_t)cs.n_geo - 1;
        }
    }
    for (uint32_t c = 0; c < nc; c++) {
        const ChunkSummary &cs = batch[c]->sum;
        if (cs.n_light) {
            tree_node_off[2 * c + 1] = (uint32_t)node_cursor;
            trees.push_back(SahTree{cs.n_light, (uint32_t)tot_geo + light_off[c], (uint32_t)node_cursor, 0});
            node_cursor += 2 * (uint64_t)cs.n_light - 1;
        }
    }
    SahInputs sin{wa.lo, wa.hi, wa.cen, wa.id};
    SahOutputs sout{(vrg_bvh_node *)(B + o_nodes), (uint32_t *)(B + o_perm), (uint32_t *)(B + o_leaf)};
    uint32_t levels = 0;
    VRG_TRY(sah_build(s, trees, (uint32_t)n_prims, (uint32_t)n_nodes, sin, sout, &levels));
    // leaf payloads of the light trees
    for (uint32_t c = 0; c < nc; c++) {
        const ChunkSummary &cs = batch[c]->sum;
        if (!cs.n_light) continue;
        uint32_t nn = 2 * cs.n_light - 1;
        uint32_t off = tree_node_off[2 * c + 1];
        uint32_t payload_off = off - (uint32_t)tot_geo_nodes;
        k_light_leaf_payload<<<(nn + 255) / 256, 256, 0, s>>>(sout.leaf_prim + off, wa.light_tri + light_off[c],
                                                             (uint32_t *)(B + o_payload) + payload_off, nn);
    }
    VRG_CUDA_TRY(cudaGetLastError());
    // root summaries (build_bl_bvh return convention, build.rs:359-371)
    std::vector<vrg_bvh_node> roots(2 * (size_t)nc);
    std::vector<float4> first_lo(2 * (size_t)nc), first_hi(2 * (size_t)nc), first_cen(2 * (size_t)nc);
    for (uint32_t c = 0; c < nc; c++) {
        for (int k = 0; k < 2; k++) {
            uint32_t off = tree_node_off[2 * c + k];
            if (off == INVALID) continue;
            VRG_CUDA_TRY(cudaMemcpyAsync(&roots[2 * c + k], sout.nodes + off, sizeof(vrg_bvh_node),
                                         cudaMemcpyDeviceToHost, s));
            uint32_t p0 = k == 0 ? geo_off[c] : (uint32_t)tot_geo + light_off[c];
            VRG_CUDA_TRY(cudaMemcpyAsync(&first_lo[2 * c + k], wa.lo + p0, 16, cudaMemcpyDeviceToHost, s));
            VRG_CUDA_TRY(cudaMemcpyAsync(&first_hi[2 * c + k], wa.hi + p0, 16, cudaMemcpyDeviceToHost, s));
            VRG_CUDA_TRY(cudaMemcpyAsync(&first_cen[2 * c + k], wa.cen + p0, 16, cudaMemcpyDeviceToHost, s));
        }
    }
    VRG_CUDA_TRY(cudaStreamSynchronize(s));
    for (uint32_t c = 0; c < nc; c++) {
        Object *ob = batch[c];
        ChunkSummary &cs = ob->sum;
        ob->batch = batch_buf;
        ob->geo_local = (const int2 *)(B + o_geo_local) + geo_off[c];
        ob->light_tri = (const uint32_t *)(B + o_light_tri) + light_off[c];
        if (cs.n_geo) {
            uint32_t off = tree_node_off[2 * c];
            ob->geo_nodes = sout.nodes + off;
            ob->geo_leaf = sout.leaf_prim + off;
            ob->geo_perm = sout.perm + geo_off[c];
            const vrg_bvh_node &r = roots[2 * c];
            if (r.left_node_idx == INVALID) {
                const float4 &l = first_lo[2 * c], &h = first_hi[2 * c];
                cs.geo_lo[0] = l.x; cs.geo_lo[1] = l.y; cs.geo_lo[2] = l.z;
                cs.geo_hi[0] = h.x; cs.geo_hi[1] = h.y; cs.geo_hi[2] = h.z;
            } else {
                for (int k = 0; k < 3; k++) { cs.geo_lo[k] = r.min[k]; cs.geo_hi[k] = r.max[k]; }
            }
        }
        if (cs.n_light) {
            uint32_t off = tree_node_off[2 * c + 1];
            ob->light_nodes = sout.nodes + off;
            ob->light_leaf = sout.leaf_prim + off;
            ob->light_perm = sout.perm + tot_geo + light_off[c];
            ob->light_leaf_tri = (const uint32_t *)(B + o_payload) + (off - tot_geo_nodes);
            const vrg_bvh_node &r = roots[2 * c + 1];
            if (r.left_node_idx == INVALID) {
                const float4 &l = first_lo[2 * c + 1], &h = first_hi[2 * c + 1];
                cs.light_lo[0] = l.x; cs.light_lo[1] = l.y; cs.light_lo[2] = l.z;
                cs.light_hi[0] = h.x; cs.light_hi[1] = h.y; cs.light_hi[2] = h.z;
                cs.light_power = first_cen[2 * c + 1].w;
            } else {
                for (int k = 0; k < 3; k++) { cs.light_lo[k] = r.min[k]; cs.light_hi[k] = r.max[k]; }
                cs.light_power = r.power;
            }
        }
        ob->levels = levels;
        ob->flushed = true;
        ob->blocks.clear();
        ob->blocks.shrink_to_fit();
        ob->slabs.clear();
        ob->slabs.shrink_to_fit();
    }
    return VRG_OK;
}

}  // namespace vrg
