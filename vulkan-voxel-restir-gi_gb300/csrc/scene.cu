// Scene commit: the GB300 replacement of Scene::get_tlas (scene.rs:234-497).
//
// On change it rebuilds, on the GPU:
//   * the light top-level BVH over objects with lights (build_tl_bvh over
//     light root AABBs and powers, scene.rs:248-279) and the prim2node map
//     (light_bvh_tl_idx, scene.rs:282-287);
//   * the geometry top-level BVH over objects (same builder), replacing the
//     driver TLAS (scene.rs:728-971);
//   * the traversal layouts: one world-space BVH2 per structure in which
//     each 64-byte node holds both children's boxes (translated to world
//     space and widened by BOX_MARGIN, so culling is conservative) and child
//     references (>= 0 node, < 0 ~record), with top-level leaves linked
//     straight to the object's BLAS root; and 16-byte world-space records per
//     surface block / light triangle.
#include <algorithm>

#include "vrg_internal.h"

namespace vrg {

namespace {

struct InstBuild {
    const vrg_bvh_node *bl;    // BLAS nodes (chunk-local)
    const uint32_t *leaf;      // leaf -> local prim
    const int2 *geo_local;     // geometry only
    const uint32_t *light_tri; // light only
    uint32_t n_prims;
    uint32_t wbase, rbase;
    float off[3];
    int ioff[3];
};

__device__ __forceinline__ int bl_root_ref(const InstBuild &I) {
    return I.bl[0].left_node_idx != INVALID ? (int)I.wbase : ~(int)(I.rbase + I.leaf[0]);
}

// one thread per node of the combined index space [TL nodes | BLAS nodes...]
__global__ void k_wide(const vrg_bvh_node *tl, uint32_t n_tl, const InstBuild *inst, uint32_t n_inst,
                       uint32_t n_total, float4 *wide) {
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n_total) return;
    const vrg_bvh_node *node;
    int k = -1;
    uint32_t j;
    if (g < n_tl) {
        node = &tl[g];
        j = g;
    } else {
        int lo = 0, hi = (int)n_inst - 1;
        while (lo < hi) {  // last instance with wbase <= g
            int mid = (lo + hi + 1) >> 1;
            if (inst[mid].wbase <= g) lo = mid; else hi = mid - 1;
        }
        k = lo;
        j = g - inst[k].wbase;
        node = &inst[k].bl[j];
    }
    if (node->left_node_idx == INVALID) return;
    uint32_t ch[2] = {node->left_node_idx, node->right_node_idx_or_prim_idx};
    float box[2][6];
    int ref[2];
    for (int s = 0; s < 2; s++) {
        const vrg_bvh_node *c;
        float off[3] = {0.0f, 0.0f, 0.0f};
        if (k < 0) {
            c = &tl[ch[s]];
            if (c->left_node_idx != INVALID) ref[s] = (int)ch[s];
            else ref[s] = bl_root_ref(inst[c->right_node_idx_or_prim_idx]);
        } else {
            const InstBuild &I = inst[k];
            c = &I.bl[ch[s]];
            off[0] = I.off[0]; off[1] = I.off[1]; off[2] = I.off[2];
            if (c->left_node_idx != INVALID) ref[s] = (int)(I.wbase + ch[s]);
            else ref[s] = ~(int)(I.rbase + I.leaf[ch[s]]);
        }
        for (int a = 0; a < 3; a++) {
            box[s][a] = (c->min[a] + off[a]) - BOX_MARGIN;
            box[s][3 + a] = (c->max[a] + off[a]) + BOX_MARGIN;
        }
    }
    float4 *w = wide + 4 * (size_t)g;
    w[0] = make_float4(box[0][0], box[0][3], box[0][1], box[0][4]);
    w[1] = make_float4(box[0][2], box[0][5], box[1][0], box[1][3]);
    w[2] = make_float4(box[1][1], box[1][4], box[1][2], box[1][5]);
    w[3] = make_float4(__int_as_float(ref[0]), __int_as_float(ref[1]), 0.0f, 0.0f);
}

// 4-wide traversal node for every inner node g of the combined index space:
// g's children, with each inner child replaced by its own two children
// (so inner children of a 4-wide node are nodes two levels down).  Layout
// (8 float4): lo.x[4], hi.x[4], lo.y[4], hi.y[4], lo.z[4], hi.z[4], refs[4], pad.
// Unused slots hold ref EMPTY_ROOT (skipped by the walk) and a box at +inf.
struct ChildRef {
    const vrg_bvh_node *node;
    float off[3];
    int ref;        // node / ~record
    int inner;      // combined index of an inner child (to expand), -1 otherwise
    int k;          // instance of a BLAS child, -1 for top level
};

__device__ __forceinline__ void child_of(const vrg_bvh_node *tl, const InstBuild *inst, int k, uint32_t c,
                                         ChildRef &out) {
    out.off[0] = out.off[1] = out.off[2] = 0.0f;
    if (k < 0) {
        const vrg_bvh_node *n = &tl[c];
        if (n->left_node_idx != INVALID) {
            out.node = n;
            out.ref = (int)c;
            out.inner = (int)c;
            out.k = -1;
            return;
        }
        // a top-level leaf stands for its object's BLAS root (translated)
        const int kk = (int)n->right_node_idx_or_prim_idx;
        const InstBuild &I = inst[kk];
        out.node = &I.bl[0];
        out.off[0] = I.off[0]; out.off[1] = I.off[1]; out.off[2] = I.off[2];
        out.k = kk;
        if (I.bl[0].left_node_idx != INVALID) {
            out.ref = (int)I.wbase;
            out.inner = (int)I.wbase;
        } else {
            out.ref = ~(int)(I.rbase + I.leaf[0]);
            out.inner = -1;
        }
        return;
    }
    const InstBuild &I = inst[k];
    out.node = &I.bl[c];
    out.off[0] = I.off[0]; out.off[1] = I.off[1]; out.off[2] = I.off[2];
    out.k = k;
    if (out.node->left_node_idx != INVALID) {
        out.ref = (int)(I.wbase + c);
        out.inner = (int)(I.wbase + c);
    } else {
        out.ref = ~(int)(I.rbase + I.leaf[c]);
        out.inner = -1;
    }
}

__global__ void k_wide4(const vrg_bvh_node *tl, uint32_t n_tl, const InstBuild *inst, uint32_t n_inst,
                        uint32_t n_total, float4 *wide4) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n_total) return;
    int k = -1;
    const vrg_bvh_node *node;
    if (g < n_tl) {
        node = &tl[g];
    } else {
        int lo = 0, hi = (int)n_inst - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (inst[mid].wbase <= g) lo = mid; else hi = mid - 1;
        }
        k = lo;
        node = &inst[k].bl[g - inst[k].wbase];
    }
    if (node->left_node_idx == INVALID) return;
    ChildRef lv1[2], out[4];
    child_of(tl, inst, k, node->left_node_idx, lv1[0]);
    child_of(tl, inst, k, node->right_node_idx_or_prim_idx, lv1[1]);
    int n = 0;
    for (int s = 0; s < 2; s++) {
        if (lv1[s].inner >= 0) {
            const vrg_bvh_node *c = lv1[s].node;
            child_of(tl, inst, lv1[s].k, c->left_node_idx, out[n++]);
            child_of(tl, inst, lv1[s].k, c->right_node_idx_or_prim_idx, out[n++]);
        } else {
            out[n++] = lv1[s];
        }
    }
    float b[6][4];
    int refs[4];
    for (int i = 0; i < 4; i++) {
        if (i < n) {
            const vrg_bvh_node *c = out[i].node;
            for (int a = 0; a < 3; a++) {
                b[2 * a][i] = (c->min[a] + out[i].off[a]) - BOX_MARGIN;
                b[2 * a + 1][i] = (c->max[a] + out[i].off[a]) + BOX_MARGIN;
            }
            refs[i] = out[i].ref;
        } else {
            for (int a = 0; a < 3; a++) {
                b[2 * a][i] = INFINITY;
                b[2 * a + 1][i] = INFINITY;
            }
            refs[i] = EMPTY_ROOT;
        }
    }
    float4 *w = wide4 + 8 * (size_t)g;
    for (int r = 0; r < 6; r++) w[r] = make_float4(b[r][0], b[r][1], b[r][2], b[r][3]);
    w[6] = make_float4(__int_as_float(refs[0]), __int_as_float(refs[1]), __int_as_float(refs[2]),
                       __int_as_float(refs[3]));
    w[7] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

__global__ void k_geo_records(const InstBuild *inst, uint32_t k, int4 *rec) {
    const InstBuild I = inst[k];
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < I.n_prims; p += gridDim.x * blockDim.x) {
        int2 l = I.geo_local[p];
        uint32_t blk = (uint32_t)l.x & 0x7FFFu;
        int wx = (int)(blk >> 10) + I.ioff[0], wy = (int)((blk >> 5) & 31u) + I.ioff[1],
            wz = (int)(blk & 31u) + I.ioff[2];
        rec[I.rbase + p] = make_int4((wx & 0xFFFF) | (wz << 16), (wy & 0xFFFF) | (int)(k << 16), l.x, l.y);
    }
}

__global__ void k_light_records(const InstBuild *inst, uint32_t k, int4 *rec) {
    const InstBuild I = inst[k];
    uint32_t n_nodes = 2 * I.n_prims - 1;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n_nodes; j += gridDim.x * blockDim.x) {
        uint32_t p = I.leaf[j];
        if (p == INVALID) continue;
        uint32_t t = I.light_tri[p];
        int wx = (int)(t & 31u) + I.ioff[0], wy = (int)((t >> 5) & 31u) + I.ioff[1],
            wz = (int)((t >> 10) & 31u) + I.ioff[2];
        uint32_t f = (t >> 15) & 7u, h = (t >> 18) & 1u;
        rec[I.rbase + p] = make_int4((wx & 0xFFFF) | (wz << 16), (wy & 0xFFFF) | (int)(k << 16), (int)(f | (h << 3)),
                                     (int)j);
    }
}

// top-level inputs: translated AABB (aabb.rs:75-92 for a translation) and
// centroid (min+max)/2 (build.rs:391-400)
__global__ void k_tl_inputs(const float *in /*[n][10]: lo3 hi3 off3 power*/, const uint32_t *ids, uint32_t n,
                            float4 *lo, float4 *hi, float4 *cen, uint32_t *id_out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *r = in + 10 * (size_t)i;
    float l[3], h[3];
    for (int a = 0; a < 3; a++) {
        float x0 = r[a] + r[6 + a], x1 = r[3 + a] + r[6 + a];
        l[a] = fminf(x0, x1);
        h[a] = fmaxf(x0, x1);
    }
    lo[i] = make_float4(l[0], l[1], l[2], 0.0f);
    hi[i] = make_float4(h[0], h[1], h[2], 0.0f);
    cen[i] = make_float4((l[0] + h[0]) / 2.0f, (l[1] + h[1]) / 2.0f, (l[2] + h[2]) / 2.0f, r[9]);
    id_out[i] = ids[i];
}

// build_bl_bvh inputs (build.rs:262-270): AABB from the three points,
// centroid (v0+v1+v2)/3, power = luminance
__global__ void k_tri_inputs(const float *tris, const float *lum, uint32_t n, float4 *lo, float4 *hi, float4 *cen) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *t = tris + 9 * (size_t)i;
    f3 v0 = f3{t[0], t[1], t[2]}, v1 = f3{t[3], t[4], t[5]}, v2 = f3{t[6], t[7], t[8]};
    lo[i] = make_float4(fminf(fminf(fminf(v0.x, v0.x), v1.x), v2.x), fminf(fminf(fminf(v0.y, v0.y), v1.y), v2.y),
                        fminf(fminf(fminf(v0.z, v0.z), v1.z), v2.z), 0.0f);
    hi[i] = make_float4(fmaxf(fmaxf(fmaxf(v0.x, v0.x), v1.x), v2.x), fmaxf(fmaxf(fmaxf(v0.y, v0.y), v1.y), v2.y),
                        fmaxf(fmaxf(fmaxf(v0.z, v0.z), v1.z), v2.z), 0.0f);
    f3 s = add3(add3(v0, v1), v2);
    cen[i] = make_float4(s.x / 3.0f, s.y / 3.0f, s.z / 3.0f, lum[i]);
}

// ---- lamp-block layout of the light any-hit walk ------------------------
// Light triangles of one block are consecutive in the light records (gen_mesh
// order: block, face, half), so a block boundary is a change of coordinates.
__global__ void k_lamp_flags(const int4 *rec, uint32_t n, uint32_t *flag) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int4 r = rec[i];
    bool start = (i == 0);
    if (!start) {
        const int4 q = rec[i - 1];
        start = (r.x != q.x) || (r.y != q.y);
    }
    flag[i] = start ? 1u : 0u;
}

// single-CTA inclusive scan in place; *total = sum
__global__ void __launch_bounds__(1024) k_scan_inclusive(uint32_t *v, uint32_t n, uint32_t *total) {
    __shared__ uint32_t sh[32];
    __shared__ uint32_t s_carry;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < n; base += 1024) {
        const uint32_t i = base + threadIdx.x;
        uint32_t x = i < n ? v[i] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += t;
        }
        if (lane == 31) sh[w] = x;
        __syncthreads();
        if (w == 0) {
            uint32_t y = sh[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, y, o);
                if (lane >= o) y += t;
            }
            sh[lane] = y;
        }
        __syncthreads();
        const uint32_t carry = s_carry;
        const uint32_t incl = carry + x + (w ? sh[w - 1] : 0u);
        if (i < n) v[i] = incl;
        __syncthreads();
        if (threadIdx.x == 1023) s_carry = incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = s_carry;
}

__global__ void k_lamp_fill(const int4 *rec, const uint32_t *grp, uint32_t n, int4 *lamp, uint32_t *table,
                            float4 *lo, float4 *hi, float4 *cen, uint32_t *id) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int4 r = rec[i];
    const uint32_t g = grp[i] - 1u;
    const int f = r.z & 7, h = (r.z >> 3) & 1;
    table[12u * g + 2u * (uint32_t)f + (uint32_t)h] = (uint32_t)r.w;
    atomicOr(&lamp[g].z, 1 << f);
    if (i == 0 || grp[i - 1] != grp[i]) {
        lamp[g].x = r.x;
        lamp[g].y = r.y;
        lamp[g].w = (int)(12u * g);
        const float x = (float)rec_wx(r), y = (float)rec_wy(r), z = (float)rec_wz(r);
        lo[g] = make_float4(x, y, z, 0.0f);
        hi[g] = make_float4(x + 1.0f, y + 1.0f, z + 1.0f, 0.0f);
        cen[g] = make_float4(x + 0.5f, y + 0.5f, z + 0.5f, 0.0f);
        id[g] = g;
    }
}

// traversal layout of a single-level tree whose leaf prim p is record p
__global__ void k_wide_single(const vrg_bvh_node *nodes, const uint32_t *leaf, uint32_t n_nodes, float4 *wide) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n_nodes) return;
    const vrg_bvh_node &nd = nodes[g];
    if (nd.left_node_idx == INVALID) return;
    const uint32_t ch[2] = {nd.left_node_idx, nd.right_node_idx_or_prim_idx};
    float box[2][6];
    int ref[2];
    for (int s = 0; s < 2; s++) {
        const vrg_bvh_node &c = nodes[ch[s]];
        ref[s] = c.left_node_idx != INVALID ? (int)ch[s] : ~(int)leaf[ch[s]];
        for (int a = 0; a < 3; a++) {
            box[s][a] = c.min[a] - BOX_MARGIN;
            box[s][3 + a] = c.max[a] + BOX_MARGIN;
        }
    }
    float4 *w = wide + 4 * (size_t)g;
    w[0] = make_float4(box[0][0], box[0][3], box[0][1], box[0][4]);
    w[1] = make_float4(box[0][2], box[0][5], box[1][0], box[1][3]);
    w[2] = make_float4(box[1][1], box[1][4], box[1][2], box[1][5]);
    w[3] = make_float4(__int_as_float(ref[0]), __int_as_float(ref[1]), 0.0f, 0.0f);
}

}  // namespace

// The light any-hit walk (nee_pdf's candidate enumeration) runs over a
// world-space SAH BVH of the lamp blocks: a leaf tests the block's emissive
// faces and maps the hit (face, half) to its light-BLAS leaf, so the set of
// light triangles found is the same as walking the triangle light BVH.
static vrg_status build_lamp_layout(Scene *sc, const int4 *light_rec, uint32_t n_light, uint32_t *depth) {
    cudaStream_t s = sc->ctx->stream;
    DevScene &D = sc->dev;
    D.lamp_root = EMPTY_ROOT;
    *depth = 0;
    if (n_light == 0) return VRG_OK;
    auto al = [](uint64_t x) { return (x + 255) & ~255ull; };
    const uint64_t n = n_light;
    uint64_t o = 0;
    uint64_t o_flag = o; o += al(n * 4);
    uint64_t o_tot = o; o += 256;
    uint64_t o_lo = o; o += al(n * 16);
    uint64_t o_hi = o; o += al(n * 16);
    uint64_t o_cen = o; o += al(n * 16);
    uint64_t o_id = o; o += al(n * 4);
    uint64_t o_perm = o; o += al(n * 4);
    uint64_t o_nodes = o; o += al(2 * n * sizeof(vrg_bvh_node));
    uint64_t o_leaf = o; o += al(2 * n * 4);
    uint64_t o_rec = o; o += al(n * 16);
    uint64_t o_tab = o; o += al(n * 12 * 4);
    uint64_t o_wide = o; o += al(2 * n * 64);
    DevBufPtr buf;
    VRG_TRY(dev_alloc(s, o, buf));
    uint8_t *B = (uint8_t *)buf->ptr;
    uint32_t *flag = (uint32_t *)(B + o_flag), *tot = (uint32_t *)(B + o_tot);
    int4 *lamp = (int4 *)(B + o_rec);
    uint32_t *table = (uint32_t *)(B + o_tab);
    VRG_CUDA_TRY(cudaMemsetAsync(lamp, 0, n * 16, s));
    VRG_CUDA_TRY(cudaMemsetAsync(table, 0xFF, n * 48, s));
    k_lamp_flags<<<(uint32_t)((n + 255) / 256), 256, 0, s>>>(light_rec, n_light, flag);
    k_scan_inclusive<<<1, 1024, 0, s>>>(flag, n_light, tot);
    k_lamp_fill<<<(uint32_t)((n + 255) / 256), 256, 0, s>>>(light_rec, flag, n_light, lamp, table,
                                                           (float4 *)(B + o_lo), (float4 *)(B + o_hi),
                                                           (float4 *)(B + o_cen), (uint32_t *)(B + o_id));
    VRG_CUDA_TRY(cudaGetLastError());
    uint32_t n_lamps = 0;
    VRG_CUDA_TRY(cudaMemcpyAsync(&n_lamps, tot, 4, cudaMemcpyDeviceToHost, s));
    VRG_CUDA_TRY(cudaStreamSynchronize(s));
    std::vector<SahTree> trees{SahTree{n_lamps, 0, 0, 0}};
    SahInputs in{(const float4 *)(B + o_lo), (const float4 *)(B + o_hi), (const float4 *)(B + o_cen),
                 (const uint32_t *)(B + o_id)};
    vrg_bvh_node *nodes = (vrg_bvh_node *)(B + o_nodes);
    uint32_t *leaf = (uint32_t *)(B + o_leaf);
    SahOutputs out{nodes, (uint32_t *)(B + o_perm), leaf};
    uint32_t levels = 0;
    VRG_TRY(sah_build(s, trees, n_lamps, 2 * n_lamps - 1, in, out, &levels));
    float4 *wide = (float4 *)(B + o_wide);
    if (n_lamps > 1) {
        k_wide_single<<<(2 * n_lamps - 1 + 255) / 256, 256, 0, s>>>(nodes, leaf, 2 * n_lamps - 1, wide);
        VRG_CUDA_TRY(cudaGetLastError());
        D.lamp_root = 0;
    } else {
        D.lamp_root = ~0;
    }
    D.lamp_wide = wide;
    D.lamp_rec = lamp;
    D.lamp_table = table;
    sc->lamp_buf = buf;
    *depth = levels + 2;
    return VRG_OK;
}

vrg_status standalone_sah(Context *ctx, bool tri, uint32_t count, const uint32_t *n, const uint32_t *prim_offset,
                          const uint32_t *node_offset, const float *prims, const float *translations,
                          const float *power, const uint32_t *ids, vrg_bvh_node *nodes_out, uint32_t *order_out) {
    cudaStream_t s = ctx->stream;
    uint64_t total_prims = 0, total_nodes = 0;
    std::vector<SahTree> trees(count);
    for (uint32_t t = 0; t < count; t++) {
        trees[t] = SahTree{n[t], prim_offset[t], node_offset[t], 0};
        total_prims = std::max<uint64_t>(total_prims, (uint64_t)prim_offset[t] + n[t]);
        if (n[t]) total_nodes = std::max<uint64_t>(total_nodes, (uint64_t)node_offset[t] + 2 * (uint64_t)n[t] - 1);
    }
    if (total_prims == 0) return VRG_OK;
    if (total_prims > 0x3FFFFFFFull || total_nodes > 0x7FFFFFFFull) return VRG_ERR_UNSUPPORTED;
    auto al = [](uint64_t x) { return (x + 255) & ~255ull; };
    const uint64_t in_floats = tri ? 9 : 10;
    uint64_t o = 0;
    uint64_t o_raw = o; o += al(total_prims * in_floats * 4);
    uint64_t o_pw = o; o += al(total_prims * 4);
    uint64_t o_lo = o; o += al(total_prims * 16);
    uint64_t o_hi = o; o += al(total_prims * 16);
    uint64_t o_cen = o; o += al(total_prims * 16);
    uint64_t o_id = o; o += al(total_prims * 4);
    uint64_t o_perm = o; o += al(total_prims * 4);
    uint64_t o_nodes = o; o += al(total_nodes * sizeof(vrg_bvh_node));
    uint64_t o_leaf = o; o += al(total_nodes * 4);
    DevBufPtr b;
    VRG_TRY(dev_alloc(s, o, b));
    uint8_t *B = (uint8_t *)b->ptr;
    if (tri) {
        VRG_CUDA_TRY(cudaMemcpyAsync(B + o_raw, prims, total_prims * 36, cudaMemcpyHostToDevice, s));
        VRG_CUDA_TRY(cudaMemcpyAsync(B + o_pw, power, total_prims * 4, cudaMemcpyHostToDevice, s));
        k_tri_inputs<<<(uint32_t)((total_prims + 255) / 256), 256, 0, s>>>(
            (const float *)(B + o_raw), (const float *)(B + o_pw), (uint32_t)total_prims, (float4 *)(B + o_lo),
            (float4 *)(B + o_hi), (float4 *)(B + o_cen));
        VRG_CUDA_TRY(cudaMemcpyAsync(B + o_id, ids, total_prims * 4, cudaMemcpyHostToDevice, s));
    } else {
        std::vector<float> tin(10 * total_prims);
        for (uint64_t i = 0; i < total_prims; i++) {
            for (int a = 0; a < 3; a++) {
                tin[10 * i + a] = prims[6 * i + a];
                tin[10 * i + 3 + a] = prims[6 * i + 3 + a];
                tin[10 * i + 6 + a] = translations ? translations[3 * i + a] : 0.0f;
            }
            tin[10 * i + 9] = power[i];
        }
        VRG_CUDA_TRY(cudaMemcpyAsync(B + o_raw, tin.data(), total_prims * 40, cudaMemcpyHostToDevice, s));
        VRG_CUDA_TRY(cudaMemcpyAsync(B + o_pw, ids, total_prims * 4, cudaMemcpyHostToDevice, s));
        k_tl_inputs<<<(uint32_t)((total_prims + 255) / 256), 256, 0, s>>>(
            (const float *)(B + o_raw), (const uint32_t *)(B + o_pw), (uint32_t)total_prims, (float4 *)(B + o_lo),
            (float4 *)(B + o_hi), (float4 *)(B + o_cen), (uint32_t *)(B + o_id));
        VRG_CUDA_TRY(cudaStreamSynchronize(s));  // tin goes out of scope
    }
    VRG_CUDA_TRY(cudaGetLastError());
    SahInputs in{(const float4 *)(B + o_lo), (const float4 *)(B + o_hi), (const float4 *)(B + o_cen),
                 (const uint32_t *)(B + o_id)};
    SahOutputs out{(vrg_bvh_node *)(B + o_nodes), (uint32_t *)(B + o_perm), (uint32_t *)(B + o_leaf)};
    uint32_t levels = 0;
    VRG_TRY(sah_build(s, trees, (uint32_t)total_prims, (uint32_t)total_nodes, in, out, &levels));
    if (nodes_out)
        VRG_CUDA_TRY(cudaMemcpyAsync(nodes_out, out.nodes, total_nodes * sizeof(vrg_bvh_node), cudaMemcpyDeviceToHost, s));
    if (order_out) VRG_CUDA_TRY(cudaMemcpyAsync(order_out, out.perm, total_prims * 4, cudaMemcpyDeviceToHost, s));
    VRG_CUDA_TRY(cudaStreamSynchronize(s));
    return VRG_OK;
}

vrg_status scene_commit(Scene *sc) {
    Context *ctx = sc->ctx;
    cudaStream_t s = ctx->stream;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        std::vector<Object *> pend;
        pend.swap(ctx->pending);
        vrg_status st = extract_and_build(ctx, pend);
        if (st != VRG_OK) {
            ctx->pending.insert(ctx->pending.end(), pend.begin(), pend.end());
            return st;
        }
        for (Object *o : pend)  // drop the pending list's reference
            if (--o->refs == 0) delete o;
    }
    if (!sc->dirty) return VRG_OK;
    // instances: non-empty objects in key order (scene.rs:245-260)
    sc->inst_objs.clear();
    sc->inst_off.clear();
    for (auto &kv : sc->objects) {
        Object *o = kv.second.obj;
        if (!o->flushed) {
            set_error("object not flushed");
            return VRG_ERR_STATE;
        }
        if (o->sum.n_tris == 0) continue;
        sc->inst_objs.push_back(o);
        sc->inst_off.push_back({kv.second.off[0], kv.second.off[1], kv.second.off[2]});
    }
    const uint32_t ni = (uint32_t)sc->inst_objs.size();
    if (ni > 65535) {
        set_error("more than 65535 instances");
        return VRG_ERR_UNSUPPORTED;
    }
    // top-level inputs
    std::vector<float> tl_in;
    std::vector<uint32_t> tl_ids;
    uint32_t n_light_inst = 0, n_geo_inst = 0;
    for (uint32_t i = 0; i < ni; i++) {
        const ChunkSummary &cs = sc->inst_objs[i]->sum;
        if (cs.n_light == 0) continue;
        const float *o = sc->inst_off[i].data();
        float r[10] = {cs.light_lo[0], cs.light_lo[1], cs.light_lo[2], cs.light_hi[0], cs.light_hi[1],
                       cs.light_hi[2], o[0], o[1], o[2], cs.light_power};
        tl_in.insert(tl_in.end(), r, r + 10);
        tl_ids.push_back(i);
        n_light_inst++;
    }
    for (uint32_t i = 0; i < ni; i++) {
        const ChunkSummary &cs = sc->inst_objs[i]->sum;
        if (cs.n_geo == 0) continue;
        const float *o = sc->inst_off[i].data();
        float r[10] = {cs.geo_lo[0], cs.geo_lo[1], cs.geo_lo[2], cs.geo_hi[0], cs.geo_hi[1], cs.geo_hi[2],
                       o[0], o[1], o[2], 0.0f};
        tl_in.insert(tl_in.end(), r, r + 10);
        tl_ids.push_back(i);
        n_geo_inst++;
    }
    const uint32_t n_tl_prims = n_light_inst + n_geo_inst;
    const uint32_t n_light_tl = n_light_inst ? 2 * n_light_inst - 1 : 1;
    const uint32_t n_geo_tl = n_geo_inst ? 2 * n_geo_inst - 1 : 0;
    // per-instance layout
    uint64_t geo_nodes = 0, geo_recs = 0, light_nodes = 0, light_recs = 0;
    std::vector<InstBuild> gb(ni), lb(ni);
    uint32_t max_levels = 0;
    for (uint32_t i = 0; i < ni; i++) {
        Object *o = sc->inst_objs[i];
        const ChunkSummary &cs = o->sum;
        for (int a = 0; a < 3; a++) {
            float t = sc->inst_off[i][a];
            if (t != floorf(t) || fabsf(t) > 16384.0f) {
                set_error("instance translation must be integral and within +-16384");
                return VRG_ERR_UNSUPPORTED;
            }
            gb[i].off[a] = lb[i].off[a] = t;
            gb[i].ioff[a] = lb[i].ioff[a] = (int)t;
        }
        gb[i].bl = o->geo_nodes;
        gb[i].leaf = o->geo_leaf;
        gb[i].geo_local = o->geo_local;
        gb[i].light_tri = nullptr;
        gb[i].n_prims = cs.n_geo;
        gb[i].wbase = n_geo_tl + (uint32_t)geo_nodes;
        gb[i].rbase = (uint32_t)geo_recs;
        geo_nodes += cs.n_geo ? 2 * (uint64_t)cs.n_geo - 1 : 0;
        geo_recs += cs.n_geo;
        lb[i].bl = o->light_nodes;
        lb[i].leaf = o->light_leaf;
        lb[i].geo_local = nullptr;
        lb[i].light_tri = o->light_tri;
        lb[i].n_prims = cs.n_light;
        lb[i].wbase = n_light_tl + (uint32_t)light_nodes;
        lb[i].rbase = (uint32_t)light_recs;
        light_nodes += cs.n_light ? 2 * (uint64_t)cs.n_light - 1 : 0;
        light_recs += cs.n_light;
        max_levels = std::max(max_levels, o->levels);
    }
    // instances without geometry/lights must not appear in the binary search
    // of k_wide (wbase stays monotone: they own zero nodes), fine as is.
    auto al = [](uint64_t x) { return (x + 255) & ~255ull; };
    uint64_t o = 0;
    const uint64_t n_geo_wide = n_geo_tl + geo_nodes;
    uint64_t o_gw = o; o += al(n_geo_wide * 128);
    uint64_t o_gr = o; o += al(geo_recs * 16);
    uint64_t o_lr = o; o += al(light_recs * 16);
    uint64_t o_tln = o; o += al((uint64_t)(n_light_tl + n_geo_tl) * sizeof(vrg_bvh_node));
    uint64_t o_inst = o; o += al((uint64_t)ni * sizeof(InstDev));
    uint64_t o_gb = o; o += al((uint64_t)ni * sizeof(InstBuild));
    uint64_t o_lb = o; o += al((uint64_t)ni * sizeof(InstBuild));
    // TL build scratch
    uint64_t o_tin = o; o += al((uint64_t)n_tl_prims * 40);
    uint64_t o_tid = o; o += al((uint64_t)n_tl_prims * 4);
    uint64_t o_tlo = o; o += al((uint64_t)n_tl_prims * 16);
    uint64_t o_thi = o; o += al((uint64_t)n_tl_prims * 16);
    uint64_t o_tcen = o; o += al((uint64_t)n_tl_prims * 16);
    uint64_t o_tidd = o; o += al((uint64_t)n_tl_prims * 4);
    uint64_t o_tperm = o; o += al((uint64_t)n_tl_prims * 4);
    uint64_t o_tleaf = o; o += al((uint64_t)(n_light_tl + n_geo_tl) * 4);
    DevBufPtr buf;
    VRG_TRY(dev_alloc(s, std::max<uint64_t>(o, 256), buf));
    uint8_t *B = (uint8_t *)buf->ptr;
    vrg_bvh_node *d_tl = (vrg_bvh_node *)(B + o_tln);  // [light TL | geometry TL]
    uint32_t tl_levels = 0;
    if (n_tl_prims) {
        VRG_CUDA_TRY(cudaMemcpyAsync(B + o_tin, tl_in.data(), tl_in.size() * 4, cudaMemcpyHostToDevice, s));
        VRG_CUDA_TRY(cudaMemcpyAsync(B + o_tid, tl_ids.data(), tl_ids.size() * 4, cudaMemcpyHostToDevice, s));
        k_tl_inputs<<<(n_tl_prims + 127) / 128, 128, 0, s>>>((const float *)(B + o_tin), (const uint32_t *)(B + o_tid),
                                                              n_tl_prims, (float4 *)(B + o_tlo), (float4 *)(B + o_thi),
                                                              (float4 *)(B + o_tcen), (uint32_t *)(B + o_tidd));
        VRG_CUDA_TRY(cudaGetLastError());
        std::vector<SahTree> trees;
        if (n_light_inst) trees.push_back(SahTree{n_light_inst, 0, 0, 0});
        if (n_geo_inst) trees.push_back(SahTree{n_geo_inst, n_light_inst, n_light_tl, 0});
        SahInputs in{(const float4 *)(B + o_tlo), (const float4 *)(B + o_thi), (const float4 *)(B + o_tcen),
                     (const uint32_t *)(B + o_tidd)};
        SahOutputs out{d_tl, (uint32_t *)(B + o_tperm), (uint32_t *)(B + o_tleaf)};
        VRG_TRY(sah_build(s, trees, n_tl_prims, n_light_tl + n_geo_tl, in, out, &tl_levels));
    }
    if (!n_light_inst) {  // dummy node (BvhNode::default, bvh/mod.rs:27-38; scene.rs:276-277)
        vrg_bvh_node d;
        d.left_node_idx = d.right_node_idx_or_prim_idx = d.parent_idx = INVALID;
        for (int a = 0; a < 3; a++) d.min[a] = d.max[a] = 0.0f;
        d.power = 0.0f;
        VRG_CUDA_TRY(cudaMemcpyAsync(d_tl, &d, sizeof(d), cudaMemcpyHostToDevice, s));
    }
    sc->h_light_tl.resize(n_light_tl);
    sc->h_geo_tl.resize(n_geo_tl);
    VRG_CUDA_TRY(cudaMemcpyAsync(sc->h_light_tl.data(), d_tl, n_light_tl * sizeof(vrg_bvh_node),
                                 cudaMemcpyDeviceToHost, s));
    if (n_geo_tl)
        VRG_CUDA_TRY(cudaMemcpyAsync(sc->h_geo_tl.data(), d_tl + n_light_tl, n_geo_tl * sizeof(vrg_bvh_node),
                                     cudaMemcpyDeviceToHost, s));
    VRG_CUDA_TRY(cudaStreamSynchronize(s));
    // instance table (prim2node)
    std::vector<InstDev> idev(ni);
    for (uint32_t i = 0; i < ni; i++) {
        for (int a = 0; a < 3; a++) idev[i].off[a] = sc->inst_off[i][a];
        idev[i].light_bvh_tl_idx = 0;
        idev[i].light_bl = sc->inst_objs[i]->light_nodes;
        idev[i].light_leaf_tri = sc->inst_objs[i]->light_leaf_tri;
    }
    if (n_light_inst)
        for (uint32_t j = 0; j < n_light_tl; j++)
            if (sc->h_light_tl[j].left_node_idx == INVALID) idev[sc->h_light_tl[j].right_node_idx_or_prim_idx].light_bvh_tl_idx = j;
    VRG_CUDA_TRY(cudaMemcpyAsync(B + o_inst, idev.data(), ni * sizeof(InstDev), cudaMemcpyHostToDevice, s));
    VRG_CUDA_TRY(cudaMemcpyAsync(B + o_gb, gb.data(), ni * sizeof(InstBuild), cudaMemcpyHostToDevice, s));
    VRG_CUDA_TRY(cudaMemcpyAsync(B + o_lb, lb.data(), ni * sizeof(InstBuild), cudaMemcpyHostToDevice, s));
    const InstBuild *d_gb = (const InstBuild *)(B + o_gb), *d_lb = (const InstBuild *)(B + o_lb);
    // wide layouts + records
    if (n_geo_wide) {
        k_wide4<<<(uint32_t)((n_geo_wide + 255) / 256), 256, 0, s>>>(d_tl + n_light_tl, n_geo_tl, d_gb, ni,
                                                                    (uint32_t)n_geo_wide, (float4 *)(B + o_gw));
        VRG_CUDA_TRY(cudaGetLastError());
    }
    for (uint32_t i = 0; i < ni; i++) {
        if (gb[i].n_prims) {
            k_geo_records<<<std::min(64u, (gb[i].n_prims + 255) / 256), 256, 0, s>>>(d_gb, i, (int4 *)(B + o_gr));
        }
        if (lb[i].n_prims) {
            k_light_records<<<std::min(64u, (2 * lb[i].n_prims + 254) / 256), 256, 0, s>>>(d_lb, i, (int4 *)(B + o_lr));
        }
    }
    VRG_CUDA_TRY(cudaGetLastError());
    // roots
    DevScene &D = sc->dev;
    D.geo_wide = (const float4 *)(B + o_gw);
    D.geo_rec = (const int4 *)(B + o_gr);

    D.light_tl = d_tl;
    D.inst = (const InstDev *)(B + o_inst);
    D.mats = (const vrg_material *)ctx->d_mats->ptr;
    D.n_inst = ni;
    auto root_of = [&](const std::vector<vrg_bvh_node> &tl, uint32_t n_tl, const std::vector<InstBuild> &ib,
                       bool light) -> vrg_status {
        (void)light;
        int *dst = &D.geo_root;
        if (n_tl == 0) { *dst = EMPTY_ROOT; return VRG_OK; }
        if (tl[0].left_node_idx != INVALID) { *dst = 0; return VRG_OK; }
        // single object: the TL root is a leaf -> its BLAS root
        uint32_t k = tl[0].right_node_idx_or_prim_idx;
        vrg_bvh_node r;
        VRG_CUDA_TRY(cudaMemcpy(&r, ib[k].bl, sizeof(r), cudaMemcpyDeviceToHost));
        if (r.left_node_idx != INVALID) { *dst = (int)ib[k].wbase; return VRG_OK; }
        uint32_t p0;
        VRG_CUDA_TRY(cudaMemcpy(&p0, ib[k].leaf, 4, cudaMemcpyDeviceToHost));
        *dst = ~(int)(ib[k].rbase + p0);
        return VRG_OK;
    };
    VRG_TRY(root_of(sc->h_geo_tl, n_geo_tl, gb, false));
    uint32_t lamp_depth = 0;
    VRG_TRY(build_lamp_layout(sc, (const int4 *)(B + o_lr), (uint32_t)light_recs, &lamp_depth));
    // the 4-wide walk pushes up to 3 refs per 4-wide level (half the binary depth)
    sc->depth_bound = std::max(3 * ((tl_levels + max_levels + 4 + 1) / 2) + 1, lamp_depth);
    if (sc->depth_bound >= (uint32_t)TRAV_STACK) {
        set_error("BVH depth bound %u exceeds the traversal stack (%d)", sc->depth_bound, TRAV_STACK);
        return VRG_ERR_UNSUPPORTED;
    }
    VRG_CUDA_TRY(cudaStreamSynchronize(s));
    sc->d_buf = buf;
    sc->dirty = false;
    for (Object *r : sc->retired) {
        if (--r->refs == 0) delete r;
    }
    sc->retired.clear();
    return VRG_OK;
}

}  // namespace vrg
