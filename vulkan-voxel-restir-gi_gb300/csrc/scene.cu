// Scene commit: the GB300 replacement of Scene::get_tlas (scene.rs:234-497).
//
// On change it rebuilds, on the GPU:
//   * the light top-level BVH over objects with lights (build_tl_bvh over
//     light root AABBs and powers, scene.rs:248-279) and the prim2node map
//     (light_bvh_tl_idx, scene.rs:282-287);
//   * the geometry top-level BVH over objects (same builder), replacing the
//     driver TLAS (scene.rs:728-971);
//   * the closest-hit traversal layout: a world-space 4-wide BVH over the
//     combined [top level | every object's BLAS] tree, in which each
//     128-byte node holds its (up to) four grandchild-level children's boxes
//     as SoA (translated to world space and widened by BOX_MARGIN, so culling
//     is conservative) and child references (>= 0 node, < 0 ~record), with
//     top-level leaves linked straight to the object's BLAS root; and
//     16-byte world-space records per surface block / light triangle;
//   * the light any-hit layout: a 2-wide world-space BVH over lamp blocks.
// Several scenes commit together with one SAH build for all their top-level
// trees and one for all their lamp trees.
#include <algorithm>
#include <cstring>

#include "vrg_internal.h"

namespace vrg {

namespace {

struct InstBuild {
    const vrg_bvh_node *bl;    // BLAS nodes (object space)
    const uint32_t *leaf;      // leaf -> local prim
    const int2 *geo_local;     // geometry of a chunk only
    const uint32_t *light_tri; // light only (mesh: triangle index per light prim)
    const float4 *mesh_tri;    // mesh only: object-space triangles
    uint32_t n_prims;
    uint32_t wbase, rbase;     // first traversal node; first record (blocks / light prims) it owns
    uint32_t tbase;            // first world-space triangle record it owns (meshes)
    uint32_t refbase;          // record index of its local prim 0 in the leaf references
    uint32_t flags;            // INST_*
    float off[3];
    int ioff[3];
    float m[12];               // the transform, row-major [R|t]
};

__device__ __forceinline__ int bl_root_ref(const InstBuild &I) {
    return I.bl[0].left_node_idx != INVALID ? (int)I.wbase : ~(int)(I.refbase + I.leaf[0]);
}

// world-space box of an object-space node box: translated, or for another
// transform the AABB of its 8 transformed corners (Aabb::transform, aabb.rs:75-92)
__device__ __forceinline__ void world_box(const vrg_bvh_node *c, const InstBuild *I, const float off[3], float lo[3],
                                          float hi[3]) {
    if (!I || !(I->flags & INST_XFORM)) {
        for (int a = 0; a < 3; a++) {
            lo[a] = c->min[a] + off[a];
            hi[a] = c->max[a] + off[a];
        }
        return;
    }
    const float4 r0 = make_float4(I->m[0], I->m[1], I->m[2], I->m[3]);
    const float4 r1 = make_float4(I->m[4], I->m[5], I->m[6], I->m[7]);
    const float4 r2 = make_float4(I->m[8], I->m[9], I->m[10], I->m[11]);
    for (int k = 0; k < 8; k++) {
        const f3 p = xf_rows(r0, r1, r2, f3{(k & 4) ? c->max[0] : c->min[0], (k & 2) ? c->max[1] : c->min[1],
                                            (k & 1) ? c->max[2] : c->min[2]});
        if (k == 0) {
            lo[0] = hi[0] = p.x; lo[1] = hi[1] = p.y; lo[2] = hi[2] = p.z;
        } else {
            lo[0] = fminf(lo[0], p.x); hi[0] = fmaxf(hi[0], p.x);
            lo[1] = fminf(lo[1], p.y); hi[1] = fmaxf(hi[1], p.y);
            lo[2] = fminf(lo[2], p.z); hi[2] = fmaxf(hi[2], p.z);
        }
    }
}

// 4-wide traversal node for every inner node g of the combined index space:
// g's children, with each inner child replaced by its own two children
// (so inner children of a 4-wide node are nodes two levels down).  Layout
// (8 float4): lo.x[4], hi.x[4], lo.y[4], hi.y[4], lo.z[4], hi.z[4], refs[4], pad.
// Unused slots hold ref EMPTY_ROOT and the inverted box lo = +inf, hi = -inf,
// which the slab test never enters (see slab4 in trace.cu).
struct ChildRef {
    const vrg_bvh_node *node;
    float off[3];
    int ref;        // node / ~record
    int inner;      // combined index of an inner child (to expand), -1 otherwise
    int k;          // instance of a BLAS child (its box is in that instance's object space), -1 for top level
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
            out.ref = ~(int)(I.refbase + I.leaf[0]);
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
        out.ref = ~(int)(I.refbase + I.leaf[c]);
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
            float lo[3], hi[3];
            world_box(out[i].node, out[i].k >= 0 ? &inst[out[i].k] : nullptr, out[i].off, lo, hi);
            for (int a = 0; a < 3; a++) {
                b[2 * a][i] = lo[a] - BOX_MARGIN;
                b[2 * a + 1][i] = hi[a] + BOX_MARGIN;
            }
            refs[i] = out[i].ref;
        } else {
            for (int a = 0; a < 3; a++) {  // an inverted box: no ray enters it
                b[2 * a][i] = INFINITY;
                b[2 * a + 1][i] = -INFINITY;
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

// last instance k with key(k) <= g (keys non-decreasing, key(0) <= g).  An
// instance that owns no nodes or records shares its key with the next one,
// so the last of equal keys is the owner.
template <typename Key>
__device__ __forceinline__ uint32_t inst_of(const InstBuild *inst, uint32_t n_inst, uint32_t g, Key key) {
    uint32_t lo = 0, hi = n_inst - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (key(inst[mid]) <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// world-space surface-block records of every instance, one thread per record
// (records of instance k start at its rbase)
__global__ void k_geo_records(const InstBuild *inst, uint32_t n_inst, uint32_t n_rec, int4 *rec) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < n_rec; g += gridDim.x * blockDim.x) {
        const uint32_t k = inst_of(inst, n_inst, g, [](const InstBuild &I) { return I.rbase; });
        const InstBuild &I = inst[k];
        const uint32_t p = g - I.rbase;
        const int2 l = I.geo_local[p];
        const uint32_t blk = (uint32_t)l.x & 0x7FFFu;
        const int wx = (int)(blk >> 10) + I.ioff[0], wy = (int)((blk >> 5) & 31u) + I.ioff[1],
                  wz = (int)(blk & 31u) + I.ioff[2];
        rec[g] = make_int4((wx & 0xFFFF) | (wz << 16), (wy & 0xFFFF) | (int)(k << 16), l.x, l.y);
    }
}

// world-space triangle records of every mesh instance, one thread per record
// (records of instance k start at its tbase): (v0, instance) (v1, triangle)
// (v2, material slot) — the triangleTransform of the vertex buffer
// (raytrace.rs:155-159)
__global__ void k_tri_records(const InstBuild *inst, uint32_t n_inst, uint32_t n_rec, float4 *rec) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < n_rec; g += gridDim.x * blockDim.x) {
        const uint32_t k = inst_of(inst, n_inst, g, [](const InstBuild &I) { return I.tbase; });
        const InstBuild &I = inst[k];
        const uint32_t t = g - I.tbase;
        const float4 *q = I.mesh_tri + 3 * (size_t)t;
        const float4 r0 = make_float4(I.m[0], I.m[1], I.m[2], I.m[3]);
        const float4 r1 = make_float4(I.m[4], I.m[5], I.m[6], I.m[7]);
        const float4 r2 = make_float4(I.m[8], I.m[9], I.m[10], I.m[11]);
        const uint32_t w[3] = {k, t, __float_as_uint(q[0].w)};
        for (int j = 0; j < 3; j++) {
            const f3 p = f3{q[j].x, q[j].y, q[j].z};
            const f3 v = (I.flags & INST_XFORM) ? xf_rows(r0, r1, r2, p) : add3(p, f3{I.off[0], I.off[1], I.off[2]});
            rec[3 * (size_t)g + j] = make_float4(v.x, v.y, v.z, __uint_as_float(w[j]));
        }
    }
}

// The light-BLAS nodes of an instance whose transform is not a translation,
// with min and max replaced by the transform applied to them: the v000 and
// v111 of nodeImportance (raytrace.rs:184-185, nee_pdf.rs:127-128), computed
// once here so the light walks move these nodes by a zero translation
__global__ void k_xform_light_nodes(const vrg_bvh_node *in, uint32_t n, float4 r0, float4 r1, float4 r2,
                                    vrg_bvh_node *out) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    vrg_bvh_node nd = in[j];
    const f3 a = xf_rows(r0, r1, r2, f3{nd.min[0], nd.min[1], nd.min[2]});
    const f3 b = xf_rows(r0, r1, r2, f3{nd.max[0], nd.max[1], nd.max[2]});
    nd.min[0] = a.x; nd.min[1] = a.y; nd.min[2] = a.z;
    nd.max[0] = b.x; nd.max[1] = b.y; nd.max[2] = b.z;
    out[j] = nd;
}

// world-space light-triangle records of every instance, one thread per light
// BLAS node (node j of instance k is index wbase - base + j); leaves write
// their prim's record
__global__ void k_light_records(const InstBuild *inst, uint32_t n_inst, uint32_t base, uint32_t n_nodes_all,
                                int4 *rec) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < n_nodes_all; g += gridDim.x * blockDim.x) {
        const uint32_t k =
            inst_of(inst, n_inst, g + base, [](const InstBuild &I) { return I.wbase; });
        const InstBuild &I = inst[k];
        if (I.n_prims == 0) continue;
        const uint32_t j = g + base - I.wbase;
        if (j >= 2 * I.n_prims - 1) continue;
        const uint32_t p = I.leaf[j];
        if (p == INVALID) continue;
        const uint32_t t = I.light_tri[p];
        if (I.flags & INST_MESH) {
            // a light triangle of a mesh: its own lamp (x is the record index,
            // unique), z = bit 31 | its world-space triangle record
            rec[I.rbase + p] = make_int4((int)(I.rbase + p), (int)(0xFFFFu | (k << 16)),
                                         (int)(0x80000000u | (I.tbase + t)), (int)j);
            continue;
        }
        const int wx = (int)(t & 31u) + I.ioff[0], wy = (int)((t >> 5) & 31u) + I.ioff[1],
                  wz = (int)((t >> 10) & 31u) + I.ioff[2];
        const uint32_t f = (t >> 15) & 7u, h = (t >> 18) & 1u;
        rec[I.rbase + p] = make_int4((wx & 0xFFFF) | (wz << 16), (wy & 0xFFFF) | (int)(k << 16),
                                     (int)(f | (h << 3)), (int)j);
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

__global__ void k_lamp_fill(const int4 *rec, const uint32_t *grp, uint32_t n, const float4 *tri_rec, int4 *lamp,
                            uint32_t *table, float4 *lo, float4 *hi, float4 *cen, uint32_t *id) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int4 r = rec[i];
    const uint32_t g = grp[i] - 1u;
    if (r.z < 0) {  // a mesh light triangle: table (leaf, triangle record), its world AABB
        const uint32_t t = (uint32_t)r.z & 0x7FFFFFFFu;
        table[12u * g] = (uint32_t)r.w;
        table[12u * g + 1u] = t;
        lamp[g] = make_int4(r.x, r.y, (int)0x80000000u, (int)(12u * g));
        const float4 a = tri_rec[3 * (size_t)t], b = tri_rec[3 * (size_t)t + 1], c = tri_rec[3 * (size_t)t + 2];
        const float4 l = make_float4(fminf(fminf(a.x, b.x), c.x), fminf(fminf(a.y, b.y), c.y),
                                     fminf(fminf(a.z, b.z), c.z), 0.0f);
        const float4 h = make_float4(fmaxf(fmaxf(a.x, b.x), c.x), fmaxf(fmaxf(a.y, b.y), c.y),
                                     fmaxf(fmaxf(a.z, b.z), c.z), 0.0f);
        lo[g] = l;
        hi[g] = h;
        cen[g] = make_float4((l.x + h.x) * 0.5f, (l.y + h.y) * 0.5f, (l.z + h.z) * 0.5f, 0.0f);
        id[g] = g;
        return;
    }
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

// 4-wide traversal layout of a single-level tree whose leaf prim p is record p
// (the lamp-block tree): for every inner node, its children with each inner
// child replaced by that child's two children; the layout of k_wide4
// (lo/hi x, y, z SoA, refs: >= 0 node, < 0 ~record, EMPTY_ROOT unused)
__global__ void k_wide4_single(const vrg_bvh_node *nodes, const uint32_t *leaf, uint32_t n_nodes, float4 *wide4) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n_nodes) return;
    const vrg_bvh_node &nd = nodes[g];
    if (nd.left_node_idx == INVALID) return;
    uint32_t out[4];
    int n = 0;
    const uint32_t ch[2] = {nd.left_node_idx, nd.right_node_idx_or_prim_idx};
    for (int s = 0; s < 2; s++) {
        const vrg_bvh_node &c = nodes[ch[s]];
        if (c.left_node_idx != INVALID) {
            out[n++] = c.left_node_idx;
            out[n++] = c.right_node_idx_or_prim_idx;
        } else {
            out[n++] = ch[s];
        }
    }
    float b[6][4];
    int refs[4];
    for (int i = 0; i < 4; i++) {
        if (i < n) {
            const vrg_bvh_node &c = nodes[out[i]];
            for (int a = 0; a < 3; a++) {
                b[2 * a][i] = c.min[a] - BOX_MARGIN;
                b[2 * a + 1][i] = c.max[a] + BOX_MARGIN;
            }
            refs[i] = c.left_node_idx != INVALID ? (int)out[i] : ~(int)leaf[out[i]];
        } else {
            for (int a = 0; a < 3; a++) {  // an inverted box: no ray enters it
                b[2 * a][i] = INFINITY;
                b[2 * a + 1][i] = -INFINITY;
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

// ---- scene commit ----------------------------------------------------------
//
// Several scenes commit together: their top-level trees (light and geometry)
// are built by ONE level-synchronous SAH build, and so are their lamp-block
// trees, so the per-level host round trips of the builder are paid once per
// commit, not once per scene.  Each scene's result is the same as a commit of
// that scene alone (the builder's trees are independent).
//
// The light any-hit walk (nee_pdf's candidate enumeration) runs over a
// world-space SAH BVH of the lamp blocks: a leaf tests the block's emissive
// faces and maps the hit (face, half) to its light-BLAS leaf, so the set of
// light triangles found is the same as walking the triangle light BVH.

namespace {

struct CommitPrep {
    Scene *sc = nullptr;
    uint32_t ni = 0, n_light_inst = 0, n_geo_inst = 0, n_light_tl = 1, n_geo_tl = 0;
    std::vector<float> tl_in;        // [prims][10]: lo3 hi3 off3 power
    std::vector<uint32_t> tl_ids;
    std::vector<InstBuild> gb, lb;
    uint64_t geo_recs = 0, light_recs = 0, tri_recs = 0, n_geo_wide = 0, n_light_nodes_all = 0;
    uint64_t blk_cursor = 0;
    uint32_t max_levels = 0;
    DevBufPtr buf;
    uint8_t *B = nullptr;
    uint64_t o_gw = 0, o_gr = 0, o_tr = 0, o_lr = 0, o_tln = 0, o_inst = 0, o_gb = 0, o_lb = 0, o_xln = 0;
    uint64_t xf_light_nodes = 0;     // light-BLAS nodes of the instances with a transform that is not a translation
    uint32_t tl_prim_off = 0, tl_node_off = 0;  // in the shared top-level build
    uint64_t lamp_off = 0;                      // in the shared lamp build
    uint32_t n_lamps = 0;
    DevBufPtr lamp_buf;
    uint32_t lamp_depth = 0;
    DevScene dev{};                             // installed only when the whole commit succeeds
};

vrg_status commit_prepare(Scene *sc, CommitPrep &cp) {
    cp.sc = sc;
    // instances: non-empty objects in key order (scene.rs:245-260)
    sc->inst_objs.clear();
    sc->inst_off.clear();
    sc->inst_xf.clear();
    sc->inst_tonly.clear();
    for (auto &kv : sc->objects) {
        Object *o = kv.second.obj;
        if (!o->flushed) {
            set_error("object not flushed");
            return VRG_ERR_STATE;
        }
        if (o->sum.n_tris == 0) continue;
        sc->inst_objs.push_back(o);
        sc->inst_off.push_back({kv.second.off[0], kv.second.off[1], kv.second.off[2]});
        std::array<float, 12> m;
        memcpy(m.data(), kv.second.m, sizeof(kv.second.m));
        sc->inst_xf.push_back(m);
        sc->inst_tonly.push_back(kv.second.tonly ? 1 : 0);
    }
    const uint32_t ni = (uint32_t)sc->inst_objs.size();
    if (ni > 65535) {
        set_error("more than 65535 instances");
        return VRG_ERR_UNSUPPORTED;
    }
    cp.ni = ni;
    // Top-level inputs: light roots, then geometry roots.  An instance's prim
    // is its root AABB moved by its transform (Aabb::transform, build.rs:391-395):
    // a translation goes to the builder as such; any other transform is
    // applied here, to the 8 corners in the reference's order, and the
    // builder gets a zero translation.
    auto tl_prim = [&](uint32_t i, const float lo[3], const float hi[3], float power) {
        float r[10];
        if (sc->inst_tonly[i]) {
            const float *o = sc->inst_off[i].data();
            for (int a = 0; a < 3; a++) {
                r[a] = lo[a];
                r[3 + a] = hi[a];
                r[6 + a] = o[a];
            }
        } else {
            const float *m = sc->inst_xf[i].data();
            const float4 r0 = make_float4(m[0], m[1], m[2], m[3]), r1 = make_float4(m[4], m[5], m[6], m[7]),
                         r2 = make_float4(m[8], m[9], m[10], m[11]);
            f3 c[8];
            for (int k = 0; k < 8; k++)
                c[k] = xf_rows(r0, r1, r2, f3{(k & 4) ? hi[0] : lo[0], (k & 2) ? hi[1] : lo[1], (k & 1) ? hi[2] : lo[2]});
            float mn[3] = {c[0].x, c[0].y, c[0].z}, mx[3] = {c[0].x, c[0].y, c[0].z};
            for (int k = 0; k < 8; k++) {  // aabb.rs:10-22 (from_points)
                mn[0] = fminf(mn[0], c[k].x); mx[0] = fmaxf(mx[0], c[k].x);
                mn[1] = fminf(mn[1], c[k].y); mx[1] = fmaxf(mx[1], c[k].y);
                mn[2] = fminf(mn[2], c[k].z); mx[2] = fmaxf(mx[2], c[k].z);
            }
            for (int a = 0; a < 3; a++) {
                r[a] = mn[a];
                r[3 + a] = mx[a];
                r[6 + a] = 0.0f;
            }
        }
        r[9] = power;
        cp.tl_in.insert(cp.tl_in.end(), r, r + 10);
        cp.tl_ids.push_back(i);
    };
    for (uint32_t i = 0; i < ni; i++) {
        const ChunkSummary &cs = sc->inst_objs[i]->sum;
        if (cs.n_light == 0) continue;
        tl_prim(i, cs.light_lo, cs.light_hi, cs.light_power);
        cp.n_light_inst++;
    }
    for (uint32_t i = 0; i < ni; i++) {
        const ChunkSummary &cs = sc->inst_objs[i]->sum;
        if (cs.n_geo == 0) continue;
        tl_prim(i, cs.geo_lo, cs.geo_hi, 0.0f);
        cp.n_geo_inst++;
    }
    cp.n_light_tl = cp.n_light_inst ? 2 * cp.n_light_inst - 1 : 1;
    cp.n_geo_tl = cp.n_geo_inst ? 2 * cp.n_geo_inst - 1 : 0;
    // Per-instance layout.  Leaf references: the surface-block records of all
    // chunks first (geo_rec), then the world-space triangles of all meshes
    // (tri_rec), so a reference ~r with r >= geo_recs names triangle
    // r - geo_recs.  Each instance owns a range of each record kind (empty
    // for the kind it does not have), in instance order.
    uint64_t geo_nodes = 0, light_nodes = 0;
    cp.gb.resize(ni);
    cp.lb.resize(ni);
    for (uint32_t i = 0; i < ni; i++) {
        const Object *o = sc->inst_objs[i];
        if (!o->mesh) cp.geo_recs += o->sum.n_geo;
    }
    for (uint32_t i = 0; i < ni; i++) {
        Object *o = sc->inst_objs[i];
        const ChunkSummary &cs = o->sum;
        InstBuild &g = cp.gb[i], &l = cp.lb[i];
        for (int a = 0; a < 3; a++) {
            const float t = sc->inst_off[i][a];
            g.off[a] = l.off[a] = t;
            g.ioff[a] = l.ioff[a] = o->mesh ? 0 : (int)t;
        }
        memcpy(g.m, sc->inst_xf[i].data(), sizeof(g.m));
        memcpy(l.m, g.m, sizeof(g.m));
        g.flags = l.flags = (o->mesh ? INST_MESH : 0u) | (sc->inst_tonly[i] ? 0u : INST_XFORM);
        g.mesh_tri = l.mesh_tri = o->mesh_tri;
        g.bl = o->geo_nodes;
        g.leaf = o->geo_leaf;
        g.geo_local = o->geo_local;
        g.light_tri = nullptr;
        g.n_prims = cs.n_geo;
        g.wbase = cp.n_geo_tl + (uint32_t)geo_nodes;
        g.rbase = (uint32_t)cp.blk_cursor;
        g.tbase = l.tbase = (uint32_t)cp.tri_recs;
        if (o->mesh) {
            g.refbase = (uint32_t)(cp.geo_recs + cp.tri_recs);
            cp.tri_recs += cs.n_tris;
        } else {
            g.refbase = g.rbase;
            cp.blk_cursor += cs.n_geo;
        }
        geo_nodes += cs.n_geo ? 2 * (uint64_t)cs.n_geo - 1 : 0;
        l.bl = o->light_nodes;
        l.leaf = o->light_leaf;
        l.geo_local = nullptr;
        l.light_tri = o->light_tri;
        l.n_prims = cs.n_light;
        l.wbase = cp.n_light_tl + (uint32_t)light_nodes;
        l.rbase = (uint32_t)cp.light_recs;
        l.refbase = l.rbase;
        light_nodes += cs.n_light ? 2 * (uint64_t)cs.n_light - 1 : 0;
        cp.light_recs += cs.n_light;
        if (!sc->inst_tonly[i] && cs.n_light) cp.xf_light_nodes += 2 * (uint64_t)cs.n_light - 1;
        cp.max_levels = std::max(cp.max_levels, o->levels);
    }
    cp.n_light_nodes_all = light_nodes;
    if (cp.n_geo_tl + geo_nodes >= 0x7FFFFFFFull || cp.geo_recs + cp.tri_recs >= 0x7FFFFFFFull) {
        set_error("scene too large for 31-bit node references");
        return VRG_ERR_UNSUPPORTED;
    }
    auto al = [](uint64_t x) { return (x + 255) & ~255ull; };
    uint64_t o = 0;
    cp.n_geo_wide = cp.n_geo_tl + geo_nodes;
    cp.o_gw = o; o += al(cp.n_geo_wide * 128);
    cp.o_gr = o; o += al(cp.geo_recs * 16);
    cp.o_tr = o; o += al(cp.tri_recs * 48);
    cp.o_xln = o; o += al(cp.xf_light_nodes * sizeof(vrg_bvh_node));
    cp.o_lr = o; o += al(cp.light_recs * 16);
    cp.o_tln = o; o += al((uint64_t)(cp.n_light_tl + cp.n_geo_tl) * sizeof(vrg_bvh_node));
    cp.o_inst = o; o += al((uint64_t)ni * sizeof(InstDev));
    cp.o_gb = o; o += al((uint64_t)ni * sizeof(InstBuild));
    cp.o_lb = o; o += al((uint64_t)ni * sizeof(InstBuild));
    VRG_TRY(dev_alloc(sc->ctx->stream, std::max<uint64_t>(o, 256), cp.buf));
    cp.B = (uint8_t *)cp.buf->ptr;
    return VRG_OK;
}

// all scenes' top-level trees in one SAH build; fills h_light_tl / h_geo_tl
// and each scene's device copy of its nodes ([light TL | geometry TL])
vrg_status commit_top_levels(cudaStream_t s, std::vector<CommitPrep> &cps, uint32_t *tl_levels) {
    uint32_t n_prims = 0, n_nodes = 0;
    for (auto &cp : cps) {
        cp.tl_prim_off = n_prims;
        cp.tl_node_off = n_nodes;
        n_prims += cp.n_light_inst + cp.n_geo_inst;
        n_nodes += cp.n_light_tl + cp.n_geo_tl;
    }
    *tl_levels = 0;
    std::vector<vrg_bvh_node> h_nodes(n_nodes);
    if (n_prims) {
        auto al = [](uint64_t x) { return (x + 255) & ~255ull; };
        uint64_t o = 0;
        uint64_t o_tin = o; o += al((uint64_t)n_prims * 40);
        uint64_t o_tid = o; o += al((uint64_t)n_prims * 4);
        uint64_t o_lo = o; o += al((uint64_t)n_prims * 16);
        uint64_t o_hi = o; o += al((uint64_t)n_prims * 16);
        uint64_t o_cen = o; o += al((uint64_t)n_prims * 16);
        uint64_t o_id = o; o += al((uint64_t)n_prims * 4);
        uint64_t o_perm = o; o += al((uint64_t)n_prims * 4);
        uint64_t o_nodes = o; o += al((uint64_t)n_nodes * sizeof(vrg_bvh_node));
        uint64_t o_leaf = o; o += al((uint64_t)n_nodes * 4);
        DevBufPtr sb;
        VRG_TRY(dev_alloc(s, o, sb));
        uint8_t *S = (uint8_t *)sb->ptr;
        std::vector<float> tin;
        std::vector<uint32_t> tid;
        tin.reserve((size_t)n_prims * 10);
        tid.reserve(n_prims);
        std::vector<SahTree> trees;
        for (auto &cp : cps) {
            tin.insert(tin.end(), cp.tl_in.begin(), cp.tl_in.end());
            tid.insert(tid.end(), cp.tl_ids.begin(), cp.tl_ids.end());
            if (cp.n_light_inst) trees.push_back(SahTree{cp.n_light_inst, cp.tl_prim_off, cp.tl_node_off, 0});
            if (cp.n_geo_inst)
                trees.push_back(SahTree{cp.n_geo_inst, cp.tl_prim_off + cp.n_light_inst,
                                        cp.tl_node_off + cp.n_light_tl, 0});
        }
        VRG_CUDA_TRY(cudaMemcpyAsync(S + o_tin, tin.data(), tin.size() * 4, cudaMemcpyHostToDevice, s));
        VRG_CUDA_TRY(cudaMemcpyAsync(S + o_tid, tid.data(), tid.size() * 4, cudaMemcpyHostToDevice, s));
        k_tl_inputs<<<(n_prims + 127) / 128, 128, 0, s>>>((const float *)(S + o_tin), (const uint32_t *)(S + o_tid),
                                                           n_prims, (float4 *)(S + o_lo), (float4 *)(S + o_hi),
                                                           (float4 *)(S + o_cen), (uint32_t *)(S + o_id));
        VRG_CUDA_TRY(cudaGetLastError());
        SahInputs in{(const float4 *)(S + o_lo), (const float4 *)(S + o_hi), (const float4 *)(S + o_cen),
                     (const uint32_t *)(S + o_id)};
        vrg_bvh_node *nodes = (vrg_bvh_node *)(S + o_nodes);
        SahOutputs out{nodes, (uint32_t *)(S + o_perm), (uint32_t *)(S + o_leaf)};
        VRG_TRY(sah_build(s, trees, n_prims, n_nodes, in, out, tl_levels));
        for (auto &cp : cps) {
            vrg_bvh_node *d_tl = (vrg_bvh_node *)(cp.B + cp.o_tln);
            VRG_CUDA_TRY(cudaMemcpyAsync(d_tl, nodes + cp.tl_node_off,
                                         (size_t)(cp.n_light_tl + cp.n_geo_tl) * sizeof(vrg_bvh_node),
                                         cudaMemcpyDeviceToDevice, s));
        }
        VRG_CUDA_TRY(cudaMemcpyAsync(h_nodes.data(), nodes, (size_t)n_nodes * sizeof(vrg_bvh_node),
                                     cudaMemcpyDeviceToHost, s));
    }
    // a scene without lights gets the dummy node (BvhNode::default, bvh/mod.rs:27-38; scene.rs:276-277)
    vrg_bvh_node dummy;
    dummy.left_node_idx = dummy.right_node_idx_or_prim_idx = dummy.parent_idx = INVALID;
    for (int a = 0; a < 3; a++) dummy.min[a] = dummy.max[a] = 0.0f;
    dummy.power = 0.0f;
    for (auto &cp : cps) {
        if (cp.n_light_inst) continue;
        VRG_CUDA_TRY(cudaMemcpyAsync(cp.B + cp.o_tln, &dummy, sizeof(dummy), cudaMemcpyHostToDevice, s));
    }
    VRG_CUDA_TRY(cudaStreamSynchronize(s));
    for (auto &cp : cps) {
        const vrg_bvh_node *h = h_nodes.data() + cp.tl_node_off;
        cp.sc->h_light_tl.assign(h, h + cp.n_light_tl);
        if (!cp.n_light_inst) cp.sc->h_light_tl[0] = dummy;
        cp.sc->h_geo_tl.assign(h + cp.n_light_tl, h + cp.n_light_tl + cp.n_geo_tl);
    }
    return VRG_OK;
}

// instance table, traversal layouts and records of one scene
vrg_status commit_layouts(cudaStream_t s, CommitPrep &cp, const vrg_bvh_node *d_tl) {
    Scene *sc = cp.sc;
    const uint32_t ni = cp.ni;
    uint8_t *B = cp.B;
    // instance table (prim2node, scene.rs:282-287)
    std::vector<InstDev> idev(ni);
    uint64_t xln = 0;
    for (uint32_t i = 0; i < ni; i++) {
        const Object *ob = sc->inst_objs[i];
        for (int a = 0; a < 3; a++) idev[i].off[a] = sc->inst_off[i][a];
        idev[i].light_bvh_tl_idx = 0;
        idev[i].light_bl = ob->light_nodes;
        idev[i].light_leaf_tri = ob->light_leaf_tri;
        idev[i].flags = cp.gb[i].flags;
        idev[i].tri_base = cp.gb[i].tbase;
        idev[i].uv = ob->mesh_uv;
        if (!sc->inst_tonly[i] && ob->sum.n_light) {
            // the light walks read this instance's nodes already transformed
            const uint32_t nn = 2 * ob->sum.n_light - 1;
            const float *m = sc->inst_xf[i].data();
            vrg_bvh_node *dst = (vrg_bvh_node *)(B + cp.o_xln) + xln;
            k_xform_light_nodes<<<(nn + 127) / 128, 128, 0, s>>>(
                ob->light_nodes, nn, make_float4(m[0], m[1], m[2], m[3]), make_float4(m[4], m[5], m[6], m[7]),
                make_float4(m[8], m[9], m[10], m[11]), dst);
            VRG_CUDA_TRY(cudaGetLastError());
            idev[i].light_bl = dst;
            idev[i].off[0] = idev[i].off[1] = idev[i].off[2] = 0.0f;
            xln += nn;
        }
    }
    if (cp.n_light_inst)
        for (uint32_t j = 0; j < cp.n_light_tl; j++)
            if (sc->h_light_tl[j].left_node_idx == INVALID)
                idev[sc->h_light_tl[j].right_node_idx_or_prim_idx].light_bvh_tl_idx = j;
    if (ni) {
        VRG_CUDA_TRY(cudaMemcpyAsync(B + cp.o_inst, idev.data(), ni * sizeof(InstDev), cudaMemcpyHostToDevice, s));
        VRG_CUDA_TRY(cudaMemcpyAsync(B + cp.o_gb, cp.gb.data(), ni * sizeof(InstBuild), cudaMemcpyHostToDevice, s));
        VRG_CUDA_TRY(cudaMemcpyAsync(B + cp.o_lb, cp.lb.data(), ni * sizeof(InstBuild), cudaMemcpyHostToDevice, s));
    }
    const InstBuild *d_gb = (const InstBuild *)(B + cp.o_gb), *d_lb = (const InstBuild *)(B + cp.o_lb);
    if (cp.n_geo_wide) {
        k_wide4<<<(uint32_t)((cp.n_geo_wide + 255) / 256), 256, 0, s>>>(d_tl + cp.n_light_tl, cp.n_geo_tl, d_gb, ni,
                                                                       (uint32_t)cp.n_geo_wide,
                                                                       (float4 *)(B + cp.o_gw));
        VRG_CUDA_TRY(cudaGetLastError());
    }
    if (cp.geo_recs) {
        const uint32_t n = (uint32_t)cp.geo_recs;
        k_geo_records<<<std::min(4096u, (n + 255) / 256), 256, 0, s>>>(d_gb, ni, n, (int4 *)(B + cp.o_gr));
    }
    if (cp.tri_recs) {
        const uint32_t n = (uint32_t)cp.tri_recs;
        k_tri_records<<<std::min(4096u, (n + 255) / 256), 256, 0, s>>>(d_gb, ni, n, (float4 *)(B + cp.o_tr));
    }
    if (cp.light_recs) {
        const uint32_t n = (uint32_t)(cp.n_light_nodes_all);
        k_light_records<<<std::min(4096u, (n + 255) / 256), 256, 0, s>>>(d_lb, ni, cp.n_light_tl, n,
                                                                        (int4 *)(B + cp.o_lr));
    }
    VRG_CUDA_TRY(cudaGetLastError());
    DevScene &D = cp.dev;
    D.geo_wide = (const float4 *)(B + cp.o_gw);
    D.geo_rec = (const int4 *)(B + cp.o_gr);
    D.tri_rec = (const float4 *)(B + cp.o_tr);
    D.n_blk_rec = (uint32_t)cp.geo_recs;
    D.n_tri_rec = (uint32_t)cp.tri_recs;
    D.light_tl = d_tl;
    D.inst = (const InstDev *)(B + cp.o_inst);
    D.mats = (const vrg_material *)sc->ctx->d_mats->ptr;
    D.n_inst = ni;
    // geometry root: the TL root, or with one object its BLAS root / single record
    if (cp.n_geo_tl == 0) {
        D.geo_root = EMPTY_ROOT;
    } else if (sc->h_geo_tl[0].left_node_idx != INVALID) {
        D.geo_root = 0;
    } else {
        const uint32_t k = sc->h_geo_tl[0].right_node_idx_or_prim_idx;
        vrg_bvh_node r;
        VRG_CUDA_TRY(cudaMemcpy(&r, cp.gb[k].bl, sizeof(r), cudaMemcpyDeviceToHost));
        if (r.left_node_idx != INVALID) {
            D.geo_root = (int)cp.gb[k].wbase;
        } else {
            uint32_t p0;
            VRG_CUDA_TRY(cudaMemcpy(&p0, cp.gb[k].leaf, 4, cudaMemcpyDeviceToHost));
            D.geo_root = ~(int)(cp.gb[k].refbase + p0);
        }
    }
    return VRG_OK;
}

// all scenes' lamp-block trees in one SAH build
vrg_status commit_lamps(cudaStream_t s, std::vector<CommitPrep> &cps) {
    uint64_t L = 0;
    for (auto &cp : cps) {
        cp.lamp_off = L;
        L += cp.light_recs;
        cp.dev.lamp_root = EMPTY_ROOT;
    }
    if (L == 0) return VRG_OK;
    if (2 * L >= 0x7FFFFFFFull) {
        set_error("too many light triangles in one commit");
        return VRG_ERR_UNSUPPORTED;
    }
    const uint32_t nc = (uint32_t)cps.size();
    auto al = [](uint64_t x) { return (x + 255) & ~255ull; };
    uint64_t o = 0;
    uint64_t o_flag = o; o += al(L * 4);
    uint64_t o_tot = o; o += al((uint64_t)nc * 4);
    uint64_t o_lo = o; o += al(L * 16);
    uint64_t o_hi = o; o += al(L * 16);
    uint64_t o_cen = o; o += al(L * 16);
    uint64_t o_id = o; o += al(L * 4);
    uint64_t o_perm = o; o += al(L * 4);
    uint64_t o_nodes = o; o += al(2 * L * sizeof(vrg_bvh_node));
    uint64_t o_leaf = o; o += al(2 * L * 4);
    DevBufPtr sb;
    VRG_TRY(dev_alloc(s, o, sb));
    uint8_t *S = (uint8_t *)sb->ptr;
    uint32_t *tot = (uint32_t *)(S + o_tot);
    VRG_CUDA_TRY(cudaMemsetAsync(tot, 0, (size_t)nc * 4, s));
    for (uint32_t c = 0; c < nc; c++) {
        CommitPrep &cp = cps[c];
        const uint64_t n = cp.light_recs;
        if (n == 0) continue;
        uint64_t q = 0;
        const uint64_t q_rec = q; q += al(n * 16);
        const uint64_t q_tab = q; q += al(n * 12 * 4);
        const uint64_t q_wide = q; q += al(2 * n * 128);
        VRG_TRY(dev_alloc(s, q, cp.lamp_buf));
        uint8_t *Q = (uint8_t *)cp.lamp_buf->ptr;
        int4 *lamp = (int4 *)(Q + q_rec);
        uint32_t *table = (uint32_t *)(Q + q_tab);
        VRG_CUDA_TRY(cudaMemsetAsync(lamp, 0, n * 16, s));
        VRG_CUDA_TRY(cudaMemsetAsync(table, 0xFF, n * 48, s));
        const int4 *light_rec = (const int4 *)(cp.B + cp.o_lr);
        uint32_t *flag = (uint32_t *)(S + o_flag) + cp.lamp_off;
        k_lamp_flags<<<(uint32_t)((n + 255) / 256), 256, 0, s>>>(light_rec, (uint32_t)n, flag);
        k_scan_inclusive<<<1, 1024, 0, s>>>(flag, (uint32_t)n, tot + c);
        k_lamp_fill<<<(uint32_t)((n + 255) / 256), 256, 0, s>>>(
            light_rec, flag, (uint32_t)n, (const float4 *)(cp.B + cp.o_tr), lamp, table, (float4 *)(S + o_lo) + cp.lamp_off,
            (float4 *)(S + o_hi) + cp.lamp_off, (float4 *)(S + o_cen) + cp.lamp_off,
            (uint32_t *)(S + o_id) + cp.lamp_off);
        VRG_CUDA_TRY(cudaGetLastError());
        DevScene &D = cp.dev;
        D.lamp_wide = (const float4 *)(Q + q_wide);
        D.lamp_rec = lamp;
        D.lamp_table = table;
    }
    std::vector<uint32_t> n_lamps(nc);
    VRG_CUDA_TRY(cudaMemcpyAsync(n_lamps.data(), tot, (size_t)nc * 4, cudaMemcpyDeviceToHost, s));
    VRG_CUDA_TRY(cudaStreamSynchronize(s));
    std::vector<SahTree> trees;
    for (uint32_t c = 0; c < nc; c++) {
        cps[c].n_lamps = n_lamps[c];
        if (n_lamps[c]) trees.push_back(SahTree{n_lamps[c], (uint32_t)cps[c].lamp_off, 2 * (uint32_t)cps[c].lamp_off, 0});
    }
    SahInputs in{(const float4 *)(S + o_lo), (const float4 *)(S + o_hi), (const float4 *)(S + o_cen),
                 (const uint32_t *)(S + o_id)};
    vrg_bvh_node *nodes = (vrg_bvh_node *)(S + o_nodes);
    uint32_t *leaf = (uint32_t *)(S + o_leaf);
    SahOutputs out{nodes, (uint32_t *)(S + o_perm), leaf};
    uint32_t levels = 0;
    VRG_TRY(sah_build(s, trees, (uint32_t)L, (uint32_t)(2 * L), in, out, &levels));
    for (auto &cp : cps) {
        if (!cp.n_lamps) continue;
        DevScene &D = cp.dev;
        if (cp.n_lamps > 1) {
            const uint32_t nn = 2 * cp.n_lamps - 1;
            k_wide4_single<<<(nn + 255) / 256, 256, 0, s>>>(nodes + 2 * cp.lamp_off, leaf + 2 * cp.lamp_off, nn,
                                                            (float4 *)D.lamp_wide);
            VRG_CUDA_TRY(cudaGetLastError());
            D.lamp_root = 0;
        } else {
            D.lamp_root = ~0;
        }
        cp.lamp_depth = 3 * ((levels + 2 + 1) / 2) + 1;  // up to 3 pushes per 4-wide level
    }
    return VRG_OK;
}

}  // namespace

vrg_status scene_commit_many(Scene *const *scs, uint32_t n) {
    if (n == 0) return VRG_OK;
    Context *ctx = scs[0]->ctx;
    for (uint32_t i = 1; i < n; i++)
        if (scs[i]->ctx != ctx) {
            set_error("scenes of one commit share a context");
            return VRG_ERR_INVALID_ARGUMENT;
        }
    cudaStream_t s = ctx->stream;
    {  // chunks uploaded since the last commit: one batched extraction + BLAS build
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
    std::vector<CommitPrep> cps;
    for (uint32_t i = 0; i < n; i++) {
        Scene *sc = scs[i];
        if (!sc->dirty) continue;
        bool seen = false;
        for (auto &cp : cps) seen |= cp.sc == sc;
        if (seen) continue;
        cps.emplace_back();
        VRG_TRY(commit_prepare(sc, cps.back()));
    }
    if (cps.empty()) return VRG_OK;
    uint32_t tl_levels = 0;
    VRG_TRY(commit_top_levels(s, cps, &tl_levels));
    for (auto &cp : cps) VRG_TRY(commit_layouts(s, cp, (const vrg_bvh_node *)(cp.B + cp.o_tln)));
    VRG_TRY(commit_lamps(s, cps));
    for (auto &cp : cps) {
        // the 4-wide walk pushes up to 3 refs per 4-wide level (half the binary depth)
        const uint32_t bound = std::max(3 * ((tl_levels + cp.max_levels + 4 + 1) / 2) + 1, cp.lamp_depth);
        if (bound >= (uint32_t)TRAV_STACK) {
            set_error("BVH depth bound %u exceeds the traversal stack (%d)", bound, TRAV_STACK);
            return VRG_ERR_UNSUPPORTED;
        }
        cp.sc->depth_bound = bound;
    }
    VRG_CUDA_TRY(cudaStreamSynchronize(s));
    for (auto &cp : cps) {
        Scene *sc = cp.sc;
        sc->dev = cp.dev;
        sc->d_buf = cp.buf;
        sc->lamp_buf = cp.lamp_buf;
        sc->dirty = false;
        for (Object *r : sc->retired)
            if (--r->refs == 0) delete r;
        sc->retired.clear();
    }
    return VRG_OK;
}

vrg_status scene_commit(Scene *sc) { return scene_commit_many(&sc, 1); }

DevScene frame_scene(const Scene *sc) {
    DevScene D = sc->dev;
    const Context *ctx = sc->ctx;
    D.mats = ctx->d_mats ? (const vrg_material *)ctx->d_mats->ptr : nullptr;
    D.atlas = ctx->d_atlas ? (const uchar4 *)ctx->d_atlas->ptr : nullptr;
    D.srgb = ctx->d_srgb;
    D.atlas_w = ctx->atlas_w;
    D.atlas_h = ctx->atlas_h;
    return D;
}

}  // namespace vrg
