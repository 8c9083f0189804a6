// Wavefront bounce kernels: per bounce, the closest hit over the world-space
// voxel BVH (k_trace, with ray generation at bounce 0), the shading with its
// light-BVH next-event estimation (k_shade), and the light-sampling pdf of the
// chosen direction in three passes (k_anyhit, k_hit_eval, k_hit_sum), which
// run on their own stream beside the next bounce.
//
// Reference stages covered here (one dispatch each in the reference):
//   raygen        raygen.rs:84-111
//   raytrace      raytrace.rs:390-578 (closest hit replaces the driver ray
//                 query; traverseBvh 218-281 is the light descent)
//   nee_pdf       nee_pdf.rs:281-337 (any-hit over light triangles along the
//                 chosen direction; reverseTraverseBvh 154-228)
// Work distribution: the closest hit and the any-hit walk are persistent
// warps in which each lane takes a new ray from the bounce's queue when its
// walk ends; rays that continue, and light-pdf jobs, are compacted into the
// next queues with one warp ballot + one atomic per warp.  State per pixel
// stays in SoA float4 arrays; the per-bounce record (E, w=pdf/q) (R, q) feeds
// the backward radiance recurrence of the resolve kernel.
#include <mutex>

#include "vrg_frame.cuh"
#include "vrg_internal.h"

namespace vrg {

__constant__ Frame c_frames[12];

namespace {

struct NodeV {
    uint32_t left, right;
    f3 mn;
    float power;
    f3 mx;
    uint32_t parent;
};

__device__ __forceinline__ NodeV ldnode(const vrg_bvh_node *n) {
    const float2 *p = reinterpret_cast<const float2 *>(n);
    float2 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3), e = __ldg(p + 4);
    NodeV r;
    r.left = __float_as_uint(a.x);
    r.right = __float_as_uint(a.y);
    r.mn = f3{b.x, b.y, c.x};
    r.power = c.y;
    r.mx = f3{d.x, d.y, e.x};
    r.parent = __float_as_uint(e.y);
    return r;
}

// The shading point's part of nodeImportance, the same for every node of a
// walk, worked out once per walk (the descent and the reverse walk are
// bound by instruction issue; this took the 1080p frame from 1.114 to 1.086
// ms).  Voxel-face normals are one of +-x, +-y, +-z: then dot(c - p, n) is
// exactly +-(c_a - p_a) (the other two products are +-0), so the 8 corners
// reduce to the box's min and max along the normal axis, 4 corners each.
struct ImpPt {
    f3 point, normal;
    int ax;     // the normal's axis (| 4 when it is -1 there) when it is +-1 on one axis and 0 on
                // the others, else -1
    float pa;   // point[ax]
};
__device__ __forceinline__ ImpPt imp_point(f3 point, f3 normal) {
    ImpPt P;
    P.point = point;
    P.normal = normal;
    P.ax = -1;
    P.pa = 0.0f;
    const bool nx = normal.x != 0.0f, ny = normal.y != 0.0f, nz = normal.z != 0.0f;
    if ((int)nx + (int)ny + (int)nz == 1) {
        const int ax = nx ? 0 : (ny ? 1 : 2);
        const float na = cmp3(normal, ax);
        if (na == 1.0f || na == -1.0f) {
            P.ax = ax | (na < 0.0f ? 4 : 0);
            P.pa = cmp3(point, ax);
        }
    }
    return P;
}

// nodeImportance (raytrace.rs:181-208: uint visibility, EPS 1e-3;
// nee_pdf.rs:125-152: float visibility, EPS 1e-4).  v000 and v111 are the
// instance transform applied to the node's min and max; the 8 corners are the
// axis-aligned box they span (as in the reference, not the transformed box).
// An instance moves its light-BLAS nodes by the translation off here; an
// instance with any other transform has its nodes' min and max transformed
// once at commit (its off is 0), which gives the same importance bits.
template <bool NEE>
__device__ __forceinline__ float node_importance(const ImpPt &P, const float off[3], const NodeV &n) {
    const f3 point = P.point, normal = P.normal;
    f3 v000 = f3{n.mn.x + off[0], n.mn.y + off[1], n.mn.z + off[2]};
    f3 v111 = f3{n.mx.x + off[0], n.mx.y + off[1], n.mx.z + off[2]};
    f3 e = sub3(v111, v000);
    f3 cc = sub3(lscl3(0.5f, add3(v000, v111)), point);
    float dist_sq = fmaxf(dot3(e, e), dot3(cc, cc));
    const float eps = NEE ? EPS_NEE : EPS_TRACE;
    if (P.ax >= 0) {
        const int ax = P.ax & 3;
        float dlo = cmp3(v000, ax) - P.pa, dhi = cmp3(v111, ax) - P.pa;
        if (P.ax & 4) { dlo = -dlo; dhi = -dhi; }
        const uint32_t visible = (dlo >= eps ? 4u : 0u) + (dhi >= eps ? 4u : 0u);
        if (!NEE) return n.power / dist_sq * ((float)visible / 8.0f);
        return n.power / dist_sq * ((float)visible * 0.125f);  // = the sum of 0.125 terms, exact
    }
    f3 c[8] = {v000, f3{v000.x, v000.y, v111.z}, f3{v000.x, v111.y, v000.z}, f3{v000.x, v111.y, v111.z},
               f3{v111.x, v000.y, v000.z}, f3{v111.x, v000.y, v111.z}, f3{v111.x, v111.y, v000.z}, v111};
    if (!NEE) {
        uint32_t visible = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) visible += (dot3(sub3(c[k], point), normal) >= eps) ? 1u : 0u;
        return n.power / dist_sq * ((float)visible / 8.0f);
    }
    float visible = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; k++) visible += 0.125f * ((dot3(sub3(c[k], point), normal) >= eps) ? 1.0f : 0.0f);
    return n.power / dist_sq * visible;
}

struct Descent {
    bool success;
    uint32_t inst, leaf;
    float importance;
};

// traverseBvh (raytrace.rs:218-281)
__device__ Descent light_descent(const DevScene &sc, f3 point, f3 normal, uint32_t seed) {
    Descent R;
    R.success = false;
    R.inst = 0;
    R.leaf = 0;
    R.importance = 0.0f;
    const vrg_bvh_node *root = sc.light_tl;
    NodeV node = ldnode(&root[0]);
    if (node.left == INVALID && node.right == INVALID) return R;
    const ImpPt P = imp_point(point, normal);
    float importance = 0.0f;
    float off[3] = {0.0f, 0.0f, 0.0f};
    uint32_t inst = INVALID, node_idx = 0;
    bool top = true;
    for (int guard = 0; guard < 256; guard++) {
        if (top && node.left == INVALID) {
            inst = node.right;
            const InstDev &I = sc.inst[inst];
            off[0] = I.off[0]; off[1] = I.off[1]; off[2] = I.off[2];
            top = false;
            root = I.light_bl;
            node = ldnode(&root[0]);
            node_idx = 0;
            if (importance == 0.0f) importance = node_importance<false>(P, off, node);
        }
        if (!top && node.left == INVALID) {
            R.success = true;
            R.inst = inst;
            R.leaf = node_idx;
            R.importance = importance;
            return R;
        }
        uint32_t li = node.left, ri = node.right;
        NodeV left = ldnode(&root[li]), right = ldnode(&root[ri]);
        float lI = node_importance<false>(P, off, left);
        float rI = node_importance<false>(P, off, right);
        float tot = lI + rI;
        const float ln = lI / tot;  // the shader's right ratio is never read
        if (mm_rand(seed) < ln) { node = left; node_idx = li; importance = lI; }
        else { node = right; node_idx = ri; importance = rI; }
        seed = mm_combine(seed, 0);
    }
    return R;
}

// reverseTraverseBvh (nee_pdf.rs:154-228)
__device__ float reverse_walk(const DevScene &sc, f3 point, f3 normal, uint32_t ii, uint32_t leaf) {
    const InstDev &I = sc.inst[ii];
    const vrg_bvh_node *root = I.light_bl;
    float probability = 1.0f;
    float off[3] = {I.off[0], I.off[1], I.off[2]};
    bool top = false;
    NodeV node = ldnode(&root[leaf]);
    uint32_t node_idx = leaf;
    const ImpPt P = imp_point(point, normal);
    for (int guard = 0; guard < 256; guard++) {
        uint32_t old = node_idx;
        if (node.parent == INVALID) {
            if (top) return probability;
            top = true;
            root = sc.light_tl;
            old = I.light_bvh_tl_idx;
            NodeV tl_leaf = ldnode(&root[I.light_bvh_tl_idx]);
            if (tl_leaf.parent == INVALID) return probability;
            node_idx = tl_leaf.parent;
            node = ldnode(&root[node_idx]);
            off[0] = off[1] = off[2] = 0.0f;
        } else {
            node_idx = node.parent;
            node = ldnode(&root[node_idx]);
        }
        NodeV left = ldnode(&root[node.left]), right = ldnode(&root[node.right]);
        float lI = node_importance<true>(P, off, left);
        float rI = node_importance<true>(P, off, right);
        float tot = lI + rI;
        float ln = lI / tot, rn = rI / tot;
        if (old == node.left) probability *= ln;
        else probability *= rn;
    }
    return probability;
}

// world-space vertices of the light triangle of light-BLAS leaf `leaf` of
// instance ii (the triangleTransform of raytrace.rs:155-159, nee_pdf.rs:95-101)
__device__ __forceinline__ void light_tri_world(const DevScene &sc, uint32_t ii, uint32_t leaf, f3 tv[3]) {
    const InstDev &I = sc.inst[ii];
    uint32_t t = __ldg(I.light_leaf_tri + leaf);
    if (I.flags & INST_MESH) {
        const float4 *r = sc.tri_rec + 3 * (size_t)(I.tri_base + t);
        tv[0] = ld3(__ldg(r));
        tv[1] = ld3(__ldg(r + 1));
        tv[2] = ld3(__ldg(r + 2));
        return;
    }
    int lx = (int)(t & 31u), ly = (int)((t >> 5) & 31u), lz = (int)((t >> 10) & 31u);
    int f = (int)((t >> 15) & 7u), h = (int)((t >> 18) & 1u);
#pragma unroll
    for (int j = 0; j < 3; j++) {
        f3 p = corner_pos(lx, ly, lz, face_corner(f, h, j));
        tv[j] = f3{p.x + I.off[0], p.y + I.off[1], p.z + I.off[2]};
    }
}

// computeNeePdf (nee_pdf.rs:240-279)
__device__ float nee_pdf_of(const DevScene &sc, f3 point, f3 normal, f3 dir, uint32_t ii, uint32_t leaf, float b1,
                            float b2) {
    f3 tv[3];
    light_tri_world(sc, ii, leaf, tv);
    f3 p = add3(add3(lscl3(b1, tv[0]), lscl3(b2, tv[1])), lscl3((1.0f - b1) - b2, tv[2]));
    float light_distance = len3(sub3(p, point));
    float light_area = 0.5f * len3(cross3(sub3(tv[0], tv[1]), sub3(tv[2], tv[1])));
    float cos_theta = dot3(normal, dir);
    float ppp = light_distance * light_distance / (cos_theta * light_area);
    float P = reverse_walk(sc, point, normal, ii, leaf);
    return P * ppp;
}

constexpr int LIGHT_LIST = 32;
constexpr uint32_t FULL = 0xffffffffu;

__device__ __forceinline__ void st3(float *a, size_t i, f3 v) {
    a[3 * i] = v.x;
    a[3 * i + 1] = v.y;
    a[3 * i + 2] = v.z;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// raygen (raygen.rs:84-111): pixel corner, jitter multiplied by 0.00
// lp: the pixel's index within its view
__device__ __forceinline__ void raygen(const ViewDev &V, uint32_t lp, f3 &o, f3 &d) {
    uint32_t x = lp % V.W, y = lp / V.W;
    float u = 2.0f * (float)x / (float)V.W - 1.0f;
    float v = 2.0f * (float)y / (float)V.H - 1.0f;
    float aspect = (float)V.W / (float)V.H;
    o = V.eye;
    d = norm3(add3(add3(scl3(lscl3(u, V.right), aspect), lscl3(v, V.up)), V.front));
}

// Conservative slab test of a traversal box (boxes carry BOX_MARGIN, so the
// rounding of the FMA form never culls a box that holds a candidate face).
__device__ __forceinline__ bool slab_fma(float lox, float hix, float loy, float hiy, float loz, float hiz, f3 inv,
                                         f3 oi, float tmin, float tmax, float &tn) {
    float t0x = __fmaf_rn(lox, inv.x, oi.x), t1x = __fmaf_rn(hix, inv.x, oi.x);
    float t0y = __fmaf_rn(loy, inv.y, oi.y), t1y = __fmaf_rn(hiy, inv.y, oi.y);
    float t0z = __fmaf_rn(loz, inv.z, oi.z), t1z = __fmaf_rn(hiz, inv.z, oi.z);
    tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
    float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), tmax));
    return tn <= tf;
}

// Pops the next pending child whose box starts at or before best_t (boxes
// are culled only when strictly beyond it); false when none is left.
__device__ __forceinline__ bool pop_near(const int2 *stack, int &sp, float best_t, int &node) {
    while (sp > 0) {
        const int2 e = stack[--sp];  // (ref, entry distance bits)
        if (__int_as_float(e.y) <= best_t) {
            node = e.x;
            return true;
        }
    }
    return false;
}

__device__ __forceinline__ void cswap(float &ta, int &ra, float &tb, int &rb) {
    if (tb < ta) {
        const float t = ta; ta = tb; tb = t;
        const int r = ra; ra = rb; rb = r;
    }
}

// three-input min / max (sm_100+); NaN inputs are ignored as by fminf/fmaxf
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// slab test of the 4 children of a 4-wide node; returns the entry distances
// sorted ascending (+inf for a miss) with their refs.  NX..FZ are the near and
// far planes per axis, picked per ray by the sign of its direction (so the
// per-axis min/max of the classic slab test is not needed).  For such a pick
// the near distance of a non-empty box is <= its far distance, exactly, since
// rounding is monotonic; a NaN distance (only possible for a direction
// component below 1e-30 in magnitude, whose inverse overflows) is ignored by
// min/max, which only keeps more boxes: the test stays conservative and the
// closest hit does not depend on it.  A component of exactly 0 has the finite
// inverse +-1e30 (slab_inv), so that axis culls like any other.  An unused
// slot holds the inverted box lo = +inf, hi = -inf: on an axis with a finite
// inverse its near distance is +inf, so the slot is never entered and needs
// no test of its ref.
__device__ __forceinline__ void slab4(float4 NX, float4 FX, float4 NY, float4 FY, float4 NZ, float4 FZ, float4 RF,
                                      f3 inv, f3 oi, float tmin, float tmax, float tk[4], int rk[4]) {
    const float nx[4] = {NX.x, NX.y, NX.z, NX.w}, fx[4] = {FX.x, FX.y, FX.z, FX.w};
    const float ny[4] = {NY.x, NY.y, NY.z, NY.w}, fy[4] = {FY.x, FY.y, FY.z, FY.w};
    const float nz[4] = {NZ.x, NZ.y, NZ.z, NZ.w}, fz[4] = {FZ.x, FZ.y, FZ.z, FZ.w};
    const int rf[4] = {__float_as_int(RF.x), __float_as_int(RF.y), __float_as_int(RF.z), __float_as_int(RF.w)};
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const float tn = fmax3(__fmaf_rn(nx[i], inv.x, oi.x), __fmaf_rn(ny[i], inv.y, oi.y),
                               fmaxf(__fmaf_rn(nz[i], inv.z, oi.z), tmin));
        const float tf = fmin3(__fmaf_rn(fx[i], inv.x, oi.x), __fmaf_rn(fy[i], inv.y, oi.y),
                               fminf(__fmaf_rn(fz[i], inv.z, oi.z), tmax));
        tk[i] = (tn <= tf) ? tn : INFINITY;
        rk[i] = rf[i];
    }
    // sorting network for 4
    cswap(tk[0], rk[0], tk[1], rk[1]);
    cswap(tk[2], rk[2], tk[3], rk[3]);
    cswap(tk[0], rk[0], tk[2], rk[2]);
    cswap(tk[1], rk[1], tk[3], rk[3]);
    cswap(tk[1], rk[1], tk[2], rk[2]);
}

// ---------------------------------------------------------------------------
// k_trace: closest hit over the voxel faces (replaces getIntersectionInfo,
// raytrace.rs:354-388).  Persistent warps; each lane owns one ray and, when
// its traversal ends, takes a new ray from the bounce queue (warp-aggregated
// fetch once a.refill_trace lanes are idle), so a warp does not wait for its
// longest ray.  The result is independent of traversal order: ties on t go
// to the smaller (instance, triangle) key and boxes are culled only when
// strictly beyond the current best t.  In a batched frame each lane reads the
// scene of its ray's view when it takes the ray.
// ---------------------------------------------------------------------------
template <bool BATCH, bool MESH>
__global__ void __launch_bounds__(128) k_trace(const __grid_constant__ FrameArgs a, uint32_t b) {
    const int lane = threadIdx.x & 31;
    const int REFILL = (int)a.refill_trace;
    const uint32_t n_in = (b == 0) ? a.n0 : a.counters[a.qsel ? CNT_TQUEUE : CNT_QUEUE + b];
    const uint32_t *qin = a.qsel ? a.tq : a.queue[(b + 1) & 1];
    uint32_t *fetch = a.counters + (a.qsel ? CNT_TFETCH : CNT_FETCH + b);
    uint32_t *err = a.counters + CNT_ERROR;
    const float4 *wide = a.v0.sc.geo_wide;
    const int4 *recs = a.v0.sc.geo_rec;
    const float4 *tris = a.v0.sc.tri_rec;
    uint32_t nblk = a.v0.sc.n_blk_rec;
    int root = a.v0.sc.geo_root;
    bool has = false, exhausted = false;
    uint32_t p = 0, steps = 0, traced = 0, n_nodes = 0, n_leaves = 0;
    f3 o = f3{0, 0, 0}, d = f3{0, 0, 0}, inv = f3{0, 0, 0}, oi = f3{0, 0, 0};
    float best_t = 0.0f, hb1 = 0.0f, hb2 = 0.0f;
    uint64_t best_key = 0;
    int node = 0, sp = 0, hrec = -1;
    uint32_t hfh = 0;
    int px = 0, py = 2, pz = 4;  // float4 index of the near plane per axis (the far one is next to it)
    // pending children with their entry distances: a popped entry whose box
    // starts beyond the current best t is dropped unvisited (every box below
    // it starts no nearer, so each would be culled by its own test)
    int2 stack[TRAV_STACK];
    while (true) {
        const uint32_t need = __ballot_sync(FULL, !has);
        if (!exhausted && need && (__popc(need) >= REFILL || need == FULL)) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(fetch, (uint32_t)__popc(need));
            base = __shfl_sync(FULL, base, 0);
            if (base + (uint32_t)__popc(need) >= n_in) exhausted = true;
            if (!has) {
                const uint32_t idx = base + (uint32_t)__popc(need & lanemask_lt());
                if (idx < n_in && (b == 0 ? bounce0_pixel<BATCH>(a, idx, p) : (p = qin[idx], true))) {
                    has = true;
                    traced++;
                    const ViewDev &V = view_of<BATCH>(a, p);
                    if constexpr (BATCH) {
                        wide = V.sc.geo_wide;
                        recs = V.sc.geo_rec;
                        tris = V.sc.tri_rec;
                        nblk = V.sc.n_blk_rec;
                        root = V.sc.geo_root;
                    }
                    if (b == 0) raygen(V, p - V.pix_off, o, d);
                    else { o = ld3(a.ray_o[p]); d = ld3(a.ray_d[p]); }
                    inv = f3{slab_inv(d.x), slab_inv(d.y), slab_inv(d.z)};
                    oi = f3{-o.x * inv.x, -o.y * inv.y, -o.z * inv.z};
                    px = signbit(inv.x) ? 1 : 0;
                    py = signbit(inv.y) ? 3 : 2;
                    pz = signbit(inv.z) ? 5 : 4;
                    best_t = 1000.0f;
                    best_key = ~0ull;
                    node = root;
                    sp = 0;
                    hrec = -1;
                    steps = 0;
                }
            }
        }
        if (!__any_sync(FULL, has)) break;
        if (has) {
            bool done = (node == EMPTY_ROOT);
            // descend through 4-wide inner nodes to the next leaf
            while (!done && node >= 0) {
                const float4 *w = wide + 8 * (size_t)node;
                const float4 NX = __ldg(w + px), FX = __ldg(w + (px ^ 1)), NY = __ldg(w + py);
                const float4 FY = __ldg(w + (py ^ 1)), NZ = __ldg(w + pz), FZ = __ldg(w + (pz ^ 1));
                const float4 RF = __ldg(w + 6);
                n_nodes++;
                float tk[4];
                int rk[4];
                slab4(NX, FX, NY, FY, NZ, FZ, RF, inv, oi, EPS_TRACE, best_t, tk, rk);
                // tk sorted ascending (misses at +inf)
                if (tk[0] == INFINITY) {
                    done = !pop_near(stack, sp, best_t, node);
                } else {
                    node = rk[0];
                    if (sp + 3 <= TRAV_STACK) {
                        if (tk[3] != INFINITY) stack[sp++] = make_int2(rk[3], __float_as_int(tk[3]));
                        if (tk[2] != INFINITY) stack[sp++] = make_int2(rk[2], __float_as_int(tk[2]));
                        if (tk[1] != INFINITY) stack[sp++] = make_int2(rk[1], __float_as_int(tk[1]));
                    } else {
                        atomicOr(err, ERR_STACK);
                    }
                }
                if (++steps > TRAV_GUARD) {  // only reachable with a malformed layout
                    atomicOr(err, ERR_GUARD);
                    done = true;
                }
            }
            if (MESH && !done && (uint32_t)(~node) >= nblk) {  // leaf: one world-space mesh triangle
                const float4 *tr = tris + 3 * (size_t)((uint32_t)(~node) - nblk);
                const float4 A = __ldg(tr), B = __ldg(tr + 1), C = __ldg(tr + 2);
                n_leaves++;
                TriHit th;
                if (tri_test(ld3(A), ld3(B), ld3(C), o, d, EPS_TRACE, best_t, th)) {
                    const uint64_t key = ((uint64_t)__float_as_uint(A.w) << 32) | __float_as_uint(B.w);
                    if (th.t < best_t || key < best_key) {
                        best_t = th.t;
                        best_key = key;
                        hrec = ~node;
                        hfh = 0;
                        hb1 = th.b1;
                        hb2 = th.b2;
                    }
                }
                done = !pop_near(stack, sp, best_t, node);
            } else if (!done) {  // leaf: the exposed faces of one surface block
                const int4 r = __ldg(recs + (~node));
                n_leaves++;
                const int wx = rec_wx(r), wy = rec_wy(r), wz = rec_wz(r);
                const uint32_t mask = ((uint32_t)r.z >> 15) & 63u;
                const uint64_t ikey = (uint64_t)rec_inst(r) << 32;
                for (uint32_t m = mask; m; m &= m - 1u) {
                    const int f = __ffs(m) - 1;
                    FaceHit fh;
                    if (face_test(wx, wy, wz, f, o, d, inv, EPS_TRACE, best_t, fh)) {
                        const uint32_t rank = __popc(mask & ((1u << f) - 1u));
                        const uint64_t key = ikey | ((uint32_t)r.w + 2u * rank + (uint32_t)fh.half);
                        if (fh.t < best_t || key < best_key) {
                            best_t = fh.t;
                            best_key = key;
                            hrec = ~node;
                            hfh = (uint32_t)f | ((uint32_t)fh.half << 3);
                            hb1 = fh.b1;
                            hb2 = fh.b2;
                        }
                    }
                }
                done = !pop_near(stack, sp, best_t, node);
            }
            if (done) {
                a.hits[p] = make_int4(hrec, (int)hfh, __float_as_int(hb1), __float_as_int(hb2));
                has = false;
            }
        }
    }
    for (int off = 16; off; off >>= 1) {
        traced += __shfl_xor_sync(FULL, traced, off);
        n_nodes += __shfl_xor_sync(FULL, n_nodes, off);
        n_leaves += __shfl_xor_sync(FULL, n_leaves, off);
    }
    if (lane == 0 && traced) {
        atomicAdd(reinterpret_cast<unsigned long long *>(a.counters + CNT_RAYS), (unsigned long long)traced);
        atomicAdd(reinterpret_cast<unsigned long long *>(a.counters + CNT_NODES), (unsigned long long)n_nodes);
        atomicAdd(reinterpret_cast<unsigned long long *>(a.counters + CNT_LEAVES), (unsigned long long)n_leaves);
    }
}

// Shading of one path vertex (raytrace.rs:405-577): the hit's material
// (constant slot colours or the texture atlas), emission, and the sampled
// continuation (mirror, transmission, or Lambertian with light-BVH NEE
// sampling).
struct ShadeOut {
    f3 n, E, R, new_o, new_d;
    float mis, pdf;
    int face, half;
    int4 rc;
};

// need_dir false: the path ends at this vertex (its last bounce, or a cache
// frame's query vertex of a path that does not train; no capture) and only
// its emission (or the cache's prediction) reaches the image: the outgoing radiance of the last
// vertex is E + (R * 0) * w = E for any finite R >= 0 and w > 0, and the
// vertex position keeps its offset; the Lambertian continuation (light-BVH
// descent and direction sampling) is skipped, with mis 0 and pdf 1.
template <bool MESH>
__device__ __forceinline__ void shade_vertex(const DevScene &S, uint32_t nee_type, uint32_t b, uint32_t seed, f3 o,
                                             f3 d, int4 hv, bool need_dir, ShadeOut &out) {
    f3 n, E, R, new_o, new_d;
    float mis = 0.0f, pdf = 1.0f;
    int face = 0, half = 0;
    int4 rc = make_int4(0, 0, 0, 0);
    if (hv.x < 0) {
        new_o = add3(o, scl3(d, 5000.0f));
        new_d = f3{0.0f, 0.0f, 0.0f};
        n = f3{0.0f, 0.0f, 0.0f};
        const float sky = (dot3(d, f3{0.0f, 1.0f, 0.0f}) > 0.9f) ? 50.0f : 0.0f;
        E = f3{sky, sky, sky};
        R = f3{0.0f, 0.0f, 0.0f};
    } else {
        const float b1 = __int_as_float(hv.z), b2 = __int_as_float(hv.w);
        const float b0 = (1.0f - b1) - b2;
        f3 t0, t1, t2;
        Frame fr;
        uint32_t slot;
        float u = 0.0f, v = 0.0f;  // the texture coordinate (read with an atlas only)
        if (MESH && (uint32_t)hv.x >= S.n_blk_rec) {
            // a mesh triangle: its world-space vertices and material slot;
            // localCoordinateSystem of the triangle (raytrace.rs:319-331);
            // face carries bit 31 | its record (the normal of the light-pdf walk)
            const uint32_t tr = (uint32_t)hv.x - S.n_blk_rec;
            const float4 *q = S.tri_rec + 3 * (size_t)tr;
            const float4 A = __ldg(q), B = __ldg(q + 1), C = __ldg(q + 2);
            t0 = ld3(A);
            t1 = ld3(B);
            t2 = ld3(C);
            fr = tri_frame(t0, t1, t2);
            slot = __float_as_uint(C.w);
            face = (int)(0x80000000u | tr);
            rc = make_int4((int)__float_as_uint(A.w), (int)__float_as_uint(B.w), -1, 0);
            if (S.atlas) {  // uv = v0.uv * b0 + v1.uv * b1 + v2.uv * b2 (raytrace.rs:457)
                const float *uv = S.inst[rc.x].uv + 6 * (size_t)rc.y;
                u = ((__ldg(uv) * b0) + (__ldg(uv + 2) * b1)) + (__ldg(uv + 4) * b2);
                v = ((__ldg(uv + 1) * b0) + (__ldg(uv + 3) * b1)) + (__ldg(uv + 5) * b2);
            }
        } else {
            rc = __ldg(S.geo_rec + hv.x);
            face = hv.y & 7;
            half = (hv.y >> 3) & 1;
            const int wx = rec_wx(rc), wy = rec_wy(rc), wz = rec_wz(rc);
            t0 = corner_pos(wx, wy, wz, face_corner(face, half, 0));
            t1 = corner_pos(wx, wy, wz, face_corner(face, half, 1));
            t2 = corner_pos(wx, wy, wz, face_corner(face, half, 2));
            fr = c_frames[2 * face + half];
            const uint32_t blk_id = ((uint32_t)rc.z >> 21) & 0xFFu;
            slot = 6u * blk_id + (uint32_t)face;
            if (S.atlas) {  // gen_mesh's corner uvs
                const uint32_t q0 = face_uv(face, half, 0), q1 = face_uv(face, half, 1),
                               q2 = face_uv(face, half, 2);
                u = (((float)(q0 & 1u) * b0) + ((float)(q1 & 1u) * b1)) + ((float)(q2 & 1u) * b2);
                v = (((float)(q0 >> 1) * b0) + ((float)(q1 >> 1) * b1)) + ((float)(q2 >> 1) * b2);
            }
        }
        n = fr.n;
        new_o = add3(add3(scl3(t0, b0), scl3(t1, b1)), scl3(t2, b2));
        const float ndd = -dot3(d, n);
        float alpha, metal;
        if (S.atlas) {
            // texture atlas: the three maps at the interpolated uv
            // (raytrace.rs:457-480), nearest texel clamped to the edge
            const int aw = (int)S.atlas_w, ah = (int)S.atlas_h;
            const int ix = min(max((int)floorf(u * (float)aw), 0), aw - 1);
            const int iy = min(max((int)floorf(v * (float)ah), 0), ah - 1);
            const size_t texel = (size_t)slot * 3 * aw * ah + (size_t)iy * aw + ix, map = (size_t)aw * ah;
            const uchar4 x0 = __ldg(S.atlas + texel), x1 = __ldg(S.atlas + texel + map),
                         x2 = __ldg(S.atlas + texel + 2 * map);
            const float *lin = S.srgb;
            R = f3{__ldg(lin + x0.x), __ldg(lin + x0.y), __ldg(lin + x0.z)};
            alpha = (float)x0.w / 255.0f;
            E = f3{(1000.0f * __ldg(lin + x1.x)) * ndd, (1000.0f * __ldg(lin + x1.y)) * ndd,
                   (1000.0f * __ldg(lin + x1.z)) * ndd};
            metal = __ldg(lin + x2.x);
        } else {
            const vrg_material &m = S.mats[slot];
            R = f3{__ldg(&m.reflectivity[0]), __ldg(&m.reflectivity[1]), __ldg(&m.reflectivity[2])};
            alpha = __ldg(&m.alpha);
            metal = __ldg(&m.metallic);
            E = f3{__ldg(&m.emission[0]) * ndd, __ldg(&m.emission[1]) * ndd, __ldg(&m.emission[2]) * ndd};
        }
        const float r0 = mm_rand(mm_combine(seed, 0));
        if (r0 < metal) {
            pdf = 1.0f;
            new_d = sub3(d, lscl3(2.0f * dot3(n, d), n));
        } else if (r0 < metal + (1.0f - alpha)) {
            new_d = d;
            R = f3{1.0f, 1.0f, 1.0f};
            pdf = 1.0f;
        } else {
            new_o = add3(new_o, lscl3(EPS_TRACE * 1.5f, n));
            R = f3{R.x / PI_F, R.y / PI_F, R.z / PI_F};
            if (!need_dir) {
                new_d = f3{0.0f, 0.0f, 0.0f};
                goto done;
            }
            Descent res;
            res.success = false;
            res.importance = 0.0f;
            if (nee_type == 1 || (nee_type == 2 && b == 1))
                res = light_descent(S, new_o, n, mm_combine(seed, 2));
            if (res.success && res.importance > 0.0f) mis = 0.3f;
            const float mis_rand = mm_rand(mm_combine(seed, 3));
            float ux = mm_rand(mm_combine(seed, 4)), uy = mm_rand(mm_combine(seed, 5));
            if (mis_rand < mis) {
                f3 lt[3];
                light_tri_world(S, res.inst, res.leaf, lt);
                if (ux + uy > 1.0f) { ux = 1.0f - ux; uy = 1.0f - uy; }  // triangleSample
                const float bx = (1.0f - ux) - uy;
                const f3 sp = add3(add3(lscl3(bx, lt[0]), lscl3(ux, lt[1])), lscl3(uy, lt[2]));
                new_d = norm3(sub3(sp, new_o));
            } else {
                float s, c;
                sincos_turns(ux, &s, &c);
                const float vv = sqrtf(fmaxf(0.0f, 1.0f - uy * uy));
                const f3 hs = f3{vv * c, uy, vv * s};
                new_d = norm3(add3(add3(lscl3(hs.x, fr.t), lscl3(hs.y, fr.n)), lscl3(hs.z, fr.b)));
            }
            pdf = dot3(new_d, n) / PI_F;
        }
    }
done:
    out.n = n;
    out.E = E;
    out.R = R;
    out.new_o = new_o;
    out.new_d = new_d;
    out.mis = mis;
    out.pdf = pdf;
    out.face = face;
    out.half = half;
    out.rc = rc;
}

// ---------------------------------------------------------------------------
// k_shade: shading of the hit, light-BVH descent and direction sampling
// (raytrace.rs:405-577).  Rays whose light pdf is needed are queued for
// k_anyhit; the others get their (E, w) (R, q) record here.
// ---------------------------------------------------------------------------
constexpr uint32_t SHADE_BATCH = 4;  // queue entries per lane of a surface-first shading batch

// the bounces whose shading takes its queue in routed batches (k_shade)
__host__ __device__ __forceinline__ bool shade_split(const FrameArgs &a, uint32_t b) {
    return b > 0 && b + 1 < a.nb;
}

// A cache frame's query vertex continues on one path in 16: the training
// paths, picked by a hash of the frame and the view's pixel.
__device__ __forceinline__ bool want_train_of(const ViewDev &V, uint32_t lp) {
    return (mm_finalize(mm_combine(V.frame * 0x9E3779B9u + 0x7a11u, lp)) & 15u) == 0u;
}

template <bool CAPTURE, bool BATCH, bool MESH, bool SPLIT>
__global__ void __launch_bounds__(128, 8) k_shade(const __grid_constant__ FrameArgs a, uint32_t b) {
    // per warp: the batch's pixels, surface hits first
    __shared__ uint32_t s_route[SPLIT ? 4 : 1][SPLIT ? 32 * SHADE_BATCH : 1];
    const int lane = threadIdx.x & 31;
    const uint32_t P = a.P, nb = a.nb;
    const uint32_t n_in = (b == 0) ? a.n0 : a.counters[a.qsel ? CNT_TQUEUE : CNT_QUEUE + b];
    const uint32_t *qin = a.qsel ? a.tq : a.queue[(b + 1) & 1];
    uint32_t *qout = a.queue[b & 1];
    // the bounce before a split query bounce: training candidates go to tq
    const bool to_tq = a.tq_split && b + 2 == a.nb_render;
    const float inv2pi = 1.0f / (2.0f * PI_F);
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    const uint32_t wid = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    // SPLIT (secondary bounces that continue): each warp takes SHADE_BATCH x
    // 32 queue entries and shades first those that sample a continuation (the
    // light-BVH descent and the direction), 32 at a time, then the others, so
    // that a lane with little to do does not sit out its neighbours'
    // descents.  Those are the surface hits, and at a cache frame's query
    // vertex (without capture) the surface hits of the training paths; the
    // others are the sky misses, and the query vertices that end into the
    // cache.  Every pixel's results are independent of the order of shading.
    const bool split = SPLIT && shade_split(a, b);
    const bool route_train = !CAPTURE && a.cache && b + 1 == a.nb_render;
    const uint32_t span = split ? 32u * SHADE_BATCH : 32u;
    uint32_t *route = s_route[threadIdx.x >> 5];
    for (uint32_t base = wid * span; base < n_in; base += warps * span) {
        uint32_t n_route = 0;
        if (split) {
            uint32_t pk[SHADE_BATCH], surf[SHADE_BATCH], valid[SHADE_BATCH];
            uint32_t n_surf = 0;
#pragma unroll
            for (uint32_t k = 0; k < SHADE_BATCH; k++) {
                const uint32_t i = base + 32 * k + lane;
                const bool v = i < n_in;
                pk[k] = v ? qin[i] : 0u;
                bool sf = v && a.hits[pk[k]].x >= 0;
                if (sf && route_train) {
                    const ViewDev &V = view_of<BATCH>(a, pk[k]);
                    sf = want_train_of(V, pk[k] - V.pix_off);
                }
                surf[k] = __ballot_sync(FULL, sf);
                valid[k] = __ballot_sync(FULL, v);
                n_surf += __popc(surf[k]);
            }
            uint32_t before_s = 0, before_m = n_surf;
#pragma unroll
            for (uint32_t k = 0; k < SHADE_BATCH; k++) {
                const uint32_t miss = valid[k] & ~surf[k];
                if ((surf[k] >> lane) & 1u) route[before_s + __popc(surf[k] & lanemask_lt())] = pk[k];
                else if ((miss >> lane) & 1u) route[before_m + __popc(miss & lanemask_lt())] = pk[k];
                before_s += __popc(surf[k]);
                before_m += __popc(miss);
            }
            n_route = before_m;
            __syncwarp();
        }
        const uint32_t passes = split ? (n_route + 31u) / 32u : 1u;
        for (uint32_t pass = 0; pass < passes; pass++) {
            uint32_t p = 0;
            bool active;
            if (split) {
                const uint32_t r = 32 * pass + lane;
                active = r < n_route;
                if (active) p = route[r];
            } else {
                const uint32_t i = base + lane;
                active = i < n_in && (b == 0 ? bounce0_pixel<BATCH>(a, i, p) : (p = qin[i], true));
            }
            bool cont = false, anyj = false, qhit = false, want_train = false;
            const bool at_query = a.cache && b + 1 == a.nb_render;
            f3 stash_E = f3{0, 0, 0}, stash_R = f3{0, 0, 0}, stash_n = f3{0, 0, 0};
            float stash_mis = 0.0f;
            int4 stash_hit = make_int4(-1, 0, 0, 0), stash_rc = make_int4(0, 0, 0, 0);
            int stash_half = 0;
            f3 new_o = f3{0, 0, 0}, new_d = f3{0, 0, 0};
            float pdf = 1.0f;
            int face = 0;
            if (active) {
                const ViewDev &V = view_of<BATCH>(a, p);
                const uint32_t lp = p - V.pix_off;
                f3 o, d;
                if (b == 0) {
                    raygen(V, lp, o, d);
                    if (CAPTURE) {
                        st3(a.c_origin, p, o);
                        st3(a.c_dir, p, d);
                    }
                } else {
                    o = ld3(a.ray_o[p]);
                    d = ld3(a.ray_d[p]);
                }
                const uint32_t seed = mm_combine(V.frame * nb + b, lp);  // interactive_rendering.rs:1189
                const int4 hv = a.hits[p];
                // A cache frame's query vertex continues only on its training paths
                // (one in 16): on the others the cache's prediction replaces the
                // vertex's outgoing radiance, and its record, direction and light
                // pdf are never read, so they skip the continuation as a last
                // vertex does.
                if (at_query || to_tq) want_train = want_train_of(V, lp);
                ShadeOut so;
                shade_vertex<MESH>(V.sc, a.nee_type, b, seed, o, d, hv,
                                   CAPTURE || (b + 1 < nb && (!at_query || want_train)), so);
                const f3 n = so.n, E = so.E;
                f3 R = so.R;
                const float mis = so.mis;
                const int half = so.half;
                const int4 rc = so.rc;
                new_o = so.new_o;
                new_d = so.new_d;
                pdf = so.pdf;
                face = so.face;
                // the light pdf of the chosen direction (nee_pdf pass, bounce nb-1 never computed)
                if (hv.x >= 0) anyj = (b + 1 < nb) && mis != 0.0f && len3(new_d) != 0.0f;
                // radiance cache: the vertex where rendered paths end into the cache
                // (every pixel's flag is cleared at bounce 0, so a path that ends
                // before the query vertex never reads a stale one)
                if (a.cache && b == 0 && !at_query) a.qflag[p] = 0;
                if (at_query) {
                    qhit = hv.x >= 0;
                    a.qflag[p] = qhit ? 1 : 0;
                    if (qhit) {
                        // the cache's normal: a face index, or a mesh normal packed in 32 bits
                        a.q_pos[p] = make_float4(new_o.x, new_o.y, new_o.z,
                                                 face >= 0 ? __int_as_float(face) : __uint_as_float(pack_normal10(so.n)));
                        a.q_dir[p] = make_float4(d.x, d.y, d.z, 0.0f);
                    }
                }
                // stash for the second half (after the warp-level training-slot grant)
                stash_E = E;
                stash_R = R;
                stash_n = n;
                stash_mis = mis;
                stash_hit = hv;
                stash_rc = rc;
                stash_half = half;
            }
            // training paths: up to train_cap per frame, granted per warp
            bool is_train = false;
            if (at_query) {
                const uint32_t tm = __ballot_sync(FULL, active && qhit && want_train);
                const uint32_t im = __ballot_sync(FULL, active && qhit);
                uint32_t tb = 0, ib = 0;
                if (lane == 0) {
                    if (tm) tb = atomicAdd(&a.counters[CNT_TRAIN], (uint32_t)__popc(tm));
                    if (im) ib = atomicAdd(&a.counters[CNT_INFER], (uint32_t)__popc(im));
                }
                tb = __shfl_sync(FULL, tb, 0);
                ib = __shfl_sync(FULL, ib, 0);
                if (active && qhit) a.infer_list[ib + __popc(im & lanemask_lt())] = p;
                if (active && qhit && want_train) {
                    const uint32_t slot = tb + __popc(tm & lanemask_lt());
                    if (slot < a.train_cap) {
                        a.train_list[slot] = p;
                        is_train = true;
                    }
                }
                if (!is_train) anyj = false;  // the record of this bounce is replaced by the cache
            }
            if (active) {
                const f3 E = stash_E, R = stash_R, n = stash_n;
                const float mis = stash_mis;
                const int4 hv = stash_hit, rc = stash_rc;
                const int half = stash_half;
                const size_t rb = (size_t)b * 2 * P;
                if (anyj) {
                    a.rec[rb + p] = make_float4(E.x, E.y, E.z, 0.0f);
                    a.rec[rb + P + p] = make_float4(R.x, R.y, R.z, 0.0f);
                } else {
                    const float q = 0.0f * mis + (1.0f - mis) * inv2pi;
                    const float w = pdf / q;
                    a.rec[rb + p] = make_float4(E.x, E.y, E.z, w);
                    a.rec[rb + P + p] = make_float4(R.x, R.y, R.z, q);
                }
                if (b == 0) {
                    a.xv[p] = make_float4(new_o.x, new_o.y, new_o.z, 0.0f);
                    a.nv[p] = make_float4(n.x, n.y, n.z, 0.0f);
                } else if (b == 1) {
                    a.xs[p] = make_float4(new_o.x, new_o.y, new_o.z, 0.0f);
                    a.ns[p] = make_float4(n.x, n.y, n.z, 0.0f);
                }
                cont = !zero3(new_d) && (b + 1 < nb) && (!at_query || is_train);
                if (cont) {
                    // .w of the ray carries the face and the bsdf pdf to k_anyhit
                    a.ray_o[p] = make_float4(new_o.x, new_o.y, new_o.z, __int_as_float(face));
                    a.ray_d[p] = make_float4(new_d.x, new_d.y, new_d.z, pdf);
                } else {
                    a.nlive[p] = (uint8_t)(b + 1);
                }
                if (CAPTURE) {
                    const size_t s1 = (size_t)(b + 1) * P + p, s0 = (size_t)b * P + p;
                    st3(a.c_origin, s1, new_o);
                    st3(a.c_dir, s1, new_d);
                    st3(a.c_normal, s0, n);
                    st3(a.c_emis, s0, E);
                    st3(a.c_refl, s0, R);
                    a.c_mis[s0] = mis;
                    a.c_pdf[s0] = pdf;
                    a.c_nee[s0] = 0.0f;
                    uint4 hw;
                    if (face < 0) {  // a mesh triangle: (instance, triangle)
                        hw = make_uint4((uint32_t)rc.x, (uint32_t)rc.y, INVALID, 0u);
                    } else if (hv.x >= 0) {
                        const uint32_t mask = ((uint32_t)rc.z >> 15) & 63u;
                        hw.x = rec_inst(rc);
                        hw.y = (uint32_t)rc.w + 2u * __popc(mask & ((1u << face) - 1u)) + (uint32_t)half;
                        hw.z = (uint32_t)rc.z & 0x7FFFu;
                        hw.w = (uint32_t)face | ((uint32_t)half << 8);
                    } else {
                        hw = make_uint4(INVALID, INVALID, INVALID, INVALID);
                    }
                    reinterpret_cast<uint4 *>(a.c_hit)[s0] = hw;
                }
            }
            // compaction: continuing rays into the next bounce queue, light-pdf jobs
            // into the any-hit queue (one ballot + one atomic per warp each)
            const bool cont_t = cont && to_tq && want_train;  // a training candidate's ray
            const uint32_t cm = __ballot_sync(FULL, cont && !cont_t);
            const uint32_t am = __ballot_sync(FULL, anyj);
            uint32_t qb = 0, ab = 0;
            if (lane == 0) {
                if (cm) qb = atomicAdd(&a.counters[CNT_QUEUE + b + 1], (uint32_t)__popc(cm));
                if (am) ab = atomicAdd(&a.counters[CNT_AQUEUE + b], (uint32_t)__popc(am));
            }
            qb = __shfl_sync(FULL, qb, 0);
            ab = __shfl_sync(FULL, ab, 0);
            if (cont && !cont_t) qout[qb + __popc(cm & lanemask_lt())] = p;
            if (to_tq) {
                const uint32_t tm = __ballot_sync(FULL, cont_t);
                uint32_t tb = 0;
                if (lane == 0 && tm) tb = atomicAdd(&a.counters[CNT_TQUEUE], (uint32_t)__popc(tm));
                tb = __shfl_sync(FULL, tb, 0);
                if (cont_t) a.tq[tb + __popc(tm & lanemask_lt())] = p;
            }
            if (anyj) {
                const uint32_t j = ab + __popc(am & lanemask_lt());
                a.aqueue[b & 1][j] = p;
                a.ajob[b & 1][2 * (size_t)j] = make_float4(new_o.x, new_o.y, new_o.z, __int_as_float(face));
                a.ajob[b & 1][2 * (size_t)j + 1] = make_float4(new_d.x, new_d.y, new_d.z, pdf);
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// The nee_pdf pass (nee_pdf.rs:281-337) for the queued rays, in three passes
// so that each runs with coherent lanes:
//   k_anyhit     every light triangle the ray crosses in [1e-4, 1000] is
//                collected (persistent warps, per-lane job replacement), in
//                ascending (instance, leaf) order; rays that cross none get
//                their record here;
//   k_hit_eval   one thread per hit: computeNeePdf (nee_pdf.rs:240-279) with
//                its reverse walk up the light BVH;
//   k_hit_sum    one thread per job: the sum in key order, then q and
//                w = bsdf_pdf / q complete the bounce record.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void finish_job(const FrameArgs &a, uint32_t b, uint32_t p, float pdf, float nee) {
    const float inv2pi = 1.0f / (2.0f * PI_F);
    const float mis = 0.3f;
    const float q = nee * mis + (1.0f - mis) * inv2pi;
    const float w = pdf / q;
    const size_t rb = (size_t)b * 2 * a.P;
    reinterpret_cast<float *>(a.rec + rb + p)[3] = w;
    reinterpret_cast<float *>(a.rec + rb + a.P + p)[3] = q;
}

template <bool CAPTURE, bool BATCH>
__global__ void __launch_bounds__(128, 8) k_anyhit(const __grid_constant__ FrameArgs a, uint32_t b) {
    // walk statistics, per lane: lamp nodes fetched, lamp blocks tested, light hits
    __shared__ uint32_t s_stat[3][128];
    const int lane = threadIdx.x & 31;
    const int REFILL = (int)a.refill_any;
    const uint32_t n_in = a.counters[CNT_AQUEUE + b];
    uint32_t *err = a.counters + CNT_ERROR;
    const float4 *wide = a.v0.sc.lamp_wide;
    const int4 *recs = a.v0.sc.lamp_rec;
    const uint32_t *table = a.v0.sc.lamp_table;
    const float4 *tris = a.v0.sc.tri_rec;
    int root = a.v0.sc.lamp_root;
    const float tmin = EPS_NEE, tmax = 1000.0f;
    bool has = false, exhausted = false;
    uint32_t p = 0, idx = 0, steps = 0;
    f3 o = f3{0, 0, 0}, d = f3{0, 0, 0}, inv = f3{0, 0, 0}, oi = f3{0, 0, 0};
    float pdf = 0.0f;
    int node = 0, sp = 0, nh = 0;
    int px = 0, py = 2, pz = 4;  // near-plane float4 per axis, picked by the ray's direction signs
    int stack[TRAV_STACK];
    uint64_t keys[LIGHT_LIST];
    float b1s[LIGHT_LIST], b2s[LIGHT_LIST];
    if (blockIdx.x == 0 && threadIdx.x == 0 && n_in)
        atomicAdd(reinterpret_cast<unsigned long long *>(a.counters + CNT_ANY), (unsigned long long)n_in);
    s_stat[0][threadIdx.x] = 0;
    s_stat[1][threadIdx.x] = 0;
    s_stat[2][threadIdx.x] = 0;
    while (true) {
        const uint32_t need = __ballot_sync(FULL, !has);
        if (!exhausted && need && (__popc(need) >= REFILL || need == FULL)) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(&a.counters[CNT_AFETCH + b], (uint32_t)__popc(need));
            base = __shfl_sync(FULL, base, 0);
            if (base + (uint32_t)__popc(need) >= n_in) exhausted = true;
            if (!has) {
                idx = base + (uint32_t)__popc(need & lanemask_lt());
                if (idx < n_in) {
                    has = true;
                    p = a.aqueue[b & 1][idx];
                    if constexpr (BATCH) {
                        const ViewDev &V = view_of<BATCH>(a, p);
                        wide = V.sc.lamp_wide;
                        recs = V.sc.lamp_rec;
                        table = V.sc.lamp_table;
                        tris = V.sc.tri_rec;
                        root = V.sc.lamp_root;
                    }
                    const float4 ro = a.ajob[b & 1][2 * (size_t)idx], rd = a.ajob[b & 1][2 * (size_t)idx + 1];
                    o = ld3(ro);
                    d = ld3(rd);
                    pdf = rd.w;
                    inv = f3{slab_inv(d.x), slab_inv(d.y), slab_inv(d.z)};
                    oi = f3{-o.x * inv.x, -o.y * inv.y, -o.z * inv.z};
                    px = signbit(inv.x) ? 1 : 0;
                    py = signbit(inv.y) ? 3 : 2;
                    pz = signbit(inv.z) ? 5 : 4;
                    node = root;
                    sp = 0;
                    nh = 0;
                    steps = 0;
                }
            }
        }
        if (!__any_sync(FULL, has)) break;
        if (has) {
            bool done = (node == EMPTY_ROOT);
            // 4-wide lamp nodes: every crossed light counts, so children are
            // visited in slot order (no sorting); the first hit child is taken,
            // the others pushed
            while (!done && node >= 0) {
                const float4 *w = wide + 8 * (size_t)node;
                const float4 NX = __ldg(w + px), FX = __ldg(w + (px ^ 1)), NY = __ldg(w + py);
                const float4 FY = __ldg(w + (py ^ 1)), NZ = __ldg(w + pz), FZ = __ldg(w + (pz ^ 1));
                const float4 RF = __ldg(w + 6);
                const float nx[4] = {NX.x, NX.y, NX.z, NX.w}, fx[4] = {FX.x, FX.y, FX.z, FX.w};
                const float ny[4] = {NY.x, NY.y, NY.z, NY.w}, fy[4] = {FY.x, FY.y, FY.z, FY.w};
                const float nz[4] = {NZ.x, NZ.y, NZ.z, NZ.w}, fz[4] = {FZ.x, FZ.y, FZ.z, FZ.w};
                const int rf[4] = {__float_as_int(RF.x), __float_as_int(RF.y), __float_as_int(RF.z),
                                   __float_as_int(RF.w)};
                int next = EMPTY_ROOT;
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const float tn = fmax3(__fmaf_rn(nx[i], inv.x, oi.x), __fmaf_rn(ny[i], inv.y, oi.y),
                                           fmaxf(__fmaf_rn(nz[i], inv.z, oi.z), tmin));
                    const float tf = fmin3(__fmaf_rn(fx[i], inv.x, oi.x), __fmaf_rn(fy[i], inv.y, oi.y),
                                           fminf(__fmaf_rn(fz[i], inv.z, oi.z), tmax));
                    if (tn <= tf) {  // (an unused slot's inverted box is never entered)
                        if (next == EMPTY_ROOT) {
                            next = rf[i];
                        } else if (sp < TRAV_STACK) {
                            stack[sp++] = rf[i];
                        } else {
                            atomicOr(err, ERR_STACK);
                        }
                    }
                }
                if (next != EMPTY_ROOT) node = next;
                else if (sp == 0) done = true;
                else node = stack[--sp];
                if (++steps > TRAV_GUARD) {
                    atomicOr(err, ERR_GUARD);
                    done = true;
                }
            }
            if (!done) {  // leaf: one lamp block; each emissive face hit names one light triangle
                s_stat[1][threadIdx.x]++;
                const int4 r = __ldg(recs + (~node));
                const int wx = rec_wx(r), wy = rec_wy(r), wz = rec_wz(r);
                const uint32_t ii = rec_inst(r);
                if (r.z < 0) {  // a mesh light triangle: (leaf, world-space triangle record) in the table
                    const uint32_t leaf = __ldg(table + r.w), t = __ldg(table + r.w + 1);
                    const float4 *q = tris + 3 * (size_t)t;
                    TriHit th;
                    if (tri_test(ld3(__ldg(q)), ld3(__ldg(q + 1)), ld3(__ldg(q + 2)), o, d, tmin, tmax, th)) {
                        const uint64_t key = ((uint64_t)ii << 32) | leaf;
                        if (nh < LIGHT_LIST) {
                            int j = nh++;
                            while (j > 0 && keys[j - 1] > key) {
                                keys[j] = keys[j - 1];
                                b1s[j] = b1s[j - 1];
                                b2s[j] = b2s[j - 1];
                                j--;
                            }
                            keys[j] = key;
                            b1s[j] = th.b1;
                            b2s[j] = th.b2;
                        } else {
                            atomicOr(err, ERR_LIGHT_LIST);
                        }
                    }
                }
                for (uint32_t fm = r.z < 0 ? 0u : (uint32_t)r.z; fm; fm &= fm - 1u) {
                    const int f = __ffs(fm) - 1;
                    FaceHit fh;
                    if (!face_test(wx, wy, wz, f, o, d, inv, tmin, tmax, fh)) continue;
                    const uint32_t leaf = __ldg(table + r.w + 2 * f + fh.half);
                    if (leaf == INVALID) continue;
                    const uint64_t key = ((uint64_t)ii << 32) | leaf;
                    if (nh < LIGHT_LIST) {
                        int j = nh++;
                        while (j > 0 && keys[j - 1] > key) {
                            keys[j] = keys[j - 1];
                            b1s[j] = b1s[j - 1];
                            b2s[j] = b2s[j - 1];
                            j--;
                        }
                        keys[j] = key;
                        b1s[j] = fh.b1;
                        b2s[j] = fh.b2;
                    } else {
                        atomicOr(err, ERR_LIGHT_LIST);
                    }
                }
                if (sp == 0) done = true;
                else node = stack[--sp];
            }
            if (done) {
                s_stat[0][threadIdx.x] += steps;
                s_stat[2][threadIdx.x] += (uint32_t)nh;
                uint32_t hb = 0;
                if (nh > 0) {
                    hb = atomicAdd(a.hit_count, (uint32_t)nh);
                    if (hb + (uint32_t)nh > a.hit_cap) {
                        atomicOr(err, ERR_LIGHT_LIST);
                        nh = 0;
                    }
                }
                if (nh == 0) {
                    finish_job(a, b, p, pdf, 0.0f);
                    if (CAPTURE) a.c_nee[(size_t)b * a.P + p] = 0.0f;
                } else {
                    for (int j = 0; j < nh; j++) {
                        a.hitbuf[2 * (size_t)(hb + j)] =
                            make_uint4(p, (uint32_t)(keys[j] >> 32), (uint32_t)keys[j], __float_as_uint(b1s[j]));
                        a.hitbuf[2 * (size_t)(hb + j) + 1] = make_uint4(__float_as_uint(b2s[j]), idx, 0u, 0u);
                    }
                }
                a.jmeta[idx] = make_uint2(hb, (uint32_t)nh);
                has = false;
            }
        }
    }
    const uint32_t n_nodes = __reduce_add_sync(FULL, s_stat[0][threadIdx.x]);
    const uint32_t n_leaves = __reduce_add_sync(FULL, s_stat[1][threadIdx.x]);
    const uint32_t n_hits = __reduce_add_sync(FULL, s_stat[2][threadIdx.x]);
    if (lane == 0 && n_nodes) {
        atomicAdd(reinterpret_cast<unsigned long long *>(a.counters + CNT_ANODES), (unsigned long long)n_nodes);
        atomicAdd(reinterpret_cast<unsigned long long *>(a.counters + CNT_ALEAVES), (unsigned long long)n_leaves);
        atomicAdd(reinterpret_cast<unsigned long long *>(a.counters + CNT_AHITS), (unsigned long long)n_hits);
    }
}

template <bool BATCH>
__global__ void __launch_bounds__(128) k_hit_eval(const __grid_constant__ FrameArgs a, uint32_t b) {
    const uint32_t n = min(*a.hit_count, a.hit_cap);
    for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h < n; h += gridDim.x * blockDim.x) {
        const uint4 A = a.hitbuf[2 * (size_t)h], B = a.hitbuf[2 * (size_t)h + 1];
        const uint32_t p = A.x;
        const float4 ro = a.ajob[b & 1][2 * (size_t)B.y], rd = a.ajob[b & 1][2 * (size_t)B.y + 1];
        const DevScene &sc = view_of<BATCH>(a, p).sc;
        // the shading normal of the job's vertex: a voxel face's, or a mesh
        // triangle's, recomputed as its shading computed it
        const int fw = __float_as_int(ro.w);
        f3 n3;
        if (fw >= 0) {
            n3 = c_frames[2 * fw].n;
        } else {
            const float4 *q = sc.tri_rec + 3 * (size_t)((uint32_t)fw & 0x7FFFFFFFu);
            n3 = tri_frame(ld3(__ldg(q)), ld3(__ldg(q + 1)), ld3(__ldg(q + 2))).n;
        }
        a.hitval[h] = nee_pdf_of(sc, ld3(ro), n3, ld3(rd), A.y, A.z, __uint_as_float(A.w), __uint_as_float(B.x));
    }
}

template <bool CAPTURE>
__global__ void __launch_bounds__(128) k_hit_sum(const __grid_constant__ FrameArgs a, uint32_t b) {
    const uint32_t n_in = a.counters[CNT_AQUEUE + b];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_in; i += gridDim.x * blockDim.x) {
        const uint2 m = a.jmeta[i];
        if (m.y == 0) continue;
        const uint32_t p = a.aqueue[b & 1][i];
        float nee = 0.0f;
        for (uint32_t j = 0; j < m.y; j++) nee += a.hitval[m.x + j];
        finish_job(a, b, p, a.ajob[b & 1][2 * (size_t)i + 1].w, nee);
        if (CAPTURE) a.c_nee[(size_t)b * a.P + p] = nee;
    }
}

}  // namespace

vrg_status upload_frames(cudaStream_t s) {
    Frame fr[12];
    for (int f = 0; f < 6; f++)
        for (int h = 0; h < 2; h++) fr[2 * f + h] = face_frame(f, h);
    VRG_CUDA_TRY(cudaMemcpyToSymbolAsync(c_frames, fr, sizeof(fr), 0, cudaMemcpyHostToDevice, s));
    return VRG_OK;
}

static int occupancy_grid(const void *fn, int threads) {
    int dev = 0, sms = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, threads, 0);
    return std::max(1, sms) * std::max(1, n);
}

// full-occupancy grids of the persistent bounce kernels, [single view,
// batched] (set once, before any stream capture)
static int g_trace[2] = {0, 0}, g_shade[2] = {0, 0}, g_any[2] = {0, 0};
static int g_sms = 1;
static std::once_flag g_grids_once;

static void init_grids_once() {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    g_sms = std::max(1, g_sms);
    g_shade[0] = occupancy_grid((const void *)k_shade<false, false, false, false>, 128);
    g_shade[1] = occupancy_grid((const void *)k_shade<false, true, false, false>, 128);
    g_any[0] = occupancy_grid((const void *)k_anyhit<false, false>, 128);
    g_any[1] = occupancy_grid((const void *)k_anyhit<false, true>, 128);
    g_trace[1] = occupancy_grid((const void *)k_trace<true, false>, 128);
    g_trace[0] = occupancy_grid((const void *)k_trace<false, false>, 128);
}

// (thread-safe: renderers may be created from several threads)
static void init_grids() { std::call_once(g_grids_once, init_grids_once); }

// resident CTAs per SM at full occupancy of (closest hit, shading, light
// hits), the bound of a tuned persistent grid; and the SM count
void bounce_occupancy(bool batch, int occ[3], int *sms) {
    init_grids();
    const int v = batch ? 1 : 0;
    occ[0] = std::max(1, g_trace[v] / g_sms);
    occ[1] = std::max(1, g_shade[v] / g_sms);
    occ[2] = std::max(1, g_any[v] / g_sms);
    *sms = g_sms;
}

// A bounce in two launches groups.  A batched frame (a.views set) runs the
// variants that look up each pixel's view.  max_rays > 0 bounds the rays of the
// bounce (a cache frame's training paths): the persistent grids then shrink to
// one lane per ray, leaving the other SMs to the work that runs beside them.
static void bounce_grids(const FrameArgs &a, uint32_t max_rays, int &gt, int &gs, int &ga) {
    init_grids();
    const int v = a.views ? 1 : 0;
    gt = a.grid_trace ? std::min((int)a.grid_trace, g_trace[v]) : g_trace[v];
    gs = a.grid_shade ? std::min((int)a.grid_shade, g_shade[v]) : g_shade[v];
    ga = a.grid_any ? std::min((int)a.grid_any, g_any[v]) : g_any[v];
    if (max_rays) {
        const int cap = (int)std::max<uint32_t>(1u, (max_rays + 127) / 128);
        gt = std::min(gt, cap);
        gs = std::min(gs, cap);
        ga = std::min(ga, cap);
    }
}

// closest hit of bounce b
vrg_status launch_trace(cudaStream_t s, const FrameArgs &a, uint32_t b, uint32_t max_rays) {
    int gt, gs, ga;
    bounce_grids(a, max_rays, gt, gs, ga);
    // the mesh-capable builds only for frames whose scenes hold meshes
    if (a.views) {
        if (a.mesh) k_trace<true, true><<<gt, 128, 0, s>>>(a, b);
        else k_trace<true, false><<<gt, 128, 0, s>>>(a, b);
    } else if (a.mesh) {
        k_trace<false, true><<<gt, 128, 0, s>>>(a, b);
    } else {
        k_trace<false, false><<<gt, 128, 0, s>>>(a, b);
    }
    VRG_CUDA_TRY(cudaGetLastError());
    return VRG_OK;
}

template <bool CAPTURE, bool BATCH, bool MESH>
static void shade_launch(int gs, cudaStream_t s, const FrameArgs &a, uint32_t b, bool split) {
    if (split) k_shade<CAPTURE, BATCH, MESH, true><<<gs, 128, 0, s>>>(a, b);
    else k_shade<CAPTURE, BATCH, MESH, false><<<gs, 128, 0, s>>>(a, b);
}

// shading of bounce b
vrg_status launch_shade(cudaStream_t s, const FrameArgs &a, uint32_t b, uint32_t max_rays) {
    int gt, gs, ga;
    bounce_grids(a, max_rays, gt, gs, ga);
    // (not for the few rays of a cache frame's training bounces, bounded by
    // max_rays: batches of 128 per warp would leave most of the grid idle)
    const bool split = shade_split(a, b) && max_rays == 0;
    if (a.mesh) {
        if (a.views) shade_launch<false, true, true>(gs, s, a, b, split);
        else if (a.capture) shade_launch<true, false, true>(gs, s, a, b, split);
        else shade_launch<false, false, true>(gs, s, a, b, split);
    } else {
        if (a.views) shade_launch<false, true, false>(gs, s, a, b, split);
        else if (a.capture) shade_launch<true, false, false>(gs, s, a, b, split);
        else shade_launch<false, false, false>(gs, s, a, b, split);
    }
    VRG_CUDA_TRY(cudaGetLastError());
    return VRG_OK;
}

// closest hit and shading of bounce b
vrg_status launch_trace_shade(cudaStream_t s, const FrameArgs &a, uint32_t b, cudaEvent_t ev_trace,
                              uint32_t max_rays) {
    if (a.views && a.capture) {
        set_error("capture is not available for batched frames");
        return VRG_ERR_UNSUPPORTED;
    }
    VRG_TRY(launch_trace(s, a, b, max_rays));
    if (ev_trace) VRG_CUDA_TRY(cudaEventRecord(ev_trace, s));
    return launch_shade(s, a, b, max_rays);
}

// the light-pdf walk of bounce b's jobs (bounces before the last): it reads only
// the jobs' own ray copies, so it may run beside bounce b + 1
vrg_status launch_light_pdf(cudaStream_t s, const FrameArgs &a, uint32_t b, uint32_t max_rays) {
    if (b + 1 >= a.nb) return VRG_OK;
    const bool batch = a.views != nullptr;
    int gt, gs, ga;
    bounce_grids(a, max_rays, gt, gs, ga);
    if (batch) k_anyhit<false, true><<<ga, 128, 0, s>>>(a, b);
    else if (a.capture) k_anyhit<true, false><<<ga, 128, 0, s>>>(a, b);
    else k_anyhit<false, false><<<ga, 128, 0, s>>>(a, b);
    if (batch) k_hit_eval<true><<<gs, 128, 0, s>>>(a, b);
    else k_hit_eval<false><<<gs, 128, 0, s>>>(a, b);
    if (a.capture) k_hit_sum<true><<<gs, 128, 0, s>>>(a, b);
    else k_hit_sum<false><<<gs, 128, 0, s>>>(a, b);
    VRG_CUDA_TRY(cudaMemsetAsync(a.hit_count, 0, 4, s));
    VRG_CUDA_TRY(cudaGetLastError());
    return VRG_OK;
}

}  // namespace vrg
