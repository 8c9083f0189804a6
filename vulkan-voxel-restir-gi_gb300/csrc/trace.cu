// Wavefront bounce kernel: ray generation (bounce 0), closest hit over the
// world-space voxel BVH, shading, light-BVH next-event estimation and the
// light-sampling pdf of the chosen direction, fused into one kernel per
// bounce.
//
// Reference stages fused here (one dispatch each in the reference):
//   raygen        raygen.rs:84-111
//   raytrace      raytrace.rs:390-578 (closest hit replaces the driver ray
//                 query; traverseBvh 218-281 is the light descent)
//   nee_pdf       nee_pdf.rs:281-337 (any-hit over light triangles along the
//                 chosen direction; reverseTraverseBvh 154-228)
// Work distribution: persistent warps fetch 32 rays at a time from the
// bounce's queue; rays that continue are compacted into the next queue with
// one warp ballot + one atomic per warp.  State per pixel stays in SoA
// float4 arrays; the per-bounce record (E, w=pdf/q) (R, q) feeds the
// backward radiance recurrence of the resolve kernel.
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

__device__ __forceinline__ bool slab(float lox, float hix, float loy, float hiy, float loz, float hiz, f3 o, f3 inv,
                                     float tmin, float tmax, float &tn) {
    float t0x = (lox - o.x) * inv.x, t1x = (hix - o.x) * inv.x;
    float t0y = (loy - o.y) * inv.y, t1y = (hiy - o.y) * inv.y;
    float t0z = (loz - o.z) * inv.z, t1z = (hiz - o.z) * inv.z;
    tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
    float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), tmax));
    return tn <= tf;
}

struct Hit {
    bool hit;
    float t, b1, b2;
    int face, half;
    int4 rec;
    uint32_t tri;
};

// Closest hit over the voxel faces; result independent of traversal order
// (ties on t go to the smaller (instance, triangle) key, boxes are culled
// only when strictly beyond the current best t).
__device__ Hit closest_hit(const DevScene &sc, f3 o, f3 d, float tmin, float tmax, uint32_t *err) {
    Hit h;
    h.hit = false;
    h.t = tmax;
    uint64_t best_key = ~0ull;
    int node = sc.geo_root;
    if (node == EMPTY_ROOT) return h;
    const f3 inv = f3{1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
    int stack[TRAV_STACK];
    int sp = 0;
    for (uint32_t guard = 0;; guard++) {
        if (guard > TRAV_GUARD) {  // only reachable with a malformed layout
            atomicOr(err, ERR_GUARD);
            break;
        }
        if (node >= 0) {
            const float4 *w = sc.geo_wide + 4 * (size_t)node;
            float4 A = __ldg(w), B = __ldg(w + 1), C = __ldg(w + 2), D = __ldg(w + 3);
            float tn0, tn1;
            bool h0 = slab(A.x, A.y, A.z, A.w, B.x, B.y, o, inv, tmin, h.t, tn0);
            bool h1 = slab(B.z, B.w, C.x, C.y, C.z, C.w, o, inv, tmin, h.t, tn1);
            int r0 = __float_as_int(D.x), r1 = __float_as_int(D.y);
            if (h0 && h1) {
                int nearr = r0, farr = r1;
                if (tn1 < tn0) { nearr = r1; farr = r0; }
                if (sp < TRAV_STACK) stack[sp++] = farr;
                else atomicOr(err, ERR_STACK);
                node = nearr;
                continue;
            }
            if (h0) { node = r0; continue; }
            if (h1) { node = r1; continue; }
        } else {
            const int4 r = __ldg(sc.geo_rec + (~node));
            const int wx = rec_wx(r), wy = rec_wy(r), wz = rec_wz(r);
            const uint32_t mask = ((uint32_t)r.z >> 15) & 63u;
            const uint64_t ikey = (uint64_t)rec_inst(r) << 32;
            for (uint32_t m = mask; m; m &= m - 1u) {
                int f = __ffs(m) - 1;
                FaceHit fh;
                if (face_test(wx, wy, wz, f, o, d, inv, tmin, h.t, fh)) {
                    uint32_t rank = __popc(mask & ((1u << f) - 1u));
                    uint32_t tri = (uint32_t)r.w + 2u * rank + (uint32_t)fh.half;
                    uint64_t key = ikey | tri;
                    if (fh.t < h.t || key < best_key) {
                        h.hit = true;
                        h.t = fh.t;
                        best_key = key;
                        h.b1 = fh.b1;
                        h.b2 = fh.b2;
                        h.face = f;
                        h.half = fh.half;
                        h.rec = r;
                        h.tri = tri;
                    }
                }
            }
        }
        if (sp == 0) break;
        node = stack[--sp];
    }
    return h;
}

// nodeImportance (raytrace.rs:181-208: uint visibility, EPS 1e-3;
// nee_pdf.rs:125-152: float visibility, EPS 1e-4); translation transforms
template <bool NEE>
__device__ __forceinline__ float node_importance(f3 point, f3 normal, const float off[3], const NodeV &n) {
    f3 v000 = f3{n.mn.x + off[0], n.mn.y + off[1], n.mn.z + off[2]};
    f3 v111 = f3{n.mx.x + off[0], n.mx.y + off[1], n.mx.z + off[2]};
    f3 e = sub3(v111, v000);
    f3 cc = sub3(lscl3(0.5f, add3(v000, v111)), point);
    float dist_sq = fmaxf(dot3(e, e), dot3(cc, cc));
    const float eps = NEE ? EPS_NEE : EPS_TRACE;
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
            if (importance == 0.0f) importance = node_importance<false>(point, normal, off, node);
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
        float lI = node_importance<false>(point, normal, off, left);
        float rI = node_importance<false>(point, normal, off, right);
        float tot = lI + rI;
        float ln = lI / tot, rn = rI / tot;
        (void)rn;
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
        float lI = node_importance<true>(point, normal, off, left);
        float rI = node_importance<true>(point, normal, off, right);
        float tot = lI + rI;
        float ln = lI / tot, rn = rI / tot;
        if (old == node.left) probability *= ln;
        else probability *= rn;
    }
    return probability;
}

__device__ __forceinline__ void light_tri_world(const DevScene &sc, uint32_t ii, uint32_t leaf, f3 tv[3]) {
    const InstDev &I = sc.inst[ii];
    uint32_t t = __ldg(I.light_leaf_tri + leaf);
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

// Sum of the light-sampling pdf over every light triangle the ray crosses in
// [1e-4, 1000] (nee_pdf.rs:302-336), added in ascending (instance, leaf) order.
__device__ float nee_any_hit(const DevScene &sc, f3 o, f3 d, f3 normal, uint32_t *err) {
    const float tmin = EPS_NEE, tmax = 1000.0f;
    int node = sc.light_root;
    if (node == EMPTY_ROOT) return 0.0f;
    const f3 inv = f3{1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
    uint64_t keys[LIGHT_LIST];
    float vals[LIGHT_LIST];
    int n = 0;
    int stack[TRAV_STACK];
    int sp = 0;
    for (uint32_t guard = 0;; guard++) {
        if (guard > TRAV_GUARD) {
            atomicOr(err, ERR_GUARD);
            break;
        }
        if (node >= 0) {
            const float4 *w = sc.light_wide + 4 * (size_t)node;
            float4 A = __ldg(w), B = __ldg(w + 1), C = __ldg(w + 2), D = __ldg(w + 3);
            float tn0, tn1;
            bool h0 = slab(A.x, A.y, A.z, A.w, B.x, B.y, o, inv, tmin, tmax, tn0);
            bool h1 = slab(B.z, B.w, C.x, C.y, C.z, C.w, o, inv, tmin, tmax, tn1);
            int r0 = __float_as_int(D.x), r1 = __float_as_int(D.y);
            if (h0 && h1) {
                if (sp < TRAV_STACK) stack[sp++] = r1;
                else atomicOr(err, ERR_STACK);
                node = r0;
                continue;
            }
            if (h0) { node = r0; continue; }
            if (h1) { node = r1; continue; }
        } else {
            const int4 r = __ldg(sc.light_rec + (~node));
            int f = r.z & 7, hh = (r.z >> 3) & 1;
            FaceHit fh;
            if (face_test(rec_wx(r), rec_wy(r), rec_wz(r), f, o, d, inv, tmin, tmax, fh) && fh.half == hh) {
                uint32_t ii = rec_inst(r), leaf = (uint32_t)r.w;
                float v = nee_pdf_of(sc, o, normal, d, ii, leaf, fh.b1, fh.b2);
                uint64_t key = ((uint64_t)ii << 32) | leaf;
                if (n < LIGHT_LIST) {
                    int j = n++;
                    while (j > 0 && keys[j - 1] > key) { keys[j] = keys[j - 1]; vals[j] = vals[j - 1]; j--; }
                    keys[j] = key;
                    vals[j] = v;
                } else {
                    atomicOr(err, ERR_LIGHT_LIST);
                }
            }
        }
        if (sp == 0) break;
        node = stack[--sp];
    }
    float pdf = 0.0f;
    for (int j = 0; j < n; j++) pdf += vals[j];
    return pdf;
}

__device__ __forceinline__ void st3(float *a, size_t i, f3 v) {
    a[3 * i] = v.x;
    a[3 * i + 1] = v.y;
    a[3 * i + 2] = v.z;
}

template <bool CAPTURE>
__global__ void __launch_bounds__(128) k_bounce(FrameArgs a, uint32_t b) {
    const int lane = threadIdx.x & 31;
    const uint32_t P = a.P, nb = a.nb;
    const uint32_t n_in = (b == 0) ? P : a.counters[CNT_QUEUE + b];
    const uint32_t *qin = a.queue[(b + 1) & 1];
    uint32_t *qout = a.queue[b & 1];
    uint32_t *err = a.counters + CNT_ERROR;
    const uint32_t inv_seed = a.frame * nb + b;  // interactive_rendering.rs:1189
    const float inv2pi = 1.0f / (2.0f * PI_F);
    while (true) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&a.counters[CNT_FETCH + b], 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n_in) break;
        const uint32_t i = base + lane;
        const bool active = i < n_in;
        bool cont = false, traced_any = false;
        uint32_t p = 0;
        if (active) {
            p = (b == 0) ? i : qin[i];
            f3 o, d;
            if (b == 0) {
                // raygen (raygen.rs:84-111): pixel corner, jitter x0.00
                uint32_t x = p % a.W, y = p / a.W;
                float u = 2.0f * (float)x / (float)a.W - 1.0f;
                float v = 2.0f * (float)y / (float)a.H - 1.0f;
                float aspect = (float)a.W / (float)a.H;
                o = a.eye;
                d = norm3(add3(add3(scl3(lscl3(u, a.right), aspect), lscl3(v, a.up)), a.front));
                if (CAPTURE) {
                    st3(a.c_origin, p, o);
                    st3(a.c_dir, p, d);
                }
            } else {
                o = ld3(a.ray_o[p]);
                d = ld3(a.ray_d[p]);
            }
            const uint32_t seed = mm_combine(inv_seed, p);
            Hit hit = closest_hit(a.sc, o, d, EPS_TRACE, 1000.0f, err);
            f3 new_o, new_d, n, E, R;
            float mis = 0.0f, pdf = 1.0f, nee = 0.0f;
            if (!hit.hit) {
                new_o = add3(o, scl3(d, 5000.0f));
                new_d = f3{0.0f, 0.0f, 0.0f};
                n = f3{0.0f, 0.0f, 0.0f};
                float sky = (dot3(d, f3{0.0f, 1.0f, 0.0f}) > 0.9f) ? 50.0f : 0.0f;
                E = f3{sky, sky, sky};
                R = f3{0.0f, 0.0f, 0.0f};
            } else {
                const int f = hit.face, hh = hit.half;
                const int wx = rec_wx(hit.rec), wy = rec_wy(hit.rec), wz = rec_wz(hit.rec);
                f3 t0 = corner_pos(wx, wy, wz, face_corner(f, hh, 0));
                f3 t1 = corner_pos(wx, wy, wz, face_corner(f, hh, 1));
                f3 t2 = corner_pos(wx, wy, wz, face_corner(f, hh, 2));
                const Frame fr = c_frames[2 * f + hh];
                n = fr.n;
                const uint32_t blk_id = ((uint32_t)hit.rec.z >> 21) & 0xFFu;
                const vrg_material &m = a.sc.mats[6u * blk_id + (uint32_t)f];
                float b0 = (1.0f - hit.b1) - hit.b2;
                new_o = add3(add3(scl3(t0, b0), scl3(t1, hit.b1)), scl3(t2, hit.b2));
                R = f3{__ldg(&m.reflectivity[0]), __ldg(&m.reflectivity[1]), __ldg(&m.reflectivity[2])};
                const float alpha = __ldg(&m.alpha), metal = __ldg(&m.metallic);
                const float ndd = -dot3(d, n);
                E = f3{__ldg(&m.emission[0]) * ndd, __ldg(&m.emission[1]) * ndd, __ldg(&m.emission[2]) * ndd};
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
                    Descent res;
                    res.success = false;
                    res.importance = 0.0f;
                    if (a.nee_type == 1 || (a.nee_type == 2 && b == 1))
                        res = light_descent(a.sc, new_o, n, mm_combine(seed, 2));
                    if (res.success && res.importance > 0.0f) mis = 0.3f;
                    const float mis_rand = mm_rand(mm_combine(seed, 3));
                    float ux = mm_rand(mm_combine(seed, 4)), uy = mm_rand(mm_combine(seed, 5));
                    if (mis_rand < mis) {
                        f3 lt[3];
                        light_tri_world(a.sc, res.inst, res.leaf, lt);
                        if (ux + uy > 1.0f) { ux = 1.0f - ux; uy = 1.0f - uy; }  // triangleSample
                        float bx = (1.0f - ux) - uy;
                        f3 sp = add3(add3(lscl3(bx, lt[0]), lscl3(ux, lt[1])), lscl3(uy, lt[2]));
                        new_d = norm3(sub3(sp, new_o));
                    } else {
                        float s, c;
                        sincos_turns(ux, &s, &c);
                        float vv = sqrtf(fmaxf(0.0f, 1.0f - uy * uy));
                        f3 hs = f3{vv * c, uy, vv * s};
                        new_d = norm3(add3(add3(lscl3(hs.x, fr.t), lscl3(hs.y, fr.n)), lscl3(hs.z, fr.b)));
                    }
                    pdf = dot3(new_d, n) / PI_F;
                }
                // light pdf of the chosen direction (nee_pdf pass; bounce nb-1 is never computed)
                if (b + 1 < nb && mis != 0.0f && len3(new_d) != 0.0f) {
                    nee = nee_any_hit(a.sc, new_o, new_d, n, err);
                    traced_any = true;
                }
            }
            const float q = nee * mis + (1.0f - mis) * inv2pi;
            const float w = pdf / q;
            const size_t rb = (size_t)b * 2 * P;
            a.rec[rb + p] = make_float4(E.x, E.y, E.z, w);
            a.rec[rb + P + p] = make_float4(R.x, R.y, R.z, q);
            if (b == 0) {
                a.xv[p] = make_float4(new_o.x, new_o.y, new_o.z, 0.0f);
                a.nv[p] = make_float4(n.x, n.y, n.z, 0.0f);
            } else if (b == 1) {
                a.xs[p] = make_float4(new_o.x, new_o.y, new_o.z, 0.0f);
                a.ns[p] = make_float4(n.x, n.y, n.z, 0.0f);
            }
            cont = !zero3(new_d) && (b + 1 < nb);
            if (cont) {
                a.ray_o[p] = make_float4(new_o.x, new_o.y, new_o.z, 0.0f);
                a.ray_d[p] = make_float4(new_d.x, new_d.y, new_d.z, 0.0f);
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
                a.c_nee[s0] = nee;
                uint4 hv;
                if (hit.hit) {
                    hv.x = rec_inst(hit.rec);
                    hv.y = hit.tri;
                    hv.z = (uint32_t)hit.rec.z & 0x7FFFu;
                    hv.w = (uint32_t)hit.face | ((uint32_t)hit.half << 8);
                } else {
                    hv = make_uint4(INVALID, INVALID, INVALID, INVALID);
                }
                reinterpret_cast<uint4 *>(a.c_hit)[s0] = hv;
            }
        }
        // compaction of continuing rays into the next queue
        const uint32_t cm = __ballot_sync(0xffffffffu, cont);
        const uint32_t am = __ballot_sync(0xffffffffu, active);
        const uint32_t hm = __ballot_sync(0xffffffffu, traced_any);
        uint32_t qbase = 0;
        if (lane == 0) {
            if (cm) qbase = atomicAdd(&a.counters[CNT_QUEUE + b + 1], (uint32_t)__popc(cm));
            atomicAdd(reinterpret_cast<unsigned long long *>(a.counters + CNT_RAYS), (unsigned long long)__popc(am));
            if (hm) atomicAdd(reinterpret_cast<unsigned long long *>(a.counters + CNT_ANY), (unsigned long long)__popc(hm));
        }
        qbase = __shfl_sync(0xffffffffu, qbase, 0);
        if (cont) qout[qbase + __popc(cm & ((1u << lane) - 1u))] = p;
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

vrg_status launch_bounce(cudaStream_t s, const FrameArgs &a, uint32_t b, int grid) {
    if (a.capture) k_bounce<true><<<grid, 128, 0, s>>>(a, b);
    else k_bounce<false><<<grid, 128, 0, s>>>(a, b);
    VRG_CUDA_TRY(cudaGetLastError());
    return VRG_OK;
}

int bounce_blocks_per_sm() {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_bounce<false>, 128, 0);
    return n > 0 ? n : 1;
}

}  // namespace vrg
