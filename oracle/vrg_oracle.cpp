// ORACLE — test infrastructure, not product code.
//
// A scalar CPU restatement of the reference path tracer of
// pimpale/vulkan-voxel-restir-gi, used only by tests/, __graft_entry__.smoke()
// and bench.py's cpu_baseline / --impl reference leg as the checker and the
// timed CPU baseline.  Nothing in the product links or calls this file.
//
// Parity status: the reference is Rust + GLSL and cannot be built or run on
// these machines (no rustc/cargo, no graphics API), and the reference has no
// tests or golden vectors for this path.  So this restatement is "parity
// unpinned": it follows the reference sources line by line (citations below)
// and defines the few things the reference leaves to a third party:
//   * partition::partition (crate 0.1.2, source not available): restated as
//     an in-place two-sided (Hoare) partition — the k-th predicate-false
//     element from the left swaps with the k-th predicate-true element from
//     the right; the split index is the number of true elements.
//   * the driver ray query (hardware closest hit / candidate enumeration):
//     restated as an exact closed-rectangle test against each exposed voxel
//     face (padded by 2^-12 so neighbouring faces overlap and no ray leaks
//     through an edge), the triangle half chosen by the face diagonal, ties
//     on t broken by the smaller (instance, triangle) key.  Triangles of
//     uploaded meshes are tested in world space (the instance transform
//     applied to their vertices, raytrace.rs:155-159) by the watertight
//     ray/triangle test of Woop, Benthin and Wald (JCGT 2(1), 2013), with
//     the same tie rule.  Light any-hit sums are added in ascending
//     (instance, BVH leaf) order.
//   * nalgebra's isometry arithmetic (crate 0.34.1, not available): the
//     instance transform is the row-major 3x4 matrix [R|t] of the C ABI,
//     applied as ((r0*x + r1*y) + r2*z) + t (the mat4x3 * vec4(p, 1) of the
//     shaders, raytrace.rs:155-159,184-185); an identity R takes the exact
//     translation p + t.  Aabb::transform (aabb.rs:75-92) applies that to
//     the 8 corners.
//   * GLSL built-ins with implementation-defined precision: dot/cross/length
//     evaluated left to right, normalize(v) = v / length(v) per component,
//     sin/cos(2*pi*u) from the quarter-turn reduction + Taylor polynomials
//     below, float->u8 as saturating truncation.
// Build: g++ -O2 -ffp-contract=off (no fast-math) — every float operation is
// a single IEEE binary32 operation in source order.

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <vector>

#include "../include/vrg.h"

#define ORC_API extern "C" __attribute__((visibility("default")))

namespace {

// ------------------------------------------------------------------------
// math (GLSL vec3 semantics, evaluated left to right)
// ------------------------------------------------------------------------
struct V3 {
    float x, y, z;
};
static inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
static inline V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
static inline V3 operator*(float s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
static inline V3 mul(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
static inline float dot3(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline V3 cross3(V3 a, V3 b) {
    return V3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
static inline float length3(V3 a) { return sqrtf(dot3(a, a)); }
static inline V3 normalize3(V3 a) {
    float l = length3(a);
    return V3{a.x / l, a.y / l, a.z / l};
}
static inline bool is_zero3(V3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
static inline float comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

static const float PI_F = 3.1415926535897932384626433832795f;   // raytrace.rs:12
static const float TWO_PI_F = 6.283185307179586476925286766559f;
static const float EPS_BLOCK_TRACE = 0.001f;                     // raytrace.rs:13
static const float EPS_BLOCK_NEE = 0.0001f;                      // nee_pdf.rs:15
static const float FACE_PAD = 1.0f / 4096.0f;                    // closed-face padding
static const float BOX_MARGIN = 1.0f / 128.0f;                   // conservative culling
static const float ZERO3[3] = {0.0f, 0.0f, 0.0f};

// murmur3 chaining (raygen.rs:37-78; identical copies in raytrace, temporal, spatial)
static inline uint32_t mm_combine(uint32_t h, uint32_t k) {
    k *= 0x1b873593u;
    h ^= k;
    h = (h << 13) | (h >> 19);
    h = h * 5u + 0xe6546b64u;
    return h;
}
static inline uint32_t mm_finalize(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}
static inline float float_construct(uint32_t m) {
    m &= 0x007FFFFFu;
    m |= 0x3F800000u;
    float f;
    memcpy(&f, &m, 4);
    return f - 1.0f;
}
static inline float mm_rand(uint32_t h) { return float_construct(mm_finalize(h)); }

// sin(2*pi*x), cos(2*pi*x) for x in [0,1): reduce by quarter turns (exact),
// then Taylor series of sin/cos on |a| <= pi/4 (truncation < 2e-9).
static inline void sincos_turns(float x, float *s, float *c) {
    float q = rintf(x * 4.0f);
    float r = x - q * 0.25f;
    float a = r * TWO_PI_F;
    float a2 = a * a;
    float ps = (((2.75573192e-6f * a2 - 1.98412698e-4f) * a2 + 8.33333333e-3f) * a2 - 1.66666667e-1f) * a2;
    float sn = a + a * ps;
    float pc = ((((-2.75573192e-7f * a2 + 2.48015873e-5f) * a2 - 1.38888889e-3f) * a2 + 4.16666667e-2f) * a2 - 0.5f) * a2;
    float cs = 1.0f + pc;
    int k = ((int)q) & 3;
    if (k == 0) { *s = sn; *c = cs; }
    else if (k == 1) { *s = cs; *c = -sn; }
    else if (k == 2) { *s = -sn; *c = -cs; }
    else { *s = -cs; *c = sn; }
}

static inline float luminance(V3 v) {  // restir_temporal_resampling.rs:248-250
    return (0.2126f * v.x + 0.7152f * v.y) + 0.0722f * v.z;
}

// ------------------------------------------------------------------------
// AABB (bvh/aabb.rs)
// ------------------------------------------------------------------------
struct OAabb {
    bool empty;
    float mn[3];
    float mx[3];
};
static inline OAabb aabb_empty() {
    OAabb a;
    a.empty = true;
    for (int i = 0; i < 3; i++) a.mn[i] = a.mx[i] = 0.0f;
    return a;
}
static inline OAabb aabb_make(const float mn[3], const float mx[3]) {
    OAabb a;
    a.empty = false;
    for (int i = 0; i < 3; i++) { a.mn[i] = mn[i]; a.mx[i] = mx[i]; }
    return a;
}
// aabb.rs:24-42
static inline OAabb aabb_union(const OAabb &a, const OAabb &b) {
    if (a.empty) return b;
    if (b.empty) return a;
    OAabb r;
    r.empty = false;
    for (int i = 0; i < 3; i++) {
        r.mn[i] = fminf(a.mn[i], b.mn[i]);
        r.mx[i] = fmaxf(a.mx[i], b.mx[i]);
    }
    return r;
}
// aabb.rs:44-52
static inline float aabb_area(const OAabb &a) {
    if (a.empty) return 0.0f;
    float dx = a.mx[0] - a.mn[0], dy = a.mx[1] - a.mn[1], dz = a.mx[2] - a.mn[2];
    return 2.0f * ((dx * dy + dx * dz) + dy * dz);
}
// aabb.rs:10-22
static inline OAabb aabb_from_points(const V3 *p, int n) {
    OAabb a;
    a.empty = false;
    a.mn[0] = a.mx[0] = p[0].x;
    a.mn[1] = a.mx[1] = p[0].y;
    a.mn[2] = a.mx[2] = p[0].z;
    for (int i = 0; i < n; i++) {
        a.mn[0] = fminf(a.mn[0], p[i].x); a.mx[0] = fmaxf(a.mx[0], p[i].x);
        a.mn[1] = fminf(a.mn[1], p[i].y); a.mx[1] = fmaxf(a.mx[1], p[i].y);
        a.mn[2] = fminf(a.mn[2], p[i].z); a.mx[2] = fmaxf(a.mx[2], p[i].z);
    }
    return a;
}
// aabb.rs:75-92 for an isometry with identity rotation: the 8 corners
// translated; the min/max of the corners is (min+t, max+t).
static inline OAabb aabb_translate(const OAabb &a, const float t[3]) {
    if (a.empty) return a;
    V3 c[8];
    float lo[3], hi[3];
    for (int i = 0; i < 3; i++) { lo[i] = a.mn[i] + t[i]; hi[i] = a.mx[i] + t[i]; }
    for (int k = 0; k < 8; k++)
        c[k] = v3((k & 4) ? hi[0] : lo[0], (k & 2) ? hi[1] : lo[1], (k & 1) ? hi[2] : lo[2]);
    return aabb_from_points(c, 8);
}

// Instance transform: row-major 3x4 [R|t].  tonly: R is exactly the
// identity, and points move by the exact translation p + t.
struct OXform {
    float m[12];
    bool tonly;
};
static const OXform XF_IDENTITY = {{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0}, true};
static inline V3 xf_point(const OXform &X, V3 p) {
    if (X.tonly) return v3(p.x + X.m[3], p.y + X.m[7], p.z + X.m[11]);
    return v3(((X.m[0] * p.x + X.m[1] * p.y) + X.m[2] * p.z) + X.m[3],
              ((X.m[4] * p.x + X.m[5] * p.y) + X.m[6] * p.z) + X.m[7],
              ((X.m[8] * p.x + X.m[9] * p.y) + X.m[10] * p.z) + X.m[11]);
}
// Aabb::transform (aabb.rs:75-92): the AABB of the 8 transformed corners, in
// the reference's corner order
static inline OAabb aabb_transform(const OAabb &a, const OXform &X) {
    if (a.empty) return a;
    V3 c[8];
    for (int k = 0; k < 8; k++)
        c[k] = xf_point(X, v3((k & 4) ? a.mx[0] : a.mn[0], (k & 2) ? a.mx[1] : a.mn[1], (k & 1) ? a.mx[2] : a.mn[2]));
    return aabb_from_points(c, 8);
}

// ------------------------------------------------------------------------
// binned SAH builder (bvh/build.rs)
// ------------------------------------------------------------------------
struct BNode {
    OAabb aabb;
    bool leaf;
    uint32_t parent;
    uint32_t first, count;   // leaf range
    uint32_t left, right;    // internal children
};

// Rust `f as usize` (saturating; NaN -> 0) followed by min(31) (build.rs:79-82)
static inline uint32_t bin_index(float v) {
    if (!(v > 0.0f)) return 0;     // NaN, negative, zero
    if (v >= 31.0f) return 31;
    return (uint32_t)v;
}

// build.rs:45-128
static void find_best_plane(uint32_t first, uint32_t count, const std::vector<uint32_t> &idx,
                            const std::vector<V3> &cen, const std::vector<OAabb> &aabbs,
                            uint32_t *out_dim, float *out_split) {
    const int BINS = 32;
    float best_cost = 3.40282347e+38f;  // f32::MAX
    uint32_t best_dim = 0;
    float best_split = 0.0f;
    for (int d = 0; d < 3; d++) {
        float bmin = 3.40282347e+38f, bmax = -3.40282347e+38f;
        for (uint32_t i = first; i < first + count; i++) {
            float c = comp(cen[idx[i]], d);
            bmin = fminf(bmin, c);
            bmax = fmaxf(bmax, c);
        }
        OAabb bin_bounds[BINS];
        uint32_t bin_count[BINS];
        for (int b = 0; b < BINS; b++) { bin_bounds[b] = aabb_empty(); bin_count[b] = 0; }
        float scale = (float)BINS / (bmax - bmin);
        for (uint32_t i = first; i < first + count; i++) {
            uint32_t p = idx[i];
            uint32_t b = bin_index((comp(cen[p], d) - bmin) * scale);
            bin_count[b] += 1;
            bin_bounds[b] = aabb_union(bin_bounds[b], aabbs[p]);
        }
        OAabb pl[BINS - 1], pr[BINS - 1];
        uint32_t cl[BINS - 1], cr[BINS - 1];
        OAabb al = aabb_empty(), ar = aabb_empty();
        uint32_t nl = 0, nr = 0;
        for (int pln = 0; pln < BINS - 1; pln++) {
            nl += bin_count[pln];
            cl[pln] = nl;
            al = aabb_union(al, bin_bounds[pln]);
            pl[pln] = al;
            nr += bin_count[BINS - 1 - pln];
            cr[BINS - 2 - pln] = nr;
            ar = aabb_union(ar, bin_bounds[BINS - 1 - pln]);
            pr[BINS - 2 - pln] = ar;
        }
        float scale2 = (bmax - bmin) / (float)BINS;
        for (int pln = 0; pln < BINS - 1; pln++) {
            // cost_function (build.rs:287-289)
            float cost = aabb_area(pl[pln]) * (float)cl[pln] + aabb_area(pr[pln]) * (float)cr[pln];
            if (cost < best_cost) {
                best_cost = cost;
                best_dim = (uint32_t)d;
                best_split = bmin + ((float)pln + 1.0f) * scale2;
            }
        }
    }
    *out_dim = best_dim;
    *out_split = best_split;
}

// partition::partition restated (see file header): returns the true count.
static uint32_t hoare_partition(uint32_t *data, uint32_t len, uint32_t dim, float split,
                                const std::vector<V3> &cen) {
    if (len == 0) return 0;
    auto pred = [&](uint32_t p) { return comp(cen[p], (int)dim) < split; };
    uint32_t l = 0, r = len - 1;
    for (;;) {
        while (l < len && pred(data[l])) l++;
        while (r > 0 && !pred(data[r])) r--;
        if (l >= r) return l;
        std::swap(data[l], data[r]);
    }
}

static OAabb range_bounds(uint32_t first, uint32_t count, const std::vector<uint32_t> &idx,
                          const std::vector<OAabb> &aabbs) {
    OAabb b = aabb_empty();  // build.rs:36-43
    for (uint32_t i = first; i < first + count; i++) b = aabb_union(b, aabbs[idx[i]]);
    return b;
}

// build.rs:130-233 with the recursion made an explicit LIFO stack (same
// node insertion order: left child's subtree completes before the right's).
static void build_tree(const std::vector<OAabb> &aabbs, const std::vector<V3> &cen,
                       std::vector<uint32_t> &idx, std::vector<BNode> &nodes) {
    uint32_t n = (uint32_t)aabbs.size();
    nodes.clear();
    nodes.reserve(2 * (size_t)n);
    BNode root;
    root.aabb = range_bounds(0, n, idx, aabbs);
    root.leaf = true;
    root.parent = 0xFFFFFFFFu;
    root.first = 0;
    root.count = n;
    root.left = root.right = 0;
    nodes.push_back(root);
    std::vector<uint32_t> stack;
    stack.push_back(0);
    while (!stack.empty()) {
        uint32_t ni = stack.back();
        stack.pop_back();
        BNode nd = nodes[ni];
        if (!nd.leaf || nd.count < 2) continue;
        uint32_t nleft;
        if (nd.count > 2) {
            uint32_t dim;
            float split;
            find_best_plane(nd.first, nd.count, idx, cen, aabbs, &dim, &split);
            nleft = hoare_partition(&idx[nd.first], nd.count, dim, split, cen);
            if (nleft == 0 || nleft == nd.count) nleft = nd.count / 2;  // build.rs:151-157
        } else {
            nleft = 1;
        }
        BNode l, r;
        l.leaf = r.leaf = true;
        l.parent = r.parent = ni;
        l.first = nd.first;
        l.count = nleft;
        r.first = nd.first + nleft;
        r.count = nd.count - nleft;
        l.left = l.right = r.left = r.right = 0;
        l.aabb = range_bounds(l.first, l.count, idx, aabbs);
        r.aabb = range_bounds(r.first, r.count, idx, aabbs);
        uint32_t li = (uint32_t)nodes.size();
        nodes.push_back(l);
        uint32_t ri = (uint32_t)nodes.size();
        nodes.push_back(r);
        nodes[ni].leaf = false;
        nodes[ni].left = li;
        nodes[ni].right = ri;
        stack.push_back(ri);
        stack.push_back(li);
    }
}

// flatten + bottom-up power (build.rs:300-357 and 430-477)
static void flatten(const std::vector<BNode> &nodes, const std::vector<uint32_t> &idx,
                    const std::vector<OAabb> &aabbs, const float *power, const uint32_t *ids,
                    std::vector<vrg_bvh_node> &out) {
    const float pad = 0.0001f;
    out.resize(nodes.size());
    for (size_t i = 0; i < nodes.size(); i++) {
        const BNode &b = nodes[i];
        vrg_bvh_node &o = out[i];
        if (b.leaf) {
            uint32_t p = idx[b.first];
            o.left_node_idx = 0xFFFFFFFFu;
            o.right_node_idx_or_prim_idx = ids[p];
            for (int c = 0; c < 3; c++) {
                o.min[c] = aabbs[p].empty ? 0.0f : aabbs[p].mn[c];
                o.max[c] = aabbs[p].empty ? 0.0f : aabbs[p].mx[c];
            }
            o.power = power[p];
            o.parent_idx = b.parent;
        } else {
            o.left_node_idx = b.left;
            o.right_node_idx_or_prim_idx = b.right;
            for (int c = 0; c < 3; c++) {
                float mn = b.aabb.empty ? 0.0f : b.aabb.mn[c];
                float mx = b.aabb.empty ? 0.0f : b.aabb.mx[c];
                o.min[c] = mn - pad;
                o.max[c] = mx + pad;
            }
            o.power = 0.0f;
            o.parent_idx = b.parent;
        }
    }
    for (size_t i = out.size(); i-- > 0;) {
        if (out[i].left_node_idx != 0xFFFFFFFFu) {
            float p = out[i].power;
            p += out[out[i].left_node_idx].power;
            p += out[out[i].right_node_idx_or_prim_idx].power;
            out[i].power = p;
        }
    }
}

// build_tl_bvh (build.rs:374-480): AABB prims with translation isometries.
static void build_tl(uint32_t n, const float *trans, const OAabb *in_aabbs, const float *power,
                     const uint32_t *ids, std::vector<vrg_bvh_node> &out, std::vector<uint32_t> &order) {
    std::vector<OAabb> aabbs(n);
    std::vector<V3> cen(n);
    for (uint32_t i = 0; i < n; i++) {
        aabbs[i] = aabb_translate(in_aabbs[i], trans ? trans + 3 * i : ZERO3);
        // centroid (min + max) / 2 (build.rs:397-400)
        cen[i] = v3((aabbs[i].mn[0] + aabbs[i].mx[0]) / 2.0f, (aabbs[i].mn[1] + aabbs[i].mx[1]) / 2.0f,
                    (aabbs[i].mn[2] + aabbs[i].mx[2]) / 2.0f);
    }
    order.resize(n);
    for (uint32_t i = 0; i < n; i++) order[i] = i;
    std::vector<BNode> nodes;
    build_tree(aabbs, cen, order, nodes);
    flatten(nodes, order, aabbs, power, ids, out);
}

// build_bl_bvh (build.rs:249-372): triangle prims.
static void build_bl(uint32_t n, const float *lum, const V3 *tri, const uint32_t *ids,
                     std::vector<vrg_bvh_node> &out, std::vector<uint32_t> &order, OAabb *root_aabb,
                     float *root_power) {
    std::vector<OAabb> aabbs(n);
    std::vector<V3> cen(n);
    for (uint32_t i = 0; i < n; i++) {
        aabbs[i] = aabb_from_points(tri + 3 * i, 3);
        V3 s = (tri[3 * i] + tri[3 * i + 1]) + tri[3 * i + 2];
        cen[i] = v3(s.x / 3.0f, s.y / 3.0f, s.z / 3.0f);
    }
    order.resize(n);
    for (uint32_t i = 0; i < n; i++) order[i] = i;
    std::vector<BNode> nodes;
    build_tree(aabbs, cen, order, nodes);
    flatten(nodes, order, aabbs, lum, ids, out);
    if (out[0].left_node_idx == 0xFFFFFFFFu) {
        *root_aabb = aabbs[0];
        *root_power = lum[0];
    } else {
        *root_aabb = aabb_make(out[0].min, out[0].max);
        *root_power = out[0].power;
    }
}

// ------------------------------------------------------------------------
// chunk meshing order (chunk.rs:158-292) and face geometry
// ------------------------------------------------------------------------
// corner bits (a,b,c) of v{abc} = (x+a, y+b, z+c) for face f, triangle h, vertex j
static const uint8_t FACE_TRI[6][2][3] = {
    {{0b001, 0b010, 0b000}, {0b011, 0b010, 0b001}},  // left
    {{0b110, 0b101, 0b100}, {0b110, 0b111, 0b101}},  // right
    {{0b000, 0b100, 0b001}, {0b100, 0b101, 0b001}},  // down
    {{0b011, 0b110, 0b010}, {0b011, 0b111, 0b110}},  // up
    {{0b010, 0b100, 0b000}, {0b010, 0b110, 0b100}},  // back
    {{0b001, 0b101, 0b011}, {0b101, 0b111, 0b011}},  // front
};
// gen_mesh texture coordinates of each triangle vertex (chunk.rs:225-285)
static const float FACE_UV[6][2][3][2] = {
    {{{0, 1}, {1, 0}, {1, 1}}, {{0, 0}, {1, 0}, {0, 1}}},  // left
    {{{0, 0}, {1, 1}, {0, 1}}, {{0, 0}, {1, 0}, {1, 1}}},  // right
    {{{0, 0}, {1, 0}, {0, 1}}, {{1, 0}, {1, 1}, {0, 1}}},  // down
    {{{1, 1}, {0, 0}, {1, 0}}, {{1, 1}, {0, 1}, {0, 0}}},  // up
    {{{0, 0}, {1, 1}, {0, 1}}, {{0, 0}, {1, 0}, {1, 1}}},  // back
    {{{1, 1}, {0, 1}, {1, 0}}, {{0, 1}, {0, 0}, {1, 0}}},  // front
};
static inline V3 corner_pos(int bx, int by, int bz, uint8_t bits) {
    return v3((float)(bx + ((bits >> 2) & 1)), (float)(by + ((bits >> 1) & 1)), (float)(bz + (bits & 1)));
}
static inline void face_axes(int f, int *a, int *u, int *v) {
    *a = f >> 1;
    if (*a == 0) { *u = 1; *v = 2; }
    else if (*a == 1) { *u = 0; *v = 2; }
    else { *u = 0; *v = 1; }
}

static inline uint32_t chunk_idx(int x, int y, int z) { return (uint32_t)(x * 1024 + y * 32 + z); }

struct OChunk {
    std::vector<uint8_t> blocks;
    std::vector<uint8_t> face_mask;   // per block
    std::vector<uint32_t> first_tri;  // per block
    std::vector<uint32_t> tri_block;  // per triangle
    std::vector<uint8_t> tri_fh;      // per triangle: face | half<<4
    uint32_t n_tris = 0;
    // light BLAS (upload_object, scene.rs:547-571; build_bl_bvh)
    uint32_t n_light = 0;
    std::vector<vrg_bvh_node> light_nodes;
    std::vector<uint32_t> light_order;
    OAabb light_aabb;
    float light_power = 0.0f;
    // geometry BLAS over per-block AABBs (build_tl_bvh semantics); for a
    // mesh, over its triangles (build_bl_bvh inputs, leaf prim = triangle)
    uint32_t n_geo = 0;
    std::vector<vrg_bvh_node> geo_nodes;
    std::vector<uint32_t> geo_order;
    OAabb geo_aabb;
    // an uploaded triangle mesh (upload_object, scene.rs:547-725) instead of a chunk
    bool mesh = false;
    std::vector<V3> mpos;          // 3 per triangle, object space
    std::vector<uint32_t> mslot;   // per triangle: its first vertex's t
    std::vector<float> muv;        // 6 per triangle
};

struct OMaterials {
    std::vector<vrg_material> mats;
    uint32_t n_types = 0;
    // texture atlas (interactive_rendering.rs:379-444): [slot][3 maps][h][w] RGBA8 sRGB
    std::vector<uint8_t> atlas;
    uint32_t atlas_w = 0, atlas_h = 0;
    float srgb[256];
    uint32_t air() const { return n_types; }
    bool translucent(uint8_t b) const {
        if (b == n_types) return true;
        return (mats[6 * (size_t)b].flags & VRG_MAT_TRANSLUCENT) != 0;
    }
};

static void build_chunk(OChunk &ch, const OMaterials &M, const uint8_t *const nb[6]) {
    const uint32_t air = M.air();
    ch.face_mask.assign(VRG_CHUNK_BLOCKS, 0);
    ch.first_tri.assign(VRG_CHUNK_BLOCKS, 0);
    ch.tri_block.clear();
    ch.tri_fh.clear();
    auto neighbour = [&](int x, int y, int z, int f) -> uint8_t {
        // chunk.rs:170-205
        int nx = x, ny = y, nz = z;
        const uint8_t *src = ch.blocks.data();
        switch (f) {
        case 0: if (x == 0) { src = nb[0]; nx = 31; } else nx = x - 1; break;
        case 1: if (x == 31) { src = nb[1]; nx = 0; } else nx = x + 1; break;
        case 2: if (y == 0) { src = nb[2]; ny = 31; } else ny = y - 1; break;
        case 3: if (y == 31) { src = nb[3]; ny = 0; } else ny = y + 1; break;
        case 4: if (z == 0) { src = nb[4]; nz = 31; } else nz = z - 1; break;
        default: if (z == 31) { src = nb[5]; nz = 0; } else nz = z + 1; break;
        }
        if (!src) return (uint8_t)air;
        return src[chunk_idx(nx, ny, nz)];
    };
    uint32_t tri = 0;
    std::vector<float> lum;
    std::vector<V3> ltri;
    std::vector<uint32_t> lids;
    std::vector<OAabb> gaabb;
    std::vector<uint32_t> gids;
    for (int x = 0; x < 32; x++)
        for (int y = 0; y < 32; y++)
            for (int z = 0; z < 32; z++) {
                uint32_t bi = chunk_idx(x, y, z);
                uint8_t b = ch.blocks[bi];
                if (b == air) continue;  // completely_transparent
                ch.first_tri[bi] = tri;
                uint8_t mask = 0;
                for (int f = 0; f < 6; f++) {
                    if (!M.translucent(neighbour(x, y, z, f))) continue;
                    mask |= (uint8_t)(1u << f);
                    uint32_t t = 6u * b + (uint32_t)f;
                    for (int h = 0; h < 2; h++) {
                        ch.tri_block.push_back(bi);
                        ch.tri_fh.push_back((uint8_t)(f | (h << 4)));
                        float L = M.mats[t].luminance;
                        if (L > 0.0f) {  // scene.rs:559-571
                            V3 a = corner_pos(x, y, z, FACE_TRI[f][h][0]);
                            V3 bb = corner_pos(x, y, z, FACE_TRI[f][h][1]);
                            V3 c = corner_pos(x, y, z, FACE_TRI[f][h][2]);
                            float area = length3(cross3(bb - a, c - a)) / 2.0f;
                            ltri.push_back(a);
                            ltri.push_back(bb);
                            ltri.push_back(c);
                            lum.push_back(L * area);
                            lids.push_back(tri);
                        }
                        tri++;
                    }
                }
                ch.face_mask[bi] = mask;
                if (mask) {
                    float mn[3] = {(float)x, (float)y, (float)z};
                    float mx[3] = {(float)(x + 1), (float)(y + 1), (float)(z + 1)};
                    gaabb.push_back(aabb_make(mn, mx));
                    gids.push_back(bi);
                }
            }
    ch.n_tris = tri;
    ch.n_light = (uint32_t)lum.size();
    if (ch.n_light) {
        build_bl(ch.n_light, lum.data(), ltri.data(), lids.data(), ch.light_nodes, ch.light_order,
                 &ch.light_aabb, &ch.light_power);
    } else {
        ch.light_nodes.clear();
        ch.light_order.clear();
        ch.light_aabb = aabb_empty();
        ch.light_power = 0.0f;
    }
    ch.n_geo = (uint32_t)gaabb.size();
    if (ch.n_geo) {
        std::vector<float> zero(ch.n_geo, 0.0f);
        build_tl(ch.n_geo, nullptr, gaabb.data(), zero.data(), gids.data(), ch.geo_nodes, ch.geo_order);
        if (ch.geo_nodes[0].left_node_idx == 0xFFFFFFFFu) ch.geo_aabb = gaabb[0];
        else ch.geo_aabb = aabb_make(ch.geo_nodes[0].min, ch.geo_nodes[0].max);
    } else {
        ch.geo_nodes.clear();
        ch.geo_order.clear();
        ch.geo_aabb = aabb_empty();
    }
}

// upload_object (scene.rs:547-725) of arbitrary triangles: the light BLAS over
// triangles whose slot luminance is > 0 (power = luminance * area, leaf prim
// id = triangle index), and the geometry BVH over all triangles
static bool build_mesh(OChunk &ch, const OMaterials &M, const vrg_vertex3d *v, uint64_t nverts) {
    if (nverts % 3) return false;
    const uint32_t n = (uint32_t)(nverts / 3);
    ch.mesh = true;
    ch.n_tris = n;
    ch.mpos.resize(3 * (size_t)n);
    ch.mslot.resize(n);
    ch.muv.resize(6 * (size_t)n);
    std::vector<float> lum;
    std::vector<V3> ltri;
    std::vector<uint32_t> lids;
    for (uint32_t i = 0; i < n; i++) {
        for (int j = 0; j < 3; j++) {
            const vrg_vertex3d &x = v[3 * (size_t)i + j];
            ch.mpos[3 * (size_t)i + j] = v3(x.position[0], x.position[1], x.position[2]);
            ch.muv[6 * (size_t)i + 2 * j] = x.uv[0];
            ch.muv[6 * (size_t)i + 2 * j + 1] = x.uv[1];
        }
        const uint32_t t = v[3 * (size_t)i].t;
        if (t >= M.mats.size()) return false;
        ch.mslot[i] = t;
        const float L = M.mats[t].luminance;
        if (L > 0.0f) {
            const V3 a = ch.mpos[3 * (size_t)i], b = ch.mpos[3 * (size_t)i + 1], c = ch.mpos[3 * (size_t)i + 2];
            const float area = length3(cross3(b - a, c - a)) / 2.0f;
            ltri.push_back(a);
            ltri.push_back(b);
            ltri.push_back(c);
            lum.push_back(L * area);
            lids.push_back(i);
        }
    }
    ch.n_light = (uint32_t)lum.size();
    if (ch.n_light) {
        build_bl(ch.n_light, lum.data(), ltri.data(), lids.data(), ch.light_nodes, ch.light_order, &ch.light_aabb,
                 &ch.light_power);
    } else {
        ch.light_aabb = aabb_empty();
        ch.light_power = 0.0f;
    }
    ch.n_geo = n;
    if (n) {
        std::vector<float> zero(n, 0.0f);
        std::vector<uint32_t> ids(n);
        for (uint32_t i = 0; i < n; i++) ids[i] = i;
        float pw;
        build_bl(n, zero.data(), ch.mpos.data(), ids.data(), ch.geo_nodes, ch.geo_order, &ch.geo_aabb, &pw);
    } else {
        ch.geo_aabb = aabb_empty();
    }
    return true;
}

// ------------------------------------------------------------------------
// world (Scene, scene.rs:86-497)
// ------------------------------------------------------------------------
struct OInstance {
    const OChunk *ch;
    float off[3];        // the translation (chunks: their whole transform)
    OXform X;            // the instance transform
    std::vector<V3> wpos;  // mesh: world-space vertices, 3 per triangle
    uint32_t light_bvh_tl_idx;
};

struct OWorld {
    OMaterials M;
    std::map<uint64_t, std::pair<std::shared_ptr<OChunk>, OXform>> objects;
    std::vector<OInstance> inst;
    std::vector<vrg_bvh_node> light_tl;   // light TL BVH (scene.rs:248-279)
    std::vector<vrg_bvh_node> geo_tl;     // geometry TL BVH over chunks
    std::vector<uint32_t> light_tl_order, geo_tl_order;
};

static void world_commit(OWorld &W) {
    W.inst.clear();
    for (auto &kv : W.objects) {
        if (kv.second.first->n_tris == 0) continue;  // SceneUploadedObjectHandle::Empty
        OInstance in;
        in.ch = kv.second.first.get();
        in.X = kv.second.second;
        in.off[0] = in.X.m[3];
        in.off[1] = in.X.m[7];
        in.off[2] = in.X.m[11];
        if (in.ch->mesh) {  // triangleTransform (raytrace.rs:155-159) of every triangle
            in.wpos.resize(in.ch->mpos.size());
            for (size_t k = 0; k < in.ch->mpos.size(); k++) in.wpos[k] = xf_point(in.X, in.ch->mpos[k]);
        }
        in.light_bvh_tl_idx = 0;
        W.inst.push_back(std::move(in));
    }
    // An instance's top-level prim: its root AABB moved by its transform
    // (Aabb::transform, build.rs:391-395); a translation goes to build_tl as
    // such, any other transform is applied here and build_tl gets 0.
    auto tl_prim = [](const OInstance &I, const OAabb &a, std::vector<float> &tr, std::vector<OAabb> &ab) {
        if (I.X.tonly) {
            for (int k = 0; k < 3; k++) tr.push_back(I.off[k]);
            ab.push_back(a);
        } else {
            for (int k = 0; k < 3; k++) tr.push_back(0.0f);
            ab.push_back(aabb_transform(a, I.X));
        }
    };
    // light TL (scene.rs:248-287)
    std::vector<float> tr, pw;
    std::vector<OAabb> ab;
    std::vector<uint32_t> ids;
    for (uint32_t i = 0; i < W.inst.size(); i++) {
        const OChunk *c = W.inst[i].ch;
        if (c->light_aabb.empty) continue;
        tl_prim(W.inst[i], c->light_aabb, tr, ab);
        pw.push_back(c->light_power);
        ids.push_back(i);
    }
    if (ab.empty()) {
        vrg_bvh_node d;
        d.left_node_idx = d.right_node_idx_or_prim_idx = d.parent_idx = 0xFFFFFFFFu;
        for (int k = 0; k < 3; k++) d.min[k] = d.max[k] = 0.0f;
        d.power = 0.0f;
        W.light_tl.assign(1, d);
        W.light_tl_order.clear();
    } else {
        build_tl((uint32_t)ab.size(), tr.data(), ab.data(), pw.data(), ids.data(), W.light_tl, W.light_tl_order);
        for (uint32_t i = 0; i < W.light_tl.size(); i++)
            if (W.light_tl[i].left_node_idx == 0xFFFFFFFFu)
                W.inst[W.light_tl[i].right_node_idx_or_prim_idx].light_bvh_tl_idx = i;
    }
    // geometry TL over instances (replaces the driver TLAS, scene.rs:728-971)
    tr.clear(); ab.clear(); pw.clear(); ids.clear();
    for (uint32_t i = 0; i < W.inst.size(); i++) {
        const OChunk *c = W.inst[i].ch;
        if (c->n_geo == 0) continue;
        tl_prim(W.inst[i], c->geo_aabb, tr, ab);
        pw.push_back(0.0f);
        ids.push_back(i);
    }
    if (ab.empty()) W.geo_tl.clear();
    else build_tl((uint32_t)ab.size(), tr.data(), ab.data(), pw.data(), ids.data(), W.geo_tl, W.geo_tl_order);
}

// ------------------------------------------------------------------------
// ray / voxel-face intersection
// ------------------------------------------------------------------------
struct FaceHit {
    float t;
    int half;
    float b1, b2;  // barycentrics of v1, v2 of the hit triangle
};

// weight of the triangle vertex at local corner (cu, cv) for the hit (lu, lv)
static inline float corner_weight(int cu, int cv, int half, float lu, float lv) {
    if (half == 0) {
        if (cu == 0 && cv == 0) return (1.0f - lu) - lv;
        if (cu == 1) return lu;
        return lv;
    }
    if (cu == 1 && cv == 1) return (lu + lv) - 1.0f;
    if (cu == 1) return 1.0f - lv;
    return 1.0f - lu;
}

static inline int bitsel(uint8_t bits, int axis) { return (bits >> (2 - axis)) & 1; }

static bool face_test(int bx, int by, int bz, int f, V3 o, V3 d, V3 inv, float tmin, float tmax,
                      FaceHit *h) {
    int a, u, v;
    face_axes(f, &a, &u, &v);
    int bc[3] = {bx, by, bz};
    float c = (float)(bc[a] + (f & 1));
    float t = (c - comp(o, a)) * comp(inv, a);
    if (!(t >= tmin && t <= tmax)) return false;
    float pu = comp(o, u) + t * comp(d, u);
    float pv = comp(o, v) + t * comp(d, v);
    float lu = pu - (float)bc[u];
    float lv = pv - (float)bc[v];
    if (!(lu >= -FACE_PAD && lu <= 1.0f + FACE_PAD && lv >= -FACE_PAD && lv <= 1.0f + FACE_PAD)) return false;
    int half = ((1.0f - lu) - lv >= 0.0f) ? 0 : 1;
    uint8_t c1 = FACE_TRI[f][half][1], c2 = FACE_TRI[f][half][2];
    h->t = t;
    h->half = half;
    h->b1 = corner_weight(bitsel(c1, u), bitsel(c1, v), half, lu, lv);
    h->b2 = corner_weight(bitsel(c2, u), bitsel(c2, v), half, lu, lv);
    return true;
}

// Watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2(1), 2013), both
// faces: the ray's dominant axis kz (the largest |d| component, the first on
// ties), the shear S, edge functions U, V, W of the sheared vertices (each
// recomputed in double when it is exactly 0), a hit iff they do not differ in
// sign and det = U + V + W != 0, t = T / det in [tmin, tmax]; barycentrics of
// v1, v2 are V / det, W / det.
struct TriHit {
    float t, b1, b2;
};
static bool tri_test(V3 v0, V3 v1, V3 v2, V3 o, V3 d, float tmin, float tmax, TriHit *h) {
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > (kz == 0 ? ax : ay)) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1, ky = kx + 1 == 3 ? 0 : kx + 1;
    if (comp(d, kz) < 0.0f) std::swap(kx, ky);
    const float Sx = comp(d, kx) / comp(d, kz), Sy = comp(d, ky) / comp(d, kz), Sz = 1.0f / comp(d, kz);
    const V3 A = v0 - o, B = v1 - o, C = v2 - o;
    const float Ax = comp(A, kx) - Sx * comp(A, kz), Ay = comp(A, ky) - Sy * comp(A, kz);
    const float Bx = comp(B, kx) - Sx * comp(B, kz), By = comp(B, ky) - Sy * comp(B, kz);
    const float Cx = comp(C, kx) - Sx * comp(C, kz), Cy = comp(C, ky) - Sy * comp(C, kz);
    float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = (U + V) + W;
    if (det == 0.0f) return false;
    const float Az = Sz * comp(A, kz), Bz = Sz * comp(B, kz), Cz = Sz * comp(C, kz);
    const float T = (U * Az + V * Bz) + W * Cz;
    const float t = T / det;
    if (!(t >= tmin && t <= tmax)) return false;
    h->t = t;
    h->b1 = V / det;
    h->b2 = W / det;
    return true;
}

static inline bool box_test(const float mn[3], const float mx[3], const float off[3], V3 o, V3 inv,
                            float tmin, float tmax) {
    float tn = tmin, tf = tmax;
    for (int k = 0; k < 3; k++) {
        float lo = (mn[k] + off[k]) - BOX_MARGIN;
        float hi = (mx[k] + off[k]) + BOX_MARGIN;
        float t0 = (lo - comp(o, k)) * comp(inv, k);
        float t1 = (hi - comp(o, k)) * comp(inv, k);
        float a = fminf(t0, t1), b = fmaxf(t0, t1);
        tn = fmaxf(tn, a);
        tf = fminf(tf, b);
    }
    return tn <= tf;
}

struct OHit {
    bool hit;
    uint32_t inst, tri, block;
    int face, half;
    float t, b1, b2;
    int bx, by, bz;  // world block coords
};

// closest hit over the voxel faces (replaces getIntersectionInfo, raytrace.rs:354-388)
static OHit closest_hit(const OWorld &W, V3 o, V3 d, float tmin, float tmax) {
    OHit best;
    best.hit = false;
    best.t = tmax;
    uint64_t best_key = ~0ull;
    if (W.geo_tl.empty()) return best;
    V3 inv = v3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    std::vector<uint32_t> tl_stack{0};
    while (!tl_stack.empty()) {
        uint32_t ni = tl_stack.back();
        tl_stack.pop_back();
        const vrg_bvh_node &n = W.geo_tl[ni];
        if (!box_test(n.min, n.max, ZERO3, o, inv, tmin, best.t)) continue;
        if (n.left_node_idx != 0xFFFFFFFFu) {
            tl_stack.push_back(n.right_node_idx_or_prim_idx);
            tl_stack.push_back(n.left_node_idx);
            continue;
        }
        uint32_t ii = n.right_node_idx_or_prim_idx;
        const OInstance &I = W.inst[ii];
        const OChunk &C = *I.ch;
        if (C.mesh) {  // every triangle, in world space
            for (uint32_t tri = 0; tri < C.n_tris; tri++) {
                TriHit th;
                if (!tri_test(I.wpos[3 * tri], I.wpos[3 * tri + 1], I.wpos[3 * tri + 2], o, d, tmin, best.t, &th))
                    continue;
                uint64_t key = ((uint64_t)ii << 32) | tri;
                if (th.t < best.t || (th.t == best.t && key < best_key)) {
                    best.hit = true;
                    best.t = th.t;
                    best_key = key;
                    best.inst = ii;
                    best.tri = tri;
                    best.block = 0xFFFFFFFFu;
                    best.face = 0;
                    best.half = 0;
                    best.b1 = th.b1;
                    best.b2 = th.b2;
                    best.bx = best.by = best.bz = 0;
                }
            }
            continue;
        }
        std::vector<uint32_t> st{0};
        while (!st.empty()) {
            uint32_t bi = st.back();
            st.pop_back();
            const vrg_bvh_node &b = C.geo_nodes[bi];
            if (!box_test(b.min, b.max, I.off, o, inv, tmin, best.t)) continue;
            if (b.left_node_idx != 0xFFFFFFFFu) {
                st.push_back(b.right_node_idx_or_prim_idx);
                st.push_back(b.left_node_idx);
                continue;
            }
            uint32_t blk = b.right_node_idx_or_prim_idx;
            int lx = (int)(blk >> 10), ly = (int)((blk >> 5) & 31), lz = (int)(blk & 31);
            int wx = lx + (int)I.off[0], wy = ly + (int)I.off[1], wz = lz + (int)I.off[2];
            uint8_t mask = C.face_mask[blk];
            uint32_t rank = 0;
            for (int f = 0; f < 6; f++) {
                if (!(mask & (1u << f))) continue;
                FaceHit fh;
                if (face_test(wx, wy, wz, f, o, d, inv, tmin, best.t, &fh)) {
                    uint32_t tri = C.first_tri[blk] + 2 * rank + (uint32_t)fh.half;
                    uint64_t key = ((uint64_t)ii << 32) | tri;
                    if (fh.t < best.t || (fh.t == best.t && key < best_key)) {
                        best.hit = true;
                        best.t = fh.t;
                        best_key = key;
                        best.inst = ii;
                        best.tri = tri;
                        best.block = blk;
                        best.face = f;
                        best.half = fh.half;
                        best.b1 = fh.b1;
                        best.b2 = fh.b2;
                        best.bx = wx; best.by = wy; best.bz = wz;
                    }
                }
                rank++;
            }
        }
    }
    return best;
}

// world-space vertices of triangle (inst, tri) — the reference's
// triangleTransform of the instance vertex buffer (raytrace.rs:155-161)
static void tri_vertices(const OWorld &W, uint32_t ii, uint32_t tri, V3 out[3], int *face, int *half) {
    const OInstance &I = W.inst[ii];
    const OChunk &C = *I.ch;
    if (C.mesh) {
        for (int j = 0; j < 3; j++) out[j] = I.wpos[3 * (size_t)tri + j];
        if (face) *face = -1;
        if (half) *half = 0;
        return;
    }
    uint32_t blk = C.tri_block[tri];
    int f = C.tri_fh[tri] & 15, h = C.tri_fh[tri] >> 4;
    int lx = (int)(blk >> 10), ly = (int)((blk >> 5) & 31), lz = (int)(blk & 31);
    for (int j = 0; j < 3; j++) {
        V3 p = corner_pos(lx, ly, lz, FACE_TRI[f][h][j]);
        out[j] = v3(p.x + I.off[0], p.y + I.off[1], p.z + I.off[2]);
    }
    if (face) *face = f;
    if (half) *half = h;
}

// ------------------------------------------------------------------------
// light BVH: importance, stochastic descent, reverse walk, nee pdf
// ------------------------------------------------------------------------
// raytrace.rs:174-208 (uint visibility, EPS 1e-3) and nee_pdf.rs:119-152
// (float visibility, EPS 1e-4): the corners are the axis-aligned box spanned
// by the transformed min and max (not the transformed box).
static float node_importance(bool nee_variant, V3 point, V3 normal, const OXform &X, const vrg_bvh_node &node) {
    V3 v000 = xf_point(X, v3(node.min[0], node.min[1], node.min[2]));
    V3 v111 = xf_point(X, v3(node.max[0], node.max[1], node.max[2]));
    V3 c[8] = {v000, v3(v000.x, v000.y, v111.z), v3(v000.x, v111.y, v000.z), v3(v000.x, v111.y, v111.z),
               v3(v111.x, v000.y, v000.z), v3(v111.x, v000.y, v111.z), v3(v111.x, v111.y, v000.z), v111};
    float dist_sq = fmaxf(dot3(v111 - v000, v111 - v000),
                          dot3(0.5f * (v000 + v111) - point, 0.5f * (v000 + v111) - point));
    if (!nee_variant) {
        uint32_t visible = 0;
        for (int k = 0; k < 8; k++) visible += (dot3(c[k] - point, normal) >= EPS_BLOCK_TRACE) ? 1u : 0u;
        return node.power / dist_sq * ((float)visible / 8.0f);
    }
    float visible = 0.0f;
    for (int k = 0; k < 8; k++) visible += 0.125f * ((dot3(c[k] - point, normal) >= EPS_BLOCK_NEE) ? 1.0f : 0.0f);
    return node.power / dist_sq * visible;
}

struct TraverseResult {
    bool success;
    uint32_t inst, prim, leaf;
    float probability, importance;
};

// traverseBvh (raytrace.rs:218-281)
static TraverseResult traverse_bvh(const OWorld &W, V3 point, V3 normal, uint32_t seed) {
    TraverseResult R;
    const vrg_bvh_node *root = W.light_tl.data();
    const vrg_bvh_node *node = &root[0];
    if (node->left_node_idx == 0xFFFFFFFFu && node->right_node_idx_or_prim_idx == 0xFFFFFFFFu) {
        R.success = false; R.inst = 0; R.prim = 0; R.leaf = 0; R.probability = 1.0f; R.importance = 0.0f;
        return R;
    }
    float probability = 1.0f, importance = 0.0f;
    const OXform *X = &XF_IDENTITY;  // mat4x3(1.0) at the top level
    uint32_t inst = 0xFFFFFFFFu;
    uint32_t node_idx = 0;
    bool top = true;
    for (;;) {
        if (top && node->left_node_idx == 0xFFFFFFFFu) {
            inst = node->right_node_idx_or_prim_idx;
            const OInstance &I = W.inst[inst];
            X = &I.X;
            top = false;
            root = I.ch->light_nodes.data();
            node = &root[0];
            node_idx = 0;
            if (importance == 0.0f) importance = node_importance(false, point, normal, *X, *node);
        }
        if (!top && node->left_node_idx == 0xFFFFFFFFu) {
            R.success = true; R.inst = inst; R.prim = node->right_node_idx_or_prim_idx; R.leaf = node_idx;
            R.probability = probability; R.importance = importance;
            return R;
        }
        uint32_t li = node->left_node_idx, ri = node->right_node_idx_or_prim_idx;
        const vrg_bvh_node &left = root[li];
        const vrg_bvh_node &right = root[ri];
        float lI = node_importance(false, point, normal, *X, left);
        float rI = node_importance(false, point, normal, *X, right);
        float tot = lI + rI;
        float ln = lI / tot, rn = rI / tot;
        if (mm_rand(seed) < ln) { node = &left; node_idx = li; probability *= ln; importance = lI; }
        else { node = &right; node_idx = ri; probability *= rn; importance = rI; }
        seed = mm_combine(seed, 0);
    }
}

// reverseTraverseBvh (nee_pdf.rs:154-228)
static float reverse_traverse(const OWorld &W, V3 point, V3 normal, uint32_t ii, uint32_t leaf) {
    const OInstance &I = W.inst[ii];
    const vrg_bvh_node *root = I.ch->light_nodes.data();
    float probability = 1.0f;
    const OXform *X = &I.X;
    bool top = false;
    const vrg_bvh_node *node = &root[leaf];
    uint32_t node_idx = leaf;
    for (;;) {
        uint32_t old = node_idx;
        if (node->parent_idx == 0xFFFFFFFFu) {
            if (top) return probability;
            top = true;
            root = W.light_tl.data();
            old = I.light_bvh_tl_idx;
            const vrg_bvh_node &tl_leaf = root[I.light_bvh_tl_idx];
            if (tl_leaf.parent_idx == 0xFFFFFFFFu) return probability;
            node_idx = tl_leaf.parent_idx;
            node = &root[node_idx];
            X = &XF_IDENTITY;
        } else {
            node_idx = node->parent_idx;
            node = &root[node_idx];
        }
        const vrg_bvh_node &left = root[node->left_node_idx];
        const vrg_bvh_node &right = root[node->right_node_idx_or_prim_idx];
        float lI = node_importance(true, point, normal, *X, left);
        float rI = node_importance(true, point, normal, *X, right);
        float tot = lI + rI;
        float ln = lI / tot, rn = rI / tot;
        if (old == node->left_node_idx) probability *= ln;
        else probability *= rn;
    }
}

// computeNeePdf (nee_pdf.rs:240-279)
static float compute_nee_pdf(const OWorld &W, V3 point, V3 normal, V3 dir, uint32_t ii, uint32_t leaf,
                             float b1, float b2) {
    const OInstance &I = W.inst[ii];
    uint32_t tri = I.ch->light_nodes[leaf].right_node_idx_or_prim_idx;
    V3 tv[3];
    tri_vertices(W, ii, tri, tv, nullptr, nullptr);
    // pointOnTriangle (nee_pdf.rs:230-232)
    V3 p = (b1 * tv[0] + b2 * tv[1]) + ((1.0f - b1) - b2) * tv[2];
    float light_distance = length3(p - point);
    float light_area = 0.5f * length3(cross3(tv[0] - tv[1], tv[2] - tv[1]));
    float cos_theta = dot3(normal, dir);
    float ppp = light_distance * light_distance / (cos_theta * light_area);
    float P = reverse_traverse(W, point, normal, ii, leaf);
    return P * ppp;
}

struct LightHit {
    uint64_t key;
    float value;
};

// nee_pdf main any-hit loop (nee_pdf.rs:281-337)
static float nee_pdf_any_hit(const OWorld &W, V3 o, V3 d, V3 normal) {
    const float tmin = EPS_BLOCK_NEE, tmax = 1000.0f;
    const vrg_bvh_node &r0 = W.light_tl[0];
    if (r0.left_node_idx == 0xFFFFFFFFu && r0.right_node_idx_or_prim_idx == 0xFFFFFFFFu) return 0.0f;
    V3 inv = v3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    std::vector<LightHit> hits;
    std::vector<uint32_t> tl_stack{0};
    while (!tl_stack.empty()) {
        uint32_t ni = tl_stack.back();
        tl_stack.pop_back();
        const vrg_bvh_node &n = W.light_tl[ni];
        if (!box_test(n.min, n.max, ZERO3, o, inv, tmin, tmax)) continue;
        if (n.left_node_idx != 0xFFFFFFFFu) {
            tl_stack.push_back(n.right_node_idx_or_prim_idx);
            tl_stack.push_back(n.left_node_idx);
            continue;
        }
        uint32_t ii = n.right_node_idx_or_prim_idx;
        const OInstance &I = W.inst[ii];
        const OChunk &C = *I.ch;
        if (C.mesh) {  // every light triangle (light BLAS leaf), in world space
            for (uint32_t bi = 0; bi < C.light_nodes.size(); bi++) {
                const vrg_bvh_node &b = C.light_nodes[bi];
                if (b.left_node_idx != 0xFFFFFFFFu) continue;
                const uint32_t tri = b.right_node_idx_or_prim_idx;
                TriHit th;
                if (!tri_test(I.wpos[3 * tri], I.wpos[3 * tri + 1], I.wpos[3 * tri + 2], o, d, tmin, tmax, &th))
                    continue;
                LightHit lh;
                lh.key = ((uint64_t)ii << 32) | bi;
                lh.value = compute_nee_pdf(W, o, normal, d, ii, bi, th.b1, th.b2);
                hits.push_back(lh);
            }
            continue;
        }
        std::vector<uint32_t> st{0};
        while (!st.empty()) {
            uint32_t bi = st.back();
            st.pop_back();
            const vrg_bvh_node &b = C.light_nodes[bi];
            if (!box_test(b.min, b.max, I.off, o, inv, tmin, tmax)) continue;
            if (b.left_node_idx != 0xFFFFFFFFu) {
                st.push_back(b.right_node_idx_or_prim_idx);
                st.push_back(b.left_node_idx);
                continue;
            }
            uint32_t tri = b.right_node_idx_or_prim_idx;
            uint32_t blk = C.tri_block[tri];
            int f = C.tri_fh[tri] & 15, h = C.tri_fh[tri] >> 4;
            int wx = (int)(blk >> 10) + (int)I.off[0], wy = (int)((blk >> 5) & 31) + (int)I.off[1],
                wz = (int)(blk & 31) + (int)I.off[2];
            FaceHit fh;
            if (face_test(wx, wy, wz, f, o, d, inv, tmin, tmax, &fh) && fh.half == h) {
                LightHit lh;
                lh.key = ((uint64_t)ii << 32) | bi;
                lh.value = compute_nee_pdf(W, o, normal, d, ii, bi, fh.b1, fh.b2);
                hits.push_back(lh);
            }
        }
    }
    std::sort(hits.begin(), hits.end(), [](const LightHit &a, const LightHit &b) { return a.key < b.key; });
    float pdf = 0.0f;
    for (auto &h : hits) pdf += h.value;
    return pdf;
}

// ------------------------------------------------------------------------
// frame state and stages (interactive_rendering.rs:952-1669)
// ------------------------------------------------------------------------
struct ORes {  // Reservoir (restir_temporal_resampling.rs:14-69)
    V3 x_v, n_v, x_s, n_s, l;
    float p_omega;
    uint32_t seed;
    float ucw;
    uint32_t m;
    float w_sum;
};

struct ORenderer {
    uint32_t W = 0, H = 0, nb_max = 0;
    uint32_t frame = 0;
    uint32_t nb = 0;
    // per-bounce SoA, [slice][P]
    std::vector<V3> origin, dir, normal, emis, refl, lout;
    std::vector<float> mis, pdf, nee, q;
    std::vector<uint32_t> hit;  // 4 per (bounce, pixel)
    std::vector<std::vector<ORes>> temporal;  // ring
    std::vector<ORes> spatial;
    std::vector<V3> final_target;
    std::vector<uint8_t> image;
    std::vector<V3> view;
    std::vector<double> accum;
    uint32_t accum_n = 0;
    uint32_t ring = 0;
    uint64_t rays_closest = 0, rays_any = 0;  // queries issued by the last frame
};

static void renderer_alloc(ORenderer &R, uint32_t W, uint32_t H, uint32_t nb) {
    R.W = W; R.H = H; R.nb_max = nb;
    size_t P = (size_t)W * H;
    R.origin.assign((nb + 1) * P, v3(0, 0, 0));
    R.dir.assign((nb + 1) * P, v3(0, 0, 0));
    R.normal.assign(nb * P, v3(0, 0, 0));
    R.emis.assign(nb * P, v3(0, 0, 0));
    R.refl.assign(nb * P, v3(0, 0, 0));
    R.lout.assign(nb * P, v3(0, 0, 0));
    R.mis.assign(nb * P, 0.0f);
    R.pdf.assign(nb * P, 0.0f);
    R.nee.assign(nb * P, 0.0f);
    R.q.assign(nb * P, 0.0f);
    R.hit.assign(nb * P * 4, 0u);
    R.temporal.clear();
    R.spatial.assign(P, ORes{});
    R.final_target.assign(P, v3(0, 0, 0));
    R.image.assign(P * 4, 0);
    R.view.assign(P, v3(0, 0, 0));
    R.accum.assign(P * 3, 0.0);
    R.accum_n = 0;
    R.frame = 0;
}

static inline uint8_t to_u8(float x) {
    float v = x * 255.0f;
    if (!(v > 0.0f)) return 0;
    if (v >= 255.0f) return 255;
    return (uint8_t)(int)v;
}

static void render_frame(ORenderer &R, const OWorld &W, const vrg_camera &cam, const vrg_render_params &pr,
                         int64_t pix_begin, int64_t pix_end) {
    const uint32_t Wd = R.W, Hd = R.H;
    const size_t P = (size_t)Wd * Hd;
    const uint32_t nb = pr.num_bounces;
    R.nb = nb;
    const uint32_t slots = pr.history_slots ? pr.history_slots : 3;
    if (R.temporal.size() != slots) {
        R.temporal.assign(slots, std::vector<ORes>(P, ORes{}));
        for (auto &ring : R.temporal)
            for (auto &r : ring) memset(&r, 0, sizeof(r));
    }
    const uint32_t ring = R.frame % slots;
    R.ring = ring;
    R.rays_closest = R.rays_any = 0;
    const V3 eye = v3(cam.eye[0], cam.eye[1], cam.eye[2]);
    const V3 front = v3(cam.front[0], cam.front[1], cam.front[2]);
    const V3 right = v3(cam.right[0], cam.right[1], cam.right[2]);
    const V3 up = v3(cam.up[0], cam.up[1], cam.up[2]);
    // pixels outside [pix_begin, pix_end) are not traced (bounded CPU sample)
    auto in_range = [&](int64_t p) { return p >= pix_begin && p < pix_end; };

    // raygen (raygen.rs:84-111): pixel corner, jitter multiplied by 0.00
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < (int64_t)P; p++) {
        uint32_t x = (uint32_t)(p % Wd), y = (uint32_t)(p / Wd);
        float u = 2.0f * (float)x / (float)Wd - 1.0f;
        float v = 2.0f * (float)y / (float)Hd - 1.0f;
        float aspect = (float)Wd / (float)Hd;
        R.origin[p] = eye;
        R.dir[p] = normalize3((u * right * aspect + v * up) + front);
    }

    // raytrace x nb (raytrace.rs:390-578)
    for (uint32_t b = 0; b < nb; b++) {
        const uint32_t inv_seed = R.frame * nb + b;  // interactive_rendering.rs:1189
        uint64_t n_closest = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : n_closest)
        for (int64_t p = 0; p < (int64_t)P; p++) {
            size_t in = b * P + p, out = (b + 1) * P + p, bb = b * P + p;
            uint32_t *hr = &R.hit[bb * 4];
            V3 origin = R.origin[in], direction = R.dir[in];
            uint32_t seed = mm_combine(inv_seed, (uint32_t)p);
            if (is_zero3(direction) || !in_range(p)) {
                R.origin[out] = origin;
                R.dir[out] = v3(0, 0, 0);
                R.normal[bb] = v3(0, 0, 0);
                R.emis[bb] = v3(0, 0, 0);
                R.refl[bb] = v3(0, 0, 0);
                R.mis[bb] = 0.0f;
                R.pdf[bb] = 1.0f;
                hr[0] = hr[1] = hr[2] = hr[3] = 0xFFFFFFFEu;
                continue;
            }
            n_closest++;
            OHit info = closest_hit(W, origin, direction, EPS_BLOCK_TRACE, 1000.0f);
            if (!info.hit) {
                R.origin[out] = origin + direction * 5000.0f;
                R.dir[out] = v3(0, 0, 0);
                R.normal[bb] = v3(0, 0, 0);
                float sky = (dot3(direction, v3(0, 1, 0)) > 0.9f) ? 50.0f : 0.0f;
                R.emis[bb] = v3(sky, sky, sky);
                R.refl[bb] = v3(0, 0, 0);
                R.mis[bb] = 0.0f;
                R.pdf[bb] = 1.0f;
                hr[0] = hr[1] = hr[2] = hr[3] = 0xFFFFFFFFu;
                continue;
            }
            hr[0] = info.inst;
            hr[1] = info.tri;
            hr[2] = info.block;
            hr[3] = (uint32_t)info.face | ((uint32_t)info.half << 8);
            float b0 = (1.0f - info.b1) - info.b2;
            V3 tri[3];
            tri_vertices(W, info.inst, info.tri, tri, nullptr, nullptr);
            // localCoordinateSystem (raytrace.rs:319-331)
            V3 v01 = tri[1] - tri[0], v02 = tri[2] - tri[0];
            V3 nrm = cross3(v01, v02);
            V3 tan = v01;
            V3 bit = cross3(nrm, tan);
            V3 n = normalize3(nrm), tg = normalize3(tan), bt = normalize3(bit);
            const OChunk &HC = *W.inst[info.inst].ch;
            // texture index: a mesh triangle's first vertex's t (raytrace.rs:455); a
            // chunk face's 6 * block + face (block.rs:116-119)
            const uint32_t slot = HC.mesh ? HC.mslot[info.tri] : 6u * HC.blocks[info.block] + (uint32_t)info.face;
            const vrg_material &m = W.M.mats[slot];
            V3 new_origin = (tri[0] * b0 + tri[1] * info.b1) + tri[2] * info.b2;
            V3 new_dir;
            V3 reflectivity = v3(m.reflectivity[0], m.reflectivity[1], m.reflectivity[2]);
            float alpha = m.alpha;
            float ndd = -dot3(direction, n);
            V3 emissivity = v3(m.emission[0] * ndd, m.emission[1] * ndd, m.emission[2] * ndd);
            float metallicity = m.metallic;
            if (!W.M.atlas.empty()) {
                // raytrace.rs:457-480: uv = v0.uv*b0 + v1.uv*b1 + v2.uv*b2; texture()
                // with the default sampler taken as nearest, clamp to edge
                const float(*uv)[2] = HC.mesh ? reinterpret_cast<const float(*)[2]>(&HC.muv[6 * (size_t)info.tri])
                                              : FACE_UV[info.face][info.half];
                const float u = ((uv[0][0] * b0) + (uv[1][0] * info.b1)) + (uv[2][0] * info.b2);
                const float vv = ((uv[0][1] * b0) + (uv[1][1] * info.b1)) + (uv[2][1] * info.b2);
                const int aw = (int)W.M.atlas_w, ah = (int)W.M.atlas_h;
                const int ix = std::min(std::max((int)std::floor(u * (float)aw), 0), aw - 1);
                const int iy = std::min(std::max((int)std::floor(vv * (float)ah), 0), ah - 1);
                auto texel = [&](int map) {
                    return W.M.atlas.data() + 4 * ((((size_t)slot * 3 + map) * ah + iy) * aw + ix);
                };
                const uint8_t *t0 = texel(0), *t1 = texel(1), *t2 = texel(2);
                const float *lin = W.M.srgb;
                reflectivity = v3(lin[t0[0]], lin[t0[1]], lin[t0[2]]);
                alpha = (float)t0[3] / 255.0f;
                emissivity = v3((1000.0f * lin[t1[0]]) * ndd, (1000.0f * lin[t1[1]]) * ndd, (1000.0f * lin[t1[2]]) * ndd);
                metallicity = lin[t2[0]];
            }
            float mis_w = 0.0f, bsdf_pdf;
            float r0 = mm_rand(mm_combine(seed, 0));
            if (r0 < metallicity) {
                bsdf_pdf = 1.0f;
                new_dir = direction - (2.0f * dot3(n, direction)) * n;  // reflect
            } else if (r0 < metallicity + (1.0f - alpha)) {
                new_dir = direction;
                reflectivity = v3(1.0f, 1.0f, 1.0f);
                bsdf_pdf = 1.0f;
            } else {
                new_origin = new_origin + (EPS_BLOCK_TRACE * 1.5f) * n;
                reflectivity = v3(reflectivity.x / PI_F, reflectivity.y / PI_F, reflectivity.z / PI_F);
                TraverseResult res;
                res.success = false;
                res.importance = 0.0f;
                if (pr.nee_type == 1 || (pr.nee_type == 2 && b == 1))
                    res = traverse_bvh(W, new_origin, n, mm_combine(seed, 2));
                if (res.success && res.importance > 0.0f) mis_w = 0.3f;
                float mis_rand = mm_rand(mm_combine(seed, 3));
                if (mis_rand < mis_w) {
                    V3 lt[3];
                    tri_vertices(W, res.inst, res.prim, lt, nullptr, nullptr);
                    float ux = mm_rand(mm_combine(seed, 4)), uy = mm_rand(mm_combine(seed, 5));
                    if (ux + uy > 1.0f) { ux = 1.0f - ux; uy = 1.0f - uy; }  // triangleSample
                    float bx = (1.0f - ux) - uy;
                    V3 sp = (bx * lt[0] + ux * lt[1]) + uy * lt[2];
                    new_dir = normalize3(sp - new_origin);
                } else {
                    float ux = mm_rand(mm_combine(seed, 4)), uy = mm_rand(mm_combine(seed, 5));
                    float s, c;
                    sincos_turns(ux, &s, &c);
                    float vv = sqrtf(fmaxf(0.0f, 1.0f - uy * uy));
                    V3 hs = v3(vv * c, uy, vv * s);
                    new_dir = normalize3((hs.x * tg + hs.y * n) + hs.z * bt);
                }
                float cos_theta = dot3(new_dir, n);
                bsdf_pdf = cos_theta / PI_F;
            }
            R.origin[out] = new_origin;
            R.dir[out] = new_dir;
            R.normal[bb] = n;
            R.emis[bb] = emissivity;
            R.refl[bb] = reflectivity;
            R.mis[bb] = mis_w;
            R.pdf[bb] = bsdf_pdf;
        }
        R.rays_closest += n_closest;
    }

    // nee_pdf x (nb-1) (nee_pdf.rs:281-337); slot nb-1 is never written by the
    // reference, taken as 0 here.
    for (uint32_t b = 0; b < nb; b++) {
        uint64_t n_any = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : n_any)
        for (int64_t p = 0; p < (int64_t)P; p++) {
            size_t bb = b * P + p;
            if (b + 1 >= nb) { R.nee[bb] = 0.0f; continue; }
            V3 d = R.dir[(b + 1) * P + p];
            if (length3(d) == 0.0f || R.mis[bb] == 0.0f) { R.nee[bb] = 0.0f; continue; }
            n_any++;
            R.nee[bb] = nee_pdf_any_hit(W, R.origin[(b + 1) * P + p], d, R.normal[bb]);
        }
        R.rays_any += n_any;
    }

    // outgoing_radiance (outgoing_radiance.rs:171-207)
    const float inv2pi = 1.0f / (2.0f * PI_F);
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < (int64_t)P; p++) {
        V3 L = v3(0, 0, 0);
        for (int b = (int)nb - 1; b >= 0; b--) {
            size_t bb = (size_t)b * P + p;
            float valid = is_zero3(R.dir[bb]) ? 0.0f : 1.0f;
            float q = R.nee[bb] * R.mis[bb] + (1.0f - R.mis[bb]) * inv2pi;
            float w = R.pdf[bb] / q;
            V3 E = R.emis[bb], Rf = R.refl[bb];
            L = v3(E.x + ((Rf.x * L.x) * w) * valid, E.y + ((Rf.y * L.y) * w) * valid,
                   E.z + ((Rf.z * L.z) * w) * valid);
            R.lout[bb] = L;
            R.q[bb] = q;
        }
    }

    // initial samples (interactive_rendering.rs:1359-1414) + temporal
    // resampling (restir_temporal_resampling.rs:256-301)
    std::vector<ORes> &T = R.temporal[ring];
    if (nb >= 2) {
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < (int64_t)P; p++) {
            ORes S;
            S.x_v = R.origin[1 * P + p];
            S.n_v = R.normal[0 * P + p];
            S.x_s = R.origin[2 * P + p];
            S.n_s = R.normal[1 * P + p];
            S.l = R.lout[1 * P + p];
            S.p_omega = R.q[0 * P + p];
            S.seed = 0;
            uint32_t ps = mm_combine(pr.temporal_seed, (uint32_t)p);
            ORes Rv = T[p];
            if (mm_rand(mm_combine(ps, 0)) < 0.4f) { Rv.w_sum = 0.0f; Rv.m = 0; }
            if (pr.mode == VRG_MODE_CONFIG && pr.m_cap && Rv.m > pr.m_cap) {
                Rv.w_sum = Rv.w_sum * ((float)pr.m_cap / (float)Rv.m);
                Rv.m = pr.m_cap;
            }
            float w = luminance(S.l) / S.p_omega;
            // updateReservoir (restir_temporal_resampling.rs:235-246)
            Rv.w_sum += w;
            Rv.m += 1;
            if (float_construct(mm_finalize(mm_combine(ps, 1))) < w / Rv.w_sum) {
                Rv.x_v = S.x_v; Rv.n_v = S.n_v; Rv.x_s = S.x_s; Rv.n_s = S.n_s; Rv.l = S.l;
                Rv.p_omega = S.p_omega; Rv.seed = S.seed;
            }
            float ph = luminance(Rv.l);
            Rv.ucw = (ph > 0.0f) ? Rv.w_sum / ((float)Rv.m * ph) : 0.0f;
            T[p] = Rv;
        }

        // spatial (restir_spatial_resampling.rs:316-406)
        const float cos25 = 0.906307787036649963f;
        const float radius = pr.spatial_radius;
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < (int64_t)P; p++) {
            uint32_t qx = (uint32_t)(p % Wd), qy = (uint32_t)(p / Wd);
            uint32_t ps = mm_combine(pr.spatial_seed, (uint32_t)p);
            ORes Rs = T[p];
            ORes S = Rs;
            uint32_t Z = 0;
            if (luminance(Rs.l) > 0.0f) Z += Rs.m;
            for (uint32_t s = 0; s < pr.spatial_iterations; s++) {
                uint32_t is = mm_combine(ps, s);
                float jx = radius * (mm_rand(mm_combine(is, 0)) - 0.5f);
                float jy = radius * (mm_rand(mm_combine(is, 1)) - 0.5f);
                int nx = (int)(((float)qx + 0.5f) + jx);
                int ny = (int)(((float)qy + 0.5f) + jy);
                nx = std::min(std::max(nx, 0), (int)Wd - 1);
                ny = std::min(std::max(ny, 0), (int)Hd - 1);
                const ORes &Rn = T[(size_t)nx + (size_t)ny * Wd];
                // geometricallySimilar (restir_spatial_resampling.rs:277-288)
                if (is_zero3(S.n_v) || is_zero3(Rn.n_v)) continue;
                if (dot3(S.n_v, Rn.n_v) < cos25) continue;
                // computeJacobianQToR (restir_spatial_resampling.rs:299-311)
                float J;
                if (is_zero3(Rn.n_s)) J = 1.0f;
                else {
                    V3 qvs = Rn.x_v - Rn.x_s, rvs = S.x_v - Rn.x_s;
                    float cq = fabsf(dot3(normalize3(qvs), Rn.n_s));
                    float cr = fabsf(dot3(normalize3(rvs), Rn.n_s));
                    J = (cr / cq) * (length3(qvs) / length3(rvs));
                }
                J = fminf(fmaxf(J, 0.1f), 10.0f);
                float p_adj = luminance(Rn.l) / J;
                // mergeReservoir (restir_spatial_resampling.rs:266-275)
                uint32_t m0 = Rs.m;
                float wn = (p_adj * Rn.ucw) * (float)Rn.m;
                Rs.w_sum += wn;
                Rs.m += 1;
                if (float_construct(mm_finalize(mm_combine(is, 2))) < wn / Rs.w_sum) {
                    Rs.x_v = Rn.x_v; Rs.n_v = Rn.n_v; Rs.x_s = Rn.x_s; Rs.n_s = Rn.n_s; Rs.l = Rn.l;
                    Rs.p_omega = Rn.p_omega; Rs.seed = Rn.seed;
                }
                Rs.m = m0 + Rn.m;
                if (luminance(Rn.l) > 0.0f) Z += Rn.m;
            }
            float ph = luminance(Rs.l);
            Rs.ucw = (ph == 0.0f) ? 0.0f : Rs.w_sum / ((float)Z * ph);
            R.spatial[p] = Rs;
            // finalize (restir_finalize.rs:121-141)
            V3 dir = normalize3(Rs.x_s - R.origin[1 * P + p]);
            float bp = dot3(dir, Rs.n_v) / PI_F;
            V3 E0 = R.emis[p], R0 = R.refl[p];
            R.final_target[p] = v3(E0.x + ((R0.x * Rs.l.x) * Rs.ucw) * bp, E0.y + ((R0.y * Rs.l.y) * Rs.ucw) * bp,
                                   E0.z + ((R0.z * Rs.l.z) * Rs.ucw) * bp);
        }
    }

    // postprocess (postprocess.rs:39-88), scale 1
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < (int64_t)P; p++) {
        V3 c;
        if (pr.debug_view == 0) c = R.lout[p];
        else if (pr.debug_view == 1) c = R.final_target[p];
        else { float d = R.spatial[p].ucw / 10.0f; c = v3(d, d, d); }
        c = v3(c.x / 1.0f, c.y / 1.0f, c.z / 1.0f);
        R.view[p] = c;
        R.image[4 * p + 0] = to_u8(c.z);
        R.image[4 * p + 1] = to_u8(c.y);
        R.image[4 * p + 2] = to_u8(c.x);
        R.image[4 * p + 3] = 255;
        if (pr.accumulate && std::isfinite(c.x) && std::isfinite(c.y) && std::isfinite(c.z)) {
            R.accum[3 * p + 0] += (double)c.x;
            R.accum[3 * p + 1] += (double)c.y;
            R.accum[3 * p + 2] += (double)c.z;
        }
    }
    if (pr.accumulate) R.accum_n++;
    R.frame++;
}

}  // namespace

// ------------------------------------------------------------------------
// C API (ctypes)
// ------------------------------------------------------------------------
struct orc_world {
    OWorld W;
};
struct orc_chunk {
    std::shared_ptr<OChunk> c;
};
struct orc_renderer {
    ORenderer R;
};

ORC_API int orc_build_tl_bvh(uint32_t n, const float *translations, const float *aabbs, const float *power,
                             const uint32_t *ids, vrg_bvh_node *nodes_out, uint32_t *order_out) {
    if (n == 0) return 1;
    std::vector<OAabb> ab(n);
    for (uint32_t i = 0; i < n; i++) ab[i] = aabb_make(aabbs + 6 * i, aabbs + 6 * i + 3);
    std::vector<vrg_bvh_node> out;
    std::vector<uint32_t> order;
    build_tl(n, translations, ab.data(), power, ids, out, order);
    memcpy(nodes_out, out.data(), out.size() * sizeof(vrg_bvh_node));
    if (order_out) memcpy(order_out, order.data(), n * 4);
    return 0;
}

ORC_API int orc_build_bl_bvh(uint32_t n, const float *lum, const float *tris, const uint32_t *ids,
                             vrg_bvh_node *nodes_out, uint32_t *order_out, float *root_aabb, float *root_power) {
    if (n == 0) return 1;
    std::vector<V3> t(3 * (size_t)n);
    for (size_t i = 0; i < 3 * (size_t)n; i++) t[i] = v3(tris[3 * i], tris[3 * i + 1], tris[3 * i + 2]);
    std::vector<vrg_bvh_node> out;
    std::vector<uint32_t> order;
    OAabb ra;
    float rp;
    build_bl(n, lum, t.data(), ids, out, order, &ra, &rp);
    memcpy(nodes_out, out.data(), out.size() * sizeof(vrg_bvh_node));
    if (order_out) memcpy(order_out, order.data(), n * 4);
    if (root_aabb) { for (int i = 0; i < 3; i++) { root_aabb[i] = ra.mn[i]; root_aabb[3 + i] = ra.mx[i]; } }
    if (root_power) *root_power = rp;
    return 0;
}

ORC_API void orc_sincos_turns(float x, float *s, float *c) { sincos_turns(x, s, c); }
// the watertight ray/triangle test: 1 and (t, b1, b2) on a hit, else 0
ORC_API int orc_tri_test(const float *v9, const float *o3, const float *d3, float tmin, float tmax, float *out3) {
    TriHit h;
    if (!tri_test(v3(v9[0], v9[1], v9[2]), v3(v9[3], v9[4], v9[5]), v3(v9[6], v9[7], v9[8]), v3(o3[0], o3[1], o3[2]),
                  v3(d3[0], d3[1], d3[2]), tmin, tmax, &h))
        return 0;
    out3[0] = h.t;
    out3[1] = h.b1;
    out3[2] = h.b2;
    return 1;
}
ORC_API uint32_t orc_mm_combine(uint32_t h, uint32_t k) { return mm_combine(h, k); }
ORC_API float orc_mm_rand(uint32_t h) { return mm_rand(h); }

ORC_API orc_world *orc_world_create(const vrg_material *mats, uint32_t n) {
    if (n == 0 || n % 6) return nullptr;
    orc_world *w = new orc_world();
    w->W.M.mats.assign(mats, mats + n);
    w->W.M.n_types = n / 6;
    return w;
}
ORC_API void orc_world_destroy(orc_world *w) { delete w; }

// texture atlas [slot][3 maps][h][w] RGBA8 sRGB; slot luminance = mean of
// r8+g8+b8 over the emissivity map (utils.rs:223-235).  Before building chunks.
ORC_API int orc_world_set_atlas(orc_world *w, const uint8_t *rgba8, uint32_t n_slots, uint32_t aw, uint32_t ah) {
    OMaterials &M = w->W.M;
    if (n_slots != M.mats.size() || aw == 0 || ah == 0) return 1;
    const size_t map = (size_t)aw * ah;
    M.atlas.assign(rgba8, rgba8 + (size_t)n_slots * 3 * map * 4);
    M.atlas_w = aw;
    M.atlas_h = ah;
    for (uint32_t t = 0; t < n_slots; t++) {
        const uint8_t *e = rgba8 + ((size_t)t * 3 + 1) * map * 4;
        float L = 0.0f;
        for (size_t i = 0; i < map; i++) L += ((float)e[4 * i] + (float)e[4 * i + 1]) + (float)e[4 * i + 2];
        M.mats[t].luminance = L / (float)(aw * ah);
    }
    for (int i = 0; i < 256; i++) {  // sRGB EOTF
        const double c = (double)i / 255.0;
        M.srgb[i] = (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
    }
    return 0;
}

// gen_mesh + upload_object for one chunk with explicit neighbours (NULL = air)
ORC_API orc_chunk *orc_chunk_build(orc_world *w, const uint8_t *blocks, const uint8_t *const nb[6]) {
    orc_chunk *c = new orc_chunk();
    c->c = std::make_shared<OChunk>();
    c->c->blocks.assign(blocks, blocks + VRG_CHUNK_BLOCKS);
    const uint8_t *n6[6];
    for (int i = 0; i < 6; i++) n6[i] = nb ? nb[i] : nullptr;
    build_chunk(*c->c, w->W.M, n6);
    return c;
}
ORC_API void orc_chunk_destroy(orc_chunk *c) { delete c; }
ORC_API void orc_chunk_info(orc_chunk *c, uint32_t *n_tris, uint32_t *n_light, uint32_t *n_geo) {
    *n_tris = c->c->n_tris;
    *n_light = c->c->n_light;
    *n_geo = c->c->n_geo;
}
// which: 0 light BLAS, 1 geometry BLAS
ORC_API int orc_chunk_read_bvh(orc_chunk *c, uint32_t which, vrg_bvh_node *nodes, uint32_t *order) {
    const auto &N = which ? c->c->geo_nodes : c->c->light_nodes;
    const auto &O = which ? c->c->geo_order : c->c->light_order;
    if (N.empty()) return 1;
    memcpy(nodes, N.data(), N.size() * sizeof(vrg_bvh_node));
    if (order) memcpy(order, O.data(), O.size() * 4);
    return 0;
}
ORC_API void orc_world_add(orc_world *w, uint64_t key, orc_chunk *c, float tx, float ty, float tz) {
    OXform X = XF_IDENTITY;
    X.m[3] = tx;
    X.m[7] = ty;
    X.m[11] = tz;
    w->W.objects[key] = std::make_pair(c->c, X);
}
// any row-major 3x4 transform [R|t]; an exactly identity R is a translation
ORC_API void orc_world_add_xform(orc_world *w, uint64_t key, orc_chunk *c, const float *m12) {
    OXform X;
    memcpy(X.m, m12, sizeof(X.m));
    X.tonly = true;
    for (int r = 0; r < 3; r++)
        for (int k = 0; k < 3; k++) X.tonly = X.tonly && m12[4 * r + k] == (r == k ? 1.0f : 0.0f);
    w->W.objects[key] = std::make_pair(c->c, X);
}
// upload_object of a triangle mesh (nverts a multiple of 3; slots in the table)
ORC_API orc_chunk *orc_mesh_build(orc_world *w, const vrg_vertex3d *v, uint64_t nverts) {
    orc_chunk *c = new orc_chunk();
    c->c = std::make_shared<OChunk>();
    if (!build_mesh(*c->c, w->W.M, v, nverts)) {
        delete c;
        return nullptr;
    }
    return c;
}
ORC_API void orc_world_remove(orc_world *w, uint64_t key) { w->W.objects.erase(key); }
ORC_API void orc_world_commit(orc_world *w) { world_commit(w->W); }
// which: 0 light TL, 1 geometry TL
ORC_API uint32_t orc_world_read_tl(orc_world *w, uint32_t which, vrg_bvh_node *nodes, uint32_t cap) {
    const auto &N = which ? w->W.geo_tl : w->W.light_tl;
    uint32_t n = (uint32_t)N.size();
    if (nodes) memcpy(nodes, N.data(), std::min(n, cap) * sizeof(vrg_bvh_node));
    return n;
}
ORC_API uint32_t orc_world_instance_tl_idx(orc_world *w, uint32_t inst) {
    return inst < w->W.inst.size() ? w->W.inst[inst].light_bvh_tl_idx : 0xFFFFFFFFu;
}

ORC_API orc_renderer *orc_renderer_create(uint32_t W, uint32_t H, uint32_t nb) {
    orc_renderer *r = new orc_renderer();
    renderer_alloc(r->R, W, H, nb);
    return r;
}
ORC_API void orc_renderer_destroy(orc_renderer *r) { delete r; }

// Renders one frame; only pixels in [pix_begin, pix_end) are traced (the
// rest are treated as terminated), which bounds the CPU baseline's work.
ORC_API int orc_render(orc_renderer *r, orc_world *w, const vrg_camera *cam, const vrg_render_params *pr,
                       int64_t pix_begin, int64_t pix_end) {
    if (pr->num_bounces == 0 || pr->num_bounces > r->R.nb_max) return 1;
    if (cam->width != r->R.W || cam->height != r->R.H) return 1;
    render_frame(r->R, w->W, *cam, *pr, pix_begin, pix_end);
    return 0;
}

// Same layouts as vrg_debug_readback.
ORC_API int orc_readback(orc_renderer *r, uint32_t what, void *dst, uint64_t bytes) {
    ORenderer &R = r->R;
    size_t P = (size_t)R.W * R.H;
    uint32_t nb = R.nb;
    auto put3 = [&](const std::vector<V3> &v, size_t slices) -> int {
        if (bytes < slices * P * 12) return 1;
        memcpy(dst, v.data(), slices * P * 12);
        return 0;
    };
    auto put1 = [&](const std::vector<float> &v, size_t slices) -> int {
        if (bytes < slices * P * 4) return 1;
        memcpy(dst, v.data(), slices * P * 4);
        return 0;
    };
    auto put_res = [&](const std::vector<ORes> &v) -> int {
        if (bytes < P * 80) return 1;
        float *o = (float *)dst;
        for (size_t p = 0; p < P; p++) {
            const ORes &s = v[p];
            float *d = o + 20 * p;
            V3 a[5] = {s.x_v, s.n_v, s.x_s, s.n_s, s.l};
            for (int k = 0; k < 5; k++) { d[3 * k] = a[k].x; d[3 * k + 1] = a[k].y; d[3 * k + 2] = a[k].z; }
            d[15] = s.p_omega;
            memcpy(&d[16], &s.seed, 4);
            d[17] = s.ucw;
            memcpy(&d[18], &s.m, 4);
            d[19] = s.w_sum;
        }
        return 0;
    };
    switch (what) {
    case VRG_DBG_ORIGIN: return put3(R.origin, nb + 1);
    case VRG_DBG_DIRECTION: return put3(R.dir, nb + 1);
    case VRG_DBG_NORMAL: return put3(R.normal, nb);
    case VRG_DBG_EMISSIVITY: return put3(R.emis, nb);
    case VRG_DBG_REFLECTIVITY: return put3(R.refl, nb);
    case VRG_DBG_MIS: return put1(R.mis, nb);
    case VRG_DBG_BSDF_PDF: return put1(R.pdf, nb);
    case VRG_DBG_NEE_PDF: return put1(R.nee, nb);
    case VRG_DBG_RADIANCE: return put3(R.lout, nb);
    case VRG_DBG_Q: return put1(R.q, nb);
    case VRG_DBG_HIT:
        if (bytes < nb * P * 16) return 1;
        memcpy(dst, R.hit.data(), nb * P * 16);
        return 0;
    case VRG_DBG_TEMPORAL: return put_res(R.temporal[R.ring]);
    case VRG_DBG_SPATIAL: return put_res(R.spatial);
    case VRG_DBG_FINAL: return put3(R.final_target, 1);
    default: return 1;
    }
}
ORC_API int orc_read_image(orc_renderer *r, uint8_t *bgra, float *view) {
    size_t P = (size_t)r->R.W * r->R.H;
    if (bgra) memcpy(bgra, r->R.image.data(), P * 4);
    if (view) memcpy(view, r->R.view.data(), P * 12);
    return 0;
}
// postprocess with srcscale = scale, dstscale = 1 (postprocess.rs:39-88): the
// per-pixel view colours of a W x H traced frame (row-major float RGB) to
// (W/scale) x (H/scale) output pixels, each the sum of its scale x scale
// samples (rows outer, columns inner, from vec3(0.0)) divided by
// float(scale*scale), packed as u8(bgr*255) with alpha 255.
ORC_API int orc_postprocess_scaled(const float *view, uint32_t W, uint32_t H, uint32_t scale, uint8_t *bgra,
                                   float *out) {
    if (scale == 0 || W % scale || H % scale) return 1;
    const uint32_t ow = W / scale, oh = H / scale;
    for (uint32_t oy = 0; oy < oh; oy++)
        for (uint32_t ox = 0; ox < ow; ox++) {
            V3 c = v3(0.0f, 0.0f, 0.0f);
            for (uint32_t sy = 0; sy < scale; sy++) {
                const uint32_t y = oy * scale + sy;
                for (uint32_t sx = 0; sx < scale; sx++) {
                    const uint32_t x = ox * scale + sx;
                    const size_t id = (size_t)y * W + x;
                    c = v3(c.x + view[3 * id], c.y + view[3 * id + 1], c.z + view[3 * id + 2]);
                }
            }
            const float n = (float)(scale * scale);
            c = v3(c.x / n, c.y / n, c.z / n);
            const size_t o = (size_t)oy * ow + ox;
            if (bgra) {
                bgra[4 * o] = to_u8(c.z);
                bgra[4 * o + 1] = to_u8(c.y);
                bgra[4 * o + 2] = to_u8(c.x);
                bgra[4 * o + 3] = 255;
            }
            if (out) {
                out[3 * o] = c.x;
                out[3 * o + 1] = c.y;
                out[3 * o + 2] = c.z;
            }
        }
    return 0;
}

ORC_API void orc_ray_counts(orc_renderer *r, uint64_t *closest, uint64_t *any) {
    *closest = r->R.rays_closest;
    *any = r->R.rays_any;
}
ORC_API uint32_t orc_read_accum(orc_renderer *r, double *rgb) {
    size_t P = (size_t)r->R.W * r->R.H;
    if (rgb) memcpy(rgb, r->R.accum.data(), P * 24);
    return r->R.accum_n;
}
