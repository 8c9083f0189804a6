// Device-side math shared by every kernel of the path tracer.
//
// Bit-exactness contract: every float expression here is a sequence of
// single IEEE binary32 operations in source order.  The library is compiled
// with -fmad=false (no FMA contraction), -prec-div=true and -prec-sqrt=true
// (correctly rounded division and square root), so the same expression gives
// the same bits on the GPU as on a host compiled with -ffp-contract=off.
// GLSL built-ins follow the reference shader semantics with a fixed
// evaluation order: dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z, normalize(v) =
// v / length(v) per component, reflect(I,N) = I - (2*dot(N,I))*N.
#pragma once

#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/vrg.h"

namespace vrg {

struct f3 {
    float x, y, z;
};
__host__ __device__ __forceinline__ f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
__host__ __device__ __forceinline__ f3 add3(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ f3 sub3(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ f3 scl3(f3 a, float s) { return f3{a.x * s, a.y * s, a.z * s}; }
__host__ __device__ __forceinline__ f3 lscl3(float s, f3 a) { return f3{s * a.x, s * a.y, s * a.z}; }
__host__ __device__ __forceinline__ float dot3(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__host__ __device__ __forceinline__ f3 cross3(f3 a, f3 b) {
    return f3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
__host__ __device__ __forceinline__ float len3(f3 a) { return sqrtf(dot3(a, a)); }
__host__ __device__ __forceinline__ f3 norm3(f3 a) {
    float l = len3(a);
    return f3{a.x / l, a.y / l, a.z / l};
}
__host__ __device__ __forceinline__ bool zero3(f3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
__host__ __device__ __forceinline__ float cmp3(f3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
__device__ __forceinline__ f3 ld3(float4 v) { return f3{v.x, v.y, v.z}; }

constexpr float PI_F = 3.1415926535897932384626433832795f;          // raytrace.rs:12
constexpr float TWO_PI_F = 6.283185307179586476925286766559f;
constexpr float EPS_TRACE = 0.001f;                                   // raytrace.rs:13
constexpr float EPS_NEE = 0.0001f;                                    // nee_pdf.rs:15
constexpr float FACE_PAD = 1.0f / 4096.0f;                            // closed, overlapping faces
constexpr float BOX_MARGIN = 1.0f / 128.0f;                           // conservative culling
constexpr float COS25 = 0.906307787036649963f;                        // cos(radians(25))
constexpr uint32_t INVALID = 0xFFFFFFFFu;
constexpr uint32_t TERMINATED = 0xFFFFFFFEu;

// murmur3 chaining (raygen.rs:48-78)
__host__ __device__ __forceinline__ uint32_t mm_combine(uint32_t h, uint32_t k) {
    k *= 0x1b873593u;
    h ^= k;
    h = (h << 13) | (h >> 19);
    h = h * 5u + 0xe6546b64u;
    return h;
}
__host__ __device__ __forceinline__ uint32_t mm_finalize(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}
// floatConstruct (raygen.rs:37-46)
__host__ __device__ __forceinline__ float float_construct(uint32_t m) {
    m &= 0x007FFFFFu;
    m |= 0x3F800000u;
#ifdef __CUDA_ARCH__
    return __uint_as_float(m) - 1.0f;
#else
    float f;
    __builtin_memcpy(&f, &m, 4);
    return f - 1.0f;
#endif
}
__host__ __device__ __forceinline__ float mm_rand(uint32_t h) { return float_construct(mm_finalize(h)); }

// sin(2*pi*x), cos(2*pi*x), x in [0,1): exact quarter-turn reduction, then
// the Taylor series of sin (to a^9) and cos (to a^10) on |a| <= pi/4.
__host__ __device__ __forceinline__ void sincos_turns(float x, float *s, float *c) {
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

__host__ __device__ __forceinline__ float luminance3(f3 v) {  // restir_temporal_resampling.rs:248-250
    return (0.2126f * v.x + 0.7152f * v.y) + 0.0722f * v.z;
}

// gen_mesh corner bits per (face, triangle, vertex): v{abc} = (x+a, y+b, z+c)
// (chunk.rs:225-285, faces in the order left, right, down, up, back, front)
__host__ __device__ __forceinline__ uint32_t face_corner(int f, int h, int j) {
    // packed: 3 bits per vertex, 9 bits per triangle, 18 bits per face
    constexpr uint64_t T[6] = {
        (0b001ull | 0b010ull << 3 | 0b000ull << 6) | ((0b011ull | 0b010ull << 3 | 0b001ull << 6) << 9),
        (0b110ull | 0b101ull << 3 | 0b100ull << 6) | ((0b110ull | 0b111ull << 3 | 0b101ull << 6) << 9),
        (0b000ull | 0b100ull << 3 | 0b001ull << 6) | ((0b100ull | 0b101ull << 3 | 0b001ull << 6) << 9),
        (0b011ull | 0b110ull << 3 | 0b010ull << 6) | ((0b011ull | 0b111ull << 3 | 0b110ull << 6) << 9),
        (0b010ull | 0b100ull << 3 | 0b000ull << 6) | ((0b010ull | 0b110ull << 3 | 0b100ull << 6) << 9),
        (0b001ull | 0b101ull << 3 | 0b011ull << 6) | ((0b101ull | 0b111ull << 3 | 0b011ull << 6) << 9),
    };
    return (uint32_t)((T[f] >> (9 * h + 3 * j)) & 7u);
}
// gen_mesh texture coordinates per (face, triangle, vertex) as u | v << 1
// (chunk.rs:225-285: each face's four corners carry fixed uvs)
__host__ __device__ __forceinline__ uint32_t face_uv(int f, int h, int j) {
    // packed: 2 bits per vertex, 6 bits per triangle, 12 bits per face
#define VRG_UV3(a, b, c) ((a) | (b) << 2 | (c) << 4)
    constexpr uint32_t T[6] = {
        VRG_UV3(2u, 1u, 3u) | VRG_UV3(0u, 1u, 2u) << 6,  // left:  (0,1) (1,0) (1,1) | (0,0) (1,0) (0,1)
        VRG_UV3(0u, 3u, 2u) | VRG_UV3(0u, 1u, 3u) << 6,  // right: (0,0) (1,1) (0,1) | (0,0) (1,0) (1,1)
        VRG_UV3(0u, 1u, 2u) | VRG_UV3(1u, 3u, 2u) << 6,  // down:  (0,0) (1,0) (0,1) | (1,0) (1,1) (0,1)
        VRG_UV3(3u, 0u, 1u) | VRG_UV3(3u, 2u, 0u) << 6,  // up:    (1,1) (0,0) (1,0) | (1,1) (0,1) (0,0)
        VRG_UV3(0u, 3u, 2u) | VRG_UV3(0u, 1u, 3u) << 6,  // back:  (0,0) (1,1) (0,1) | (0,0) (1,0) (1,1)
        VRG_UV3(3u, 2u, 1u) | VRG_UV3(2u, 0u, 1u) << 6,  // front: (1,1) (0,1) (1,0) | (0,1) (0,0) (1,0)
    };
#undef VRG_UV3
    return (T[f] >> (6 * h + 2 * j)) & 3u;
}

__host__ __device__ __forceinline__ f3 corner_pos(int bx, int by, int bz, uint32_t bits) {
    return f3{(float)(bx + (int)((bits >> 2) & 1u)), (float)(by + (int)((bits >> 1) & 1u)),
              (float)(bz + (int)(bits & 1u))};
}
// in-plane axes of a face: a = normal axis, u/v = the other two ascending
__host__ __device__ __forceinline__ void face_axes(int f, int &a, int &u, int &v) {
    a = f >> 1;
    u = (a == 0) ? 1 : 0;
    v = (a == 2) ? 1 : 2;
}
__host__ __device__ __forceinline__ int bitsel(uint32_t bits, int axis) { return (int)((bits >> (2 - axis)) & 1u); }

// barycentric weight of the triangle vertex at in-plane corner (cu, cv)
__host__ __device__ __forceinline__ float corner_weight(int cu, int cv, int half, float lu, float lv) {
    if (half == 0) {
        if (cu == 0 && cv == 0) return (1.0f - lu) - lv;
        if (cu == 1) return lu;
        return lv;
    }
    if (cu == 1 && cv == 1) return (lu + lv) - 1.0f;
    if (cu == 1) return 1.0f - lv;
    return 1.0f - lu;
}

// Exact test of one exposed voxel face (the pair of gen_mesh triangles) —
// the closest-hit and candidate semantics of the reference's ray query
// restated for axis-aligned unit faces: plane hit t in [tmin, tmax], the
// in-plane point inside the closed face rectangle padded by FACE_PAD, the
// triangle half chosen by the face diagonal (on the diagonal: triangle 0).
struct FaceHit {
    float t;
    int half;
    float b1, b2;
};
// The inverse direction of the traversal's slab tests and of face_test.  A
// component of exactly 0 gets +-1e30 instead of +-inf.  With +-inf the FMA
// form of the slab test, fma(plane, inv, -o * inv), is inf - inf = NaN on that
// axis for every box, min/max ignore the NaN, and a ray parallel to an axis
// plane entered every box that its other two axes cross: a Lambertian sample
// whose normal component is exactly 0 (about one in 2^23) walked up to 44,000
// nodes in the 32x32-chunk scene and held a whole bounce for ms.  With 1e30
// that axis culls as (plane - o) * inf would.  The ray's coordinate on it is
// constant, so a box that can hold a hit face has the origin at least
// BOX_MARGIN - FACE_PAD inside its widened slab there: the distances on that
// axis are beyond +-1e27 and the box is kept (the FMA rounding, about
// |o| * 2^-24, is far below that depth).  A box whose slab lies wholly on one
// side of the origin gets two distances of one sign, beyond +-1e27, and is
// culled.  face_test rejects the faces of such an axis itself, as the true
// inverse (t = +-inf or NaN) would.
__host__ __device__ __forceinline__ float slab_inv(float d) { return d == 0.0f ? copysignf(1e30f, d) : 1.0f / d; }

__host__ __device__ __forceinline__ bool face_test(int bx, int by, int bz, int f, f3 o, f3 d, f3 inv, float tmin,
                                                   float tmax, FaceHit &h) {
    int a, u, v;
    face_axes(f, a, u, v);
    int bc[3] = {bx, by, bz};
    if (cmp3(d, a) == 0.0f) return false;  // parallel to the face: t = +-inf or NaN, no hit
    float c = (float)(bc[a] + (f & 1));
    float t = (c - cmp3(o, a)) * cmp3(inv, a);
    if (!(t >= tmin && t <= tmax)) return false;
    float pu = cmp3(o, u) + t * cmp3(d, u);
    float pv = cmp3(o, v) + t * cmp3(d, v);
    float lu = pu - (float)bc[u];
    float lv = pv - (float)bc[v];
    if (!(lu >= -FACE_PAD && lu <= 1.0f + FACE_PAD && lv >= -FACE_PAD && lv <= 1.0f + FACE_PAD)) return false;
    int half = ((1.0f - lu) - lv >= 0.0f) ? 0 : 1;
    uint32_t c1 = face_corner(f, half, 1), c2 = face_corner(f, half, 2);
    h.t = t;
    h.half = half;
    h.b1 = corner_weight(bitsel(c1, u), bitsel(c1, v), half, lu, lv);
    h.b2 = corner_weight(bitsel(c2, u), bitsel(c2, v), half, lu, lv);
    return true;
}

// Shading frame of (face, half) (localCoordinateSystem, raytrace.rs:319-331).
// The triangle edges are exact small integers, so the frame does not depend
// on the block position; computed once on the host into constant memory.
struct Frame {
    f3 n, t, b;
};
__host__ __device__ inline Frame face_frame(int f, int h) {
    f3 v0 = corner_pos(0, 0, 0, face_corner(f, h, 0));
    f3 v1 = corner_pos(0, 0, 0, face_corner(f, h, 1));
    f3 v2 = corner_pos(0, 0, 0, face_corner(f, h, 2));
    f3 e1 = sub3(v1, v0), e2 = sub3(v2, v0);
    f3 n = cross3(e1, e2);
    f3 bt = cross3(n, e1);
    return Frame{norm3(n), norm3(e1), norm3(bt)};
}

// ---------------------------------------------------------------------
// device scene description (built by vrg_scene_commit)
// ---------------------------------------------------------------------
// Geometry prim record (one per surface block, world space), 16 bytes:
//   x = (wx & 0xFFFF) | wz << 16      (signed 16-bit world block coords)
//   y = (wy & 0xFFFF) | instance << 16
//   z = chunk-local block index (15 bits) | face_mask << 15 | block id << 21
//   w = first triangle index of the block in the chunk's gen_mesh order
// Light record (one per light triangle, scene build only), 16 bytes:
//   x, y as above; z = face | half << 3; w = light BLAS leaf node index
__host__ __device__ __forceinline__ int rec_wx(int4 r) { return (int)(short)(r.x & 0xFFFF); }
__host__ __device__ __forceinline__ int rec_wz(int4 r) { return r.x >> 16; }
__host__ __device__ __forceinline__ int rec_wy(int4 r) { return (int)(short)(r.y & 0xFFFF); }
__host__ __device__ __forceinline__ uint32_t rec_inst(int4 r) { return ((uint32_t)r.y) >> 16; }

// InstDev::flags
constexpr uint32_t INST_MESH = 1u;    // an uploaded triangle mesh (else a voxel chunk)
constexpr uint32_t INST_XFORM = 2u;   // a transform other than a translation

struct InstDev {
    float off[3];                     // the translation (0 with INST_XFORM)
    uint32_t light_bvh_tl_idx;        // prim2node (scene.rs:282-287)
    const vrg_bvh_node *light_bl;     // light BLAS nodes (object space; with INST_XFORM their min and
                                      // max already transformed, the v000 / v111 of nodeImportance)
    const uint32_t *light_leaf_tri;   // per light BLAS node: chunk lx | ly<<5 | lz<<10 | face<<15 | half<<18,
                                      // mesh: its triangle index
    uint32_t flags;                   // INST_*
    uint32_t tri_base;                // mesh: its first world-space triangle record (DevScene::tri_rec)
    const float *uv;                  // mesh: vertex uvs, 6 floats per triangle
};

// The instance transform applied to a point: a translation exactly (p + t),
// any other row-major 3x4 [R|t] as ((r0*x + r1*y) + r2*z) + t per row — the
// mat4x3 * vec4(p, 1) of the reference shaders (raytrace.rs:155-159,184-185).
__host__ __device__ __forceinline__ f3 xf_rows(const float4 &r0, const float4 &r1, const float4 &r2, f3 p) {
    return f3{((r0.x * p.x + r0.y * p.y) + r0.z * p.z) + r0.w, ((r1.x * p.x + r1.y * p.y) + r1.z * p.z) + r1.w,
              ((r2.x * p.x + r2.y * p.y) + r2.z * p.z) + r2.w};
}

// Watertight ray/triangle test (Woop, Benthin, Wald, "Watertight
// Ray/Triangle Intersection", JCGT 2(1), 2013), both faces: the ray's
// dominant axis kz (largest |d| component, the first on ties), the shear,
// the edge functions U, V, W of the sheared vertices (recomputed in double
// when one is exactly 0), a hit iff they do not differ in sign and
// det = U + V + W != 0, t = T / det in [tmin, tmax]; the barycentrics of v1
// and v2 are V / det and W / det.  Vertices sharing an edge give the same
// edge function, so no ray passes between two triangles of a mesh.
struct TriHit {
    float t, b1, b2;
};
__host__ __device__ __forceinline__ bool tri_test(f3 v0, f3 v1, f3 v2, f3 o, f3 d, float tmin, float tmax,
                                                  TriHit &h) {
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > (kz == 0 ? ax : ay)) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1, ky = kx + 1 == 3 ? 0 : kx + 1;
    if (cmp3(d, kz) < 0.0f) {
        const int t = kx;
        kx = ky;
        ky = t;
    }
    const float dz = cmp3(d, kz);
    const float Sx = cmp3(d, kx) / dz, Sy = cmp3(d, ky) / dz, Sz = 1.0f / dz;
    const f3 A = sub3(v0, o), B = sub3(v1, o), C = sub3(v2, o);
    const float Ax = cmp3(A, kx) - Sx * cmp3(A, kz), Ay = cmp3(A, ky) - Sy * cmp3(A, kz);
    const float Bx = cmp3(B, kx) - Sx * cmp3(B, kz), By = cmp3(B, ky) - Sy * cmp3(B, kz);
    const float Cx = cmp3(C, kx) - Sx * cmp3(C, kz), Cy = cmp3(C, ky) - Sy * cmp3(C, kz);
    float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = (U + V) + W;
    if (det == 0.0f) return false;
    const float Az = Sz * cmp3(A, kz), Bz = Sz * cmp3(B, kz), Cz = Sz * cmp3(C, kz);
    const float T = (U * Az + V * Bz) + W * Cz;
    const float t = T / det;
    if (!(t >= tmin && t <= tmax)) return false;
    h.t = t;
    h.b1 = V / det;
    h.b2 = W / det;
    return true;
}

// localCoordinateSystem (raytrace.rs:319-331) of a world-space triangle
__host__ __device__ __forceinline__ Frame tri_frame(f3 v0, f3 v1, f3 v2) {
    const f3 e1 = sub3(v1, v0), e2 = sub3(v2, v0);
    const f3 n = cross3(e1, e2);
    const f3 bt = cross3(n, e1);
    return Frame{norm3(n), norm3(e1), norm3(bt)};
}

// A shading normal carried in one 32-bit word (ray and query .w lanes): a
// voxel face index 0..5, or a mesh normal as bit 31 | three 10-bit snorm
// components (read only as an input feature of the radiance cache)
__host__ __device__ __forceinline__ uint32_t pack_normal10(f3 n) {
    auto q = [](float c) -> uint32_t { return (uint32_t)((int)rintf(fminf(fmaxf(c, -1.0f), 1.0f) * 511.0f) & 1023); };
    return 0x80000000u | q(n.x) | (q(n.y) << 10) | (q(n.z) << 20);
}
__host__ __device__ __forceinline__ f3 unpack_normal10(uint32_t w) {
    auto u = [](uint32_t v) -> float { return (float)((int)(v << 22) >> 22) / 511.0f; };
    return f3{u(w & 1023u), u((w >> 10) & 1023u), u((w >> 20) & 1023u)};
}

struct DevScene {
    const float4 *geo_wide;   // 8 float4 per node: 4-wide child boxes (world, +margin, SoA) and refs
    const int4 *geo_rec;      // records [0, n_blk_rec): surface blocks; [n_blk_rec, ...): mesh triangles
    const float4 *tri_rec;    // world-space mesh triangles, 3 float4 each: (v0, instance) (v1, triangle)
                              // (v2, material slot), .w as u32 bits
    uint32_t n_blk_rec, n_tri_rec;
    int geo_root;             // >=0 wide node, <0 ~record, INT32_MIN empty
    const float4 *lamp_wide;  // any-hit layout over lamp blocks: 8 float4 per node, 4-wide as geo_wide
    const int4 *lamp_rec;     // per lamp block: x/y packed coords + instance, z emissive face mask, w table base
    const uint32_t *lamp_table;  // 12 per lamp block: light-BLAS leaf of (face, half), INVALID if none
    int lamp_root;
    const vrg_bvh_node *light_tl;  // reference-format light TL BVH (dummy node if no light)
    const InstDev *inst;
    const vrg_material *mats;
    uint32_t n_inst;
    // texture atlas (NULL: constant slot colours): [slot][3 maps][h][w] RGBA8,
    // and the sRGB-to-linear table of the 256 byte values
    const uchar4 *atlas;
    const float *srgb;
    uint32_t atlas_w, atlas_h;
};

constexpr int EMPTY_ROOT = (int)0x80000000;
constexpr int TRAV_STACK = 96;
constexpr uint32_t ERR_STACK = 1u;
constexpr uint32_t ERR_LIGHT_LIST = 2u;
constexpr uint32_t ERR_GUARD = 4u;
constexpr uint32_t ERR_COPY = 8u;           // a bulk copy into shared memory did not complete in time
constexpr uint32_t ERR_MMA = 16u;           // a tensor-core MMA group did not complete in time
constexpr uint32_t TRAV_GUARD = 1u << 22;  // iteration bound of every traversal loop

}  // namespace vrg
