// Neural radiance cache (no reference counterpart): a multiresolution hash
// grid encoding (Müller et al. 2022, "Instant Neural Graphics Primitives")
// of the query position plus octahedral normal and view direction, followed
// by a 5 x 64 ReLU MLP with a linear RGB output, trained online on radiance
// the path tracer produces (Müller et al. 2021, "Real-time Neural Radiance
// Caching") with a relative L2 loss and Adam.
//
// GB300 mapping: BF16 weights and activations on the tensor cores, FP32
// accumulate.  Inference encodes one query per thread (many hash-grid gathers
// in flight), then runs the MLP on the 5th-generation tensor cores: tiles of
// 128 queries, tcgen05.mma from shared-memory operands into tensor-memory
// accumulators, one issuing thread per tile, ReLU epilogues from tcgen05.ld.
// Training encodes the samples with the same encoding pass, then runs the
// forward, the loss, the backward through the layers and the hash-grid
// gradient scatter on tcgen05 in the same 128-sample tiles (the backward's B
// operands are the transposed weights).  A warp-level training kernel on mma
// m16n8k16 remains selectable (the activations stay in registers: the f32 C
// fragment of layer l is repacked as the bf16 A fragment of layer l+1 without
// shuffles; the weights are resident in shared memory, row stride padded to
// 72 bf16).  Weight gradients are a split-K tensor-core reduction over the
// batch; Adam runs over FP32 master copies and refreshes the BF16 / FP16
// working copies.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cmath>
#include <cstring>

#include "vrg_internal.h"

namespace vrg {

constexpr int NRC_W = 64;            // hidden width
constexpr int NRC_LAYERS = 6;        // 5 hidden (64) + output (16 padded, 3 used)
constexpr int NRC_OUT = 16;
constexpr int NRC_STRIDE = 72;       // padded bf16 row stride of weights and tiles
constexpr int NRC_TSTRIDE5 = 24;     // padded row stride of the transposed output layer
constexpr int NRC_MAX_LEVELS = 16;

struct NrcParams {
    int levels, log2_t, base_res, features;
    float scale[NRC_MAX_LEVELS];      // per-level resolution
    uint32_t dense[NRC_MAX_LEVELS];   // 1 = dense indexing
    uint32_t res1[NRC_MAX_LEVELS];    // resolution + 1 (dense stride)
    float lo[3], inv_ext[3];          // scene box -> [0,1]^3
};

// weight pack in shared-memory layout (bf16): W_l [out][72], then WT_l [in][72 or 24]
__host__ __device__ constexpr size_t w_off(int l) { return (size_t)l * NRC_W * NRC_STRIDE; }  // l < 5
constexpr size_t W5_OFF = 5 * (size_t)NRC_W * NRC_STRIDE;
constexpr size_t WT_OFF = W5_OFF + (size_t)NRC_OUT * NRC_STRIDE;
__host__ __device__ constexpr size_t wt_off(int l) { return WT_OFF + (size_t)l * NRC_W * NRC_STRIDE; }
constexpr size_t WT5_OFF = WT_OFF + 5 * (size_t)NRC_W * NRC_STRIDE;
constexpr size_t WPACK_ELEMS = WT5_OFF + (size_t)NRC_W * NRC_TSTRIDE5;
constexpr size_t WFWD_ELEMS = WT_OFF;  // forward needs W only
// fp32 master weights: layer l has out(l) x 64
__host__ __device__ constexpr int out_dim(int l) { return l < 5 ? NRC_W : NRC_OUT; }
__host__ __device__ constexpr size_t m_off(int l) { return (size_t)l * NRC_W * NRC_W; }
constexpr size_t MASTER_ELEMS = 5 * (size_t)NRC_W * NRC_W + (size_t)NRC_OUT * NRC_W;

namespace {

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ void mma16816(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16 *p) { return *reinterpret_cast<const uint32_t *>(p); }

// octahedral map of a unit vector to [0,1]^2
__device__ __forceinline__ void oct_encode(f3 v, float &u, float &w) {
    float s = fabsf(v.x) + fabsf(v.y) + fabsf(v.z);
    float px = v.x / s, py = v.y / s;
    if (v.z < 0.0f) {
        float tx = (1.0f - fabsf(py)) * (px >= 0.0f ? 1.0f : -1.0f);
        float ty = (1.0f - fabsf(px)) * (py >= 0.0f ? 1.0f : -1.0f);
        px = tx;
        py = ty;
    }
    u = px * 0.5f + 0.5f;
    w = py * 0.5f + 0.5f;
}

__device__ __forceinline__ uint32_t grid_index(const NrcParams &P, int l, int x, int y, int z) {
    const uint32_t mask = (1u << P.log2_t) - 1u;
    if (P.dense[l]) {
        const uint32_t r = P.res1[l];
        return ((uint32_t)x + (uint32_t)y * r + (uint32_t)z * r * r) & mask;
    }
    return ((uint32_t)x ^ ((uint32_t)y * 2654435761u) ^ ((uint32_t)z * 805459861u)) & mask;
}

struct Corner {
    uint32_t idx[8];
    float w[8];
};

__device__ __forceinline__ void level_corners(const NrcParams &P, int l, f3 p, Corner &c) {
    const float s = P.scale[l];
    const float gx = p.x * s, gy = p.y * s, gz = p.z * s;
    const float fx = floorf(gx), fy = floorf(gy), fz = floorf(gz);
    const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    const float tx = gx - fx, ty = gy - fy, tz = gz - fz;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int dx = (k >> 2) & 1, dy = (k >> 1) & 1, dz = k & 1;
        c.idx[k] = grid_index(P, l, ix + dx, iy + dy, iz + dz);
        c.w[k] = (dx ? tx : 1.0f - tx) * (dy ? ty : 1.0f - ty) * (dz ? tz : 1.0f - tz);
    }
}

__device__ __forceinline__ f3 normalize_pos(const NrcParams &P, f3 x) {
    f3 p = f3{(x.x - P.lo[0]) * P.inv_ext[0], (x.y - P.lo[1]) * P.inv_ext[1], (x.z - P.lo[2]) * P.inv_ext[2]};
    p.x = fminf(fmaxf(p.x, 0.0f), 1.0f);
    p.y = fminf(fmaxf(p.y, 0.0f), 1.0f);
    p.z = fminf(fmaxf(p.z, 0.0f), 1.0f);
    return p;
}

// encodes one query into a bf16 row of 64: 2*levels hash features, oct
// normal, oct view direction, zeros
// The input row as packed bf16 pairs, word k at row32[k * stride]: the levels'
// feature pairs, then the octahedral normal and direction; with FILL the row
// is zero-filled to NRC_W columns.
template <bool FILL = true>
__device__ void encode_row(const NrcParams &P, const __half2 *table, f3 pos, f3 nrm, f3 dir, uint32_t *row32,
                           size_t stride = 1) {
    const f3 p = normalize_pos(P, pos);
    const size_t T = (size_t)1 << P.log2_t;
    // unrolled so that the gathers of several levels are in flight together
#pragma unroll 4
    for (int l = 0; l < P.levels; l++) {
        Corner c;
        level_corners(P, l, p, c);
        float f0 = 0.0f, f1 = 0.0f;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const float2 v = __half22float2(__ldg(table + (size_t)l * T + c.idx[k]));
            f0 += c.w[k] * v.x;
            f1 += c.w[k] * v.y;
        }
        // one 32-bit store per bf16 pair (rows of 144 bytes: 2-byte stores
        // of a warp's 32 rows would meet 8-way bank conflicts)
        row32[l * stride] = pack_bf16(f0, f1);
    }
    float a, b;
    oct_encode(nrm, a, b);
    row32[P.levels * stride] = pack_bf16(a, b);
    oct_encode(dir, a, b);
    row32[(P.levels + 1) * stride] = pack_bf16(a, b);
    if (FILL)
        for (int k = P.levels + 2; k < NRC_W / 2; k++) row32[k * stride] = 0u;
}

// four 8x8 b16 matrices from shared memory (ldmatrix): thread t gives the
// address of row (t & 7) of matrix t >> 3 and receives {M[g][2q], M[g][2q+1]}
// of each — the mma.m16n8k16 A / B fragment layout
__device__ __forceinline__ void ldsm_x4(const __nv_bfloat16 *p, uint32_t &r0, uint32_t &r1, uint32_t &r2,
                                        uint32_t &r3) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(a));
}

// Stages `bytes` (a multiple of 16, 16-byte aligned at both ends) from global
// into shared memory with one bulk copy (cp.async.bulk, completing on an
// mbarrier) issued by thread 0; every thread of the CTA waits for it.  The wait
// is bounded: past the limit the kernel flags ERR_COPY, waits once more
// (bounded) for the copy in flight, and the caller returns.
__device__ __forceinline__ bool stage_bulk(void *dst, const void *src, uint32_t bytes, uint64_t *bar, uint32_t *err) {
    const uint32_t b = (uint32_t)__cvta_generic_to_shared(bar), d = (uint32_t)__cvta_generic_to_shared(dst);
    if ((d & 15u) || ((uintptr_t)src & 15u) || (bytes & 15u)) {  // not a bulk-copy shape: plain copy
        const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
        uint4 *d4 = reinterpret_cast<uint4 *>(dst);
        for (uint32_t i = threadIdx.x; i < bytes / 16; i += blockDim.x) d4[i] = s4[i];
        __syncthreads();
        return true;
    }
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(b) : "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(b), "r"(bytes) : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(d),
                     "l"(src), "r"(bytes), "r"(b)
                     : "memory");
    }
    __syncthreads();
    auto wait = [&](uint32_t limit) {
        for (uint32_t it = 0; it < limit; it++) {
            uint32_t done;
            asm volatile(
                "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
                : "=r"(done)
                : "r"(b)
                : "memory");
            if (done) return true;
        }
        return false;
    };
    if (wait(1u << 22)) return true;
    if (threadIdx.x == 0 && err) atomicOr(err, ERR_COPY);
    wait(1u << 22);
    return false;
}

// A fragments of a 16-row tile held row-major in shared memory (rows of
// NRC_STRIDE bf16, 16-byte aligned): per 16-column chunk kc the matrices
// (rows 0-7, kc), (rows 8-15, kc), (rows 0-7, kc + 8), (rows 8-15, kc + 8)
__device__ __forceinline__ void load_a(const __nv_bfloat16 *tile, int g, int q, uint32_t a[4][4]) {
    const int lane = (g << 2) | q;
    const __nv_bfloat16 *row = tile + ((lane & 7) + ((lane >> 3) & 1) * 8) * NRC_STRIDE + (lane >> 4) * 8;
#pragma unroll
    for (int kc = 0; kc < 4; kc++) ldsm_x4(row + kc * 16, a[kc][0], a[kc][1], a[kc][2], a[kc][3]);
}

// B fragments of n-tile nt of a row-major [out][in] weight block for the
// chunk pair (kc, kc + 1) = (2 kp, 2 kp + 1): b0, b1 of each
__device__ __forceinline__ void load_b2(const __nv_bfloat16 *W, int nt, int kp, int lane, uint32_t &b00, uint32_t &b01,
                                        uint32_t &b10, uint32_t &b11) {
    ldsm_x4(W + (nt * 8 + (lane & 7)) * NRC_STRIDE + kp * 32 + (lane >> 3) * 8, b00, b01, b10, b11);
}

// one 64 -> 64 layer: C = A * W^T
__device__ __forceinline__ void layer64(const __nv_bfloat16 *W, const uint32_t a[4][4], int g, int q, float c[8][4]) {
    const int lane = (g << 2) | q;
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        c[nt][0] = c[nt][1] = c[nt][2] = c[nt][3] = 0.0f;
#pragma unroll
        for (int kp = 0; kp < 2; kp++) {
            uint32_t b00, b01, b10, b11;
            load_b2(W, nt, kp, lane, b00, b01, b10, b11);
            mma16816(c[nt], a[2 * kp], b00, b01);
            mma16816(c[nt], a[2 * kp + 1], b10, b11);
        }
    }
}

// ReLU + bf16 repack of the C fragments as the next layer's A fragments;
// returns the ReLU mask (bit 4*nt + i)
__device__ __forceinline__ uint32_t relu_pack(float c[8][4], uint32_t a[4][4]) {
    uint32_t mask = 0;
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
#pragma unroll
        for (int i = 0; i < 4; i++) {
            if (c[nt][i] > 0.0f) mask |= 1u << (4 * nt + i);
            else c[nt][i] = 0.0f;
        }
#pragma unroll
    for (int kc = 0; kc < 4; kc++) {
        a[kc][0] = pack_bf16(c[2 * kc][0], c[2 * kc][1]);
        a[kc][1] = pack_bf16(c[2 * kc][2], c[2 * kc][3]);
        a[kc][2] = pack_bf16(c[2 * kc + 1][0], c[2 * kc + 1][1]);
        a[kc][3] = pack_bf16(c[2 * kc + 1][2], c[2 * kc + 1][3]);
    }
    return mask;
}

// output layer (16 padded outputs): y[2][4] fragments
__device__ __forceinline__ void layer_out(const __nv_bfloat16 *W5, const uint32_t a[4][4], int g, int q, float y[2][4]) {
    const int lane = (g << 2) | q;
#pragma unroll
    for (int nt = 0; nt < 2; nt++) {
        y[nt][0] = y[nt][1] = y[nt][2] = y[nt][3] = 0.0f;
#pragma unroll
        for (int kp = 0; kp < 2; kp++) {
            uint32_t b00, b01, b10, b11;
            load_b2(W5, nt, kp, lane, b00, b01, b10, b11);
            mma16816(y[nt], a[2 * kp], b00, b01);
            mma16816(y[nt], a[2 * kp + 1], b10, b11);
        }
    }
}

// stores the A fragments of a tile (the bf16 activations) to a [16][64] global block
__device__ __forceinline__ void store_a(__nv_bfloat16 *dst, const uint32_t a[4][4], int g, int q) {
#pragma unroll
    for (int kc = 0; kc < 4; kc++) {
        *reinterpret_cast<uint32_t *>(dst + g * NRC_W + kc * 16 + 2 * q) = a[kc][0];
        *reinterpret_cast<uint32_t *>(dst + (g + 8) * NRC_W + kc * 16 + 2 * q) = a[kc][1];
        *reinterpret_cast<uint32_t *>(dst + g * NRC_W + kc * 16 + 8 + 2 * q) = a[kc][2];
        *reinterpret_cast<uint32_t *>(dst + (g + 8) * NRC_W + kc * 16 + 8 + 2 * q) = a[kc][3];
    }
}

constexpr int NRC_WARPS = 4;   // training kernel (more warps per SM only add contention on the
                               // hash-grid gradient atomics of the coarse levels)

struct InferArgs {
    NrcParams P;
    const __half2 *table;
    const __nv_bfloat16 *wpack;
    uint32_t n;                // capacity (and count when n_dev is NULL)
    const uint32_t *n_dev;     // optional device-side count
    const uint32_t *list;      // optional pixel list (NULL: direct indexing)
    const float4 *pos;         // (x, y, z, face) per pixel / query
    const float4 *dir;
    const float4 *nrm;         // optional explicit normals (NULL: from the face in pos.w)
    float4 *out;               // rgb per pixel / query
    uint32_t *err;             // error word (ERR_COPY)
    uint32_t *enc;             // encoded rows between the two passes: [levels + 2][enc_cap] words
    uint32_t enc_cap;
};

// the normal of a query: a voxel face index 0..5, or a mesh normal packed
// with bit 31 set (pack_normal10)
__device__ __forceinline__ f3 face_normal(int f) {
    if (f < 0) return unpack_normal10((uint32_t)f);
    f3 n = f3{0.0f, 0.0f, 0.0f};
    const float s = (f & 1) ? 1.0f : -1.0f;
    if ((f >> 1) == 0) n.x = s;
    else if ((f >> 1) == 1) n.y = s;
    else n.z = s;
    return n;
}

// Inference, encoding pass: one thread per query, many warps per SM so that
// many queries' hash-grid gathers are in flight (the loop covers any grid).  The packed bf16 input row
// (encode_row, without the zero columns) goes to enc[k * a.enc_cap + i].
__global__ void __launch_bounds__(256) k_nrc_encode(InferArgs a) {
    const uint32_t n = a.n_dev ? min(*a.n_dev, a.n) : a.n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t id = a.list ? a.list[i] : i;
        const float4 pp = a.pos[id], dd = a.dir[id];
        const f3 nrm = a.nrm ? ld3(a.nrm[id]) : face_normal(__float_as_int(pp.w));
        encode_row<false>(a.P, a.table, ld3(pp), nrm, f3{-dd.x, -dd.y, -dd.z}, a.enc + i, a.enc_cap);
    }
}

// ---------------------------------------------------------------------------
// Inference, MLP pass on the 5th-generation tensor cores (tcgen05).  A CTA of
// TC_GROUPS warpgroups; warpgroup g owns a tile of 128 queries:
//   - its input rows, then its activations, in shared memory as bf16 in the
//     canonical K-major layout without swizzle: 8-row x 16-byte core matrices
//     of 128 contiguous bytes, the 8 of a row group's 64 columns side by side
//     (1 KB per 8 rows);
//   - its accumulator in tensor memory: lanes 0-127 (row = query), columns
//     64 g .. 64 g + 63 (FP32).
// Per layer one thread of the group issues four M128 x N64 x K16 MMAs (N16
// for the output layer) and commits them to the group's mbarrier; each thread
// then reads its row of the accumulator (tcgen05.ld), applies ReLU and writes
// the row back as the next layer's bf16 operand.  The weights (42 KB, the same
// layout, out x in) are shared by the groups.  Every wait is bounded: past the
// limit the kernel flags ERR_MMA, waits once more (bounded) for the MMAs in
// flight, and frees its tensor memory before it returns.
// ---------------------------------------------------------------------------
constexpr int TC_GROUPS = 4;
constexpr int TC_THREADS = 128 * TC_GROUPS;
constexpr uint32_t TC_COLS = 64 * TC_GROUPS;                 // tensor-memory columns (a power of 2, >= 32)
constexpr uint32_t TC_LBYTES = (uint32_t)NRC_W * NRC_W * 2;  // one 64 x 64 layer (8 KB)
constexpr uint32_t TC_WBYTES = 5 * TC_LBYTES + (uint32_t)NRC_OUT * NRC_W * 2;
constexpr uint32_t TC_TILE = 128u * NRC_W * 2;               // one group's operand tile (16 KB)
constexpr uint32_t TC_WAIT = 1u << 22;                       // iteration bound of an mbarrier wait

// byte offset of (row r, 8-column group kg) in a K-major tile of 64 columns
__device__ __forceinline__ uint32_t kmaj_off(uint32_t r, uint32_t kg) {
    return (r >> 3) * 1024u + kg * 128u + (r & 7u) * 16u;
}

// shared-memory matrix descriptor: start address, leading byte offset (the
// next core matrix along K: 128 B), stride byte offset (the next 8 rows:
// 1 KB), the fixed 0b001 at bits 46-48, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(1024u >> 4) << 32) |
           (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N and M = 128
__host__ __device__ constexpr uint32_t tc_idesc(uint32_t n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                       uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint32_t limit) {
    for (uint32_t it = 0; it < limit; it++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void group_sync(int grp) {
    asm volatile("bar.sync %0, 128;\n" ::"r"(grp + 1) : "memory");
}

// 32 consecutive FP32 columns of this thread's lane
__device__ __forceinline__ void tc_ld32(uint32_t taddr, uint32_t v[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr)
        : "memory");
}
__device__ __forceinline__ void tc_ld4(uint32_t taddr, uint32_t v[4]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3])
                 : "r"(taddr)
                 : "memory");
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

__device__ __forceinline__ uint32_t relu_bf16x2(uint32_t a, uint32_t b) {
    return pack_bf16(fmaxf(__uint_as_float(a), 0.0f), fmaxf(__uint_as_float(b), 0.0f));
}

__global__ void __launch_bounds__(TC_THREADS, 1) k_nrc_infer_tc(InferArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[TC_GROUPS];
    __shared__ uint32_t tmem_base_s, fail_s[TC_GROUPS];
    const int tid = threadIdx.x, grp = tid >> 7, t = tid & 127, warp = tid >> 5;
    unsigned char *Wc = smem;
    unsigned char *tile = smem + TC_WBYTES + (size_t)grp * TC_TILE;
    const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&bars[grp]);
    // the forward weights (row-major, rows of NRC_STRIDE bf16) into the K-major layout
    for (uint32_t c = tid; c < (5u * NRC_W + NRC_OUT) * 8u; c += TC_THREADS) {
        const uint32_t row = c >> 3, kg = c & 7u;
        const uint32_t l = row < 5u * NRC_W ? row / NRC_W : 5u, n = l < 5u ? row % NRC_W : row - 5u * NRC_W;
        const __nv_bfloat16 *src = a.wpack + (l < 5u ? w_off((int)l) : W5_OFF) + (size_t)n * NRC_STRIDE + kg * 8u;
        *reinterpret_cast<uint4 *>(Wc + l * TC_LBYTES + kmaj_off(n, kg)) = *reinterpret_cast<const uint4 *>(src);
    }
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
        fail_s[grp] = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         (uint32_t)__cvta_generic_to_shared(&tmem_base_s)),
                     "r"(TC_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_s + (uint32_t)grp * 64u;         // this group's columns
    const uint32_t trow = tmem + ((uint32_t)((warp & 3) * 32) << 16);  // this warp's lanes
    const uint32_t n = a.n_dev ? min(*a.n_dev, a.n) : a.n;
    const int words = a.P.levels + 2;
    const uint32_t tiles = (n + 127u) / 128u;
    const uint32_t a_s = (uint32_t)__cvta_generic_to_shared(tile), w_s = (uint32_t)__cvta_generic_to_shared(Wc);
    uint32_t phase = 0;
    bool failed = false;
    for (uint32_t ti = blockIdx.x * TC_GROUPS + grp; ti < tiles && !failed; ti += gridDim.x * TC_GROUPS) {
        const uint32_t i = ti * 128u + (uint32_t)t;
        const uint32_t id = i < n ? (a.list ? a.list[i] : i) : 0u;
#pragma unroll
        for (int kg = 0; kg < 8; kg++) {
            uint32_t w4[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int k = 4 * kg + j;
                w4[j] = (i < n && k < words) ? a.enc[(size_t)k * a.enc_cap + i] : 0u;
            }
            *reinterpret_cast<uint4 *>(tile + kmaj_off((uint32_t)t, (uint32_t)kg)) = make_uint4(w4[0], w4[1], w4[2], w4[3]);
        }
        fence_async_smem();
        tc_fence_before();
        group_sync(grp);
        for (int l = 0; l < NRC_LAYERS && !failed; l++) {
            if (t == 0) {
                tc_fence_after();
                const uint32_t wl = w_s + (uint32_t)l * TC_LBYTES;
                const uint32_t idesc = tc_idesc(l < 5 ? (uint32_t)NRC_W : (uint32_t)NRC_OUT);
#pragma unroll
                for (int s = 0; s < 4; s++)
                    tc_mma(tmem, tc_desc(a_s + 256u * s), tc_desc(wl + 256u * s), idesc, s > 0 ? 1u : 0u);
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
                             : "memory");
            }
            if (!mbar_wait(bar, phase, TC_WAIT)) {
                fail_s[grp] = 1;
                atomicOr(a.err, ERR_MMA);
            }
            __syncwarp();
            tc_fence_after();
            if (l < NRC_LAYERS - 1) {
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    uint32_t v[32];
                    tc_ld32(trow + 32u * h, v);
                    tc_wait_ld();
#pragma unroll
                    for (int g4 = 0; g4 < 4; g4++) {
                        const uint32_t *u = v + 8 * g4;
                        *reinterpret_cast<uint4 *>(tile + kmaj_off((uint32_t)t, (uint32_t)(4 * h + g4))) =
                            make_uint4(relu_bf16x2(u[0], u[1]), relu_bf16x2(u[2], u[3]), relu_bf16x2(u[4], u[5]),
                                       relu_bf16x2(u[6], u[7]));
                    }
                }
                fence_async_smem();
            } else {
                uint32_t v[4];
                tc_ld4(trow, v);
                tc_wait_ld();
                if (i < n) a.out[id] = make_float4(__uint_as_float(v[0]), __uint_as_float(v[1]), __uint_as_float(v[2]), 0.0f);
            }
            tc_fence_before();
            group_sync(grp);
            failed = fail_s[grp] != 0;  // the same for the whole group (read after the barrier)
            if (!failed) phase ^= 1u;
        }
    }
    if (failed && t == 0) mbar_wait(bar, phase, TC_WAIT);  // the MMAs in flight, before their memory is freed
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem_base_s), "r"(TC_COLS)
                     : "memory");
    }
}

struct TrainArgs {
    NrcParams P;
    const __half2 *table;
    const __nv_bfloat16 *wpack;
    uint32_t n;                 // capacity (and batch when n_dev is NULL)
    const uint32_t *n_dev;      // optional device-side batch size
    const uint32_t *list;
    const float4 *pos, *dir, *nrm;  // nrm optional
    const float4 *target;
    __nv_bfloat16 *H;           // [6][n_pad][64] layer inputs (H0 = encoding)
    __nv_bfloat16 *dZ;          // [6][n_pad][64] pre-activation gradients (layer 5: 16 used)
    size_t n_pad;               // rows per layer of H and dZ (the buffers' allocation, >= n)
    float2 *gtable;             // hash-grid gradients (fp32)
    float *loss;                // summed loss
    uint32_t *err;              // error word (ERR_COPY)
    float4 *pred;               // optional: the forward pass's prediction per sample
    const uint32_t *enc;        // tensor-core pass: the encoded input rows (k_nrc_encode layout)
    uint32_t enc_cap;
};

__global__ void __launch_bounds__(NRC_WARPS * 32) k_nrc_train(TrainArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    __nv_bfloat16 *W = reinterpret_cast<__nv_bfloat16 *>(smem);
    __nv_bfloat16 *tiles = W + WPACK_ELEMS;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, g = lane >> 2, q = lane & 3;
    __shared__ __align__(8) uint64_t bar;
    if (!stage_bulk(W, a.wpack, (uint32_t)(WPACK_ELEMS * 2), &bar, a.err)) return;  // weights and transposes
    __nv_bfloat16 *tile = tiles + (size_t)w * 32 * NRC_STRIDE;
    float *ybuf = reinterpret_cast<float *>(tiles + (size_t)NRC_WARPS * 32 * NRC_STRIDE) + (size_t)w * 32 * NRC_OUT;
    const size_t n_pad = a.n_pad;
    const uint32_t warps = gridDim.x * NRC_WARPS;
    const uint32_t n = a.n_dev ? min(*a.n_dev, a.n) : a.n;
    const float inv_n = n ? 1.0f / (float)n : 0.0f;
    float loss_acc = 0.0f;
    for (uint32_t base = (blockIdx.x * NRC_WARPS + w) * 32; base < n; base += warps * 32) {
        const uint32_t i = base + lane;
        uint32_t id = 0;
        f3 pos = f3{0, 0, 0}, nrm = f3{0, 0, 1}, vdir = f3{0, 0, 1};
        float4 tg = make_float4(0, 0, 0, 0);
        if (i < n) {
            id = a.list ? a.list[i] : i;
            const float4 pp = a.pos[id], dd = a.dir[id];
            pos = ld3(pp);
            nrm = a.nrm ? ld3(a.nrm[id]) : face_normal(__float_as_int(pp.w));
            vdir = f3{-dd.x, -dd.y, -dd.z};
            tg = a.target[id];
            encode_row(a.P, a.table, pos, nrm, vdir, reinterpret_cast<uint32_t *>(tile + lane * NRC_STRIDE));
        } else {
            for (int k = 0; k < NRC_W / 2; k++) reinterpret_cast<uint32_t *>(tile + lane * NRC_STRIDE)[k] = 0u;
        }
        __syncwarp();
#pragma unroll 1
        for (int t = 0; t < 2; t++) {
            const size_t row0 = (size_t)base + 16 * t;
            uint32_t act[4][4];
            float c[8][4];
            uint32_t masks[5];
            load_a(tile + t * 16 * NRC_STRIDE, g, q, act);
            store_a(a.H + row0 * NRC_W, act, g, q);
#pragma unroll 1
            for (int l = 0; l < 5; l++) {
                layer64(W + w_off(l), act, g, q, c);
                masks[l] = relu_pack(c, act);
                store_a(a.H + ((size_t)(l + 1) * n_pad + row0) * NRC_W, act, g, q);
            }
            float y[2][4];
            layer_out(W + W5_OFF, act, g, q, y);
            float *yt = ybuf + t * 16 * NRC_OUT;
#pragma unroll
            for (int nt = 0; nt < 2; nt++) {
                yt[g * NRC_OUT + nt * 8 + 2 * q] = y[nt][0];
                yt[g * NRC_OUT + nt * 8 + 2 * q + 1] = y[nt][1];
                yt[(g + 8) * NRC_OUT + nt * 8 + 2 * q] = y[nt][2];
                yt[(g + 8) * NRC_OUT + nt * 8 + 2 * q + 1] = y[nt][3];
            }
            __syncwarp();
            // relative L2 loss (NRC): sum_c (y_c - t_c)^2 / (sg(mean y)^2 + 0.01), mean over the batch
            if (lane >= 16 * t && lane < 16 * t + 16) {
                float *yr = yt + (lane - 16 * t) * NRC_OUT;
                // a non-finite target (the path estimator's 0*inf cases) carries no gradient
                const bool finite_target = isfinite(tg.x) && isfinite(tg.y) && isfinite(tg.z);
                if (a.pred && i < n) a.pred[i] = make_float4(yr[0], yr[1], yr[2], 0.0f);
                if (i < n && finite_target) {
                    const float m = (yr[0] + yr[1] + yr[2]) * (1.0f / 3.0f);
                    const float den = m * m + 0.01f;
                    const float e0 = yr[0] - tg.x, e1 = yr[1] - tg.y, e2 = yr[2] - tg.z;
                    loss_acc += (e0 * e0 + e1 * e1 + e2 * e2) / den * inv_n;
                    yr[0] = 2.0f * e0 / den * inv_n;
                    yr[1] = 2.0f * e1 / den * inv_n;
                    yr[2] = 2.0f * e2 / den * inv_n;
                } else {
                    yr[0] = yr[1] = yr[2] = 0.0f;
                }
                for (int k = 3; k < NRC_OUT; k++) yr[k] = 0.0f;
            }
            __syncwarp();
            // dZ6 (16 wide) as A fragments: one k-chunk
            uint32_t ad[4];
            ad[0] = pack_bf16(yt[g * NRC_OUT + 2 * q], yt[g * NRC_OUT + 2 * q + 1]);
            ad[1] = pack_bf16(yt[(g + 8) * NRC_OUT + 2 * q], yt[(g + 8) * NRC_OUT + 2 * q + 1]);
            ad[2] = pack_bf16(yt[g * NRC_OUT + 8 + 2 * q], yt[g * NRC_OUT + 8 + 2 * q + 1]);
            ad[3] = pack_bf16(yt[(g + 8) * NRC_OUT + 8 + 2 * q], yt[(g + 8) * NRC_OUT + 8 + 2 * q + 1]);
            {
                __nv_bfloat16 *d5 = a.dZ + ((size_t)5 * n_pad + row0) * NRC_W;
                *reinterpret_cast<uint32_t *>(d5 + g * NRC_W + 2 * q) = ad[0];
                *reinterpret_cast<uint32_t *>(d5 + (g + 8) * NRC_W + 2 * q) = ad[1];
                *reinterpret_cast<uint32_t *>(d5 + g * NRC_W + 8 + 2 * q) = ad[2];
                *reinterpret_cast<uint32_t *>(d5 + (g + 8) * NRC_W + 8 + 2 * q) = ad[3];
            }
            // dH5 = dZ6 * W5 (K = 16): b from WT5 [in][24]
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                c[nt][0] = c[nt][1] = c[nt][2] = c[nt][3] = 0.0f;
                const __nv_bfloat16 *wr = W + WT5_OFF + (nt * 8 + g) * NRC_TSTRIDE5;
                mma16816(c[nt], ad, ld32(wr + 2 * q), ld32(wr + 8 + 2 * q));
            }
            // backward through the hidden layers: dZ_l = dH_l * relu'(Z_l), dH_{l-1} = dZ_l * W_{l-1}
#pragma unroll 1
            for (int l = 4; l >= 0; l--) {
                const uint32_t m = masks[l];
#pragma unroll
                for (int nt = 0; nt < 8; nt++)
#pragma unroll
                    for (int k = 0; k < 4; k++)
                        if (!((m >> (4 * nt + k)) & 1u)) c[nt][k] = 0.0f;
                uint32_t dz[4][4];
#pragma unroll
                for (int kc = 0; kc < 4; kc++) {
                    dz[kc][0] = pack_bf16(c[2 * kc][0], c[2 * kc][1]);
                    dz[kc][1] = pack_bf16(c[2 * kc][2], c[2 * kc][3]);
                    dz[kc][2] = pack_bf16(c[2 * kc + 1][0], c[2 * kc + 1][1]);
                    dz[kc][3] = pack_bf16(c[2 * kc + 1][2], c[2 * kc + 1][3]);
                }
                store_a(a.dZ + ((size_t)l * n_pad + row0) * NRC_W, dz, g, q);
                // dH_{l} (input of layer l) = dZ_{l+1} * W_l  (b from WT_l)
#pragma unroll
                for (int nt = 0; nt < 8; nt++) {
                    c[nt][0] = c[nt][1] = c[nt][2] = c[nt][3] = 0.0f;
                    const __nv_bfloat16 *wr = W + wt_off(l) + (nt * 8 + g) * NRC_STRIDE;
#pragma unroll
                    for (int kc = 0; kc < 4; kc++)
                        mma16816(c[nt], dz[kc], ld32(wr + kc * 16 + 2 * q), ld32(wr + kc * 16 + 8 + 2 * q));
                }
            }
            // c now holds dX, the gradient of the encoding; the hash features are
            // columns 0 .. 2*levels-1 (n-tiles 0..3), staged as floats for the scatter
            __syncwarp();
            float *dx = ybuf;  // 16 rows x 32 floats (yt of this tile is no longer needed)
#pragma unroll
            for (int j = 0; j < 4; j++) {
                dx[g * 32 + j * 8 + 2 * q] = c[j][0];
                dx[g * 32 + j * 8 + 2 * q + 1] = c[j][1];
                dx[(g + 8) * 32 + j * 8 + 2 * q] = c[j][2];
                dx[(g + 8) * 32 + j * 8 + 2 * q + 1] = c[j][3];
            }
            __syncwarp();
            if (lane >= 16 * t && lane < 16 * t + 16 && i < n) {
                const float *dr = dx + (lane - 16 * t) * 32;
                const f3 p = normalize_pos(a.P, pos);
                const size_t T = (size_t)1 << a.P.log2_t;
                for (int l = 0; l < a.P.levels; l++) {
                    Corner cr;
                    level_corners(a.P, l, p, cr);
                    const float g0 = dr[2 * l], g1 = dr[2 * l + 1];
#pragma unroll
                    for (int k = 0; k < 8; k++)
                        atomicAdd(&a.gtable[(size_t)l * T + cr.idx[k]], make_float2(cr.w[k] * g0, cr.w[k] * g1));
                }
            }
            __syncwarp();
        }
    }
    for (int o = 16; o; o >>= 1) loss_acc += __shfl_xor_sync(0xffffffffu, loss_acc, o);
    if (lane == 0 && loss_acc != 0.0f) atomicAdd(a.loss, loss_acc);
}

// ---------------------------------------------------------------------------
// Training on the 5th-generation tensor cores (tcgen05), the layout of the
// inference pass: a CTA of TC_GROUPS warpgroups, each owning a tile of 128
// samples (thread t of the group = sample row t), the tile's operand in shared
// memory (K-major, no swizzle), its accumulator in tensor memory (64 FP32
// columns per group).  Per tile:
//   - forward: the encoded rows (k_nrc_encode) through the five hidden layers
//     and the output layer, one M128 x N64 (N16) MMA group per layer; each
//     thread keeps its row's ReLU mask per layer (64 bits) and stores the
//     layer inputs H_l to global memory for the weight gradients;
//   - loss: the relative L2 loss of its sample and dY (the output layer's dZ);
//   - backward: dH_l = dZ_l * W_l, one MMA group per layer with the
//     transposed weights (in x out, K-major) as the B operand; dZ_l = dH_{l+1}
//     masked by the layer's ReLU; the dZ_l are stored for the weight
//     gradients (k_nrc_dw);
//   - the input gradient's hash-feature columns scattered into the table
//     gradient (atomics), as the warp-level kernel does.
// Every wait is bounded (ERR_MMA), and tensor memory is freed before return.
// ---------------------------------------------------------------------------
constexpr uint32_t TCT_WTBYTES = 6 * TC_LBYTES;  // WT_l (in x out) for l < 5, WT5 (in x 16) in a 64-column slot

__device__ __forceinline__ void st_row_bf16(__nv_bfloat16 *dst, const uint32_t w[32]) {
    uint4 *d = reinterpret_cast<uint4 *>(dst);
#pragma unroll
    for (int j = 0; j < 8; j++) d[j] = make_uint4(w[4 * j], w[4 * j + 1], w[4 * j + 2], w[4 * j + 3]);
}

__global__ void __launch_bounds__(TC_THREADS, 1) k_nrc_train_tc(TrainArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[TC_GROUPS];
    __shared__ uint32_t tmem_base_s, fail_s[TC_GROUPS];
    const int tid = threadIdx.x, grp = tid >> 7, t = tid & 127, warp = tid >> 5, lane = tid & 31;
    unsigned char *Wc = smem, *WTc = smem + TC_WBYTES;
    unsigned char *tile = smem + TC_WBYTES + TCT_WTBYTES + (size_t)grp * TC_TILE;
    const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&bars[grp]);
    // forward weights W_l (out x in) and backward weights WT_l (in x out) into the K-major layout
    for (uint32_t c = tid; c < (5u * NRC_W + NRC_OUT) * 8u; c += TC_THREADS) {
        const uint32_t row = c >> 3, kg = c & 7u;
        const uint32_t l = row < 5u * NRC_W ? row / NRC_W : 5u, n = l < 5u ? row % NRC_W : row - 5u * NRC_W;
        const __nv_bfloat16 *src = a.wpack + (l < 5u ? w_off((int)l) : W5_OFF) + (size_t)n * NRC_STRIDE + kg * 8u;
        *reinterpret_cast<uint4 *>(Wc + l * TC_LBYTES + kmaj_off(n, kg)) = *reinterpret_cast<const uint4 *>(src);
    }
    for (uint32_t c = tid; c < 6u * NRC_W * 8u; c += TC_THREADS) {
        const uint32_t l = c / (NRC_W * 8u), n = (c / 8u) % NRC_W, kg = c & 7u;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (l < 5u)
            v = *reinterpret_cast<const uint4 *>(a.wpack + wt_off((int)l) + (size_t)n * NRC_STRIDE + kg * 8u);
        else if (kg < 2u)  // WT5: in x 16 (rows of NRC_TSTRIDE5)
            v = *reinterpret_cast<const uint4 *>(a.wpack + WT5_OFF + (size_t)n * NRC_TSTRIDE5 + kg * 8u);
        *reinterpret_cast<uint4 *>(WTc + l * TC_LBYTES + kmaj_off(n, kg)) = v;
    }
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
        fail_s[grp] = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         (uint32_t)__cvta_generic_to_shared(&tmem_base_s)),
                     "r"(TC_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_s + (uint32_t)grp * 64u;
    const uint32_t trow = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    const uint32_t n = a.n_dev ? min(*a.n_dev, a.n) : a.n;
    const float inv_n = n ? 1.0f / (float)n : 0.0f;
    const int words = a.P.levels + 2;
    const uint32_t tiles = (n + 127u) / 128u;
    const size_t n_pad = a.n_pad;
    const uint32_t a_s = (uint32_t)__cvta_generic_to_shared(tile), w_s = (uint32_t)__cvta_generic_to_shared(Wc),
                   wt_s = (uint32_t)__cvta_generic_to_shared(WTc);
    uint32_t phase = 0;
    bool failed = false;
    float loss_acc = 0.0f;
    // one MMA group (n_k K16 steps into this group's columns), then the wait
    auto mma_round = [&](uint32_t b_base, uint32_t nn, int n_k) {
        if (t == 0) {
            tc_fence_after();
            const uint32_t idesc = tc_idesc(nn);
            for (int s = 0; s < n_k; s++)
                tc_mma(tmem, tc_desc(a_s + 256u * s), tc_desc(b_base + 256u * s), idesc, s > 0 ? 1u : 0u);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
                         : "memory");
        }
        if (mbar_wait(bar, phase, TC_WAIT)) {
            phase ^= 1u;  // each commit completes one phase
        } else {
            fail_s[grp] = 1;
            atomicOr(a.err, ERR_MMA);
        }
        __syncwarp();
        tc_fence_after();
    };
    // the tile rewritten (and the accumulator read) before the next MMA group
    auto round_end = [&]() {
        fence_async_smem();
        tc_fence_before();
        group_sync(grp);
        failed = fail_s[grp] != 0;
    };
    for (uint32_t ti = blockIdx.x * TC_GROUPS + grp; ti < tiles && !failed; ti += gridDim.x * TC_GROUPS) {
        const uint32_t i = ti * 128u + (uint32_t)t;
        const bool live = i < n;
        const uint32_t id = live ? (a.list ? a.list[i] : i) : 0u;
        {  // H_0: the encoded row
            uint32_t w[32];
#pragma unroll
            for (int k = 0; k < 32; k++) w[k] = (live && k < words) ? a.enc[(size_t)k * a.enc_cap + i] : 0u;
#pragma unroll
            for (int kg = 0; kg < 8; kg++)
                *reinterpret_cast<uint4 *>(tile + kmaj_off((uint32_t)t, (uint32_t)kg)) =
                    make_uint4(w[4 * kg], w[4 * kg + 1], w[4 * kg + 2], w[4 * kg + 3]);
            if (live) st_row_bf16(a.H + (size_t)i * NRC_W, w);
        }
        round_end();
        if (failed) break;
        uint32_t mask[5][2];
        // forward through the hidden layers
        for (int l = 0; l < 5 && !failed; l++) {
            mma_round(w_s + (uint32_t)l * TC_LBYTES, NRC_W, 4);
            uint32_t w[32];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                uint32_t v[32];
                tc_ld32(trow + 32u * h, v);
                tc_wait_ld();
                uint32_t m = 0;
#pragma unroll
                for (int k = 0; k < 32; k++) {
                    float z = __uint_as_float(v[k]);
                    if (z > 0.0f) m |= 1u << k;
                    else z = 0.0f;
                    v[k] = __float_as_uint(z);
                }
                mask[l][h] = m;
#pragma unroll
                for (int k = 0; k < 16; k++) w[16 * h + k] = pack_bf16(__uint_as_float(v[2 * k]), __uint_as_float(v[2 * k + 1]));
            }
#pragma unroll
            for (int kg = 0; kg < 8; kg++)
                *reinterpret_cast<uint4 *>(tile + kmaj_off((uint32_t)t, (uint32_t)kg)) =
                    make_uint4(w[4 * kg], w[4 * kg + 1], w[4 * kg + 2], w[4 * kg + 3]);
            if (live) st_row_bf16(a.H + ((size_t)(l + 1) * n_pad + i) * NRC_W, w);
            round_end();
        }
        if (failed) break;
        // output layer, loss and dY
        mma_round(w_s + 5u * TC_LBYTES, NRC_OUT, 4);
        {
            uint32_t v[4];
            tc_ld4(trow, v);
            tc_wait_ld();
            const float y0 = __uint_as_float(v[0]), y1 = __uint_as_float(v[1]), y2 = __uint_as_float(v[2]);
            float d0 = 0.0f, d1 = 0.0f, d2 = 0.0f;
            if (live) {
                if (a.pred) a.pred[i] = make_float4(y0, y1, y2, 0.0f);
                const float4 tg = a.target[id];
                // a non-finite target (the path estimator's 0*inf cases) carries no gradient
                if (isfinite(tg.x) && isfinite(tg.y) && isfinite(tg.z)) {
                    const float m = (y0 + y1 + y2) * (1.0f / 3.0f);
                    const float den = m * m + 0.01f;
                    const float e0 = y0 - tg.x, e1 = y1 - tg.y, e2 = y2 - tg.z;
                    loss_acc += (e0 * e0 + e1 * e1 + e2 * e2) / den * inv_n;
                    d0 = 2.0f * e0 / den * inv_n;
                    d1 = 2.0f * e1 / den * inv_n;
                    d2 = 2.0f * e2 / den * inv_n;
                }
            }
            // dZ6 (16 columns, 3 used) as the A operand of dH5 = dZ6 * W5 (K = 16)
            const uint4 q0 = make_uint4(pack_bf16(d0, d1), pack_bf16(d2, 0.0f), 0u, 0u), q1 = make_uint4(0, 0, 0, 0);
            *reinterpret_cast<uint4 *>(tile + kmaj_off((uint32_t)t, 0u)) = q0;
            *reinterpret_cast<uint4 *>(tile + kmaj_off((uint32_t)t, 1u)) = q1;
            if (live) {
                uint4 *d5 = reinterpret_cast<uint4 *>(a.dZ + ((size_t)5 * n_pad + i) * NRC_W);
                d5[0] = q0;
                d5[1] = q1;
            }
        }
        round_end();
        if (failed) break;
        // backward: dH5 = dZ6 * W5, then dZ_l = dH_{l+1} * relu'(Z_l), dH_l = dZ_l * W_l
        mma_round(wt_s + 5u * TC_LBYTES, NRC_W, 1);
        for (int l = 4; l >= 0 && !failed; l--) {
            uint32_t w[32];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                uint32_t v[32];
                tc_ld32(trow + 32u * h, v);
                tc_wait_ld();
                const uint32_t m = mask[l][h];
#pragma unroll
                for (int k = 0; k < 16; k++) {
                    const float g0 = ((m >> (2 * k)) & 1u) ? __uint_as_float(v[2 * k]) : 0.0f;
                    const float g1 = ((m >> (2 * k + 1)) & 1u) ? __uint_as_float(v[2 * k + 1]) : 0.0f;
                    w[16 * h + k] = pack_bf16(g0, g1);
                }
            }
#pragma unroll
            for (int kg = 0; kg < 8; kg++)
                *reinterpret_cast<uint4 *>(tile + kmaj_off((uint32_t)t, (uint32_t)kg)) =
                    make_uint4(w[4 * kg], w[4 * kg + 1], w[4 * kg + 2], w[4 * kg + 3]);
            if (live) st_row_bf16(a.dZ + ((size_t)l * n_pad + i) * NRC_W, w);
            round_end();
            if (failed) break;
            mma_round(wt_s + (uint32_t)l * TC_LBYTES, NRC_W, 4);
        }
        if (failed) break;
        // dX: the hash features' gradients into the table gradient
        {
            uint32_t v[32];
            tc_ld32(trow, v);
            tc_wait_ld();
            if (live) {
                const f3 p = normalize_pos(a.P, ld3(a.pos[id]));
                const size_t T = (size_t)1 << a.P.log2_t;
                for (int l = 0; l < a.P.levels; l++) {
                    Corner cr;
                    level_corners(a.P, l, p, cr);
                    const float g0 = __uint_as_float(v[2 * l]), g1 = __uint_as_float(v[2 * l + 1]);
#pragma unroll
                    for (int k = 0; k < 8; k++)
                        atomicAdd(&a.gtable[(size_t)l * T + cr.idx[k]], make_float2(cr.w[k] * g0, cr.w[k] * g1));
                }
            }
        }
        tc_fence_before();
        group_sync(grp);
    }
    for (int o = 16; o; o >>= 1) loss_acc += __shfl_xor_sync(0xffffffffu, loss_acc, o);
    if (lane == 0 && loss_acc != 0.0f) atomicAdd(a.loss, loss_acc);
    if (failed && t == 0) mbar_wait(bar, phase, TC_WAIT);  // the MMAs in flight, before their memory is freed
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem_base_s), "r"(TC_COLS)
                     : "memory");
    }
}

// 8x8 b16 matrices from shared memory, transposed (ldmatrix .trans): thread t
// gives the address of row (t & 7) of matrix t >> 3 and receives
// {M[2q][g], M[2q+1][g]} of each of the four matrices
__device__ __forceinline__ void ldsm_x4_t(const __nv_bfloat16 *p, uint32_t &r0, uint32_t &r1, uint32_t &r2,
                                          uint32_t &r3) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(a));
}

constexpr int DW_CHUNK = 64;  // samples staged per step

// dW_l[n][k] += sum_b dZ_l[b][n] * H_l[b][k]: split-K over the batch (a CTA per
// rows_per_cta samples of one layer, staged DW_CHUNK at a time for all its
// warps), one warp per 16-row block of n, atomics into the fp32 gradient

__global__ void __launch_bounds__(128) k_nrc_dw(const __nv_bfloat16 *H, const __nv_bfloat16 *dZ, size_t n_pad,
                                                uint32_t n_cap, const uint32_t *n_dev, float *dW,
                                                uint32_t rows_per_cta) {
    const int l = blockIdx.y;
    const uint32_t n = n_dev ? min(*n_dev, n_cap) : n_cap;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, g = lane >> 2, q = lane & 3;
    const int mdim = out_dim(l);
    const bool active = w * 16 < mdim;  // the 16-wide output layer uses warp 0 only
    // dZ and H of DW_CHUNK samples, staged once per CTA (row stride 72 bf16:
    // 16-byte aligned rows for ldmatrix)
    __shared__ __align__(16) __nv_bfloat16 sz[DW_CHUNK][NRC_STRIDE];
    __shared__ __align__(16) __nv_bfloat16 sh[DW_CHUNK][NRC_STRIDE];
    const __nv_bfloat16 *Hl = H + (size_t)l * n_pad * NRC_W;
    const __nv_bfloat16 *Zl = dZ + (size_t)l * n_pad * NRC_W;
    float acc[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
    const size_t r0 = (size_t)blockIdx.x * rows_per_cta;
    if (r0 >= n) return;  // uniform over the CTA
    const size_t r1 = min((size_t)n, r0 + rows_per_cta);
    const int m0 = w * 16;
    // per-thread ldmatrix row / column selectors (see ldsm_x4_t)
    const int a_row = (lane & 7) + ((lane >> 4) << 3), a_col = ((lane >> 3) & 1) * 8;
    const int b_row = (lane & 7) + (((lane >> 3) & 1) << 3), b_col = (lane >> 4) * 8;
    for (size_t s0 = r0; s0 < r1; s0 += DW_CHUNK) {
        for (int e = threadIdx.x; e < DW_CHUNK * 8; e += blockDim.x) {
            const int r = e >> 3, cc = (e & 7) * 8;
            const size_t row = s0 + r;
            uint4 vz = make_uint4(0, 0, 0, 0), vh = make_uint4(0, 0, 0, 0);
            if (row < r1) {
                vz = *reinterpret_cast<const uint4 *>(Zl + row * NRC_W + cc);
                vh = *reinterpret_cast<const uint4 *>(Hl + row * NRC_W + cc);
            }
            *reinterpret_cast<uint4 *>(&sz[r][cc]) = vz;
            *reinterpret_cast<uint4 *>(&sh[r][cc]) = vh;
        }
        __syncthreads();
        if (active) {
            // A[m = output][k = sample] = dZ[sample][m0 + m]; B[k = sample][n = input] = H[sample][n]
#pragma unroll
            for (int kk = 0; kk < DW_CHUNK / 16; kk++) {
                uint32_t af[4];
                ldsm_x4_t(&sz[kk * 16 + a_row][m0 + a_col], af[0], af[1], af[2], af[3]);
#pragma unroll
                for (int ntp = 0; ntp < 4; ntp++) {
                    uint32_t b00, b01, b10, b11;
                    ldsm_x4_t(&sh[kk * 16 + b_row][ntp * 16 + b_col], b00, b01, b10, b11);
                    mma16816(acc[2 * ntp], af, b00, b01);
                    mma16816(acc[2 * ntp + 1], af, b10, b11);
                }
            }
        }
        __syncthreads();
    }
    if (!active) return;
    float *dWl = dW + m_off(l);
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const int m = w * 16 + g, k = nt * 8 + 2 * q;
        atomicAdd(&dWl[m * NRC_W + k], acc[nt][0]);
        atomicAdd(&dWl[m * NRC_W + k + 1], acc[nt][1]);
        atomicAdd(&dWl[(m + 8) * NRC_W + k], acc[nt][2]);
        atomicAdd(&dWl[(m + 8) * NRC_W + k + 1], acc[nt][3]);
    }
}

struct AdamArgs {
    float lr, b1, b2, eps, c1, c2;  // c1 = 1/(1-b1^t), c2 = 1/(1-b2^t)
};

__global__ void k_adam_weights(float *master, float *m, float *v, float *grad, AdamArgs A) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= MASTER_ELEMS) return;
    // the padded output rows 3..15 stay zero
    if (i >= 5 * (size_t)NRC_W * NRC_W && (i - 5 * (size_t)NRC_W * NRC_W) / NRC_W >= 3) {
        grad[i] = 0.0f;
        return;
    }
    const float gr = grad[i];
    const float mi = A.b1 * m[i] + (1.0f - A.b1) * gr;
    const float vi = A.b2 * v[i] + (1.0f - A.b2) * gr * gr;
    m[i] = mi;
    v[i] = vi;
    master[i] -= A.lr * (mi * A.c1) / (sqrtf(vi * A.c2) + A.eps);
    grad[i] = 0.0f;
}

// master weights -> bf16 pack (W and W^T in the padded shared-memory layout)
__global__ void k_pack_weights(const float *master, __nv_bfloat16 *pack) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= WPACK_ELEMS) return;
    float v = 0.0f;
    if (i < W5_OFF) {
        const int l = (int)(i / (NRC_W * NRC_STRIDE)), r = (int)(i % (NRC_W * NRC_STRIDE));
        const int o = r / NRC_STRIDE, k = r % NRC_STRIDE;
        if (k < NRC_W) v = master[m_off(l) + o * NRC_W + k];
    } else if (i < WT_OFF) {
        const int r = (int)(i - W5_OFF), o = r / NRC_STRIDE, k = r % NRC_STRIDE;
        if (k < NRC_W) v = master[m_off(5) + o * NRC_W + k];
    } else if (i < WT5_OFF) {
        const int r = (int)(i - WT_OFF), l = r / (NRC_W * NRC_STRIDE), rr = r % (NRC_W * NRC_STRIDE);
        const int k = rr / NRC_STRIDE, o = rr % NRC_STRIDE;
        if (o < NRC_W) v = master[m_off(l) + o * NRC_W + k];
    } else {
        const int r = (int)(i - WT5_OFF), k = r / NRC_TSTRIDE5, o = r % NRC_TSTRIDE5;
        if (o < NRC_OUT) v = master[m_off(5) + o * NRC_W + k];
    }
    pack[i] = __float2bfloat16_rn(v);
}

__global__ void k_adam_table(float2 *master, float2 *m, float2 *v, float2 *grad, __half2 *table, size_t n,
                             AdamArgs A) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 gr = grad[i];
    if (gr.x == 0.0f && gr.y == 0.0f) return;  // untouched entries keep their moments
    float2 mi = m[i], vi = v[i], p = master[i];
    mi.x = A.b1 * mi.x + (1.0f - A.b1) * gr.x;
    mi.y = A.b1 * mi.y + (1.0f - A.b1) * gr.y;
    vi.x = A.b2 * vi.x + (1.0f - A.b2) * gr.x * gr.x;
    vi.y = A.b2 * vi.y + (1.0f - A.b2) * gr.y * gr.y;
    p.x -= A.lr * (mi.x * A.c1) / (sqrtf(vi.x * A.c2) + A.eps);
    p.y -= A.lr * (mi.y * A.c1) / (sqrtf(vi.y * A.c2) + A.eps);
    m[i] = mi;
    v[i] = vi;
    master[i] = p;
    table[i] = __floats2half2_rn(p.x, p.y);
    grad[i] = make_float2(0.0f, 0.0f);
}

__global__ void k_init_table(float2 *master, __half2 *table, size_t n, uint64_t seed) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    auto u = [&](uint64_t k) {
        uint64_t x = seed ^ (k * 0x9E3779B97F4A7C15ull);
        x ^= x >> 31; x *= 0x7fb5d329728ea185ull; x ^= x >> 27; x *= 0x81dadef4bc2dd44dull; x ^= x >> 33;
        return (float)((x >> 40) * (1.0 / 16777216.0)) * 2.0f - 1.0f;
    };
    const float2 p = make_float2(1e-4f * u(2 * i), 1e-4f * u(2 * i + 1));
    master[i] = p;
    table[i] = __floats2half2_rn(p.x, p.y);
}

}  // namespace

// ------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------
struct Nrc {
    Context *ctx = nullptr;
    vrg_nrc_desc desc{};
    NrcParams P{};
    size_t T = 0, table_entries = 0;
    DevBufPtr buf;
    float2 *t_master = nullptr, *t_m = nullptr, *t_v = nullptr, *t_grad = nullptr;
    __half2 *table = nullptr;
    float *w_master = nullptr, *w_m = nullptr, *w_v = nullptr, *w_grad = nullptr;
    __nv_bfloat16 *wpack = nullptr;
    float *loss = nullptr;
    uint32_t *err = nullptr;  // error word of the host-array entry points
    DevBufPtr act;  // training activations
    size_t act_rows = 0;
    __nv_bfloat16 *H = nullptr, *dZ = nullptr;
    uint32_t step = 0;
    int grid_train = 0, grid_tc = 0, grid_train_tc = 0;
    bool train_tc = true;             // training on tcgen05 (false: the warp-level mma.sync kernel)
    DevBufPtr train_enc_buf;          // the training samples' encoded rows (own buffer: training
    size_t train_enc_cap = 0;         // runs beside inference in a cache frame)
    DevBufPtr enc_buf;  // encoded query rows of inference
    size_t enc_cap = 0;
    DevBufPtr pred_buf;  // the last host-array training batch's predictions
    uint32_t pred_n = 0, pred_cap = 0;
    cudaEvent_t ev_alloc = nullptr;  // orders a grown buffer between the context stream and its user
    // a cache frame's gradients wait for their Adam step, which the next user
    // of the cache runs first (a cache frame: beside its own bounces)
    bool pending = false;
};

static size_t tc_smem() { return (size_t)TC_WBYTES + (size_t)TC_GROUPS * TC_TILE; }
static size_t train_tc_smem() { return (size_t)TC_WBYTES + TCT_WTBYTES + (size_t)TC_GROUPS * TC_TILE; }
static size_t train_smem() {
    return WPACK_ELEMS * 2 + (size_t)NRC_WARPS * 32 * NRC_STRIDE * 2 + (size_t)NRC_WARPS * 32 * NRC_OUT * 4;
}

vrg_status nrc_set_bounds(Nrc *N, const float lo[3], const float hi[3]) {
    for (int k = 0; k < 3; k++) {
        N->P.lo[k] = lo[k];
        float e = hi[k] - lo[k];
        N->P.inv_ext[k] = e > 0.0f ? 1.0f / e : 1.0f;
    }
    return VRG_OK;
}

vrg_status nrc_create(Context *ctx, const vrg_nrc_desc *d, Nrc **out) {
    Nrc *N = new Nrc();
    N->ctx = ctx;
    N->desc = *d;
    NrcParams &P = N->P;
    P.levels = (int)d->levels;
    P.log2_t = (int)d->log2_table;
    P.base_res = (int)d->base_resolution;
    P.features = 2;
    if (P.levels < 1 || P.levels > NRC_MAX_LEVELS || 2 * P.levels + 4 > NRC_W || P.log2_t < 4 || P.log2_t > 24 ||
        d->features != 2) {
        delete N;
        set_error("nrc: levels 1..16, log2_table 4..24, features 2");
        return VRG_ERR_INVALID_ARGUMENT;
    }
    // every CTA of the tensor-memory inference kernel that fits on an SM
    // must get its columns (512 per SM), or its allocation would wait
    int bc = 0;
    if (cudaFuncSetAttribute(k_nrc_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem()) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bc, k_nrc_infer_tc, TC_THREADS, tc_smem()) != cudaSuccess ||
        bc < 1 || (uint32_t)bc * TC_COLS > 512u) {
        delete N;
        set_error("radiance cache: %d tensor-core inference CTAs per SM, %u tensor-memory columns each", bc, TC_COLS);
        return VRG_ERR_UNSUPPORTED;
    }
    N->grid_tc = ctx->num_sms * bc;
    // the tensor-memory training kernel likewise, also beside inference CTAs
    // when both fit on an SM
    int bt_tc = 0, smem_sm = 0;
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx->device);
    if (cudaFuncSetAttribute(k_nrc_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_tc_smem()) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bt_tc, k_nrc_train_tc, TC_THREADS, train_tc_smem()) !=
            cudaSuccess ||
        bt_tc < 1 || (uint32_t)bt_tc * TC_COLS > 512u ||
        (tc_smem() + train_tc_smem() <= (size_t)smem_sm && (uint32_t)(bc + bt_tc) * TC_COLS > 512u)) {
        delete N;
        set_error("radiance cache: %d tensor-core training CTAs per SM, %u tensor-memory columns each", bt_tc, TC_COLS);
        return VRG_ERR_UNSUPPORTED;
    }
    N->grid_train_tc = ctx->num_sms * bt_tc;
    N->train_tc = (d->flags & VRG_NRC_TRAIN_WARP_MMA) == 0;
    N->T = (size_t)1 << P.log2_t;
    const double b = P.levels > 1 ? std::exp((std::log((double)d->max_resolution) - std::log((double)d->base_resolution)) /
                                             (double)(P.levels - 1))
                                  : 1.0;
    for (int l = 0; l < P.levels; l++) {
        const double res = std::floor((double)d->base_resolution * std::pow(b, (double)l));
        P.scale[l] = (float)res;
        const double cells = (res + 1.0) * (res + 1.0) * (res + 1.0);
        P.dense[l] = cells <= (double)N->T ? 1u : 0u;
        P.res1[l] = (uint32_t)(res + 1.0);
    }
    nrc_set_bounds(N, d->scene_min, d->scene_max);
    N->table_entries = N->T * (size_t)P.levels;
    const size_t te = N->table_entries;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    size_t o = 0;
    size_t o_tm = o; o += al(te * 8);
    size_t o_t1 = o; o += al(te * 8);
    size_t o_t2 = o; o += al(te * 8);
    size_t o_tg = o; o += al(te * 8);
    size_t o_th = o; o += al(te * 4);
    size_t o_wm = o; o += al(MASTER_ELEMS * 4);
    size_t o_w1 = o; o += al(MASTER_ELEMS * 4);
    size_t o_w2 = o; o += al(MASTER_ELEMS * 4);
    size_t o_wg = o; o += al(MASTER_ELEMS * 4);
    size_t o_wp = o; o += al(WPACK_ELEMS * 2);
    size_t o_ls = o; o += 256;
    cudaStream_t s = ctx->stream;
    vrg_status st = dev_alloc(s, o, N->buf);
    if (st != VRG_OK) {
        delete N;
        return st;
    }
    if (cudaEventCreateWithFlags(&N->ev_alloc, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        N->ev_alloc = nullptr;
        delete N;
        set_error("cudaEventCreateWithFlags failed");
        return VRG_ERR_CUDA;
    }
    uint8_t *B = (uint8_t *)N->buf->ptr;
    N->t_master = (float2 *)(B + o_tm);
    N->t_m = (float2 *)(B + o_t1);
    N->t_v = (float2 *)(B + o_t2);
    N->t_grad = (float2 *)(B + o_tg);
    N->table = (__half2 *)(B + o_th);
    N->w_master = (float *)(B + o_wm);
    N->w_m = (float *)(B + o_w1);
    N->w_v = (float *)(B + o_w2);
    N->w_grad = (float *)(B + o_wg);
    N->wpack = (__nv_bfloat16 *)(B + o_wp);
    N->loss = (float *)(B + o_ls);
    N->err = (uint32_t *)(B + o_ls + 4);
    VRG_CUDA_TRY(cudaMemsetAsync(B, 0, o, s));
    k_init_table<<<(uint32_t)((te + 255) / 256), 256, 0, s>>>(N->t_master, N->table, te, d->seed ^ 0x7ab1eull);
    // He-uniform hidden layers, Xavier-uniform output layer (rows 0..2)
    std::vector<float> wm(MASTER_ELEMS, 0.0f);
    uint64_t x = d->seed * 0x9E3779B97F4A7C15ull + 1;
    auto rnd = [&]() {
        x ^= x << 13; x ^= x >> 7; x ^= x << 17;
        return (float)((x >> 40) * (1.0 / 16777216.0)) * 2.0f - 1.0f;
    };
    for (int l = 0; l < 5; l++) {
        const float a = std::sqrt(6.0f / (float)NRC_W);
        for (int i = 0; i < NRC_W * NRC_W; i++) wm[m_off(l) + i] = a * rnd();
    }
    const float a5 = std::sqrt(6.0f / (float)(NRC_W + 3));
    for (int o5 = 0; o5 < 3; o5++)
        for (int k = 0; k < NRC_W; k++) wm[m_off(5) + o5 * NRC_W + k] = a5 * rnd();
    VRG_CUDA_TRY(cudaMemcpyAsync(N->w_master, wm.data(), MASTER_ELEMS * 4, cudaMemcpyHostToDevice, s));
    k_pack_weights<<<(uint32_t)((WPACK_ELEMS + 255) / 256), 256, 0, s>>>(N->w_master, N->wpack);
    VRG_CUDA_TRY(cudaGetLastError());
    VRG_CUDA_TRY(cudaFuncSetAttribute(k_nrc_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem()));
    int bt = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bt, k_nrc_train, NRC_WARPS * 32, train_smem());
    N->grid_train = std::max(1, ctx->num_sms * std::max(1, bt));

    VRG_CUDA_TRY(cudaStreamSynchronize(s));
    ctx_retain(ctx);  // dropped by nrc_destroy
    *out = N;
    return VRG_OK;
}

// Grows one of the cache's scratch buffers for use on stream s.  The buffer
// lives on the context's stream, not on s: a cache frame trains on a
// renderer's stream, and the renderer (with its streams) may be destroyed
// before the cache frees the buffer.  The context stream frees the buffer
// being replaced after s's earlier work (its last reader) and s waits for the
// new allocation (and its zero fill, when asked).
static vrg_status cache_alloc(Nrc *N, cudaStream_t s, size_t bytes, bool zero, DevBufPtr &buf) {
    cudaStream_t cs = N->ctx->stream;
    if (s != cs) {
        VRG_CUDA_TRY(cudaEventRecord(N->ev_alloc, s));
        VRG_CUDA_TRY(cudaStreamWaitEvent(cs, N->ev_alloc, 0));
    }
    DevBufPtr b;
    VRG_TRY(dev_alloc(cs, bytes, b));
    if (zero) VRG_CUDA_TRY(cudaMemsetAsync(b->ptr, 0, bytes, cs));
    buf = b;
    if (s != cs) {
        VRG_CUDA_TRY(cudaEventRecord(N->ev_alloc, cs));
        VRG_CUDA_TRY(cudaStreamWaitEvent(s, N->ev_alloc, 0));
    }
    return VRG_OK;
}

vrg_status nrc_infer(Nrc *N, cudaStream_t s, uint32_t n, const uint32_t *n_dev, const uint32_t *list,
                     const float4 *pos, const float4 *dir, const float4 *nrm, float4 *out, uint32_t *err) {
    if (n == 0) return VRG_OK;
    if (N->enc_cap < n) {
        VRG_TRY(cache_alloc(N, s, (size_t)(N->P.levels + 2) * n * 4, false, N->enc_buf));
        N->enc_cap = n;
    }
    InferArgs a{N->P, N->table, N->wpack, n, n_dev, list, pos, dir, nrm, out, err ? err : N->err,
                (uint32_t *)N->enc_buf->ptr, (uint32_t)N->enc_cap};
    // one query per thread: short-lived CTAs, so that a higher-priority
    // stream's kernels (a cache frame's training branch) get SMs in between
    k_nrc_encode<<<(n + 255) / 256, 256, 0, s>>>(a);
    const uint32_t tiles = (n + 127) / 128;
    const uint32_t blocks = std::min<uint32_t>((uint32_t)N->grid_tc, (tiles + TC_GROUPS - 1) / TC_GROUPS);
    k_nrc_infer_tc<<<blocks, TC_THREADS, tc_smem(), s>>>(a);
    VRG_CUDA_TRY(cudaGetLastError());
    return VRG_OK;
}

static vrg_status ensure_act(Nrc *N, cudaStream_t s, size_t rows) {
    const size_t n_pad = (rows + 31) & ~(size_t)31;
    if (N->act && N->act_rows >= n_pad) return VRG_OK;
    DevBufPtr b;
    VRG_TRY(cache_alloc(N, s, 2 * 6 * n_pad * NRC_W * 2, true, b));
    N->act = b;
    N->act_rows = n_pad;
    N->H = (__nv_bfloat16 *)b->ptr;
    N->dZ = N->H + 6 * n_pad * NRC_W;
    return VRG_OK;
}

// gradients of one batch (accumulated into w_grad / t_grad); update == true
// also runs the Adam step
vrg_status nrc_train(Nrc *N, cudaStream_t s, uint32_t n, const uint32_t *n_dev, const uint32_t *list,
                     const float4 *pos, const float4 *dir, const float4 *nrm, const float4 *target, bool update,
                     uint32_t *err, float4 *pred) {
    if (n == 0) return VRG_OK;
    VRG_TRY(nrc_flush(N, s));  // new gradients start from the updated cache
    VRG_TRY(ensure_act(N, s, n));
    const size_t n_pad = N->act_rows;
    // H and dZ hold n_pad rows per layer (the allocation, possibly made for a
    // larger batch): the training pass writes and k_nrc_dw reads with that pitch
    TrainArgs a{N->P,  N->table, N->wpack, n,         n_dev,   list,  pos, dir, nrm, target,
                N->H,  N->dZ,    n_pad,    N->t_grad, N->loss, err ? err : N->err, pred, nullptr, 0};
    if (N->train_tc) {
        // the samples' encoded rows (the inference encoding pass), then the
        // tensor-memory training pass over 128-sample tiles
        if (N->train_enc_cap < n) {
            VRG_TRY(cache_alloc(N, s, (size_t)(N->P.levels + 2) * n * 4, false, N->train_enc_buf));
            N->train_enc_cap = n;
        }
        a.enc = (const uint32_t *)N->train_enc_buf->ptr;
        a.enc_cap = (uint32_t)N->train_enc_cap;
        InferArgs e{N->P, N->table, N->wpack, n, n_dev, list, pos, dir, nrm, nullptr, a.err,
                    (uint32_t *)N->train_enc_buf->ptr, (uint32_t)N->train_enc_cap};
        k_nrc_encode<<<(n + 255) / 256, 256, 0, s>>>(e);
        const uint32_t tiles = (n + 127) / 128;
        const uint32_t blocks = std::min<uint32_t>((uint32_t)N->grid_train_tc, (tiles + TC_GROUPS - 1) / TC_GROUPS);
        k_nrc_train_tc<<<blocks, TC_THREADS, train_tc_smem(), s>>>(a);
    } else {
        const uint32_t blocks =
            std::min<uint32_t>((uint32_t)N->grid_train, (n + NRC_WARPS * 32 - 1) / (NRC_WARPS * 32));
        k_nrc_train<<<blocks, NRC_WARPS * 32, train_smem(), s>>>(a);
    }
    VRG_CUDA_TRY(cudaGetLastError());
    const uint32_t rows_per_cta = 512;
    dim3 g((n + rows_per_cta - 1) / rows_per_cta, NRC_LAYERS);
    k_nrc_dw<<<g, 128, 0, s>>>(N->H, N->dZ, n_pad, n, n_dev, N->w_grad, rows_per_cta);
    VRG_CUDA_TRY(cudaGetLastError());
    return update ? nrc_update(N, s) : VRG_OK;
}

// the Adam step of a previous cache frame's gradients, if one waits
vrg_status nrc_flush(Nrc *N, cudaStream_t s) {
    if (!N->pending) return VRG_OK;
    N->pending = false;
    return nrc_update(N, s);
}

bool nrc_pending(const Nrc *N) { return N->pending; }
void nrc_defer_update(Nrc *N) { N->pending = true; }

// the Adam step of the accumulated gradients: rewrites the weights and the
// table that inference reads
vrg_status nrc_update(Nrc *N, cudaStream_t s) {
    N->step++;
    AdamArgs A;
    A.lr = N->desc.learning_rate;
    A.b1 = 0.9f;
    A.b2 = 0.99f;
    A.eps = 1e-8f;
    A.c1 = (float)(1.0 / (1.0 - std::pow(0.9, (double)N->step)));
    A.c2 = (float)(1.0 / (1.0 - std::pow(0.99, (double)N->step)));
    k_adam_weights<<<(uint32_t)((MASTER_ELEMS + 255) / 256), 256, 0, s>>>(N->w_master, N->w_m, N->w_v, N->w_grad, A);
    k_pack_weights<<<(uint32_t)((WPACK_ELEMS + 255) / 256), 256, 0, s>>>(N->w_master, N->wpack);
    k_adam_table<<<(uint32_t)((N->table_entries + 255) / 256), 256, 0, s>>>(N->t_master, N->t_m, N->t_v, N->t_grad,
                                                                           N->table, N->table_entries, A);
    VRG_CUDA_TRY(cudaGetLastError());
    return VRG_OK;
}

uint32_t nrc_batch(const Nrc *N) { return N->desc.batch ? N->desc.batch : 65536u; }

void nrc_destroy(Nrc *N) {
    if (!N) return;
    cudaStreamSynchronize(N->ctx->stream);
    if (N->ev_alloc) cudaEventDestroy(N->ev_alloc);
    Context *c = N->ctx;
    delete N;  // its buffers are freed on the context's stream, before the context may go
    ctx_release(c);
}

// ---- host-array entry points (tests and tools) ------------------------------

static vrg_status stage4(cudaStream_t s, const float *src, uint32_t n, int comps, float4 *dst) {
    std::vector<float4> h(n);
    for (uint32_t i = 0; i < n; i++)
        h[i] = make_float4(src[comps * i], src[comps * i + 1], src[comps * i + 2], comps > 3 ? src[comps * i + 3] : 0.0f);
    VRG_CUDA_TRY(cudaMemcpyAsync(dst, h.data(), (size_t)n * 16, cudaMemcpyHostToDevice, s));
    VRG_CUDA_TRY(cudaStreamSynchronize(s));
    return VRG_OK;
}

vrg_status nrc_query_host(Nrc *N, uint32_t n, const float *pos, const float *nrm, const float *dir, float *rgb) {
    cudaStream_t s = N->ctx->stream;
    VRG_TRY(nrc_flush(N, s));
    DevBufPtr b;
    VRG_TRY(dev_alloc(s, (size_t)n * 16 * 4 + 64, b));
    float4 *dp = (float4 *)b->ptr, *dd = dp + n, *dn = dd + n, *dout = dn + n;
    VRG_TRY(stage4(s, pos, n, 3, dp));
    VRG_TRY(stage4(s, dir, n, 3, dd));
    VRG_TRY(stage4(s, nrm, n, 3, dn));
    VRG_CUDA_TRY(cudaMemsetAsync(N->err, 0, 4, s));
    VRG_TRY(nrc_infer(N, s, n, nullptr, nullptr, dp, dd, dn, dout, nullptr));
    std::vector<float4> h(n);
    uint32_t err = 0;
    VRG_CUDA_TRY(cudaMemcpyAsync(h.data(), dout, (size_t)n * 16, cudaMemcpyDeviceToHost, s));
    VRG_CUDA_TRY(cudaMemcpyAsync(&err, N->err, 4, cudaMemcpyDeviceToHost, s));
    VRG_CUDA_TRY(cudaStreamSynchronize(s));
    if (err) {
        set_error("radiance cache kernel error flags 0x%x", err);
        return VRG_ERR_OVERFLOW;
    }
    for (uint32_t i = 0; i < n; i++) { rgb[3 * i] = h[i].x; rgb[3 * i + 1] = h[i].y; rgb[3 * i + 2] = h[i].z; }
    return VRG_OK;
}

vrg_status nrc_train_host(Nrc *N, uint32_t n, const float *pos, const float *nrm, const float *dir, const float *target,
                          uint32_t update, float *loss_out) {
    cudaStream_t s = N->ctx->stream;
    DevBufPtr b;
    VRG_TRY(dev_alloc(s, (size_t)n * 16 * 4 + 64, b));
    float4 *dp = (float4 *)b->ptr, *dd = dp + n, *dn = dd + n, *dt = dn + n;
    VRG_TRY(stage4(s, pos, n, 3, dp));
    VRG_TRY(stage4(s, dir, n, 3, dd));
    VRG_TRY(stage4(s, nrm, n, 3, dn));
    VRG_TRY(stage4(s, target, n, 3, dt));
    VRG_CUDA_TRY(cudaMemsetAsync(N->loss, 0, 8, s));  // loss and error word
    if (N->pred_cap < n) {
        VRG_TRY(cache_alloc(N, s, (size_t)n * 16, false, N->pred_buf));
        N->pred_cap = n;
    }
    N->pred_n = n;
    VRG_TRY(nrc_train(N, s, n, nullptr, nullptr, dp, dd, dn, dt, update != 0, nullptr, (float4 *)N->pred_buf->ptr));
    float l = 0.0f;
    uint32_t err = 0;
    VRG_CUDA_TRY(cudaMemcpyAsync(&l, N->loss, 4, cudaMemcpyDeviceToHost, s));
    VRG_CUDA_TRY(cudaMemcpyAsync(&err, N->err, 4, cudaMemcpyDeviceToHost, s));
    VRG_CUDA_TRY(cudaStreamSynchronize(s));
    if (err) {
        set_error("radiance cache kernel error flags 0x%x", err);
        return VRG_ERR_OVERFLOW;
    }
    if (loss_out) *loss_out = l;
    return VRG_OK;
}

vrg_status nrc_read(Nrc *N, uint32_t what, void *dst, uint64_t bytes) {
    cudaStream_t s = N->ctx->stream;
    VRG_TRY(nrc_flush(N, s));
    const void *src = nullptr;
    size_t nb = 0;
    switch (what) {
    case VRG_NRC_WEIGHTS: src = N->w_master; nb = MASTER_ELEMS * 4; break;
    case VRG_NRC_WEIGHT_GRADS: src = N->w_grad; nb = MASTER_ELEMS * 4; break;
    case VRG_NRC_TABLE: src = N->t_master; nb = N->table_entries * 8; break;
    case VRG_NRC_TABLE_GRADS: src = N->t_grad; nb = N->table_entries * 8; break;
    case VRG_NRC_TRAIN_PREDICTIONS: {
        if (!N->pred_buf) return VRG_ERR_STATE;
        if (bytes < (uint64_t)N->pred_n * 12) return VRG_ERR_INVALID_ARGUMENT;
        std::vector<float4> h(N->pred_n);
        VRG_CUDA_TRY(cudaMemcpyAsync(h.data(), N->pred_buf->ptr, (size_t)N->pred_n * 16, cudaMemcpyDeviceToHost, s));
        VRG_CUDA_TRY(cudaStreamSynchronize(s));
        float *d = (float *)dst;
        for (uint32_t i = 0; i < N->pred_n; i++) { d[3 * i] = h[i].x; d[3 * i + 1] = h[i].y; d[3 * i + 2] = h[i].z; }
        return VRG_OK;
    }
    default: return VRG_ERR_INVALID_ARGUMENT;
    }
    if (bytes < nb) return VRG_ERR_INVALID_ARGUMENT;
    VRG_CUDA_TRY(cudaMemcpyAsync(dst, src, nb, cudaMemcpyDeviceToHost, s));
    VRG_CUDA_TRY(cudaStreamSynchronize(s));
    return VRG_OK;
}

vrg_status nrc_write(Nrc *N, uint32_t what, const void *src, uint64_t bytes) {
    cudaStream_t s = N->ctx->stream;
    VRG_TRY(nrc_flush(N, s));
    if (what == VRG_NRC_WEIGHTS) {
        if (bytes < MASTER_ELEMS * 4) return VRG_ERR_INVALID_ARGUMENT;
        VRG_CUDA_TRY(cudaMemcpyAsync(N->w_master, src, MASTER_ELEMS * 4, cudaMemcpyHostToDevice, s));
        k_pack_weights<<<(uint32_t)((WPACK_ELEMS + 255) / 256), 256, 0, s>>>(N->w_master, N->wpack);
    } else if (what == VRG_NRC_TABLE) {
        if (bytes < N->table_entries * 8) return VRG_ERR_INVALID_ARGUMENT;
        std::vector<float2> h(N->table_entries);
        memcpy(h.data(), src, N->table_entries * 8);
        std::vector<__half2> hh(N->table_entries);
        for (size_t i = 0; i < h.size(); i++) hh[i] = __floats2half2_rn(h[i].x, h[i].y);
        VRG_CUDA_TRY(cudaMemcpyAsync(N->t_master, h.data(), N->table_entries * 8, cudaMemcpyHostToDevice, s));
        VRG_CUDA_TRY(cudaMemcpyAsync(N->table, hh.data(), N->table_entries * 4, cudaMemcpyHostToDevice, s));
        VRG_CUDA_TRY(cudaStreamSynchronize(s));
    } else if (what == VRG_NRC_ZERO_GRADS) {
        VRG_CUDA_TRY(cudaMemsetAsync(N->w_grad, 0, MASTER_ELEMS * 4, s));
        VRG_CUDA_TRY(cudaMemsetAsync(N->t_grad, 0, N->table_entries * 8, s));
    } else {
        return VRG_ERR_INVALID_ARGUMENT;
    }
    VRG_CUDA_TRY(cudaGetLastError());
    VRG_CUDA_TRY(cudaStreamSynchronize(s));
    return VRG_OK;
}

void nrc_layout(uint32_t *levels, float *scales, uint32_t *dense, uint32_t *res1, const Nrc *N) {
    *levels = (uint32_t)N->P.levels;
    for (int l = 0; l < N->P.levels; l++) {
        scales[l] = N->P.scale[l];
        dense[l] = N->P.dense[l];
        res1[l] = N->P.res1[l];
    }
}

}  // namespace vrg
