// Streaming kernels after the bounces:
//   k_resolve: backward outgoing-radiance recurrence (outgoing_radiance.rs:
//     171-207), assembly of the initial ReSTIR sample from the bounce slices
//     (the six copy_buffer calls, interactive_rendering.rs:1359-1414, now a
//     register move) and temporal resampling (restir_temporal_resampling.rs:
//     256-301) — one read and one write of the 80-byte reservoir per pixel.
//   k_spatial: spatial resampling (restir_spatial_resampling.rs:316-406),
//     finalize (restir_finalize.rs:121-141) and postprocess pack
//     (postprocess.rs:39-88) fused; the spatial reservoir is consumed in
//     registers and written only for parity capture.
// Reservoirs are five float4 planes per pixel (SoA, coalesced 16-byte loads):
//   0 (x_v, ucw)  1 (n_v, w_sum)  2 (x_s, m)  3 (n_s, p_omega)  4 (l_o_hat, seed)
// Both passes are latency-bound streams: they are compiled for 5 CTAs of 256
// threads per SM (at most 51 registers, a few bytes of spills), not 4; on the
// 1080p frame the spatial pass went from 0.111 to 0.103-0.104 ms.
#include <cuda.h>

#include "vrg_frame.cuh"
#include "vrg_internal.h"

namespace vrg {

namespace {

struct Res {
    f3 x_v, n_v, x_s, n_s, l;
    float p_omega;
    uint32_t seed;
    float ucw;
    uint32_t m;
    float w_sum;
};

__device__ __forceinline__ Res load_res(const float4 *base, uint32_t P, uint32_t p) {
    float4 a = base[p], b = base[P + p], c = base[2 * (size_t)P + p], d = base[3 * (size_t)P + p],
           e = base[4 * (size_t)P + p];
    Res r;
    r.x_v = ld3(a); r.ucw = a.w;
    r.n_v = ld3(b); r.w_sum = b.w;
    r.x_s = ld3(c); r.m = __float_as_uint(c.w);
    r.n_s = ld3(d); r.p_omega = d.w;
    r.l = ld3(e); r.seed = __float_as_uint(e.w);
    return r;
}
__device__ __forceinline__ void store_res(float4 *base, uint32_t P, uint32_t p, const Res &r) {
    base[p] = make_float4(r.x_v.x, r.x_v.y, r.x_v.z, r.ucw);
    base[P + p] = make_float4(r.n_v.x, r.n_v.y, r.n_v.z, r.w_sum);
    base[2 * (size_t)P + p] = make_float4(r.x_s.x, r.x_s.y, r.x_s.z, __uint_as_float(r.m));
    base[3 * (size_t)P + p] = make_float4(r.n_s.x, r.n_s.y, r.n_s.z, r.p_omega);
    base[4 * (size_t)P + p] = make_float4(r.l.x, r.l.y, r.l.z, __uint_as_float(r.seed));
}

__device__ __forceinline__ void st3(float *a, size_t i, f3 v) {
    a[3 * i] = v.x;
    a[3 * i + 1] = v.y;
    a[3 * i + 2] = v.z;
}

template <bool CAPTURE, bool BATCH>
__global__ void __launch_bounds__(256, 5) k_resolve(const __grid_constant__ FrameArgs a) {
    const uint32_t P = a.P;
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const uint32_t nb = a.nb;
    // a path that reached the cache's query vertex with a hit needs no more of
    // its length here (its training continuation may still be running on
    // another stream and writing nlive); every other path ended by then
    const uint32_t nl = (!CAPTURE && a.cache && a.qflag[p]) ? a.nb_render : a.nlive[p];
    const float inv2pi = 1.0f / (2.0f * PI_F);
    f3 L = f3{0.0f, 0.0f, 0.0f}, L1 = f3{0.0f, 0.0f, 0.0f};
    float q0 = inv2pi;
    if (CAPTURE) {
        // terminal slices (raytrace.rs:406-416 for rays with direction 0)
        for (uint32_t b = nl; b < nb; b++) {
            size_t s0 = (size_t)b * P + p, s1 = (size_t)(b + 1) * P + p, sp = (size_t)b * P + p;
            a.c_origin[3 * s1] = a.c_origin[3 * sp];
            a.c_origin[3 * s1 + 1] = a.c_origin[3 * sp + 1];
            a.c_origin[3 * s1 + 2] = a.c_origin[3 * sp + 2];
            st3(a.c_dir, s1, f3{0.0f, 0.0f, 0.0f});
            st3(a.c_normal, s0, f3{0.0f, 0.0f, 0.0f});
            st3(a.c_emis, s0, f3{0.0f, 0.0f, 0.0f});
            st3(a.c_refl, s0, f3{0.0f, 0.0f, 0.0f});
            a.c_mis[s0] = 0.0f;
            a.c_pdf[s0] = 1.0f;
            a.c_nee[s0] = 0.0f;
            reinterpret_cast<uint4 *>(a.c_hit)[s0] = make_uint4(TERMINATED, TERMINATED, TERMINATED, TERMINATED);
            st3(a.c_L, s0, f3{0.0f, 0.0f, 0.0f});
            a.c_q[s0] = inv2pi;
        }
    }
    int top = (int)nl - 1;
    if (a.cache && nl >= a.nb_render) {
        // the path ends into the radiance cache at vertex nb_render-1: its
        // outgoing radiance is the cache's prediction when the ray hit geometry,
        // the record's emission (sky) when it missed
        const int qb = (int)a.nb_render - 1;
        if (a.qflag[p]) {
            const float4 pr = a.pred[p];
            L = f3{pr.x, pr.y, pr.z};
        } else {
            const float4 e = a.rec[(size_t)qb * 2 * P + p];
            L = f3{e.x, e.y, e.z};
        }
        if (qb == 1) L1 = L;
        top = qb - 1;
    }
    for (int b = top; b >= 0; b--) {
        const size_t rb = (size_t)b * 2 * P;
        const float4 e = a.rec[rb + p], r = a.rec[rb + P + p];
        // L = E + R * L * (bsdf_pdf / q) * valid, valid = 1 for traced rays
        L = f3{e.x + (r.x * L.x) * e.w, e.y + (r.y * L.y) * e.w, e.z + (r.z * L.z) * e.w};
        if (b == 1) L1 = L;
        if (b == 0) q0 = r.w;
        if (CAPTURE) {
            st3(a.c_L, (size_t)b * P + p, L);
            a.c_q[(size_t)b * P + p] = r.w;
        }
    }
    a.plain[p] = make_float4(L.x, L.y, L.z, 0.0f);
    if (nb < 2 || !a.restir) return;
    // initial sample (interactive_rendering.rs:1359-1414)
    Res S;
    S.x_v = ld3(a.xv[p]);
    S.n_v = ld3(a.nv[p]);
    if (nl >= 2) {
        S.x_s = ld3(a.xs[p]);
        S.n_s = ld3(a.ns[p]);
    } else {  // bounce 1 never traced: origin passes through, normal 0
        S.x_s = S.x_v;
        S.n_s = f3{0.0f, 0.0f, 0.0f};
    }
    S.l = L1;
    S.p_omega = q0;
    S.seed = 0;
    // temporal resampling (restir_temporal_resampling.rs:256-301)
    const ViewDev &V = view_of<BATCH>(a, p);
    const uint32_t ps = mm_combine(V.temporal_seed, p - V.pix_off);
    Res R = load_res(a.res, P, p);
    if (mm_rand(mm_combine(ps, 0)) < 0.4f) {
        R.w_sum = 0.0f;
        R.m = 0;
    }
    if (a.mode == VRG_MODE_CONFIG && a.m_cap && R.m > a.m_cap) {  // M-cap (no reference counterpart)
        R.w_sum = R.w_sum * ((float)a.m_cap / (float)R.m);
        R.m = a.m_cap;
    }
    const float w = luminance3(S.l) / S.p_omega;
    R.w_sum += w;
    R.m += 1;
    if (float_construct(mm_finalize(mm_combine(ps, 1))) < w / R.w_sum) {
        R.x_v = S.x_v; R.n_v = S.n_v; R.x_s = S.x_s; R.n_s = S.n_s; R.l = S.l;
        R.p_omega = S.p_omega; R.seed = S.seed;
    }
    const float ph = luminance3(R.l);
    R.ucw = (ph > 0.0f) ? R.w_sum / ((float)R.m * ph) : 0.0f;
    store_res(a.res, P, p, R);
}

__device__ __forceinline__ uint8_t to_u8(float x) {
    float v = x * 255.0f;
    if (!(v > 0.0f)) return 0;
    if (v >= 255.0f) return 255;
    return (uint8_t)(int)v;
}

// Where the spatial pass reads reservoirs: straight from the ring slot, or
// (ResTile) from the CTA's tile of it staged in shared memory when the pixel
// lies in that tile.  The arithmetic is the same either way.
struct ResGlobal {
    const float4 *res;
    uint32_t P;
    __device__ __forceinline__ float4 plane(int k, uint32_t p, uint32_t, uint32_t) const {
        return res[(size_t)k * P + p];
    }
};
constexpr uint32_t ST_W = 32, ST_H = 8;  // staged tile: 32 x 8 pixels, 5 planes (20 KB)
struct ResTile {
    const float4 *res;
    uint32_t P, x0, y0;
    const float4 *tile;  // [5][ST_H][ST_W]
    __device__ __forceinline__ float4 plane(int k, uint32_t p, uint32_t x, uint32_t y) const {
        if (x - x0 < ST_W && y - y0 < ST_H) return tile[((uint32_t)k * ST_H + (y - y0)) * ST_W + (x - x0)];
        return res[(size_t)k * P + p];
    }
};

template <typename Src>
__device__ __forceinline__ Res load_res_src(const Src &src, uint32_t p, uint32_t x, uint32_t y) {
    const float4 a = src.plane(0, p, x, y), b = src.plane(1, p, x, y), c = src.plane(2, p, x, y),
                 d = src.plane(3, p, x, y), e = src.plane(4, p, x, y);
    Res r;
    r.x_v = ld3(a); r.ucw = a.w;
    r.n_v = ld3(b); r.w_sum = b.w;
    r.x_s = ld3(c); r.m = __float_as_uint(c.w);
    r.n_s = ld3(d); r.p_omega = d.w;
    r.l = ld3(e); r.seed = __float_as_uint(e.w);
    return r;
}

// spatial resampling, finalize, pack and accumulation of pixel p
template <bool CAPTURE, bool BATCH, typename Src>
__device__ __forceinline__ void spatial_pixel(const FrameArgs &a, uint32_t p, const Src &src) {
    const uint32_t P = a.P;
    f3 fin = f3{0.0f, 0.0f, 0.0f};
    float ucw_view = 0.0f;
    if (a.nb >= 2 && a.restir) {
        // neighbours are taken within the pixel's own view
        const ViewDev &V = view_of<BATCH>(a, p);
        const uint32_t lp = p - V.pix_off;
        const uint32_t qx = lp % V.W, qy = lp / V.W;
        const uint32_t ps = mm_combine(V.spatial_seed, lp);
        Res Rs = load_res_src(src, p, qx, qy);
        const f3 Sx_v = Rs.x_v, Sn_v = Rs.n_v;
        uint32_t Z = (luminance3(Rs.l) > 0.0f) ? Rs.m : 0u;
        for (uint32_t s = 0; s < a.spatial_iters; s++) {
            const uint32_t is = mm_combine(ps, s);
            const float jx = a.spatial_radius * (mm_rand(mm_combine(is, 0)) - 0.5f);
            const float jy = a.spatial_radius * (mm_rand(mm_combine(is, 1)) - 0.5f);
            int nx = (int)(((float)qx + 0.5f) + jx);
            int ny = (int)(((float)qy + 0.5f) + jy);
            nx = min(max(nx, 0), (int)V.W - 1);
            ny = min(max(ny, 0), (int)V.H - 1);
            const uint32_t np = V.pix_off + (uint32_t)nx + (uint32_t)ny * V.W;
            // geometricallySimilar (restir_spatial_resampling.rs:277-288)
            const float4 nvn = src.plane(1, np, (uint32_t)nx, (uint32_t)ny);
            const f3 nn = ld3(nvn);
            if (zero3(Sn_v) || zero3(nn)) continue;
            if (dot3(Sn_v, nn) < COS25) continue;
            const Res Rn = load_res_src(src, np, (uint32_t)nx, (uint32_t)ny);
            // computeJacobianQToR (restir_spatial_resampling.rs:299-311)
            float J;
            if (zero3(Rn.n_s)) {
                J = 1.0f;
            } else {
                const f3 qvs = sub3(Rn.x_v, Rn.x_s), rvs = sub3(Sx_v, Rn.x_s);
                const float cq = fabsf(dot3(norm3(qvs), Rn.n_s));
                const float cr = fabsf(dot3(norm3(rvs), Rn.n_s));
                J = (cr / cq) * (len3(qvs) / len3(rvs));
            }
            J = fminf(fmaxf(J, 0.1f), 10.0f);
            const float p_adj = luminance3(Rn.l) / J;
            // mergeReservoir (restir_spatial_resampling.rs:266-275)
            const uint32_t m0 = Rs.m;
            const float wn = (p_adj * Rn.ucw) * (float)Rn.m;
            Rs.w_sum += wn;
            Rs.m += 1;
            if (float_construct(mm_finalize(mm_combine(is, 2))) < wn / Rs.w_sum) {
                Rs.x_v = Rn.x_v; Rs.n_v = Rn.n_v; Rs.x_s = Rn.x_s; Rs.n_s = Rn.n_s; Rs.l = Rn.l;
                Rs.p_omega = Rn.p_omega; Rs.seed = Rn.seed;
            }
            Rs.m = m0 + Rn.m;
            if (luminance3(Rn.l) > 0.0f) Z += Rn.m;
        }
        const float ph = luminance3(Rs.l);
        Rs.ucw = (ph == 0.0f) ? 0.0f : Rs.w_sum / ((float)Z * ph);
        // finalize (restir_finalize.rs:121-141)
        const f3 dir = norm3(sub3(Rs.x_s, ld3(a.xv[p])));
        const float bp = dot3(dir, Rs.n_v) / PI_F;
        const float4 e0 = a.rec[p], r0 = a.rec[P + p];
        fin = f3{e0.x + ((r0.x * Rs.l.x) * Rs.ucw) * bp, e0.y + ((r0.y * Rs.l.y) * Rs.ucw) * bp,
                 e0.z + ((r0.z * Rs.l.z) * Rs.ucw) * bp};
        ucw_view = Rs.ucw;
        if (CAPTURE) {
            store_res(a.spatial, P, p, Rs);
            a.final_t[p] = make_float4(fin.x, fin.y, fin.z, 0.0f);
        }
    }
    // postprocess (postprocess.rs:39-88), scale 1
    f3 c;
    if (a.debug_view == 0) c = ld3(a.plain[p]);
    else if (a.debug_view == 1) c = fin;
    else { const float dv = ucw_view / 10.0f; c = f3{dv, dv, dv}; }
    if (a.pack && a.scale <= 1) {
        uchar4 px = make_uchar4(to_u8(c.z), to_u8(c.y), to_u8(c.x), 255);
        reinterpret_cast<uchar4 *>(a.bgra)[p] = px;
    }
    if (a.radiance) st3(a.radiance, p, c);
    if (a.accumulate && isfinite(c.x) && isfinite(c.y) && isfinite(c.z)) {
        // non-finite samples (the estimator's 0*inf cases) are left out of the sum
        a.accum[3 * (size_t)p] += (double)c.x;
        a.accum[3 * (size_t)p + 1] += (double)c.y;
        a.accum[3 * (size_t)p + 2] += (double)c.z;
    }
}

template <bool CAPTURE, bool BATCH>
__global__ void __launch_bounds__(256, 5) k_spatial(const __grid_constant__ FrameArgs a) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.P) return;
    spatial_pixel<CAPTURE, BATCH>(a, p, ResGlobal{a.res, a.P});
}

// The spatial pass over 32 x 8 pixel tiles of a single view, the CTA's own
// reservoirs staged in shared memory by one tensor copy (cp.async.bulk.tensor,
// a 3-D box of the ring slot: 32 pixels x 8 rows x 5 planes, completing on an
// mbarrier; parts outside the view are zero-filled and never read).  A pixel
// reads its own reservoir, and its neighbours' when they fall in the tile,
// from shared memory, the rest from L2 / HBM as k_spatial does.  The wait is
// bounded: past the limit the kernel flags ERR_COPY, waits once more
// (bounded) for the copy in flight, and returns.
template <bool CAPTURE>
__global__ void __launch_bounds__(256, 5) k_spatial_tma(const __grid_constant__ FrameArgs a,
                                                     const __grid_constant__ CUtensorMap map) {
    __shared__ __align__(128) float4 tile[5 * ST_H * ST_W];
    __shared__ __align__(8) uint64_t bar;
    const uint32_t W = a.v0.W, H = a.v0.H;
    const uint32_t x0 = blockIdx.x * ST_W, y0 = blockIdx.y * ST_H;
    const uint32_t b = (uint32_t)__cvta_generic_to_shared(&bar), d = (uint32_t)__cvta_generic_to_shared(tile);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(b) : "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(b),
                     "r"((uint32_t)sizeof(tile))
                     : "memory");
        // x in floats: 4 per pixel, so 16-byte aligned
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
            "[%5];\n" ::"r"(d),
            "l"(&map), "r"((int)(4 * x0)), "r"((int)y0), "r"(0), "r"(b)
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
    if (!wait(1u << 22)) {
        if (threadIdx.x == 0) atomicOr(a.counters + CNT_ERROR, ERR_COPY);
        wait(1u << 22);
        return;
    }
    const uint32_t x = x0 + (threadIdx.x % ST_W), y = y0 + (threadIdx.x / ST_W);
    if (x >= W || y >= H) return;
    spatial_pixel<CAPTURE, false>(a, y * W + x, ResTile{a.res, a.P, x0, y0, tile});
}

// postprocess with scale > 1 (postprocess.rs:39-88, srcscale = scale,
// dstscale = 1): each output pixel is the mean of its scale x scale traced
// pixels, summed row by row from zero as the shader does, then packed
__global__ void __launch_bounds__(256) k_downsample(const __grid_constant__ FrameArgs a) {
    const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= a.out_w * a.out_h) return;
    const uint32_t ox = o % a.out_w, oy = o / a.out_w, s = a.scale, src_w = a.out_w * s;
    f3 c = f3{0.0f, 0.0f, 0.0f};
    for (uint32_t sy = 0; sy < s; sy++) {
        const uint32_t y = oy * s + sy;
        for (uint32_t sx = 0; sx < s; sx++) {
            const uint32_t x = ox * s + sx;
            const size_t id = (size_t)y * src_w + x;
            c = f3{c.x + a.radiance[3 * id], c.y + a.radiance[3 * id + 1], c.z + a.radiance[3 * id + 2]};
        }
    }
    const float n = (float)(s * s);
    c = f3{c.x / n, c.y / n, c.z / n};
    if (a.pack) reinterpret_cast<uchar4 *>(a.out_bgra)[o] = make_uchar4(to_u8(c.z), to_u8(c.y), to_u8(c.x), 255);
    if (a.out_radiance) st3(a.out_radiance, o, c);
}

// training targets of the radiance cache: the outgoing radiance at vertex
// nb_render-1 of each long training path (its full backward recurrence)
__global__ void __launch_bounds__(256) k_train_targets(const __grid_constant__ FrameArgs a) {
    const uint32_t n = min(a.counters[CNT_TRAIN], a.train_cap);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t P = a.P, p = a.train_list[i];
    const int nl = a.nlive[p], qb = (int)a.nb_render - 1;
    f3 L = f3{0.0f, 0.0f, 0.0f};
    for (int b = nl - 1; b >= qb; b--) {
        const size_t rb = (size_t)b * 2 * P;
        const float4 e = a.rec[rb + p], r = a.rec[rb + P + p];
        L = f3{e.x + (r.x * L.x) * e.w, e.y + (r.y * L.y) * e.w, e.z + (r.z * L.z) * e.w};
    }
    a.target[p] = make_float4(L.x, L.y, L.z, 0.0f);
}

}  // namespace

vrg_status launch_train_targets(cudaStream_t s, const FrameArgs &a) {
    k_train_targets<<<(a.train_cap + 255) / 256, 256, 0, s>>>(a);
    VRG_CUDA_TRY(cudaGetLastError());
    return VRG_OK;
}

// per-pixel kernels: CTAs of a.stream_block threads (64, 128 or 256)
static uint32_t stream_block(const FrameArgs &a) { return a.stream_block ? a.stream_block : 256u; }

vrg_status launch_resolve(cudaStream_t s, const FrameArgs &a) {
    const uint32_t t = stream_block(a);
    dim3 g((a.P + t - 1) / t);
    if (a.views) k_resolve<false, true><<<g, t, 0, s>>>(a);
    else if (a.capture) k_resolve<true, false><<<g, t, 0, s>>>(a);
    else k_resolve<false, false><<<g, t, 0, s>>>(a);
    VRG_CUDA_TRY(cudaGetLastError());
    return VRG_OK;
}

vrg_status launch_spatial(cudaStream_t s, const FrameArgs &a, const CUtensorMap *res_map) {
    const uint32_t t = stream_block(a);
    dim3 g((a.P + t - 1) / t);
    if (res_map && !a.views) {  // single view with its ring slot's tensor map: tiles staged by TMA
        const dim3 gt((a.v0.W + ST_W - 1) / ST_W, (a.v0.H + ST_H - 1) / ST_H);
        if (a.capture) k_spatial_tma<true><<<gt, ST_W * ST_H, 0, s>>>(a, *res_map);
        else k_spatial_tma<false><<<gt, ST_W * ST_H, 0, s>>>(a, *res_map);
    } else if (a.views) k_spatial<false, true><<<g, t, 0, s>>>(a);
    else if (a.capture) k_spatial<true, false><<<g, t, 0, s>>>(a);
    else k_spatial<false, false><<<g, t, 0, s>>>(a);
    VRG_CUDA_TRY(cudaGetLastError());
    if (a.scale > 1 && (a.pack || a.out_radiance)) {
        const uint32_t n = a.out_w * a.out_h;
        k_downsample<<<(n + 255) / 256, 256, 0, s>>>(a);
        VRG_CUDA_TRY(cudaGetLastError());
    }
    return VRG_OK;
}

}  // namespace vrg
