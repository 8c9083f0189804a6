// Per-frame kernel arguments shared by the wavefront stages.
#pragma once

#include "vrg_device.cuh"

namespace vrg {

// counters[] layout (u32 words)
constexpr int CNT_QUEUE = 0;     // [0..7]  rays queued for bounce b
constexpr int CNT_FETCH = 8;     // [8..15] closest-hit work-fetch cursor of bounce b
constexpr int CNT_ERROR = 16;    // error word
constexpr int CNT_RAYS = 18;     // u64 at words 18-19: closest-hit queries
constexpr int CNT_TQUEUE = 22;   // a cache frame's training candidates queued for its query bounce (FrameArgs::tq)
constexpr int CNT_TFETCH = 23;   // their closest-hit work-fetch cursor
constexpr int CNT_ANY = 20;      // u64 at words 20-21: light any-hit queries
constexpr int CNT_AQUEUE = 24;   // [24..31] any-hit jobs queued by bounce b
constexpr int CNT_AFETCH = 32;   // [32..39] any-hit work-fetch cursor of bounce b
constexpr int CNT_SFETCH = 40;   // [40..47] shading work-fetch cursor of bounce b
constexpr int CNT_NODES = 50;    // u64 at words 50-51: inner nodes fetched by k_trace
constexpr int CNT_LEAVES = 52;   // u64 at words 52-53: leaf records tested by k_trace
constexpr int CNT_HITS = 54;     // light hits collected by k_anyhit for the current bounce
constexpr int CNT_HITS_TRAIN = 55;  // the same for a cache frame's training branch (its own job and hit buffers)
constexpr int CNT_ANODES = 56;   // u64 at words 56-57: 4-wide lamp nodes fetched by k_anyhit
constexpr int CNT_ALEAVES = 58;  // u64 at words 58-59: lamp-block records tested by k_anyhit
constexpr int CNT_AHITS = 60;    // u64 at words 60-61: light hits collected by k_anyhit
constexpr int CNT_INFER = 48;    // radiance-cache queries of the frame
constexpr int CNT_TRAIN = 49;    // radiance-cache training paths of the frame
constexpr int CNT_WORDS = 64;
constexpr int MAX_BOUNCES = 8;

// One camera view of one scene.  A frame renders either one view (the
// FrameArgs::v0 fields, passed as kernel parameters) or a batch of views whose
// pixels are numbered view after view in one pixel space (FrameArgs::views in
// device memory, so that a captured launch sequence reads each frame's
// cameras, seeds and scenes from there).  Pixel streams and reservoir
// neighbourhoods use the view-local pixel index p - pix_off, so a view renders
// the same image alone or inside a batch.
struct ViewDev {
    DevScene sc;
    f3 eye, front, right, up;
    uint32_t W, H, pix_off, pix_end;
    uint32_t frame, temporal_seed, spatial_seed, pad;
};
constexpr int VIEW_SHIFT = 8;  // vtab entry per 256 pixels: the view of the group's first pixel

struct FrameArgs {
    ViewDev v0;                   // the view of a single-view frame
    const ViewDev *views;         // batched frame: the views (device), else null
    const uint16_t *vtab;         // batched frame: view of pixel group p >> VIEW_SHIFT
    uint32_t n_views;
    uint32_t mesh;                // a scene of the frame holds mesh triangles (the bounce kernels
                                  // built with mesh support run; voxel-only frames run without it)
    uint32_t P;                   // pixels of the frame (all views)
    uint32_t n0, tiles_x;         // bounce-0 slots and 8x4 tiles per row (bounce0_pixel)
    uint32_t nb, nee_type;
    uint32_t mode, spatial_iters;
    float spatial_radius;
    uint32_t m_cap, debug_view, accumulate, pack;
    // launch configuration (scheduling only, never a result): idle lanes that
    // trigger a warp's refill, persistent grids (CTAs), per-pixel CTA size
    uint32_t refill_trace, refill_any;
    // supersampling (Renderer.scale): the frame is traced at scale x the
    // output extent; k_downsample packs out_w x out_h pixels
    uint32_t scale, out_w, out_h;
    uint8_t *out_bgra;
    float *out_radiance;
    uint32_t grid_trace, grid_shade, grid_any, stream_block;
    // wavefront state
    float4 *ray_o, *ray_d;
    uint32_t *queue[2];
    // A single-view cache frame traces its query bounce in two launches: the
    // training candidates (one pixel in 16) first, so that the training
    // branch forks early, then the other paths.  tq_split: the shading of the
    // bounce before the query bounce queues the candidates' rays in tq
    // (CNT_TQUEUE) instead of queue[]; qsel: this launch of the query bounce
    // takes its rays from tq.
    uint32_t *tq;
    uint32_t tq_split, qsel;
    // light-pdf jobs of bounce b in [b & 1] (double-buffered by bounce parity:
    // the jobs of bounce b are walked while bounce b + 1 traces and shades):
    // the pixel, and a copy of its ray (origin | face, direction | bsdf pdf)
    uint32_t *aqueue[2];
    float4 *ajob[2];              // 2 float4 per job
    uint4 *hitbuf;                // light hits: (pixel, instance, leaf, b1 bits), then (b2 bits, 0, 0, 0)
    float *hitval;                // light-sampling pdf of each hit
    uint2 *jmeta;                 // per any-hit job: (first hit, hit count)
    uint32_t hit_cap;
    uint32_t *hit_count;          // the hits collected for the current bounce (a counter word)
    int4 *hits;                   // closest hit per pixel: (~record or -1, face|half<<3, b1, b2)
    uint32_t *counters;
    uint8_t *nlive;
    float4 *rec;                  // [nb][2][P]: (E.xyz, w), (R.xyz, q)
    float4 *xv, *nv, *xs, *ns;
    float4 *plain;                // L[0]
    float4 *res;                  // temporal ring slot [5][P]
    float4 *spatial;              // [5][P] (written when capture)
    float4 *final_t;              // [P] (written when capture)
    uint8_t *bgra;
    float *radiance;
    double *accum;
    // radiance cache (VRG_RENDER_CACHE): paths end into the cache after
    // nb_render bounces; 1/16 of them (up to train_cap) trace to nb and train it
    uint32_t nb_render, cache, train_cap, restir;  // restir: run the ReSTIR stages
    float4 *q_pos, *q_dir, *pred, *target;
    uint32_t *infer_list, *train_list;
    uint8_t *qflag;
    // capture (reference SoA layout, for parity readback)
    uint32_t capture;
    float *c_origin, *c_dir, *c_normal, *c_emis, *c_refl, *c_mis, *c_pdf, *c_nee, *c_L, *c_q;
    uint32_t *c_hit;
};

// The view that owns pixel p of the frame.
template <bool BATCH>
__device__ __forceinline__ const ViewDev &view_of(const FrameArgs &a, uint32_t p) {
    if constexpr (BATCH) {
        uint32_t v = a.vtab[p >> VIEW_SHIFT];
        while (p >= a.views[v].pix_end) v++;  // views smaller than a pixel group
        return a.views[v];
    } else {
        (void)p;
        return a.v0;
    }
}

// Bounce 0 of a single view takes its pixels in 8x4 tiles, so that a warp's
// primary rays, and through the queue order the secondary rays they spawn,
// start close together.  Slot i (< n0) is pixel p, or no pixel in the part of
// an edge tile outside the view.  A batched frame keeps the pixel order.
template <bool BATCH>
__device__ __forceinline__ bool bounce0_pixel(const FrameArgs &a, uint32_t i, uint32_t &p) {
    if constexpr (BATCH) {
        p = i;
        return i < a.P;
    } else {
        const uint32_t t = i >> 5, k = i & 31u;
        const uint32_t x = (t % a.tiles_x) * 8u + (k & 7u), y = (t / a.tiles_x) * 4u + (k >> 3);
        p = y * a.v0.W + x;
        return x < a.v0.W && y < a.v0.H;
    }
}

}  // namespace vrg
