// Batched GPU binned-SAH BVH builder reproducing bvh/build.rs exactly.
//
// The reference builds recursively (subdivide, build.rs:130-233): a node
// with n > 2 prims is split at the best of 3 axes x 31 planes over 32
// centroid bins (find_best_plane, build.rs:45-128), its prim indices are
// partitioned in place, and the two children are appended to the node list
// together before the left subtree is built.  The index of every node is
// therefore a closed form of the split sizes: a node whose children start at
// `base` puts its left child at base, its right child at base+1, the left
// child's children at base+2 and the right child's at base + 2*n_left (a
// subtree of k leaves has 2k-1 nodes).  This builder runs the recursion
// level by level over all trees of a batch at once, one warp per node,
// carrying (node index, children base) so the node array comes out in the
// reference's order without a renumbering pass.
//
// Per node the warp: reduces the node AABB and centroid bounds
// (order-independent min/max), bins prims per axis with shared-memory atomic
// counts and ordered-integer atomic min/max (exact), evaluates the 93 plane
// costs with the reference's float expression, takes the first minimum in
// (axis, plane) order, and partitions the node's slice with a warp-parallel
// two-sided (Hoare) pass: the k-th predicate-false element from the left is
// swapped with the k-th predicate-true element from the right, the pairing
// of the serial two-pointer partition.
#include <cfloat>
#include <mutex>

#include "vrg_internal.h"

namespace vrg {

namespace {

struct Item {
    uint32_t tree, node, base, first, count, parent;
};

constexpr int SAH_WARPS = 8;
constexpr int NB = 32;

__device__ __forceinline__ int f2o(float f) {
    int b = __float_as_int(f);
    return b ^ ((b >> 31) & 0x7FFFFFFF);
}
__device__ __forceinline__ float o2f(int o) { return __int_as_float(o ^ ((o >> 31) & 0x7FFFFFFF)); }

__device__ __forceinline__ uint32_t bin_index(float v) {  // Rust `as usize` then min(31)
    if (!(v > 0.0f)) return 0;
    if (v >= 31.0f) return 31;
    return (uint32_t)v;
}

__device__ __forceinline__ float area_of(float lx, float ly, float lz, float hx, float hy, float hz) {
    float dx = hx - lx, dy = hy - ly, dz = hz - lz;
    return 2.0f * ((dx * dy + dx * dz) + dy * dz);  // aabb.rs:44-52
}

__device__ __forceinline__ float wmin(float v) {
    for (int o = 16; o; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float wmax(float v) {
    for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ void write_leaf(const SahInputs &in, const SahOutputs &out, const SahTree &T, uint32_t node,
                           uint32_t parent, uint32_t p) {
    uint32_t g = T.prim_off + p;
    float4 lo = in.lo[g], hi = in.hi[g], c = in.cen[g];
    vrg_bvh_node n;
    n.left_node_idx = INVALID;
    n.right_node_idx_or_prim_idx = in.id[g];
    n.min[0] = lo.x; n.min[1] = lo.y; n.min[2] = lo.z;
    n.power = c.w;
    n.max[0] = hi.x; n.max[1] = hi.y; n.max[2] = hi.z;
    n.parent_idx = parent;
    out.nodes[T.node_off + node] = n;
    out.leaf_prim[T.node_off + node] = p;
}

__device__ void write_internal(const SahOutputs &out, const SahTree &T, uint32_t node, uint32_t parent,
                               uint32_t base, const float lo[3], const float hi[3]) {
    const float pad = 0.0001f;  // build.rs:300
    vrg_bvh_node n;
    n.left_node_idx = base;
    n.right_node_idx_or_prim_idx = base + 1;
    for (int k = 0; k < 3; k++) { n.min[k] = lo[k] - pad; n.max[k] = hi[k] + pad; }
    n.power = 0.0f;
    n.parent_idx = parent;
    out.nodes[T.node_off + node] = n;
    out.leaf_prim[T.node_off + node] = INVALID;
}

// node with exactly two prims: internal node + two leaves in current order
__device__ void write_pair(const SahInputs &in, const SahOutputs &out, const SahTree &T, uint32_t node,
                           uint32_t parent, uint32_t base, uint32_t first) {
    uint32_t p0 = out.perm[T.prim_off + first], p1 = out.perm[T.prim_off + first + 1];
    float4 a0 = in.lo[T.prim_off + p0], b0 = in.hi[T.prim_off + p0];
    float4 a1 = in.lo[T.prim_off + p1], b1 = in.hi[T.prim_off + p1];
    float lo[3] = {fminf(a0.x, a1.x), fminf(a0.y, a1.y), fminf(a0.z, a1.z)};
    float hi[3] = {fmaxf(b0.x, b1.x), fmaxf(b0.y, b1.y), fmaxf(b0.z, b1.z)};
    write_internal(out, T, node, parent, base, lo, hi);
    write_leaf(in, out, T, base, node, p0);
    write_leaf(in, out, T, base + 1, node, p1);
}

__global__ void k_perm_init(const SahTree *trees, uint32_t *perm) {
    SahTree T = trees[blockIdx.y];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < T.n; i += gridDim.x * blockDim.x)
        perm[T.prim_off + i] = i;
}

__global__ void __launch_bounds__(SAH_WARPS * 32) k_sah_level(const SahTree *trees, SahInputs in, SahOutputs out,
                                                              const Item *items, const uint32_t *n_items_p,
                                                              Item *next, uint32_t *n_next) {
    __shared__ int s_cnt[SAH_WARPS][3 * NB];
    __shared__ int s_lo[SAH_WARPS][3 * NB][3];
    __shared__ int s_hi[SAH_WARPS][3 * NB][3];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t n_items = *n_items_p;
    for (uint32_t it = blockIdx.x * SAH_WARPS + w; it < n_items; it += gridDim.x * SAH_WARPS) {
        const Item I = items[it];
        const SahTree T = trees[I.tree];
        const uint32_t c = I.count;
        uint32_t *perm = out.perm + T.prim_off + I.first;
        if (c == 1) {
            if (lane == 0) write_leaf(in, out, T, I.node, I.parent, perm[0]);
            continue;
        }
        if (c == 2) {
            if (lane == 0) write_pair(in, out, T, I.node, I.parent, I.base, I.first);
            continue;
        }
        // node AABB (blas_leaf_bounds, build.rs:36-43) and centroid bounds (build.rs:60-66)
        float nlo[3] = {INFINITY, INFINITY, INFINITY}, nhi[3] = {-INFINITY, -INFINITY, -INFINITY};
        float clo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, chi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (uint32_t i = lane; i < c; i += 32) {
            uint32_t g = T.prim_off + perm[i];
            float4 a = in.lo[g], b = in.hi[g], m = in.cen[g];
            nlo[0] = fminf(nlo[0], a.x); nlo[1] = fminf(nlo[1], a.y); nlo[2] = fminf(nlo[2], a.z);
            nhi[0] = fmaxf(nhi[0], b.x); nhi[1] = fmaxf(nhi[1], b.y); nhi[2] = fmaxf(nhi[2], b.z);
            clo[0] = fminf(clo[0], m.x); clo[1] = fminf(clo[1], m.y); clo[2] = fminf(clo[2], m.z);
            chi[0] = fmaxf(chi[0], m.x); chi[1] = fmaxf(chi[1], m.y); chi[2] = fmaxf(chi[2], m.z);
        }
        for (int k = 0; k < 3; k++) {
            nlo[k] = wmin(nlo[k]); nhi[k] = wmax(nhi[k]);
            clo[k] = wmin(clo[k]); chi[k] = wmax(chi[k]);
        }
        // bins (build.rs:68-85)
        for (int b = lane; b < 3 * NB; b += 32) {
            s_cnt[w][b] = 0;
            for (int k = 0; k < 3; k++) { s_lo[w][b][k] = f2o(INFINITY); s_hi[w][b][k] = f2o(-INFINITY); }
        }
        __syncwarp();
        float scale[3];
        for (int d = 0; d < 3; d++) scale[d] = (float)NB / (chi[d] - clo[d]);
        for (uint32_t i = lane; i < c; i += 32) {
            uint32_t g = T.prim_off + perm[i];
            float4 a = in.lo[g], b = in.hi[g], m = in.cen[g];
            float cc[3] = {m.x, m.y, m.z};
            for (int d = 0; d < 3; d++) {
                int bi = d * NB + (int)bin_index((cc[d] - clo[d]) * scale[d]);
                atomicAdd(&s_cnt[w][bi], 1);
                atomicMin(&s_lo[w][bi][0], f2o(a.x)); atomicMin(&s_lo[w][bi][1], f2o(a.y));
                atomicMin(&s_lo[w][bi][2], f2o(a.z));
                atomicMax(&s_hi[w][bi][0], f2o(b.x)); atomicMax(&s_hi[w][bi][1], f2o(b.y));
                atomicMax(&s_hi[w][bi][2], f2o(b.z));
            }
        }
        __syncwarp();
        // plane costs (build.rs:87-125): lane p < 31 evaluates plane p of each axis
        float best_cost = FLT_MAX;
        int best_key = 0x7FFFFFFF;
        if (lane < NB - 1) {
            for (int d = 0; d < 3; d++) {
                uint32_t nl = 0, nr = 0;
                float l0 = INFINITY, l1 = INFINITY, l2 = INFINITY, h0 = -INFINITY, h1 = -INFINITY, h2 = -INFINITY;
                float r0 = INFINITY, r1 = INFINITY, r2 = INFINITY, g0 = -INFINITY, g1 = -INFINITY, g2 = -INFINITY;
                for (int b = 0; b < NB; b++) {
                    int bi = d * NB + b;
                    int cnt = s_cnt[w][bi];
                    if (cnt == 0) continue;
                    float a0 = o2f(s_lo[w][bi][0]), a1 = o2f(s_lo[w][bi][1]), a2 = o2f(s_lo[w][bi][2]);
                    float b0 = o2f(s_hi[w][bi][0]), b1 = o2f(s_hi[w][bi][1]), b2 = o2f(s_hi[w][bi][2]);
                    if (b <= lane) {
                        nl += (uint32_t)cnt;
                        l0 = fminf(l0, a0); l1 = fminf(l1, a1); l2 = fminf(l2, a2);
                        h0 = fmaxf(h0, b0); h1 = fmaxf(h1, b1); h2 = fmaxf(h2, b2);
                    } else {
                        nr += (uint32_t)cnt;
                        r0 = fminf(r0, a0); r1 = fminf(r1, a1); r2 = fminf(r2, a2);
                        g0 = fmaxf(g0, b0); g1 = fmaxf(g1, b1); g2 = fmaxf(g2, b2);
                    }
                }
                float al = nl ? area_of(l0, l1, l2, h0, h1, h2) : 0.0f;
                float ar = nr ? area_of(r0, r1, r2, g0, g1, g2) : 0.0f;
                float cost = al * (float)nl + ar * (float)nr;
                int key = d * (NB - 1) + lane;
                if (cost < best_cost) { best_cost = cost; best_key = key; }  // strict <, first in order
            }
        }
        // first minimum over (axis, plane) order; NaN costs never compare less
        for (int o = 16; o; o >>= 1) {
            float oc = __shfl_xor_sync(0xffffffffu, best_cost, o);
            int ok = __shfl_xor_sync(0xffffffffu, best_key, o);
            if (oc < best_cost || (oc == best_cost && ok < best_key)) { best_cost = oc; best_key = ok; }
        }
        uint32_t dim = 0;
        float split = 0.0f;
        if (best_key != 0x7FFFFFFF && best_cost < FLT_MAX) {
            dim = (uint32_t)(best_key / (NB - 1));
            int pl = best_key % (NB - 1);
            float lo_d = dim == 0 ? clo[0] : (dim == 1 ? clo[1] : clo[2]);
            float hi_d = dim == 0 ? chi[0] : (dim == 1 ? chi[1] : chi[2]);
            split = lo_d + ((float)pl + 1.0f) * ((hi_d - lo_d) / (float)NB);
        }
        // count trues
        uint32_t n_true = 0;
        for (uint32_t base = 0; base < c; base += 32) {
            uint32_t i = base + lane;
            bool pr = false;
            if (i < c) {
                float4 m = in.cen[T.prim_off + perm[i]];
                pr = (dim == 0 ? m.x : (dim == 1 ? m.y : m.z)) < split;
            }
            n_true += __popc(__ballot_sync(0xffffffffu, pr));
        }
        uint32_t n_left;
        if (n_true == 0 || n_true == c) {
            n_left = c / 2;  // build.rs:151-157, current order kept
        } else {
            n_left = n_true;
            // two-sided partition: left region [0, n_true) ascending looking for
            // false, right region [n_true, c) descending looking for true
            uint32_t L = 0;
            int32_t R = (int32_t)c - 1;
            uint32_t lmask = 0, rmask = 0;
            uint32_t lval = 0, rval = 0;
            bool lload = true, rload = true;
            while (true) {
                if (lload) {
                    if (L >= n_true) break;
                    uint32_t i = L + lane;
                    bool f = false;
                    if (i < n_true) {
                        lval = perm[i];
                        float4 m = in.cen[T.prim_off + lval];
                        f = !((dim == 0 ? m.x : (dim == 1 ? m.y : m.z)) < split);
                    }
                    lmask = __ballot_sync(0xffffffffu, f);
                    lload = false;
                }
                if (rload) {
                    if (R < (int32_t)n_true) break;  // unreachable: both regions hold m misplaced
                    int32_t i = R - lane;
                    bool t = false;
                    if (i >= (int32_t)n_true) {
                        rval = perm[i];
                        float4 m = in.cen[T.prim_off + rval];
                        t = (dim == 0 ? m.x : (dim == 1 ? m.y : m.z)) < split;
                    }
                    rmask = __ballot_sync(0xffffffffu, t);
                    rload = false;
                }
                if (lmask == 0) { L += 32; lload = true; continue; }
                if (rmask == 0) { R -= 32; rload = true; continue; }
                uint32_t k = min(__popc(lmask), __popc(rmask));
                // lanes holding the first k set bits of each mask pair by rank
                uint32_t lrank = __popc(lmask & ((1u << lane) - 1u));
                uint32_t rrank = __popc(rmask & ((1u << lane) - 1u));
                bool lact = ((lmask >> lane) & 1u) && lrank < k;
                bool ract = ((rmask >> lane) & 1u) && rrank < k;
                int lpartner = lact ? (int)__fns(rmask, 0, (int)lrank + 1) : lane;
                int rpartner = ract ? (int)__fns(lmask, 0, (int)rrank + 1) : lane;
                uint32_t from_r = __shfl_sync(0xffffffffu, rval, lpartner);
                uint32_t from_l = __shfl_sync(0xffffffffu, lval, rpartner);
                if (lact) perm[L + lane] = from_r;
                if (ract) perm[R - lane] = from_l;
                __syncwarp();
                // drop the paired bits (the lowest k set bits of each mask)
                for (uint32_t j = 0; j < k; j++) { lmask &= lmask - 1u; rmask &= rmask - 1u; }
            }
        }
        __syncwarp();
        if (lane == 0) {
            write_internal(out, T, I.node, I.parent, I.base, nlo, nhi);
            uint32_t ln = I.base, rn = I.base + 1;
            uint32_t lbase = I.base + 2, rbase = I.base + 2 * n_left;
            uint32_t counts[2] = {n_left, c - n_left};
            uint32_t nodes[2] = {ln, rn};
            uint32_t bases[2] = {lbase, rbase};
            uint32_t firsts[2] = {I.first, I.first + n_left};
            for (int s = 0; s < 2; s++) {
                if (counts[s] == 1) write_leaf(in, out, T, nodes[s], I.node, out.perm[T.prim_off + firsts[s]]);
                else if (counts[s] == 2) write_pair(in, out, T, nodes[s], I.node, bases[s], firsts[s]);
                else {
                    uint32_t slot = atomicAdd(n_next, 1u);
                    next[slot] = Item{I.tree, nodes[s], bases[s], firsts[s], counts[s], I.node};
                }
            }
        }
        __syncwarp();
    }
}

// power of an internal node = (0 + left) + right, bottom-up (build.rs:341-357)
__global__ void k_power_up(const SahTree *trees, vrg_bvh_node *nodes, uint32_t *arrive) {
    SahTree T = trees[blockIdx.y];
    if (T.n == 0) return;
    uint32_t n_nodes = 2 * T.n - 1;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_nodes; i += gridDim.x * blockDim.x) {
        vrg_bvh_node *base = nodes + T.node_off;
        if (base[i].left_node_idx != INVALID) continue;
        uint32_t cur = i;
        for (uint32_t guard = 0; guard < n_nodes; guard++) {
            uint32_t parent = base[cur].parent_idx;
            if (parent == INVALID) break;
            __threadfence();
            if (atomicAdd(&arrive[T.node_off + parent], 1u) == 0) break;  // sibling not done yet
            __threadfence();
            volatile vrg_bvh_node *vb = base;
            float lp = vb[vb[parent].left_node_idx].power;
            float rp = vb[vb[parent].right_node_idx_or_prim_idx].power;
            float p = 0.0f;
            p += lp;
            p += rp;
            vb[parent].power = p;
            cur = parent;
        }
    }
}

}  // namespace

vrg_status sah_build(cudaStream_t s, const std::vector<SahTree> &trees, uint32_t total_prims,
                     uint32_t total_nodes, const SahInputs &in, const SahOutputs &out, uint32_t *levels) {
    if (trees.empty() || total_prims == 0) {
        if (levels) *levels = 0;
        return VRG_OK;
    }
    const uint32_t nt = (uint32_t)trees.size();
    if (nt > 65535) {
        set_error("sah_build: %u trees exceeds one launch (65535)", nt);
        return VRG_ERR_UNSUPPORTED;
    }
    uint32_t max_n = 0;
    std::vector<Item> roots;
    for (uint32_t t = 0; t < nt; t++) {
        max_n = std::max(max_n, trees[t].n);
        if (trees[t].n) roots.push_back(Item{t, 0, 1, 0, trees[t].n, INVALID});
    }
    // scratch: trees, two item queues, counters, arrival flags
    size_t q_cap = std::max<size_t>(roots.size(), total_prims / 3 + 1);
    size_t bytes = nt * sizeof(SahTree) + 2 * q_cap * sizeof(Item) + 64 + (size_t)total_nodes * 4;
    DevBufPtr scratch;
    VRG_TRY(dev_alloc(s, bytes, scratch));
    uint8_t *p = (uint8_t *)scratch->ptr;
    SahTree *d_trees = (SahTree *)p; p += nt * sizeof(SahTree);
    Item *q0 = (Item *)p; p += q_cap * sizeof(Item);
    Item *q1 = (Item *)p; p += q_cap * sizeof(Item);
    uint32_t *cnt = (uint32_t *)p; p += 64;
    uint32_t *arrive = (uint32_t *)p;
    uint32_t *h_cnt = nullptr;
    VRG_CUDA_TRY(cudaMallocHost(&h_cnt, 16));
    std::unique_ptr<uint32_t, void (*)(uint32_t *)> h_guard(h_cnt, [](uint32_t *x) { cudaFreeHost(x); });
    VRG_CUDA_TRY(cudaMemcpyAsync(d_trees, trees.data(), nt * sizeof(SahTree), cudaMemcpyHostToDevice, s));
    VRG_CUDA_TRY(cudaMemcpyAsync(q0, roots.data(), roots.size() * sizeof(Item), cudaMemcpyHostToDevice, s));
    uint32_t n_roots = (uint32_t)roots.size();
    VRG_CUDA_TRY(cudaMemcpyAsync(cnt, &n_roots, 4, cudaMemcpyHostToDevice, s));
    VRG_CUDA_TRY(cudaMemsetAsync(arrive, 0, (size_t)total_nodes * 4, s));
    {
        dim3 g(std::max(1u, std::min(1024u, (max_n + 255) / 256)), nt);
        k_perm_init<<<g, 256, 0, s>>>(d_trees, out.perm);
        VRG_CUDA_TRY(cudaGetLastError());
    }
    uint32_t n_cur = n_roots, lv = 0;
    Item *cur = q0, *nxt = q1;
    uint32_t cur_slot = 0;
    while (n_cur > 0) {
        uint32_t next_slot = cur_slot ^ 1u;
        VRG_CUDA_TRY(cudaMemsetAsync(cnt + next_slot, 0, 4, s));
        uint32_t blocks = std::min<uint32_t>((n_cur + SAH_WARPS - 1) / SAH_WARPS, 152u * 16u);
        k_sah_level<<<blocks, SAH_WARPS * 32, 0, s>>>(d_trees, in, out, cur, cnt + cur_slot, nxt, cnt + next_slot);
        VRG_CUDA_TRY(cudaGetLastError());
        VRG_CUDA_TRY(cudaMemcpyAsync(h_cnt, cnt + next_slot, 4, cudaMemcpyDeviceToHost, s));
        VRG_CUDA_TRY(cudaStreamSynchronize(s));
        n_cur = *h_cnt;
        std::swap(cur, nxt);
        cur_slot = next_slot;
        lv++;
        if (lv > 100000) {
            set_error("sah_build: level loop did not terminate");
            return VRG_ERR_STATE;
        }
    }
    {
        uint32_t max_nodes = 2 * max_n - 1;
        dim3 g(std::max(1u, std::min(1024u, (max_nodes + 255) / 256)), nt);
        k_power_up<<<g, 256, 0, s>>>(d_trees, out.nodes, arrive);
        VRG_CUDA_TRY(cudaGetLastError());
    }
    if (levels) *levels = lv;
    return VRG_OK;
}

}  // namespace vrg

namespace vrg {

// ---------------------------------------------------------------------------
// Build without allocating: vrg_build_tl_bvh_noalloc
//
// For callers that must not allocate device memory while they run: a game or
// engine that owns the whole device-memory budget and hands this library
// only the buffers it has set aside, or a chunk-streaming worker that builds
// BVHs next to a frame in flight, where cudaMalloc/cudaFree may synchronize
// the device and stall the frame.  The builder's scratch (work queues,
// level counters, bottom-up arrival flags, prepared prim bounds) lives in
// the fixed device array below instead of a cudaMallocAsync allocation.
// ---------------------------------------------------------------------------

namespace {

constexpr uint32_t NOALLOC_MAX_PRIMS = 32768;  // one chunk's worth of blocks
constexpr size_t NOALLOC_QCAP = NOALLOC_MAX_PRIMS / 3 + 2;
constexpr size_t NOALLOC_OFF_LO = 0;
constexpr size_t NOALLOC_OFF_HI = NOALLOC_OFF_LO + (size_t)NOALLOC_MAX_PRIMS * 16;
constexpr size_t NOALLOC_OFF_CEN = NOALLOC_OFF_HI + (size_t)NOALLOC_MAX_PRIMS * 16;
constexpr size_t NOALLOC_OFF_Q0 = NOALLOC_OFF_CEN + (size_t)NOALLOC_MAX_PRIMS * 16;
constexpr size_t NOALLOC_OFF_Q1 = NOALLOC_OFF_Q0 + NOALLOC_QCAP * sizeof(Item);
constexpr size_t NOALLOC_OFF_CNT = (NOALLOC_OFF_Q1 + NOALLOC_QCAP * sizeof(Item) + 255) & ~(size_t)255;
constexpr size_t NOALLOC_OFF_TREE = NOALLOC_OFF_CNT + 256;
constexpr size_t NOALLOC_OFF_ARRIVE = NOALLOC_OFF_TREE + 256;
constexpr size_t NOALLOC_OFF_LEAF = NOALLOC_OFF_ARRIVE + (size_t)2 * NOALLOC_MAX_PRIMS * 4;
constexpr size_t NOALLOC_BYTES = NOALLOC_OFF_LEAF + (size_t)2 * NOALLOC_MAX_PRIMS * 4;  // about 2.4 MiB

// inputs of build_tl_bvh with identity isometries: AABB as given, centroid
// (min+max)/2 (build.rs:391-400), w = power
__global__ void k_noalloc_prep(const float *aabbs, const float *power, uint32_t n, float4 *lo, float4 *hi,
                               float4 *cen) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *a = aabbs + 6 * (size_t)i;
    float l[3], h[3];
    for (int k = 0; k < 3; k++) {
        float x0 = a[k] + 0.0f, x1 = a[3 + k] + 0.0f;  // translation by zero, as k_tl_inputs
        l[k] = fminf(x0, x1);
        h[k] = fmaxf(x0, x1);
    }
    lo[i] = make_float4(l[0], l[1], l[2], 0.0f);
    hi[i] = make_float4(h[0], h[1], h[2], 0.0f);
    cen[i] = make_float4((l[0] + h[0]) / 2.0f, (l[1] + h[1]) / 2.0f, (l[2] + h[2]) / 2.0f, power[i]);
}

}  // namespace
}  // namespace vrg

// The scratch array every call of vrg_build_tl_bvh_noalloc shares.  Each GPU
// that loads the library holds it until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[vrg::NOALLOC_BYTES];

extern "C" VRG_API vrg_status vrg_build_tl_bvh_noalloc(const float *aabbs, const float *power, const uint32_t *ids,
                                                       uint32_t n, vrg_bvh_node *nodes, uint32_t *prim_order,
                                                       void *stream) {
    using namespace vrg;
    if (!aabbs || !power || !ids || !nodes || !prim_order || n == 0) {
        set_error("vrg_build_tl_bvh_noalloc: null pointer or n == 0");
        return VRG_ERR_INVALID_ARGUMENT;
    }
    if (n > NOALLOC_MAX_PRIMS) {
        set_error("vrg_build_tl_bvh_noalloc: %u prims exceed the fixed scratch capacity of %u prims", n,
                  NOALLOC_MAX_PRIMS);
        return VRG_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t s = (cudaStream_t)stream;
    // The device address of the array in the context current now (its name in
    // host code is only a host-side stand-in).  Looked up on every call, so a
    // device reset or another current context never leaves a stale address;
    // the lookup allocates nothing.
    void *base = nullptr;
    {
        cudaError_t e = cudaGetSymbolAddress(&base, g_noalloc_scratch);
        if (e != cudaSuccess || !base) {
            set_error("cudaGetSymbolAddress(g_noalloc_scratch) failed: %s", cudaGetErrorString(e));
            return VRG_ERR_CUDA;
        }
    }
    // Everything from the first enqueue on: on an error return the stream is
    // synchronized first, so no work that uses the shared array is still
    // queued when the call returns.
    auto build = [&]() -> vrg_status {
        uint8_t *B = (uint8_t *)base;
        float4 *lo = (float4 *)(B + NOALLOC_OFF_LO), *hi = (float4 *)(B + NOALLOC_OFF_HI),
               *cen = (float4 *)(B + NOALLOC_OFF_CEN);
        Item *q0 = (Item *)(B + NOALLOC_OFF_Q0), *q1 = (Item *)(B + NOALLOC_OFF_Q1);
        uint32_t *cnt = (uint32_t *)(B + NOALLOC_OFF_CNT);
        SahTree *d_tree = (SahTree *)(B + NOALLOC_OFF_TREE);
        uint32_t *arrive = (uint32_t *)(B + NOALLOC_OFF_ARRIVE);
        uint32_t *leaf = (uint32_t *)(B + NOALLOC_OFF_LEAF);
        const uint32_t n_nodes = 2 * n - 1;
        // the array keeps the previous call's contents: reset what must start at zero
        VRG_CUDA_TRY(cudaMemsetAsync(arrive, 0, (size_t)n_nodes * 4, s));
        VRG_CUDA_TRY(cudaMemsetAsync(cnt, 0, 256, s));
        // tree descriptor and root work item: copies of host stack values
        SahTree tree{n, 0, 0, 0};
        Item root{0, 0, 1, 0, n, INVALID};
        uint32_t one = 1;
        VRG_CUDA_TRY(cudaMemcpyAsync(d_tree, &tree, sizeof(tree), cudaMemcpyHostToDevice, s));
        VRG_CUDA_TRY(cudaMemcpyAsync(q0, &root, sizeof(root), cudaMemcpyHostToDevice, s));
        VRG_CUDA_TRY(cudaMemcpyAsync(cnt, &one, 4, cudaMemcpyHostToDevice, s));
        k_noalloc_prep<<<(n + 255) / 256, 256, 0, s>>>(aabbs, power, n, lo, hi, cen);
        VRG_CUDA_TRY(cudaGetLastError());
        SahInputs in{lo, hi, cen, ids};
        SahOutputs out{nodes, prim_order, leaf};
        k_perm_init<<<dim3(std::max(1u, (n + 255) / 256), 1), 256, 0, s>>>(d_tree, prim_order);
        VRG_CUDA_TRY(cudaGetLastError());
        uint32_t n_cur = 1, cur_slot = 0, lv = 0;
        Item *cur = q0, *nxt = q1;
        while (n_cur > 0) {
            uint32_t next_slot = cur_slot ^ 1u;
            VRG_CUDA_TRY(cudaMemsetAsync(cnt + next_slot, 0, 4, s));
            uint32_t blocks = std::min<uint32_t>((n_cur + SAH_WARPS - 1) / SAH_WARPS, 152u * 16u);
            k_sah_level<<<blocks, SAH_WARPS * 32, 0, s>>>(d_tree, in, out, cur, cnt + cur_slot, nxt, cnt + next_slot);
            VRG_CUDA_TRY(cudaGetLastError());
            uint32_t h_next = 0;
            VRG_CUDA_TRY(cudaMemcpyAsync(&h_next, cnt + next_slot, 4, cudaMemcpyDeviceToHost, s));
            VRG_CUDA_TRY(cudaStreamSynchronize(s));
            n_cur = h_next;
            std::swap(cur, nxt);
            cur_slot = next_slot;
            if (++lv > 4 * NOALLOC_MAX_PRIMS) {
                set_error("vrg_build_tl_bvh_noalloc: level loop did not terminate");
                return VRG_ERR_STATE;
            }
        }
        k_power_up<<<dim3(std::max(1u, (n_nodes + 255) / 256), 1), 256, 0, s>>>(d_tree, nodes, arrive);
        VRG_CUDA_TRY(cudaGetLastError());
        VRG_CUDA_TRY(cudaStreamSynchronize(s));
        return VRG_OK;
    };
    const vrg_status st = build();
    if (st != VRG_OK) (void)cudaStreamSynchronize(s);
    return st;
}
