// Roofline denominator measured on the device (no reference counterpart):
// the L2 read bandwidth that the BVH walks (closest hit, light-hit
// collection) are held against.  Their node and record fetches are served
// from L1/L2 while the trees fit in L2, so an HBM copy peak is the wrong
// yardstick for them.
//
// k_l2_read sweeps a buffer that fits in L2 (the GB300 has 126 MB over two
// dies) `reps` times with 16-byte loads that bypass L1 (ld.global.cg), four
// independent loads per thread and iteration, from a grid of several CTAs
// per SM; the XOR of the data goes to a sink only on an impossible value, so
// the loads cannot be dropped.
#include "vrg_internal.h"

namespace vrg {
namespace {

__global__ void __launch_bounds__(512) k_l2_read(const uint4 *__restrict__ buf, size_t n16, uint32_t reps,
                                                  uint32_t *sink) {
    uint32_t acc = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (uint32_t r = 0; r < reps; r++) {
        size_t i = t0;
        for (; i + 3 * stride < n16; i += 4 * stride) {
            const uint4 a = __ldcg(buf + i), b = __ldcg(buf + i + stride);
            const uint4 c = __ldcg(buf + i + 2 * stride), d = __ldcg(buf + i + 3 * stride);
            acc ^= ((a.x ^ a.y) ^ (a.z ^ a.w)) + ((b.x ^ b.y) ^ (b.z ^ b.w));
            acc ^= ((c.x ^ c.y) ^ (c.z ^ c.w)) + ((d.x ^ d.y) ^ (d.z ^ d.w));
        }
        for (; i < n16; i += stride) {
            const uint4 a = __ldcg(buf + i);
            acc ^= (a.x ^ a.y) ^ (a.z ^ a.w);
        }
    }
    if (acc == 0x9E3779B9u) atomicAdd(sink, 1u);
}

}  // namespace
}  // namespace vrg

using namespace vrg;

struct vrg_context : Context {};

extern "C" VRG_API vrg_status vrg_measure_l2_bandwidth(vrg_context *ctx, uint64_t bytes, uint32_t reps, float *gbs) {
    if (!ctx || !gbs || bytes < (1u << 20) || bytes > (96ull << 20) || reps == 0 || reps > 4096) {
        set_error("vrg_measure_l2_bandwidth: bytes must be 1..96 MiB, reps 1..4096");
        return VRG_ERR_INVALID_ARGUMENT;
    }
    *gbs = 0.0f;
    cudaStream_t s = ctx->stream;
    const size_t n16 = (size_t)bytes / 16;
    DevBufPtr buf;
    VRG_TRY(dev_alloc(s, n16 * 16 + 256, buf));
    uint4 *d = (uint4 *)buf->ptr;
    uint32_t *sink = (uint32_t *)((uint8_t *)buf->ptr + n16 * 16);
    VRG_CUDA_TRY(cudaMemsetAsync(buf->ptr, 0x5a, n16 * 16 + 256, s));
    int per_sm = 0;
    VRG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_l2_read, 512, 0));
    const int grid = std::max(1, ctx->num_sms) * std::max(1, per_sm);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    VRG_CUDA_TRY(cudaEventCreate(&e0));
    VRG_CUDA_TRY(cudaEventCreate(&e1));
    vrg_status st = VRG_OK;
    float ms = 0.0f;
    k_l2_read<<<grid, 512, 0, s>>>(d, n16, 2, sink);  // brings the buffer into L2
    if (cudaEventRecord(e0, s) != cudaSuccess) st = VRG_ERR_CUDA;
    k_l2_read<<<grid, 512, 0, s>>>(d, n16, reps, sink);
    if (cudaGetLastError() != cudaSuccess || cudaEventRecord(e1, s) != cudaSuccess ||
        cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
        set_error("vrg_measure_l2_bandwidth: launch or timing failed");
        st = VRG_ERR_CUDA;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st == VRG_OK && ms > 0.0f) *gbs = (float)((double)n16 * 16.0 * reps / (ms * 1e-3) / 1e9);
    return st;
}
