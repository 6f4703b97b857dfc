// probe.cu -- the random-access ceiling the push kernel is measured against.
//
// A push is a 4-byte atomic add on a residual entry chosen by the graph, so
// the relevant ceiling is not the streaming HBM bandwidth but the rate of
// uniformly random float atomics (with their return value, which the
// crossing test needs) over an array of the residual slabs' size.  This
// kernel measures that rate: every thread issues `kIters` atomics at
// hashed-random indices, all taken modulo the array length, with the grid
// sized at 8 blocks of 256 threads per SM.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "gde.h"
#include "gde_common.cuh"
#include "gde_internal.h"

int gde_internal_fail(gde_ctx* ctx, int code, const char* msg);
void* gde_internal_wsget(gde_ctx* ctx, const char* name, size_t bytes);

namespace {

constexpr int kProbeThreads = 256;
constexpr int kProbeIters = 64;

// A 32-bit integer mix (xor-shift / multiply): spreads consecutive thread
// and step numbers over the whole index range.
__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

__global__ void probe_atomics_kernel(float* a, uint32_t n, int with_return, float* sink) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    float acc = 0.f;
    for (int k = 0; k < kProbeIters; ++k) {
        const uint32_t i = mix32(t * 977u + (uint32_t)k * 131u) % n;
        if (with_return) acc += atomicAdd(a + i, 1e-9f);
        else atomicAdd(a + i, 1e-9f);
    }
    if (acc == -1.f) sink[0] = acc;  // keeps the returned values live
}

}  // namespace

extern "C" int gde_probe_random_atomics(gde_ctx* ctx, int64_t n_floats, int with_return, double* gops_out) {
    if (!ctx) return GDE_EINVAL;
    if (!gops_out || n_floats < 1 || n_floats > (int64_t)UINT32_MAX)
        return gde_internal_fail(ctx, GDE_EINVAL, "probe size must be in [1, 2^32)");
    cudaSetDevice(ctx->device);
    float* a = (float*)gde_internal_wsget(ctx, "probe", (size_t)n_floats * 4 + 256);
    if (!a) return gde_internal_fail(ctx, GDE_ENOMEM, "probe array");
    float* sink = a + n_floats;
    cudaStream_t st = ctx->stream;
    if (cudaMemsetAsync(a, 0, (size_t)n_floats * 4, st) != cudaSuccess)
        return gde_internal_fail(ctx, GDE_ECUDA, "probe memset");
    const int blocks = std::max(1, ctx->sms) * 8;
    const double ops = (double)blocks * kProbeThreads * kProbeIters;
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {  // the first launch warms up; the best of the rest counts
        cudaEventRecord(ctx->ev[0], st);
        probe_atomics_kernel<<<blocks, kProbeThreads, 0, st>>>(a, (uint32_t)n_floats, with_return, sink);
        cudaEventRecord(ctx->ev[1], st);
        if (cudaEventSynchronize(ctx->ev[1]) != cudaSuccess || cudaGetLastError() != cudaSuccess)
            return gde_internal_fail(ctx, GDE_ECUDA, "probe kernel");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
        if (rep > 0) best = std::min(best, ms);
    }
    *gops_out = ops / (best * 1e-3) / 1e9;
    return GDE_OK;
}
