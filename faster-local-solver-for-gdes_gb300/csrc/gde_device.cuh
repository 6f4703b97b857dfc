// gde_device.cuh -- small device helpers shared by the kernel translation units.
#pragma once
#include <cstdint>

#include "gde_common.cuh"

namespace gde {

constexpr unsigned long long kSpinLimit = 1ull << 26;  // ~ seconds of polling

// ---------------------------------------------------------------------------
// Bounded grid barrier (sense by generation counter).  Co-residency of all
// blocks is guaranteed by the cooperative launch; the spin limit only guards
// against a bug turning into a hang: on expiry the block records GDE_EHANG
// and every block leaves its loop at the next barrier.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned ld_volatile(const unsigned* p) { return *(volatile const unsigned*)p; }
__device__ __forceinline__ int ld_volatile_i(const int* p) { return *(volatile const int*)p; }
// A load that later loads of this thread cannot pass (device-scope acquire).
__device__ __forceinline__ int ld_acquire_gpu_i(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// `limit` polls (0: kSpinLimit) before a waiting block gives up; `members`
// blocks meet at `bar` (0: the whole grid).
__device__ __forceinline__ bool grid_barrier(GridBarrier* bar, int* err, unsigned long long limit = 0,
                                             unsigned members = 0) {
    if (limit == 0) limit = kSpinLimit;
    if (members == 0) members = gridDim.x;
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        unsigned gen = ld_volatile(&bar->gen);
        __threadfence();
        unsigned arrived = atomicAdd(&bar->count, 1u);
        if (arrived == members - 1) {
            atomicExch(&bar->count, 0u);
            __threadfence();
            atomicAdd(&bar->gen, 1u);
        } else {
            unsigned long long spins = 0;
            while (ld_volatile(&bar->gen) == gen) {
                if (ld_volatile_i(err) != 0) { ok = 0; break; }
                if (++spins > limit) { atomicCAS(err, 0, GDE_EHANG); ok = 0; break; }
                __nanosleep(100);
            }
        }
        __threadfence();
        if (ld_volatile_i(err) != 0) ok = 0;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}


// Device-wide nanosecond clock (PTX %globaltimer).
__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Append v to a candidate list once per stamp (mark dedup), one atomic per
// warp for all appending lanes.  `mask` must name every lane executing the
// call.
__device__ __forceinline__ void append_once(bool want, int v, int32_t* mark, int stamp, int32_t* list, int* cnt,
                                            unsigned mask) {
    bool app = false;
    if (want) {
        if (mark[v] != stamp) app = (atomicExch(&mark[v], stamp) != stamp);
    }
    unsigned b = __ballot_sync(mask, app);
    if (b) {
        int lane = threadIdx.x & 31;
        int leader = __ffs(b) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(cnt, __popc(b));
        base = __shfl_sync(mask, base, leader);
        if (app) list[base + __popc(b & ((1u << lane) - 1u))] = v;
    }
}

}  // namespace gde
