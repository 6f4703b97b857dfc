// gde_device.cuh -- small device helpers shared by the kernel translation units.
#pragma once
#include <cstdint>

namespace gde {

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
