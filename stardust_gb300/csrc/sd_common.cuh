// sd_common.cuh -- shared device helpers for the stardust-gb300 kernels.
//
// Every kernel in this library is compiled with -fmad=false: each float
// operation rounds once, in the order written, so results are reproducible
// bit-for-bit by the plain-C restatement that the tests compare against.
// Where a fused multiply-add is part of the specification (the reference's
// in-cell offset, sh_collision_detection.cu:66) it is written explicitly
// as __fmaf_rn.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/stardust.h"
#include "sd_internal.h"

namespace sd {

constexpr int kWarp = 32;

// Bounded spin: a wait on another CTA's flag gives up after this many polls
// (with a short back-off), records kErrLookbackTimeout and carries on, so a
// kernel never hangs the GPU.  Far above any legitimate wait (a predecessor
// CTA that is already resident publishes within microseconds).
constexpr uint32_t kSpinLimit = 1u << 22;

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & (kWarp - 1); }

// Inclusive warp scan of a u32.
__device__ __forceinline__ uint32_t warp_inclusive_scan(uint32_t v) {
#pragma unroll
    for (int o = 1; o < kWarp; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane_id() >= (uint32_t)o) v += t;
    }
    return v;
}

// Exclusive scan over the block of one u32 per thread (blockDim.x <= 1024,
// a multiple of 32).  `ws` is shared scratch of >= 33 words.  Returns the
// exclusive prefix; *total receives the block sum.  Contains __syncthreads.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* ws, uint32_t* total) {
    const int nwarps = blockDim.x / kWarp;
    const int w = threadIdx.x / kWarp;
    uint32_t inc = warp_inclusive_scan(v);
    if (lane_id() == kWarp - 1) ws[w] = inc;
    __syncthreads();
    if (w == 0) {
        uint32_t x = lane_id() < (uint32_t)nwarps ? ws[lane_id()] : 0u;
        uint32_t xi = warp_inclusive_scan(x);
        if (lane_id() < (uint32_t)nwarps) ws[lane_id()] = xi - x;
        if (lane_id() == (uint32_t)nwarps - 1) ws[32] = xi;
    }
    __syncthreads();
    uint32_t r = ws[w] + inc - v;
    *total = ws[32];
    __syncthreads();
    return r;
}

}  // namespace sd
