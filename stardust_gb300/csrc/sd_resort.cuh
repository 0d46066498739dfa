// sd_resort.cuh -- device side of the incremental re-sort, shared by the
// scan kernel (sd_resort.cu) and the contact kernel, which does the scan's
// work itself for scenes without clumps (it holds each sphere's new key).
//
// A block appends its moved slots -- new key differs from the sorted key the
// slot sits under -- to a list as (key << 32 | slot), one atomic per block
// (the list's order does not matter: it is sorted next).  The last block to
// finish (a fence and an arrival counter, no waiting) publishes the count M
// and, in 8 KB of shared memory, sorts the list by (key, slot), then the
// moved slots alone; moved entry r (rank r in (key, slot) order) goes to
// sorted position r + (unmoved slots sorting before it).  The previous
// step's cell table bounds the slots of its key, so that count is its slot
// clamped to that range minus the moved slots below the clamp.  The reorder
// then reads the whole order from these lists.
#pragma once

#include <stdint.h>

#include "sd_common.cuh"
#include "sd_internal.h"

namespace sd {

struct ResortArgs {
    const uint32_t* keys_prev;  // null: the re-sort is off for this launch
    unsigned long long* list;   // kResortMaxCap entries
    uint32_t* pos;              // per moved entry: its sorted position
    uint32_t* q;                // per moved slot, ascending: slot - rank
    uint32_t* scratch;          // [0] running count, [1] M, [2] arrivals
    const uint32_t* cell_start;
    uint32_t n, ncells, mmax;
};

// Sorts v[0, P) ascending in shared memory (P a power of two; every thread
// of the block calls it).
__device__ __forceinline__ void rs_bitonic(unsigned long long* v, uint32_t P) {
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
                const uint32_t l = i ^ j;
                if (l > i) {
                    const unsigned long long a = v[i], b = v[l];
                    if ((a > b) == ((i & k) == 0)) {
                        v[i] = b;
                        v[l] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// One slot per thread (every thread of the block calls it): appends the
// block's moved entries to the list.
__device__ __forceinline__ void resort_collect_one(const ResortArgs& ra, bool moved, uint32_t key, uint32_t slot) {
    __shared__ uint32_t s_wcnt[32], s_base;
    const uint32_t w = threadIdx.x / kWarp, lane = lane_id(), nw = blockDim.x / kWarp;
    const uint32_t m = __ballot_sync(0xffffffffu, moved);
    if (lane == 0) s_wcnt[w] = __popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t tot = 0;
        for (uint32_t v = 0; v < nw; ++v) tot += s_wcnt[v];
        s_base = tot ? atomicAdd(&ra.scratch[0], tot) : 0u;
    }
    __syncthreads();
    if (moved) {
        uint32_t rank = s_base + __popc(m & lanemask_lt());
        for (uint32_t v = 0; v < w; ++v) rank += s_wcnt[v];
        if (rank < ra.mmax) ra.list[rank] = ((unsigned long long)key << 32) | slot;
    }
}

// Every thread of every block calls it after its block's entries are in
// the list; the last block to arrive sorts and places them.  buf: kResortMaxCap
// entries of shared memory the caller no longer needs.
__device__ __forceinline__ void resort_finish(const ResortArgs& ra, unsigned long long* buf) {
    __shared__ uint32_t s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(&ra.scratch[2], 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const uint32_t M = ld_relaxed(&ra.scratch[0]);
    if (threadIdx.x == 0) {
        ra.scratch[1] = M;
        ra.scratch[0] = 0u;
        ra.scratch[2] = 0u;
    }
    if (M == 0 || M > ra.mmax) return;
    uint32_t P = 2;
    while (P < M) P <<= 1;
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) buf[i] = i < M ? __ldcg(&ra.list[i]) : ~0ull;
    __syncthreads();
    rs_bitonic(buf, P);
    for (uint32_t i = threadIdx.x; i < M; i += blockDim.x) {
        ra.list[i] = buf[i];
        buf[i] &= 0xffffffffull;  // its slot
    }
    __syncthreads();
    rs_bitonic(buf, P);
    const uint32_t n = ra.n;
    for (uint32_t r = threadIdx.x; r < M; r += blockDim.x) {
        const unsigned long long c = __ldcg(&ra.list[r]);
        const uint32_t key = (uint32_t)(c >> 32), slot = (uint32_t)c;
        // the previous order's slots of keys below `key` are [0, L), those
        // of `key` itself [L, U); the unmoved ones among [0, clamp(slot, L,
        // U)) sort before (key, slot)
        const uint32_t L = min(ra.cell_start[min(key, ra.ncells)], n);
        const uint32_t U = min(ra.cell_start[min(key + 1, ra.ncells)], n);
        const uint32_t x = min(max(slot, L), U);
        uint32_t lo = 0, hi = M;  // moved slots below x
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (buf[mid] < x) lo = mid + 1;
            else hi = mid;
        }
        ra.pos[r] = r + x - lo;
        ra.q[r] = (uint32_t)buf[r] - r;
    }
}

// The contact kernel's epilogue, one slot per thread: list the moved slot
// and, in the last block, sort and place.  Kept out of line so that it does
// not change the register allocation of the kernel's main loop.
static __device__ __noinline__ void resort_epilogue(ResortArgs ra, bool moved, uint32_t key, uint32_t slot,
                                             unsigned long long* buf) {
    resort_collect_one(ra, moved, key, slot);
    resort_finish(ra, buf);
}

// The arguments for b's re-sort; keys_prev null when it is off or b.rs_max is
// not a power of two up to kResortMaxCap.
ResortArgs resort_args(const DemBuffers& b);

}  // namespace sd
