// sd_resort.cu -- the step's cell sort as an incremental re-sort.
//
// Every step sorts the spheres' new cell keys (key, slot) stably, slot order
// being the sorted order of the previous step.  Between two steps almost
// every sphere keeps its cell (1,048,576 settling spheres: 0-3 changes per
// step), so the result is the previous order with a few entries moved, and
// it can be built without a radix sort:
//
//   1. resort_scan_kernel: per block of 4096 slots, the slots whose new key
//      differs from the sorted key they sit under ("moved"), appended to a
//      list as (key << 32 | slot) (one atomic per block: the list's order
//      does not matter, it is sorted next).  The last block to finish (a
//      fence and an arrival counter, no waiting) publishes the count M and,
//      in shared memory, sorts the list by (key, slot) and the moved slots
//      alone (bitonic); moved entry r (rank r in (key, slot) order) goes to
//      r plus the unmoved slots that sort before it -- the previous step's
//      cell table bounds the slots of its key, so that count is its slot
//      clamped to that range minus the moved slots below it;
//   2. the in-place reorder (dem_fix_gather_kernel, dem_fix_place_kernel in
//      sd_dem.cu) reads the order from these lists: position k holds a moved
//      entry where one was placed, else the unmoved slot of rank
//      k - (moved entries placed before k).
//
// The unmoved slots are already in (key, slot) order, so this is a merge of
// two sorted sequences and the result is exactly the stable LSD sort's.
// When more than `mmax` keys change the step's radix passes run instead (they
// are in the graph and return at once otherwise) and the reorder reads their
// sorted arrays.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sd_common.cuh"
#include "sd_internal.h"

namespace sd {
namespace {

// 1024 threads, so that the last block sorts the moved list with 1024
// threads; 4 words of 32 slots per warp, 4096 slots per block
constexpr int kRsThreads = 1024;
constexpr uint32_t kRsWordsPerWarp = 4;
constexpr uint32_t kRsBlockWords = kRsWordsPerWarp * kRsThreads / kWarp;  // 128 words: 4096 slots

// Sorts v[0, P) ascending in shared memory (P a power of two; every thread
// of the block calls it).
__device__ void bitonic_sort(unsigned long long* v, uint32_t P) {
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

// scratch: [0] running count, [1] M (published by the last block),
// [2] arrivals.  [0] and [2] are zero again when the kernel ends.
__global__ void __launch_bounds__(kRsThreads)
resort_scan_kernel(const uint32_t* __restrict__ keys_new, const uint32_t* __restrict__ keys_prev, uint32_t n,
                   unsigned long long* __restrict__ list, uint32_t* __restrict__ pos_out, uint32_t* __restrict__ q_out,
                   uint32_t mmax, uint32_t* __restrict__ scratch, const uint32_t* __restrict__ cell_start,
                   uint32_t ncells, uint32_t* __restrict__ vl_flags) {
    __shared__ uint32_t s_wcnt[kRsThreads / kWarp], s_base, s_last;
    __shared__ unsigned long long s_a[kResortMaxCap], s_b[kResortMaxCap];
    const uint32_t w = threadIdx.x / kWarp, lane = lane_id();
    const uint32_t word0 = blockIdx.x * kRsBlockWords + w * kRsWordsPerWarp;
    uint32_t m[kRsWordsPerWarp];
    uint32_t cnt = 0;
#pragma unroll
    for (uint32_t j = 0; j < kRsWordsPerWarp; ++j) {
        const uint32_t s = (word0 + j) * 32 + lane;
        const bool moved = s < n && keys_new[s] != keys_prev[s];
        m[j] = __ballot_sync(0xffffffffu, moved);
        cnt += __popc(m[j]);
    }
    if (lane == 0) s_wcnt[w] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t tot = 0;
        for (uint32_t v = 0; v < kRsThreads / kWarp; ++v) tot += s_wcnt[v];
        s_base = tot ? atomicAdd(&scratch[0], tot) : 0u;
    }
    __syncthreads();
    if (cnt) {
        uint32_t rank0 = s_base;
        for (uint32_t v = 0; v < w; ++v) rank0 += s_wcnt[v];
#pragma unroll
        for (uint32_t j = 0; j < kRsWordsPerWarp; ++j) {
            if ((m[j] >> lane) & 1u) {
                const uint32_t rank = rank0 + __popc(m[j] & lanemask_lt());
                const uint32_t s = (word0 + j) * 32 + lane;
                if (rank < mmax) list[rank] = ((unsigned long long)keys_new[s] << 32) | s;
            }
            rank0 += __popc(m[j]);
        }
    }
    // the last block to arrive sees every block's count and list entries
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(&scratch[2], 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const uint32_t M = ld_relaxed(&scratch[0]);
    if (threadIdx.x == 0) {
        scratch[1] = M;
        scratch[0] = 0u;
        scratch[2] = 0u;
        if (vl_flags) {  // the skin lists: build next step if a sphere left its skin this step
            if (vl_flags[0]) ++vl_flags[2];  // steps that built the lists
            else ++vl_flags[3];              // steps that used them
            vl_flags[0] = vl_flags[1];
            vl_flags[1] = 0u;
        }
    }
    if (M == 0 || M > mmax) return;
    uint32_t P = 2;
    while (P < M) P <<= 1;
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) s_a[i] = i < M ? __ldcg(&list[i]) : ~0ull;
    __syncthreads();
    bitonic_sort(s_a, P);
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) s_b[i] = i < M ? (s_a[i] & 0xffffffffull) : ~0ull;
    __syncthreads();
    bitonic_sort(s_b, P);
    for (uint32_t r = threadIdx.x; r < M; r += blockDim.x) {
        const unsigned long long c = s_a[r];
        const uint32_t key = (uint32_t)(c >> 32), slot = (uint32_t)c;
        // the previous order's slots of keys below `key` are [0, L), those
        // of `key` itself [L, U); the unmoved ones among [0, clamp(slot, L,
        // U)) sort before (key, slot)
        const uint32_t L = min(cell_start[min(key, ncells)], n);
        const uint32_t U = min(cell_start[min(key + 1, ncells)], n);
        const uint32_t x = min(max(slot, L), U);
        uint32_t lo = 0, hi = M;  // moved slots below x
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (s_b[mid] < x) lo = mid + 1;
            else hi = mid;
        }
        list[r] = c;
        pos_out[r] = r + x - lo;
        q_out[r] = (uint32_t)s_b[r] - r;
    }
}

}  // namespace

static uint32_t g_resort_max = 1024;

void dem_set_resort_max(uint32_t m) { g_resort_max = m; }
uint32_t dem_resort_max() { return g_resort_max; }

uint64_t resort_scratch_words(uint32_t) { return 4; }

cudaError_t resort_async(const DemBuffers& b, cudaStream_t st, uint32_t* vl_flags) {
    const uint32_t n = b.n, mmax = b.rs_max;
    if (n == 0 || mmax == 0) return cudaSuccess;
    if (mmax > kResortMaxCap || (mmax & (mmax - 1)) != 0) return cudaErrorInvalidValue;
    const uint32_t blocks = ((n + 31) / 32 + kRsBlockWords - 1) / kRsBlockWords;
    resort_scan_kernel<<<blocks, kRsThreads, 0, st>>>(b.keys, b.keys_prev, n, b.rs_list, b.rs_pos, b.rs_q, mmax,
                                                      b.rs_scratch, b.cell_start, b.ncells, vl_flags);
    return cudaGetLastError();
}

}  // namespace sd
