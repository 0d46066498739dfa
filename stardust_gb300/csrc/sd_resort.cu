// sd_resort.cu -- the step's cell sort as an incremental re-sort.
//
// Every step sorts the spheres' new cell keys (key, slot) stably, slot order
// being the sorted order of the previous step.  Between two steps almost
// every sphere keeps its cell (1,048,576 settling spheres: 0-3 changes per
// step), so the result is the previous order with a few entries moved, and
// it can be built without a radix sort: the moved entries are listed,
// sorted and placed (sd_resort.cuh), and the reorder reads the order from
// that list -- position k holds a moved entry where one was placed, else
// the unmoved slot of rank k - (moved entries placed before k).  The
// unmoved slots are already in (key, slot) order, so this is a merge of two
// sorted sequences and the result is exactly the stable LSD sort's.  When
// more than `mmax` keys change the step's radix passes run instead (they are
// in the graph and return at once otherwise) and the reorder reads their
// sorted arrays.
//
// resort_scan_kernel lists the moved slots for scenes with clumps (whose
// spheres' keys the body kernel writes after the contact kernel) and for the
// column contact kernel; the per-slot contact kernel lists them itself.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sd_common.cuh"
#include "sd_internal.h"
#include "sd_resort.cuh"

namespace sd {
namespace {

constexpr int kRsThreads = 256;
constexpr uint32_t kRsWordsPerWarp = 16;
constexpr uint32_t kRsBlockWords = kRsWordsPerWarp * kRsThreads / kWarp;  // 128 words: 4096 slots

__global__ void __launch_bounds__(kRsThreads)
resort_scan_kernel(const uint32_t* __restrict__ keys_new, ResortArgs ra) {
    __shared__ uint32_t s_wcnt[kRsThreads / kWarp], s_base;
    __shared__ unsigned long long s_buf[kResortMaxCap];
    const uint32_t n = ra.n;
    const uint32_t w = threadIdx.x / kWarp, lane = lane_id();
    const uint32_t word0 = blockIdx.x * kRsBlockWords + w * kRsWordsPerWarp;
    uint32_t m[kRsWordsPerWarp];
    uint32_t cnt = 0;
#pragma unroll
    for (uint32_t j = 0; j < kRsWordsPerWarp; ++j) {
        const uint32_t s = (word0 + j) * 32 + lane;
        const bool moved = s < n && keys_new[s] != ra.keys_prev[s];
        m[j] = __ballot_sync(0xffffffffu, moved);
        cnt += __popc(m[j]);
    }
    if (lane == 0) s_wcnt[w] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t tot = 0;
        for (uint32_t v = 0; v < kRsThreads / kWarp; ++v) tot += s_wcnt[v];
        s_base = tot ? atomicAdd(&ra.scratch[0], tot) : 0u;
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
                if (rank < ra.mmax) ra.list[rank] = ((unsigned long long)keys_new[s] << 32) | s;
            }
            rank0 += __popc(m[j]);
        }
    }
    resort_finish(ra, s_buf);
}

}  // namespace

static uint32_t g_resort_max = 1024;

void dem_set_resort_max(uint32_t m) { g_resort_max = m; }
uint32_t dem_resort_max() { return g_resort_max; }

uint64_t resort_scratch_words(uint32_t) { return 4; }

ResortArgs resort_args(const DemBuffers& b) {
    ResortArgs ra{};
    if (b.n == 0 || b.rs_max == 0 || b.rs_max > kResortMaxCap || (b.rs_max & (b.rs_max - 1)) != 0) return ra;
    ra = ResortArgs{b.keys_prev, b.rs_list, b.rs_pos, b.rs_q, b.rs_scratch, b.cell_start, b.n, b.ncells, b.rs_max};
    return ra;
}

cudaError_t resort_async(const DemBuffers& b, cudaStream_t st) {
    const ResortArgs ra = resort_args(b);
    if (!ra.keys_prev) return b.rs_max == 0 || b.n == 0 ? cudaSuccess : cudaErrorInvalidValue;
    const uint32_t blocks = ((b.n + 31) / 32 + kRsBlockWords - 1) / kRsBlockWords;
    resort_scan_kernel<<<blocks, kRsThreads, 0, st>>>(b.keys, ra);
    return cudaGetLastError();
}

}  // namespace sd
