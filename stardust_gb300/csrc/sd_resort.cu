// sd_resort.cu -- the step's cell sort as an incremental re-sort.
//
// Every step sorts the spheres' new cell keys (key, slot) stably, slot order
// being the sorted order of the previous step.  Between two steps almost
// every sphere keeps its cell (1,048,576 settling spheres: 0-100 changes per
// step), so the result is the previous order with a few entries moved, and
// it can be built without a radix sort:
//
//   1. the kernel that writes the new keys (contact or body kernel) appends
//      every slot whose new key differs from the sorted key it sits under
//      ("moved") to a list as (key << 32 | slot), one warp-aggregated atomic
//      per warp that has any (the list's order does not matter);
//   2. resort_plan_kernel, one block: publishes the count M and, in shared
//      memory, sorts the list by (key, slot) and the moved slots alone
//      (each entry placed by counting the smaller ones); moved entry r
//      (rank r in (key, slot) order) goes to r plus the unmoved slots that
//      sort before it -- the previous step's cell
//      table bounds the slots of its key, so that count is its slot clamped
//      to that range minus the moved slots below it.  Only positions between
//      a moved entry's old slot and its new position change hands, so it also
//      lists those intervals (with the prefix sums of their lengths) for the
//      reorder;
//   3. the in-place reorder (dem_fix_gather_kernel, dem_fix_place_kernel in
//      sd_dem.cu) visits the intervals' positions and reads the order from
//      these lists: position k holds a moved entry where one was placed,
//      else the unmoved slot of rank k - (moved entries placed before k).
//
// The unmoved slots are already in (key, slot) order, so this is a merge of
// two sorted sequences and the result is exactly the stable LSD sort's.
// When more than `mmax` keys change, the plan kernel clears the radix sort's
// counters and histograms and the step's fallback (histogram + passes, in
// the graph and returning at once otherwise) sorts; the reorder then reads
// their sorted arrays.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sd_common.cuh"
#include "sd_internal.h"

namespace sd {
namespace {

// one block of 1024 threads: one thread per moved entry of a full list
constexpr int kRsThreads = 1024;
// above this many moved entries the ranks are counted against sorted chunks
constexpr uint32_t kChunkedRankM = 256;
static_assert(kResortMaxCap <= (uint32_t)kRsThreads, "one thread per moved entry");

// scratch (u32): [0] moved count (appended to during the step, zero again
// when this kernel ends), [1] M of the step, [3] total length T of the
// shift intervals.  sort_clear: the radix fallback's tile counters and
// histograms, cleared when the fallback will run.
__global__ void __launch_bounds__(kRsThreads)
resort_plan_kernel(unsigned long long* __restrict__ list, uint32_t* __restrict__ pos_out,
                   uint32_t* __restrict__ q_out, uint32_t* __restrict__ iv_lo, uint32_t* __restrict__ iv_pre,
                   uint32_t mmax, uint32_t* __restrict__ scratch, const uint32_t* __restrict__ cell_start,
                   uint32_t ncells, uint32_t n, uint32_t* __restrict__ vl_flags, uint32_t* __restrict__ sort_clear,
                   uint32_t sort_clear_words) {
    __shared__ unsigned long long s_a[kResortMaxCap], s_b[kResortMaxCap];
    __shared__ uint32_t s_c[kResortMaxCap];
    __shared__ uint32_t s_M, ws[33];
    if (threadIdx.x == 0) {
        const uint32_t M = scratch[0];
        s_M = M;
        scratch[0] = 0u;
        scratch[1] = M;
        if (vl_flags) {  // the skin lists: build next step if a sphere left its skin this step
            if (vl_flags[0]) ++vl_flags[2];  // steps that built the lists
            else ++vl_flags[3];              // steps that used them
            vl_flags[0] = vl_flags[1];
            vl_flags[1] = 0u;
        }
    }
    __syncthreads();
    const uint32_t M = s_M;
    if (M > mmax) {  // the radix fallback sorts this step
        for (uint32_t i = threadIdx.x; i < sort_clear_words; i += blockDim.x) sort_clear[i] = 0u;
        return;
    }
    if (M == 0) {
        if (threadIdx.x == 0) scratch[3] = 0u;
        return;
    }
    if (M > kChunkedRankM) {
        // each entry is placed by counting the smaller ones (entries and
        // slots are distinct), chunk by chunk: every warp sorts 32 entries
        // by (key, slot) and their slots alone (bitonic network over the
        // lanes), then each entry adds up, over the chunks, the number of
        // smaller elements (binary search): M/32 chunks x 6 probes per
        // order instead of M comparisons
        const uint32_t lane = threadIdx.x & 31u, t = threadIdx.x;
        unsigned long long v = t < M ? list[t] : ~0ull;
        uint32_t sv = t < M ? (uint32_t)v : 0xffffffffu;
        const unsigned long long c = v;
        for (uint32_t k = 2; k <= 32; k <<= 1)
            for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                const unsigned long long o = __shfl_xor_sync(0xffffffffu, v, (int)j);
                const uint32_t os = __shfl_xor_sync(0xffffffffu, sv, (int)j);
                const bool take_min = ((lane & j) == 0) == ((lane & k) == 0);
                v = take_min ? (o < v ? o : v) : (o < v ? v : o);
                sv = take_min ? min(os, sv) : max(os, sv);
            }
        s_b[t] = v;  // chunks of 32, each ascending (padding last)
        s_c[t] = sv;
        __syncthreads();
        uint32_t ra = 0, rs = 0;
        if (t < M) {
            const uint32_t cs = (uint32_t)c, nch = (M + 31u) >> 5;
            for (uint32_t q = 0; q < nch; ++q) {
                const unsigned long long* A = s_b + 32u * q;
                const uint32_t* S = s_c + 32u * q;
                uint32_t pa = 0, ps = 0;  // elements of the chunk below c, below cs
#pragma unroll
                for (uint32_t step = 32; step > 0; step >>= 1) {
                    if (pa + step <= 32u && A[pa + step - 1u] < c) pa += step;
                    if (ps + step <= 32u && S[ps + step - 1u] < cs) ps += step;
                }
                ra += pa;
                rs += ps;
            }
        }
        __syncthreads();
        if (t < M) {
            s_a[ra] = c;
            s_b[rs] = c & 0xffffffffull;  // the moved slots, ascending
        }
        __syncthreads();
    } else {
        // each entry is placed by counting the smaller ones (entries and
        // slots are distinct): G threads per entry, G the largest power of two
        // up to 32 with G * M <= 1024, each counting a G-th of the list, then
        // summed across the G lanes; two barriers in all
        uint32_t G = 32;
        while (G > 1 && G * M > (uint32_t)kRsThreads) G >>= 1;
        if (threadIdx.x < M) s_b[threadIdx.x] = list[threadIdx.x];
        __syncthreads();
        const uint32_t r = threadIdx.x / G, g = threadIdx.x % G;
        const unsigned long long c = r < M ? s_b[r] : 0ull;
        uint32_t ra = 0, rs = 0;
        if (r < M) {
            for (uint32_t j = g; j < M; j += G) {
                const unsigned long long o = s_b[j];
                ra += o < c;
                rs += (o & 0xffffffffull) < (c & 0xffffffffull);
            }
        }
        for (uint32_t o = G >> 1; o > 0; o >>= 1) {
            ra += __shfl_xor_sync(0xffffffffu, ra, (int)o);
            rs += __shfl_xor_sync(0xffffffffu, rs, (int)o);
        }
        __syncthreads();
        if (r < M && g == 0) {
            s_a[ra] = c;
            s_b[rs] = c & 0xffffffffull;  // the moved slots, ascending
        }
        __syncthreads();
    }
    // one moved entry per thread (M <= kResortMaxCap = blockDim.x)
    const uint32_t r = threadIdx.x;
    uint32_t len = 0, lo = 0;
    if (r < M) {
        const unsigned long long c = s_a[r];
        const uint32_t key = (uint32_t)(c >> 32), slot = (uint32_t)c;
        // the previous order's slots of keys below `key` are [0, L), those
        // of `key` itself [L, U); the unmoved ones among [0, clamp(slot, L,
        // U)) sort before (key, slot)
        const uint32_t L = min(cell_start[min(key, ncells)], n);
        const uint32_t U = min(cell_start[min(key + 1, ncells)], n);
        const uint32_t x = min(max(slot, L), U);
        uint32_t a = 0, b = M;  // moved slots below x
        while (a < b) {
            const uint32_t mid = (a + b) >> 1;
            if (s_b[mid] < x) a = mid + 1;
            else b = mid;
        }
        const uint32_t p = r + x - a;
        list[r] = c;
        pos_out[r] = p;
        q_out[r] = (uint32_t)s_b[r] - r;
        // positions [min(slot, p), max(slot, p)] may change hands
        lo = min(slot, p);
        len = max(slot, p) - lo + 1u;
    }
    uint32_t total;
    const uint32_t ex = block_exclusive_scan(len, ws, &total);
    if (r < M) {
        iv_lo[r] = lo;
        iv_pre[r] = ex;
    }
    if (threadIdx.x == 0) {
        iv_pre[M] = total;
        scratch[3] = total;
    }
}

}  // namespace

static uint32_t g_resort_max = 1024;

void dem_set_resort_max(uint32_t m) { g_resort_max = m; }
uint32_t dem_resort_max() { return g_resort_max; }

uint64_t resort_scratch_words(uint32_t) { return 4; }

cudaError_t resort_plan_async(const DemBuffers& b, cudaStream_t st, uint32_t* vl_flags) {
    const uint32_t n = b.n, mmax = b.rs_max;
    if (n == 0 || mmax == 0) return cudaSuccess;
    if (mmax > kResortMaxCap || (mmax & (mmax - 1)) != 0) return cudaErrorInvalidValue;
    resort_plan_kernel<<<1, kRsThreads, 0, st>>>(b.rs_list, b.rs_pos, b.rs_q, b.rs_iv_lo, b.rs_iv_pre, mmax,
                                                 b.rs_scratch, b.cell_start, b.ncells, n, vl_flags,
                                                 b.sort_scratch + 4, (uint32_t)sort_fallback_clear_words());
    return cudaGetLastError();
}

}  // namespace sd
