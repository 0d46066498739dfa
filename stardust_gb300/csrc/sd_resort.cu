// sd_resort.cu -- the step's cell sort as an incremental re-sort.
//
// Every step sorts the spheres' new cell keys (key, slot) stably, slot order
// being the sorted order of the previous step.  Between two steps almost
// every sphere keeps its cell (1,048,576 settling spheres: 0-3 changes per
// step), so the result is the previous order with a few entries moved, and
// it can be built without a radix sort:
//
//   1. resort_scan_kernel: per tile of 1024 slots, the slots whose new key
//      differs from the sorted key they sit under ("moved"), as one bit per
//      slot; a single-pass scan (decoupled look-back over tiles) gives every
//      32-slot word the number of moved slots before it; the moved entries
//      are compacted, in slot order, as (key << 32 | slot).  The last block
//      to finish (a fence and an arrival counter, no waiting) sorts those M
//      entries in shared memory (bitonic) and clears the look-back state for
//      the next step;
//   2. resort_merge_kernel: an unmoved slot i keeps its key; its place is i
//      minus the moved slots before it plus the moved entries that sort
//      before (key_i << 32 | i).  Moved entry r (rank r among the moved)
//      goes to r plus the unmoved slots that sort before it; the previous
//      step's cell table bounds the slots of its key, so that count is the
//      clamped slot minus the moved slots before it.
//
// The unmoved slots are already in (key, slot) order, so this is a merge of
// two sorted sequences and the result is exactly the stable LSD sort's.
// When more than `mmax` keys change the step's radix passes run instead (they
// are in the graph and return at once otherwise) and the merge returns.
// Waits are bounded (kSpinLimit) and report through the status word.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sd_common.cuh"
#include "sd_internal.h"

namespace sd {
namespace {

constexpr int kRsThreads = 256;
constexpr uint32_t kRsTile = 1024;  // slots per tile: 8 warps x 4 words of 32
constexpr uint32_t kFlagAgg = 1u << 30, kFlagInc = 2u << 30, kCountMask = (1u << 30) - 1;

// scratch: [0] tile ticket, [1] M (moved entries), [2] arrivals, [4 ..) tile
// status.  All but M are zero again when the kernel ends.
__global__ void __launch_bounds__(kRsThreads)
resort_scan_kernel(const uint32_t* __restrict__ keys_new, const uint32_t* __restrict__ keys_prev, uint32_t n,
                   uint32_t* __restrict__ mask, uint32_t* __restrict__ wbase, unsigned long long* __restrict__ list,
                   uint32_t mmax, uint32_t* __restrict__ scratch, uint32_t ntiles, uint32_t* __restrict__ err) {
    __shared__ uint32_t s_cnt[32], s_ex[32], s_tile, s_excl, s_last;
    __shared__ unsigned long long s_list[kResortMaxCap];
    if (threadIdx.x == 0) s_tile = atomicAdd(&scratch[0], 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t w = threadIdx.x / kWarp, lane = lane_id();
    const uint32_t nwords = (n + 31) / 32;
    uint32_t* status = scratch + 4;
    uint32_t m[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const uint32_t word = tile * 32 + w * 4 + j;
        const uint32_t s = word * 32 + lane;
        const bool moved = s < n && keys_new[s] != keys_prev[s];
        m[j] = __ballot_sync(0xffffffffu, moved);
        if (lane == 0) s_cnt[w * 4 + j] = __popc(m[j]);
    }
    __syncthreads();
    if (w == 0) {
        const uint32_t c = s_cnt[lane];
        const uint32_t inc = warp_inclusive_scan(c);
        s_ex[lane] = inc - c;
        const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
        if (lane == 0) st_relaxed(&status[tile], (tile == 0 ? kFlagInc : kFlagAgg) | total);
        uint32_t excl = 0;
        if (tile > 0) {
            int64_t p = (int64_t)tile - 1;
            uint32_t spins = 0;
            while (true) {
                const int64_t q = p - (int64_t)lane;
                const uint32_t st = q >= 0 ? ld_relaxed(&status[q]) : kFlagInc;
                const uint32_t unpub = __ballot_sync(0xffffffffu, (st & ~kCountMask) == 0u);
                const uint32_t incl = __ballot_sync(0xffffffffu, (st & kFlagInc) != 0u);
                const uint32_t stop = unpub ? __ffs(unpub) - 1 : 32u;  // lanes [0, stop) are published
                const uint32_t inc_before = stop < 32 ? incl & ((1u << stop) - 1u) : incl;
                const uint32_t take = inc_before ? __ffs(inc_before) : stop;
                uint32_t x = lane < take ? (st & kCountMask) : 0u;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
                excl += x;
                if (inc_before) break;
                p -= (int64_t)take;
                if (take == 0) {
                    if (++spins > kSpinLimit) {
                        if (lane == 0) atomicOr(err, kErrLookbackTimeout);
                        break;
                    }
                    if (spins > 64) __nanosleep(32);
                }
            }
            // published after a timeout too (the error bit is set)
            if (lane == 0) st_relaxed(&status[tile], kFlagInc | ((excl + total) & kCountMask));
        }
        if (lane == 0) {
            s_excl = excl;
            if (tile == ntiles - 1) scratch[1] = excl + total;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const uint32_t word = tile * 32 + w * 4 + j;
        if (word >= nwords) continue;
        const uint32_t wb = s_excl + s_ex[w * 4 + j];
        if (lane == 0) {
            mask[word] = m[j];
            wbase[word] = wb;
        }
        const uint32_t s = word * 32 + lane;
        if ((m[j] >> lane) & 1u) {
            const uint32_t rank = wb + __popc(m[j] & lanemask_lt());
            if (rank < mmax) list[rank] = ((unsigned long long)keys_new[s] << 32) | s;
        }
    }
    // the last block to arrive sees every block's list entries and M
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(&scratch[2], 1u) == ntiles - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const uint32_t M = ld_relaxed(&scratch[1]);
    for (uint32_t t = threadIdx.x; t < ntiles; t += blockDim.x) status[t] = 0u;
    if (threadIdx.x == 0) {
        scratch[0] = 0u;
        scratch[2] = 0u;
    }
    if (M < 2 || M > mmax) return;
    uint32_t P = 2;
    while (P < M) P <<= 1;
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) s_list[i] = i < M ? __ldcg(&list[i]) : ~0ull;
    __syncthreads();
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
                const uint32_t l = i ^ j;
                if (l > i) {
                    const unsigned long long a = s_list[i], b = s_list[l];
                    if ((a > b) == ((i & k) == 0)) {
                        s_list[i] = b;
                        s_list[l] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (uint32_t i = threadIdx.x; i < M; i += blockDim.x) list[i] = s_list[i];
}

// Moved slots before slot x (x <= n).
__device__ __forceinline__ uint32_t moved_before(const uint32_t* mask, const uint32_t* wbase, uint32_t x, uint32_t n,
                                                 uint32_t M) {
    if (x >= n) return M;
    return wbase[x >> 5] + __popc(mask[x >> 5] & ((1u << (x & 31)) - 1u));
}

__global__ void __launch_bounds__(kRsThreads)
resort_merge_kernel(const uint32_t* __restrict__ keys_prev, uint32_t n, const uint32_t* __restrict__ mask,
                    const uint32_t* __restrict__ wbase, const unsigned long long* __restrict__ list,
                    const uint32_t* __restrict__ scratch, uint32_t mmax, const uint32_t* __restrict__ cell_start,
                    uint32_t ncells, uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out) {
    const uint32_t M = scratch[1];
    if (M > mmax) return;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const uint32_t mw = mask[i >> 5];
        if (!((mw >> (i & 31)) & 1u)) {  // unmoved (a moved slot is placed below)
            const uint32_t key = keys_prev[i];
            const unsigned long long c = ((unsigned long long)key << 32) | i;
            uint32_t lo = 0, hi = M;  // moved entries sorting before (key, i)
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                if (list[mid] < c) lo = mid + 1;
                else hi = mid;
            }
            const uint32_t pos = i - (wbase[i >> 5] + __popc(mw & ((1u << (i & 31)) - 1u))) + lo;
            if (pos < n) {  // always, for consistent tables
                keys_out[pos] = key;
                vals_out[pos] = i;
            }
        }
    }
    if (i < M) {
        const unsigned long long c = list[i];
        const uint32_t key = (uint32_t)(c >> 32), slot = (uint32_t)c;
        // the previous order's slots of keys below `key` are [0, L), those of
        // `key` itself [L, U); the unmoved ones among [0, clamp(slot, L, U))
        // sort before (key, slot)
        const uint32_t L = min(cell_start[min(key, ncells)], n);
        const uint32_t U = min(cell_start[min(key + 1, ncells)], n);
        const uint32_t x = min(max(slot, L), U);
        const uint32_t pos = i + x - moved_before(mask, wbase, x, n, M);
        if (pos < n) {
            keys_out[pos] = key;
            vals_out[pos] = slot;
        }
    }
}

}  // namespace

static uint32_t g_resort_max = 1024;

void dem_set_resort_max(uint32_t m) { g_resort_max = m; }
uint32_t dem_resort_max() { return g_resort_max; }

uint32_t resort_tiles(uint32_t n) { return (n + kRsTile - 1) / kRsTile; }
uint64_t resort_scratch_words(uint32_t n) { return 4 + (uint64_t)resort_tiles(n); }

cudaError_t resort_async(const DemBuffers& b, uint32_t* keys_out, uint32_t* vals_out, cudaStream_t st) {
    const uint32_t n = b.n, mmax = b.rs_max;
    if (n == 0 || mmax == 0) return cudaSuccess;
    if (mmax > kResortMaxCap || (mmax & (mmax - 1)) != 0) return cudaErrorInvalidValue;
    const uint32_t tiles = resort_tiles(n);
    resort_scan_kernel<<<tiles, kRsThreads, 0, st>>>(b.keys, b.keys_prev, n, b.rs_mask, b.rs_wbase, b.rs_list, mmax,
                                                     b.rs_scratch, tiles, b.dev_status);
    resort_merge_kernel<<<(n + kRsThreads - 1) / kRsThreads, kRsThreads, 0, st>>>(
        b.keys_prev, n, b.rs_mask, b.rs_wbase, b.rs_list, b.rs_scratch, mmax, b.cell_start, b.ncells, keys_out,
        vals_out);
    return cudaGetLastError();
}

}  // namespace sd
