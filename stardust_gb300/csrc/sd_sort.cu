// sd_sort.cu -- stable onesweep LSD radix sort of (u32 key, u32 value) pairs.
//
// Replaces the reference's three-kernel, 16-CTA radix sort
// (RadixTabulateCUDA / RadixSumCUDA / RadixReorderCUDA,
// src/engine/cuda/sh_collision_detection.cu:129-283, driven by
// sortCollisionList :310-360).  Its intended semantics -- a stable LSD sort
// of 32-bit cell words carrying 32-bit sphere words -- are kept; the
// algorithm is the single-pass-per-digit "onesweep" scheme:
//
//   1. one histogram kernel reads every key once and builds the digit
//      histograms of all passes (warp-aggregated shared atomics);
//   2. per digit pass, one kernel: each CTA takes the next tile index from an
//      atomic counter, ranks its keys per digit with __match_any_sync (stable
//      within warp, warp-ordered across the tile), publishes its per-digit
//      tile count, resolves its global digit offset by decoupled look-back
//      over the predecessors' published counts, stages the tile in shared
//      memory in digit order and writes it out in coalesced runs.
//
// Digits are up to 9 bits wide -- a key range of `key_bits` bits takes
// ceil(key_bits / 9) passes (18-bit cell keys: 2 passes; 32-bit: 4 of 8) --
// except 19- and 20-bit keys, which take 2 passes of 10-bit digits (1024
// bins) rather than 3.
// Look-back waits are bounded (kSpinLimit) and report through the status
// word instead of hanging.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sd_common.cuh"
#include "sd_internal.h"

namespace sd {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / kWarp;
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kCountMask = (1u << 30) - 1;
constexpr int kLookback = 8;  // predecessor statuses read per look-back round trip

// Scratch layout (u32 words):
//   [0]                 status word (error bits; never cleared by the sort)
//   [4 .. 8)            per-pass tile counters
//   [16 .. 16+2048)     per-pass global digit histograms, pass q at
//                       q * stride (4 x 512, or 2 x 1024)
//   [kStatusOff ..)     per-pass tile status [pass][tile][stride] (only
//                       the pass's digit bins are used)
constexpr uint64_t kHistOff = 16;
constexpr uint64_t kStatusOff = kHistOff + 4 * 512;

SortPlan sort_plan(int key_bits) {
    SortPlan p{};
    if (key_bits < 1) key_bits = 1;
    if (key_bits > 32) key_bits = 32;
    p.passes = (key_bits == 19 || key_bits == 20) ? 2 : (key_bits + 8) / 9;
    int base = key_bits / p.passes, extra = key_bits % p.passes, sh = 0;
    for (int i = 0; i < p.passes; ++i) {
        p.bits[i] = base + (i < extra ? 1 : 0);
        p.shift[i] = sh;
        sh += p.bits[i];
    }
    p.stride = p.bits[0] > 9 ? 1024 : 512;
    return p;
}

template <int ITEMS>
constexpr uint32_t tile_keys() { return kSortThreads * ITEMS; }

// --------------------------------------------------------------- histogram
__global__ void __launch_bounds__(kSortThreads)
sort_histogram_kernel(const uint32_t* __restrict__ keys, uint32_t n, SortPlan plan,
                      uint32_t* __restrict__ scratch) {
    __shared__ uint32_t hist[2048];  // pass p at p * plan.stride
    for (int i = threadIdx.x; i < 2048; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        uint32_t i = base + threadIdx.x;
        bool valid = i < n;
        uint32_t k = valid ? keys[i] : 0u;
        uint32_t active = __ballot_sync(0xffffffffu, valid);
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            if (p >= plan.passes) break;
            uint32_t d = (k >> plan.shift[p]) & ((1u << plan.bits[p]) - 1u);
            uint32_t peers = __match_any_sync(0xffffffffu, valid ? d : 0xffffffffu);
            if (valid && (peers & lanemask_lt()) == 0) atomicAdd(&hist[p * plan.stride + d], __popc(peers & active));
        }
    }
    __syncthreads();
    for (int p = 0; p < plan.passes; ++p) {
        uint32_t nb = 1u << plan.bits[p];
        for (uint32_t d = threadIdx.x; d < nb; d += blockDim.x)
            if (hist[p * plan.stride + d]) atomicAdd(&scratch[kHistOff + p * plan.stride + d], hist[p * plan.stride + d]);
    }
}

// The radix fallback of the incremental re-sort.  When more keys changed
// than the re-sort takes (skip[1] > skip_max) it clears the passes' tile
// status, writes the slot identity into vals and builds the digit
// histograms -- the re-sort's plan kernel has cleared the tile counters and
// histograms -- else it returns at once, so that a step whose moves the
// re-sort placed pays for neither.
__global__ void __launch_bounds__(kSortThreads)
sort_hist_fallback_kernel(const uint32_t* __restrict__ keys, uint32_t* __restrict__ vals, uint32_t n,
                          SortPlan plan, uint32_t* __restrict__ scratch, const uint32_t* __restrict__ skip,
                          uint32_t skip_max, uint64_t status_words) {
    if (skip[1] <= skip_max) return;
    const uint64_t gstride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < status_words; w += gstride)
        scratch[kStatusOff + w] = 0u;
    __shared__ uint32_t hist[2048];  // pass p at p * plan.stride
    for (int i = threadIdx.x; i < 2048; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < n;
        const uint32_t k = valid ? keys[i] : 0u;
        if (valid) vals[i] = i;  // the slot identity the passes carry
        const uint32_t active = __ballot_sync(0xffffffffu, valid);
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            if (p >= plan.passes) break;
            const uint32_t d = (k >> plan.shift[p]) & ((1u << plan.bits[p]) - 1u);
            const uint32_t peers = __match_any_sync(0xffffffffu, valid ? d : 0xffffffffu);
            if (valid && (peers & lanemask_lt()) == 0) atomicAdd(&hist[p * plan.stride + d], __popc(peers & active));
        }
    }
    __syncthreads();
    for (int p = 0; p < plan.passes; ++p) {
        const uint32_t nb = 1u << plan.bits[p];
        for (uint32_t d = threadIdx.x; d < nb; d += blockDim.x)
            if (hist[p * plan.stride + d]) atomicAdd(&scratch[kHistOff + p * plan.stride + d], hist[p * plan.stride + d]);
    }
}

// ------------------------------------------------------------ onesweep pass
// BINS: 256, 512 or 1024 digit bins (template so narrow passes do less
// per-digit work).  ITEMS: keys per thread (tile = 256 * ITEMS keys).
// stride: the plan's histogram and status stride.
template <int BINS, int ITEMS>
__global__ void __launch_bounds__(kSortThreads)
sort_pass_kernel(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                 uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, uint32_t n,
                 int shift, int bits, int pass, uint32_t num_tiles, uint32_t stride,
                 uint32_t* __restrict__ scratch, const uint32_t* __restrict__ skip, uint32_t skip_max) {
    if (skip && skip[1] <= skip_max) return;  // the incremental re-sort wrote the result
    constexpr int TILE = kSortThreads * ITEMS;
    constexpr int DPT = BINS / kSortThreads;  // digits per thread (1, 2 or 4)
    extern __shared__ __align__(16) uint32_t smem[];
    uint32_t* s_keys = smem;                            // TILE
    uint32_t* s_vals = s_keys + TILE;                   // TILE
    uint32_t* s_whist = s_vals + TILE;                  // kSortWarps * BINS
    uint32_t* s_tile_start = s_whist + kSortWarps * BINS;  // BINS
    uint32_t* s_gbase = s_tile_start + BINS;            // BINS
    uint32_t* s_ws = s_gbase + BINS;                    // 40 (scan scratch + tile id)

    const uint32_t mask = (1u << bits) - 1u;
    const int w = threadIdx.x / kWarp;
    const uint32_t lane = lane_id();

    if (threadIdx.x == 0) s_ws[36] = atomicAdd(&scratch[4 + pass], 1u);
    for (int i = threadIdx.x; i < kSortWarps * BINS; i += kSortThreads) s_whist[i] = 0;
    __syncthreads();
    const uint32_t tile = s_ws[36];
    const uint32_t tile_base = tile * TILE;

    // load + warp-local stable ranking
    uint32_t key[ITEMS], val[ITEMS], rank[ITEMS];
    uint32_t* wh = s_whist + w * BINS;
    // all of the thread's loads first, so their latencies overlap; read once,
    // so streaming (evict-first) loads
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        uint32_t idx = tile_base + w * (ITEMS * kWarp) + j * kWarp + lane;
        bool valid = idx < n;
        key[j] = valid ? __ldcs(keys_in + idx) : 0xffffffffu;
        val[j] = valid ? __ldcs(vals_in + idx) : 0u;
    }
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        uint32_t idx = tile_base + w * (ITEMS * kWarp) + j * kWarp + lane;
        bool valid = idx < n;
        uint32_t d = valid ? ((key[j] >> shift) & mask) : 0xffffffffu;
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t before = __popc(peers & lanemask_lt());
        uint32_t base = valid ? wh[d] : 0u;
        __syncwarp();
        if (valid && before == 0) wh[d] = base + __popc(peers);
        __syncwarp();
        rank[j] = base + before;
    }
    __syncthreads();

    // per-digit warp offsets and tile counts
    uint32_t cnt[DPT];
#pragma unroll
    for (int q = 0; q < DPT; ++q) {
        uint32_t d = threadIdx.x + q * kSortThreads, run = 0;
#pragma unroll
        for (int ww = 0; ww < kSortWarps; ++ww) {
            uint32_t c = s_whist[ww * BINS + d];
            s_whist[ww * BINS + d] = run;
            run += c;
        }
        cnt[q] = run;
    }
    // publish this tile's aggregate before anything else so successors can
    // make progress
    uint32_t* status = scratch + kStatusOff + ((uint64_t)pass * num_tiles + tile) * stride;
#pragma unroll
    for (int q = 0; q < DPT; ++q) {
        uint32_t d = threadIdx.x + q * kSortThreads;
        st_relaxed(&status[d], (tile == 0 ? kFlagInc : kFlagAgg) | cnt[q]);
    }

    // tile-local digit starts and global digit starts (exclusive scans over
    // digits; digit d = threadIdx.x + q*256)
    const uint32_t* ghist = scratch + kHistOff + pass * stride;
    uint32_t carry_t = 0, carry_g = 0;
#pragma unroll
    for (int q = 0; q < DPT; ++q) {
        uint32_t d = threadIdx.x + q * kSortThreads;
        uint32_t tot;
        uint32_t ex = block_exclusive_scan(cnt[q], s_ws, &tot);
        s_tile_start[d] = carry_t + ex;
        carry_t += tot;
        uint32_t gv = ghist[d];
        uint32_t gex = block_exclusive_scan(gv, s_ws, &tot);
        s_gbase[d] = carry_g + gex;
        carry_g += tot;
    }

    // decoupled look-back, one digit per thread per q.  The statuses of the
    // kLookback nearest unresolved predecessors are loaded together, so a
    // chain of aggregates costs one round trip per kLookback tiles.
#pragma unroll
    for (int q = 0; q < DPT; ++q) {
        const uint32_t d = threadIdx.x + q * kSortThreads;
        uint32_t excl = 0;
        if (tile > 0) {
            const uint32_t* pass_status = scratch + kStatusOff + (uint64_t)pass * num_tiles * stride + d;
            int64_t p = (int64_t)tile - 1;
            uint32_t spins = 0;
            while (true) {
                uint32_t v[kLookback];
#pragma unroll
                for (int w = 0; w < kLookback; ++w)
                    v[w] = p - w >= 0 ? ld_relaxed(pass_status + (uint64_t)(p - w) * stride) : kFlagInc;
                bool done = false;
                int used = 0;
#pragma unroll
                for (int w = 0; w < kLookback; ++w) {
                    if ((v[w] & ~kCountMask) == 0u) break;  // not published yet: retry from here
                    excl += v[w] & kCountMask;
                    used = w + 1;
                    if (v[w] & kFlagInc) {
                        done = true;
                        break;
                    }
                }
                if (done) break;
                p -= used;
                if (used == 0) {
                    if (++spins > kSpinLimit) {
                        atomicOr(&scratch[0], kErrLookbackTimeout);
                        break;
                    }
                    if (spins > 64) __nanosleep(32);
                }
            }
            st_relaxed(&status[d], kFlagInc | ((excl + cnt[q]) & kCountMask));
        }
        s_gbase[d] += excl;
    }
    __syncthreads();

    // stage the tile in digit order
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        uint32_t idx = tile_base + w * (ITEMS * kWarp) + j * kWarp + lane;
        if (idx < n) {
            uint32_t d = (key[j] >> shift) & mask;
            uint32_t pos = s_tile_start[d] + s_whist[w * BINS + d] + rank[j];
            s_keys[pos] = key[j];
            s_vals[pos] = val[j];
        }
    }
    __syncthreads();

    // coalesced write-out: consecutive staged keys of one digit go to
    // consecutive global positions
    uint32_t valid_in_tile = n - tile_base < (uint32_t)TILE ? n - tile_base : (uint32_t)TILE;
    for (uint32_t s = threadIdx.x; s < valid_in_tile; s += kSortThreads) {
        uint32_t k = s_keys[s];
        uint32_t d = (k >> shift) & mask;
        uint32_t o = s_gbase[d] + (s - s_tile_start[d]);
        // o < n whenever the histogram and look-back are consistent; the
        // check keeps a timed-out look-back from writing out of bounds
        if (o < n) {
            keys_out[o] = k;
            vals_out[o] = s_vals[s];
        }
    }
}

template <int BINS, int ITEMS>
static size_t pass_smem_bytes() {
    return sizeof(uint32_t) * (2 * (size_t)kSortThreads * ITEMS + (size_t)kSortWarps * BINS + 2 * BINS + 40);
}

// Smallest tile the pass kernel is instantiated with; sizes the status area.
constexpr int kSortItemsMin = 8;
static int g_sort_items = 16;  // keys per thread of the pass kernel (8 or 16)

void sort_set_items(int items) { g_sort_items = items >= 16 ? 16 : 8; }
int sort_items() { return g_sort_items; }

uint64_t sort_scratch_words(uint64_t n, int key_bits) {
    SortPlan p = sort_plan(key_bits);
    uint64_t tiles = (n + tile_keys<kSortItemsMin>() - 1) / tile_keys<kSortItemsMin>();
    if (tiles == 0) tiles = 1;
    return kStatusOff + (uint64_t)p.passes * tiles * (uint64_t)p.stride;
}

uint32_t* sort_hist_ptr(uint32_t* scratch) { return scratch + kHistOff; }

static uint32_t num_tiles(uint32_t n) {
    uint32_t t = kSortThreads * (uint32_t)g_sort_items;
    return (n + t - 1) / t;
}

cudaError_t sort_clear_async(uint32_t n, const SortPlan& plan, uint32_t* scratch, cudaStream_t st) {
    // counters, histograms and this sort's tile status; not the status word
    size_t clear_words = kStatusOff - 4 + (size_t)plan.passes * num_tiles(n) * (size_t)plan.stride;
    return cudaMemsetAsync(scratch + 4, 0, clear_words * sizeof(uint32_t), st);
}

cudaError_t sort_histogram_async(const uint32_t* keys, uint32_t n, const SortPlan& plan, uint32_t* scratch,
                                 cudaStream_t st) {
    int hist_blocks = (int)((n + kSortThreads * 16 - 1) / (kSortThreads * 16));
    if (hist_blocks > 152 * 8) hist_blocks = 152 * 8;
    if (hist_blocks < 1) hist_blocks = 1;
    sort_histogram_kernel<<<hist_blocks, kSortThreads, 0, st>>>(keys, n, plan, scratch);
    return cudaGetLastError();
}

template <int BINS, int ITEMS>
static cudaError_t launch_pass(const uint32_t* ki, const uint32_t* vi, uint32_t* ko, uint32_t* vo,
                               uint32_t n, int shift, int bits, int pass, uint32_t tiles, uint32_t stride,
                               uint32_t* scratch, cudaStream_t st, const uint32_t* skip, uint32_t skip_max) {
    size_t sm = pass_smem_bytes<BINS, ITEMS>();
    if (sm > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(sort_pass_kernel<BINS, ITEMS>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
    }
    sort_pass_kernel<BINS, ITEMS><<<tiles, kSortThreads, sm, st>>>(ki, vi, ko, vo, n, shift, bits,
                                                                   pass, tiles, stride, scratch, skip, skip_max);
    return cudaGetLastError();
}

// The digit passes alone: the histograms in scratch must be complete and the
// tile status cleared (sort_clear_async + a histogram producer).
cudaError_t sort_passes_async(uint32_t* keys, uint32_t* vals, uint32_t* keys_tmp, uint32_t* vals_tmp,
                              uint32_t n, const SortPlan& plan, uint32_t* scratch, cudaStream_t st,
                              bool* in_tmp, const uint32_t* skip, uint32_t skip_max) {
    *in_tmp = false;
    if (n == 0) return cudaSuccess;
    const uint32_t tiles = num_tiles(n);
    uint32_t *ki = keys, *vi = vals, *ko = keys_tmp, *vo = vals_tmp;
    for (int p = 0; p < plan.passes; ++p) {
        cudaError_t e;
        const int b = plan.bits[p], sh = plan.shift[p];
        const uint32_t sd = (uint32_t)plan.stride;
        if (g_sort_items >= 16)
            e = b > 9   ? launch_pass<1024, 16>(ki, vi, ko, vo, n, sh, b, p, tiles, sd, scratch, st, skip, skip_max)
                : b > 8 ? launch_pass<512, 16>(ki, vi, ko, vo, n, sh, b, p, tiles, sd, scratch, st, skip, skip_max)
                        : launch_pass<256, 16>(ki, vi, ko, vo, n, sh, b, p, tiles, sd, scratch, st, skip, skip_max);
        else
            e = b > 9   ? launch_pass<1024, 8>(ki, vi, ko, vo, n, sh, b, p, tiles, sd, scratch, st, skip, skip_max)
                : b > 8 ? launch_pass<512, 8>(ki, vi, ko, vo, n, sh, b, p, tiles, sd, scratch, st, skip, skip_max)
                        : launch_pass<256, 8>(ki, vi, ko, vo, n, sh, b, p, tiles, sd, scratch, st, skip, skip_max);
        if (e != cudaSuccess) return e;
        uint32_t* t;
        t = ki; ki = ko; ko = t;
        t = vi; vi = vo; vo = t;
    }
    *in_tmp = (plan.passes & 1) != 0;
    return cudaSuccess;
}

uint64_t sort_fallback_clear_words() { return kStatusOff - 4; }

cudaError_t sort_fallback_async(uint32_t* keys, uint32_t* vals, uint32_t* keys_tmp, uint32_t* vals_tmp, uint32_t n,
                                const SortPlan& plan, uint32_t* scratch, cudaStream_t st, bool* in_tmp,
                                const uint32_t* skip, uint32_t skip_max) {
    *in_tmp = false;
    if (n == 0) return cudaSuccess;
    int blocks = (int)((n + kSortThreads * 16 - 1) / (kSortThreads * 16));
    if (blocks > 152 * 4) blocks = 152 * 4;
    if (blocks < 1) blocks = 1;
    const uint64_t status_words = (uint64_t)plan.passes * num_tiles(n) * (uint64_t)plan.stride;
    sort_hist_fallback_kernel<<<blocks, kSortThreads, 0, st>>>(keys, vals, n, plan, scratch, skip, skip_max,
                                                               status_words);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return sort_passes_async(keys, vals, keys_tmp, vals_tmp, n, plan, scratch, st, in_tmp, skip, skip_max);
}

// Sorts (keys, vals) by bits [0, key_bits).  Returns via *in_tmp whether
// the result ended in the tmp buffers (odd pass count).
cudaError_t sort_pairs_async(uint32_t* keys, uint32_t* vals, uint32_t* keys_tmp, uint32_t* vals_tmp,
                             uint32_t n, int key_bits, uint32_t* scratch, cudaStream_t st,
                             bool* in_tmp) {
    SortPlan plan = sort_plan(key_bits);
    *in_tmp = false;
    if (n == 0) return cudaSuccess;
    cudaError_t e = sort_clear_async(n, plan, scratch, st);
    if (e != cudaSuccess) return e;
    if ((e = sort_histogram_async(keys, n, plan, scratch, st)) != cudaSuccess) return e;
    return sort_passes_async(keys, vals, keys_tmp, vals_tmp, n, plan, scratch, st, in_tmp);
}

int sort_num_passes(int key_bits) { return sort_plan(key_bits).passes; }

}  // namespace sd
