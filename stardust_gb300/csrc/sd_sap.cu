// sd_sap.cu -- sweep and prune over axis-aligned boxes.
//
// The reference's live broad phase (SAPCollision::processCollisions,
// src/engine/cuda/collisions/SAP/sap_detection.cu:668-706): per-object AABB
// from position and radius (computeAABBCUDA, :178-217), per-axis extents
// (projectAABBCUDA, :222-272), a radix sort of the lower x extents as
// uint32 float bits (sortLowestExtents, :278-290) and a windowed sweep
// (sweepAndPruneCUDA, :385-440).  Two operators here:
//
//  * sap_sweep_ref: that sweep's own rows, for drop-in use and parity: per
//    sorted position a row of up to 16 partner ids (padding 16, unused
//    entries -1), at most 9 filled, a window of 64 sorted positions, x then
//    y tested -- and, as written at :413-417, the x test of later window
//    entries compares against the home box's upper y once a y test has
//    run.  Rows are cleared to -1 first (the reference's initIdxCUDA,
//    :135-172, clears only entries [0, n + 15) because it indexes tid + i).
//  * sap_pairs: an exact broad phase -- every pair of overlapping closed
//    boxes -- by sorting the lower x extents (order-preserving float keys,
//    so negative coordinates sort correctly) and sweeping each box forward
//    while the next lower x is within its upper x, then per-box partner
//    lists (sorted) and the ascending unique pair list.  The sweep is binned
//    like the reference's grid prototype (src/engine/testSAP.cu:341-438,
//    objects mapped to y-z cells, one x sweep per cell): a y-z grid of
//    columns at least as wide as the largest box, each box entered in the
//    (at most 2 x 2) columns it touches, entries stably sorted by column so
//    that each column keeps the x order, and each entry swept forward
//    inside its column only.  A pair sharing several columns is reported in
//    the column of its overlap's lower y-z corner, so every pair is found
//    once, by the same tests as the unbinned sweep: the same pair set.
#include "sd_common.cuh"
#include "sd_engine_impl.h"

namespace sd {

namespace {

constexpr int kSapThreads = 256;
constexpr int kRefWindow = 64;
constexpr int kRefPadding = 16;
constexpr int kRefMaxFill = 9;

inline uint32_t grid_for(uint64_t n, int threads) { return (uint32_t)((n + threads - 1) / threads); }

// Ordered uint32 image of a float: a < b  <=>  key(a) < key(b).
__device__ __forceinline__ uint32_t float_key(float x) {
    const uint32_t b = __float_as_uint(x);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__global__ void aabb_kernel(uint32_t n, const float4* __restrict__ pos, const float* __restrict__ radius,
                            float4* __restrict__ lo, float4* __restrict__ hi) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    const float r = radius ? radius[i] : p.w;
    lo[i] = make_float4(p.x - r, p.y - r, p.z - r, 0.0f);
    hi[i] = make_float4(p.x + r, p.y + r, p.z + r, 0.0f);
}

// Keys of the lower x extents: raw float bits (the reference's cast, valid
// for non-negative x) or the order-preserving image.
__global__ void lower_x_keys_kernel(uint32_t n, const float4* __restrict__ lo, uint32_t* __restrict__ keys,
                                    uint32_t* __restrict__ vals, int ordered) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    keys[i] = ordered ? float_key(lo[i].x) : __float_as_uint(lo[i].x);
    vals[i] = i;
}

__global__ void sweep_ref_kernel(uint32_t n, const float* __restrict__ upperx, const float* __restrict__ lowerx_sorted,
                                 const float* __restrict__ uppery, const float* __restrict__ lowery,
                                 const uint32_t* __restrict__ idx_sorted, int32_t* __restrict__ rows) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= n) return;
    int32_t row[kRefPadding];
#pragma unroll
    for (int k = 0; k < kRefPadding; ++k) row[k] = -1;
    int len = 0;
    const uint32_t home = idx_sorted[tid];
    float home_upper = upperx[home];
    const uint32_t end = min(tid + (uint32_t)kRefWindow, n);
    for (uint32_t i = tid + 1; i < end; ++i) {
        const float pl = lowerx_sorted[i];
        const uint32_t ph = idx_sorted[i];
        if (pl <= home_upper) {
            home_upper = uppery[home];  // as written: later x tests use the upper y
            if (lowery[ph] <= home_upper) {
                bool unique = true;
#pragma unroll
                for (int k = 0; k < kRefPadding; ++k) unique &= row[k] != (int32_t)ph;
                if (unique && len < kRefMaxFill && ph != tid) row[len++] = (int32_t)ph;
            }
        }
    }
    int4* out = reinterpret_cast<int4*>(rows + (size_t)tid * kRefPadding);
#pragma unroll
    for (int k = 0; k < kRefPadding / 4; ++k) out[k] = make_int4(row[4 * k], row[4 * k + 1], row[4 * k + 2], row[4 * k + 3]);
}

__global__ void gather_sorted_kernel(uint32_t n, const uint32_t* __restrict__ svals, const float4* __restrict__ lo,
                                     const float4* __restrict__ hi, float4* __restrict__ slo, float4* __restrict__ shi) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t i = svals[k];
    slo[k] = lo[i];
    shi[k] = hi[i];
}

__global__ void sort_segments_kernel(uint32_t n, const uint32_t* __restrict__ off, uint32_t* __restrict__ partners,
                                     uint64_t cap) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const uint32_t base = off[b], lim = off[b + 1];
    if ((uint64_t)lim > cap) return;
    for (uint32_t e = base + 1; e < lim; ++e) {
        const uint32_t x = partners[e];
        uint32_t m = e;
        while (m > base && partners[m - 1] > x) {
            partners[m] = partners[m - 1];
            --m;
        }
        partners[m] = x;
    }
}

inline size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

// ---- the column grid of the binned sweep
constexpr uint32_t kColSentinel = 0xffffu;  // an unused entry (columns are < 255 * 255)
constexpr int kMaxCols = 255;               // per axis
constexpr int kSlots = 4;                   // entries per box: at most 2 x 2 columns

struct SapGrid {
    float y0, z0, inv;  // column of v: floor((v - v0) * inv), clamped
    int gy, gz;
};

__device__ __forceinline__ int sap_col(float v, float v0, float inv, int g) {
    const float t = floorf((v - v0) * inv);
    return t >= 0.0f ? (t < (float)g ? (int)t : g - 1) : 0;  // NaN -> 0
}

__device__ __forceinline__ float key_float(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// Bounds of the boxes in y and z and their largest y or z extent, as
// ordered keys (minima stored complemented, so every word is a maximum;
// the words start at 0).  NaN coordinates are skipped.
__global__ void sap_bounds_kernel(uint32_t n, const float4* __restrict__ lo, const float4* __restrict__ hi,
                                  uint32_t* __restrict__ w) {
    uint32_t m[5] = {0u, 0u, 0u, 0u, 0u};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = lo[i], b = hi[i];
        const float ly = fminf(a.y, b.y), hy = fmaxf(a.y, b.y), lz = fminf(a.z, b.z), hz = fmaxf(a.z, b.z);
        const float ey = hy - ly, ez = hz - lz;
        if (ly == ly) {
            m[0] = max(m[0], ~float_key(ly));
            m[1] = max(m[1], float_key(hy));
        }
        if (ey == ey) m[4] = max(m[4], float_key(ey));
        if (lz == lz) {
            m[2] = max(m[2], ~float_key(lz));
            m[3] = max(m[3], float_key(hz));
        }
        if (ez == ez) m[4] = max(m[4], float_key(ez));
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const uint32_t r = __reduce_max_sync(0xffffffffu, m[k]);
        if ((threadIdx.x & 31) == 0 && r) atomicMax(&w[k], r);
    }
}

// Columns at least 1.0001 x the largest extent wide (so a box spans at most
// two columns per axis, rounding included) and at most kMaxCols per axis.
__global__ void sap_grid_kernel(const uint32_t* __restrict__ w, SapGrid* __restrict__ g) {
    SapGrid r{0.0f, 0.0f, 0.0f, 1, 1};
    if (w[0] && w[1] && w[2] && w[3]) {
        const float y0 = key_float(~w[0]), y1 = key_float(w[1]), z0 = key_float(~w[2]), z1 = key_float(w[3]);
        const float ext = w[4] ? key_float(w[4]) : 0.0f;
        const float c = fmaxf(fmaxf(ext * 1.0001f, (y1 - y0) / (float)kMaxCols), (z1 - z0) / (float)kMaxCols);
        if (c > 0.0f && c < INFINITY) {
            r.y0 = y0;
            r.z0 = z0;
            r.inv = 1.0f / c;
            r.gy = min(kMaxCols, max(1, (int)fminf((y1 - y0) * r.inv, 1e6f) + 1));
            r.gz = min(kMaxCols, max(1, (int)fminf((z1 - z0) * r.inv, 1e6f) + 1));
        }
    }
    *g = r;
}

// Per x-sorted box k: its columns (y-major) in entries 4k .. 4k+3, unused
// entries keyed kColSentinel; values are k.
__global__ void sap_entries_kernel(uint32_t n, const float4* __restrict__ slo, const float4* __restrict__ shi,
                                   const SapGrid* __restrict__ grid, uint32_t* __restrict__ keys,
                                   uint32_t* __restrict__ vals, uint32_t* __restrict__ status) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const SapGrid g = *grid;
    const float4 a = slo[k], b = shi[k];
    const int y0 = sap_col(fminf(a.y, b.y), g.y0, g.inv, g.gy), y1 = sap_col(fmaxf(a.y, b.y), g.y0, g.inv, g.gy);
    const int z0 = sap_col(fminf(a.z, b.z), g.z0, g.inv, g.gz), z1 = sap_col(fmaxf(a.z, b.z), g.z0, g.inv, g.gz);
    if (y1 - y0 > 1 || z1 - z0 > 1) atomicOr(status, kErrBadInput);  // excluded by the column width
    int t = 0;
    for (int y = y0; y <= y0 + 1; ++y)
        for (int z = z0; z <= z0 + 1; ++z) {
            const bool on = y <= y1 && z <= z1;
            keys[(size_t)kSlots * k + t] = on ? (uint32_t)(y * g.gz + z) : kColSentinel;
            vals[(size_t)kSlots * k + t] = k;
            ++t;
        }
}

// Forward sweep of entry p inside its column: entries m > p of the same
// column with lower x <= upper x of p's box (x order within the column, the
// first miss ends it), tested on y, z and x like the unbinned sweep; a pair
// counts in the column of its overlap's lower y-z corner only.  COUNT: per
// box, the number of partners (both sides, atomics on counts).  FILL:
// partners written at off[box] + cursor (atomics), sorted later.
template <bool FILL>
__global__ void sweep_binned_kernel(uint32_t n_entries, const uint32_t* __restrict__ ckeys,
                                    const uint32_t* __restrict__ cvals, const uint32_t* __restrict__ svals,
                                    const float4* __restrict__ slo, const float4* __restrict__ shi,
                                    const SapGrid* __restrict__ grid, uint32_t* __restrict__ counts,
                                    const uint32_t* __restrict__ off, uint32_t* __restrict__ cursor,
                                    uint32_t* __restrict__ partners, uint64_t cap, uint32_t* __restrict__ status) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_entries) return;
    const uint32_t col = ckeys[p];
    if (col == kColSentinel) return;
    const SapGrid g = *grid;
    const uint32_t k = cvals[p];
    const float4 a0 = slo[k], a1 = shi[k];
    const float ay = fminf(a0.y, a1.y), az = fminf(a0.z, a1.z);
    const uint32_t i = svals[k];
    for (uint32_t q = p + 1; q < n_entries; ++q) {
        if (ckeys[q] != col) break;
        const uint32_t m = cvals[q];
        const float4 b0 = slo[m];
        if (!(b0.x <= a1.x)) break;
        const float4 b1 = shi[m];
        if (!(b0.y <= a1.y && a0.y <= b1.y && b0.z <= a1.z && a0.z <= b1.z && a0.x <= b1.x)) continue;
        const int cy = sap_col(fmaxf(ay, fminf(b0.y, b1.y)), g.y0, g.inv, g.gy);
        const int cz = sap_col(fmaxf(az, fminf(b0.z, b1.z)), g.z0, g.inv, g.gz);
        if ((uint32_t)(cy * g.gz + cz) != col) continue;
        const uint32_t j = svals[m];
        if (!FILL) {
            atomicAdd(&counts[i], 1u);
            atomicAdd(&counts[j], 1u);
        } else {
            const uint32_t ei = off[i] + atomicAdd(&cursor[i], 1u);
            const uint32_t ej = off[j] + atomicAdd(&cursor[j], 1u);
            if ((uint64_t)ei < cap && (uint64_t)ej < cap) {
                partners[ei] = j;
                partners[ej] = i;
            } else {
                atomicOr(status, kErrPairOverflow);
            }
        }
    }
}

__global__ void project_kernel(uint32_t n, const float4* __restrict__ lo, const float4* __restrict__ hi,
                               float* __restrict__ upperx, float* __restrict__ uppery, float* __restrict__ lowery) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    upperx[i] = hi[i].x;
    uppery[i] = hi[i].y;
    lowery[i] = lo[i].y;
}

}  // namespace

uint64_t sap_scratch_bytes(uint64_t n, uint64_t pair_cap) {
    const uint64_t m = n ? n : 1;
    return 4 * al256(4 * m) + al256(4 * sort_scratch_words(m, 32)) + 4 * al256(16 * m) + 3 * al256(4 * (m + 1)) +
           al256(4 * scan_scratch_words((uint32_t)m + 1)) + al256(4 * (2 * pair_cap + 1)) + al256(16) +
           4 * al256(4 * kSlots * m) + al256(4 * sort_scratch_words(kSlots * m, 16)) + al256(64);
}

cudaError_t sap_aabb_async(uint32_t n, const float4* pos, const float* radius, float4* lo, float4* hi,
                           cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    aabb_kernel<<<grid_for(n, kSapThreads), kSapThreads, 0, st>>>(n, pos, radius, lo, hi);
    return cudaGetLastError();
}

cudaError_t sap_sort_lower_x_async(uint32_t n, const float4* lo, bool ordered, uint32_t* keys, uint32_t* vals,
                                   uint32_t* keys_tmp, uint32_t* vals_tmp, uint32_t* sort_scratch, bool* in_tmp,
                                   cudaStream_t st) {
    *in_tmp = false;
    if (n == 0) return cudaSuccess;
    lower_x_keys_kernel<<<grid_for(n, kSapThreads), kSapThreads, 0, st>>>(n, lo, keys, vals, ordered ? 1 : 0);
    return sort_pairs_async(keys, vals, keys_tmp, vals_tmp, n, 32, sort_scratch, st, in_tmp);
}

cudaError_t sap_sweep_ref_async(uint32_t n, const float* upperx, const float* lowerx_sorted, const float* uppery,
                                const float* lowery, const uint32_t* idx_sorted, int32_t* rows, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    sweep_ref_kernel<<<grid_for(n, kSapThreads), kSapThreads, 0, st>>>(n, upperx, lowerx_sorted, uppery, lowery,
                                                                       idx_sorted, rows);
    return cudaGetLastError();
}

cudaError_t sap_pairs_async(uint32_t n, const float4* lo, const float4* hi, void* scratch, uint64_t pair_cap,
                            unsigned long long* out, uint32_t* d_count2, cudaStream_t st) {
    const uint64_t m = n ? n : 1;
    char* p = static_cast<char*>(scratch);
    auto take = [&](size_t bytes) {
        char* r = p;
        p += al256(bytes);
        return r;
    };
    uint32_t* keys = (uint32_t*)take(4 * m);
    uint32_t* vals = (uint32_t*)take(4 * m);
    uint32_t* keys_tmp = (uint32_t*)take(4 * m);
    uint32_t* vals_tmp = (uint32_t*)take(4 * m);
    uint32_t* sort_scratch = (uint32_t*)take(4 * sort_scratch_words(m, 32));
    float4* slo = (float4*)take(16 * m);
    float4* shi = (float4*)take(16 * m);
    take(16 * m);
    take(16 * m);
    uint32_t* counts = (uint32_t*)take(4 * (m + 1));
    uint32_t* off = (uint32_t*)take(4 * (m + 1));
    uint32_t* pos = (uint32_t*)take(4 * (m + 1));
    uint32_t* scan = (uint32_t*)take(4 * scan_scratch_words((uint32_t)m + 1));
    uint32_t* partners = (uint32_t*)take(4 * (2 * pair_cap + 1));
    uint32_t* status = (uint32_t*)take(16);
    uint32_t* ckeys = (uint32_t*)take(4 * kSlots * m);
    uint32_t* cvals = (uint32_t*)take(4 * kSlots * m);
    uint32_t* ckeys_tmp = (uint32_t*)take(4 * kSlots * m);
    uint32_t* cvals_tmp = (uint32_t*)take(4 * kSlots * m);
    uint32_t* csort = (uint32_t*)take(4 * sort_scratch_words(kSlots * m, 16));
    uint32_t* bounds = (uint32_t*)take(64);  // 5 words, then the grid
    SapGrid* grid = reinterpret_cast<SapGrid*>(bounds + 8);
    cudaError_t e = cudaMemsetAsync(status, 0, 16, st);
    if (e != cudaSuccess) return e;
    if (n == 0) return cudaMemsetAsync(d_count2, 0, 8, st);
    bool in_tmp = false;
    if ((e = sap_sort_lower_x_async(n, lo, true, keys, vals, keys_tmp, vals_tmp, sort_scratch, &in_tmp, st)) !=
        cudaSuccess)
        return e;
    const uint32_t* svals = in_tmp ? vals_tmp : vals;
    gather_sorted_kernel<<<grid_for(n, kSapThreads), kSapThreads, 0, st>>>(n, svals, lo, hi, slo, shi);
    // the column grid, each box's entries, stably sorted by column
    if ((e = cudaMemsetAsync(bounds, 0, 32, st)) != cudaSuccess) return e;
    sap_bounds_kernel<<<std::min<uint32_t>(grid_for(n, kSapThreads), 152 * 8), kSapThreads, 0, st>>>(n, lo, hi,
                                                                                                     bounds);
    sap_grid_kernel<<<1, 1, 0, st>>>(bounds, grid);
    sap_entries_kernel<<<grid_for(n, kSapThreads), kSapThreads, 0, st>>>(n, slo, shi, grid, ckeys, cvals, status);
    const uint32_t ne = kSlots * n;
    bool c_tmp = false;
    if ((e = sort_pairs_async(ckeys, cvals, ckeys_tmp, cvals_tmp, ne, 16, csort, st, &c_tmp)) != cudaSuccess)
        return e;
    const uint32_t* sk = c_tmp ? ckeys_tmp : ckeys;
    const uint32_t* sv = c_tmp ? cvals_tmp : cvals;
    if ((e = cudaMemsetAsync(counts, 0, 4 * (m + 1), st)) != cudaSuccess) return e;
    sweep_binned_kernel<false><<<grid_for(ne, kSapThreads), kSapThreads, 0, st>>>(
        ne, sk, sv, svals, slo, shi, grid, counts, nullptr, nullptr, nullptr, 0, status);
    if ((e = scan_exclusive_async(counts, off, n, scan, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(counts, 0, 4 * (m + 1), st)) != cudaSuccess) return e;  // reused as cursors
    sweep_binned_kernel<true><<<grid_for(ne, kSapThreads), kSapThreads, 0, st>>>(
        ne, sk, sv, svals, slo, shi, grid, nullptr, off, counts, partners, 2 * pair_cap, status);
    sort_segments_kernel<<<grid_for(n, kSapThreads), kSapThreads, 0, st>>>(n, off, partners, 2 * pair_cap);
    uint32_t* ucount = keys;  // free again
    if ((e = csr_unique_pairs_async(n, off, partners, 2 * pair_cap, ucount, scan, pos, out, pair_cap, st)) !=
        cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(d_count2, pos + n, 4, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
    return cudaMemcpyAsync(d_count2 + 1, status, 4, cudaMemcpyDeviceToDevice, st);
}

}  // namespace sd

// =================================================================== C ABI
extern "C" {

sd_status sd_sap_scratch_bytes(uint64_t n, uint64_t pair_cap, uint64_t* bytes) {
    if (!bytes) return sd_fail(nullptr, SD_ERR_INVALID_ARG, "bytes NULL");
    if (n >= (1ull << 30)) return sd_fail(nullptr, SD_ERR_CAPACITY, "n must be < 2^30");
    *bytes = sd::sap_scratch_bytes(n, pair_cap);
    return SD_OK;
}

sd_status sd_sap_pairs(uint64_t n, const float* d_lo4, const float* d_hi4, uint64_t* d_pairs, uint64_t cap,
                       uint32_t* d_count, void* d_scratch, uint64_t scratch_bytes, void* stream) {
    if (n && (!d_lo4 || !d_hi4 || !d_scratch)) return sd_fail(nullptr, SD_ERR_INVALID_ARG, "NULL pointer");
    if (!d_count) return sd_fail(nullptr, SD_ERR_INVALID_ARG, "d_count NULL");
    if (n >= (1ull << 30)) return sd_fail(nullptr, SD_ERR_CAPACITY, "n must be < 2^30");
    if (scratch_bytes < sd::sap_scratch_bytes(n, cap))
        return sd_fail(nullptr, SD_ERR_CAPACITY, "scratch smaller than sd_sap_scratch_bytes");
    if ((reinterpret_cast<uintptr_t>(d_lo4) | reinterpret_cast<uintptr_t>(d_hi4)) & 15u)
        return sd_fail(nullptr, SD_ERR_INVALID_ARG, "boxes must be 16-byte aligned");
    cudaError_t e = sd::sap_pairs_async((uint32_t)n, reinterpret_cast<const float4*>(d_lo4),
                                        reinterpret_cast<const float4*>(d_hi4), d_scratch, cap,
                                        reinterpret_cast<unsigned long long*>(d_pairs), d_count,
                                        static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return sd_cuda_fail(nullptr, e, "sd_sap_pairs");
    return SD_OK;
}

sd_status sd_sap_sweep(uint64_t n, const float* d_upperx, const float* d_lowerx_sorted, const float* d_uppery,
                       const float* d_lowery, const uint32_t* d_idx_sorted, int32_t* d_rows, void* stream) {
    if (n && (!d_upperx || !d_lowerx_sorted || !d_uppery || !d_lowery || !d_idx_sorted || !d_rows))
        return sd_fail(nullptr, SD_ERR_INVALID_ARG, "NULL pointer");
    if (n >= (1ull << 31) / 16) return sd_fail(nullptr, SD_ERR_CAPACITY, "n too large for 16-entry rows");
    if (reinterpret_cast<uintptr_t>(d_rows) & 15u) return sd_fail(nullptr, SD_ERR_INVALID_ARG, "rows must be 16-byte aligned");
    cudaError_t e = sd::sap_sweep_ref_async((uint32_t)n, d_upperx, d_lowerx_sorted, d_uppery, d_lowery, d_idx_sorted,
                                            d_rows, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return sd_cuda_fail(nullptr, e, "sd_sap_sweep");
    return SD_OK;
}

sd_status sd_sap_process_collisions(uint64_t n, const float* d_pos4, const float* d_radius, int32_t* d_rows,
                                    void* d_scratch, uint64_t scratch_bytes, void* stream) {
    if (n && (!d_pos4 || !d_rows || !d_scratch)) return sd_fail(nullptr, SD_ERR_INVALID_ARG, "NULL pointer");
    if (n >= (1ull << 31) / 16) return sd_fail(nullptr, SD_ERR_CAPACITY, "n too large for 16-entry rows");
    if (scratch_bytes < sd::sap_scratch_bytes(n, 0))
        return sd_fail(nullptr, SD_ERR_CAPACITY, "scratch smaller than sd_sap_scratch_bytes(n, 0)");
    if ((reinterpret_cast<uintptr_t>(d_pos4) | reinterpret_cast<uintptr_t>(d_rows)) & 15u)
        return sd_fail(nullptr, SD_ERR_INVALID_ARG, "positions and rows must be 16-byte aligned");
    const uint32_t m = n ? (uint32_t)n : 1u;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    char* p = static_cast<char*>(d_scratch);
    auto take = [&](size_t bytes) {
        char* r = p;
        p += sd::al256(bytes);
        return r;
    };
    uint32_t* keys = (uint32_t*)take(4ull * m);
    uint32_t* vals = (uint32_t*)take(4ull * m);
    uint32_t* keys_tmp = (uint32_t*)take(4ull * m);
    uint32_t* vals_tmp = (uint32_t*)take(4ull * m);
    uint32_t* sort_scratch = (uint32_t*)take(4ull * sd::sort_scratch_words(m, 32));
    float4* lo = (float4*)take(16ull * m);
    float4* hi = (float4*)take(16ull * m);
    float* proj = (float*)take(16ull * m);
    float* upperx = proj;
    float* uppery = proj + m;
    float* lowery = proj + 2ull * m;
    if (n == 0) return SD_OK;
    bool in_tmp = false;
    cudaError_t e = sd::sap_aabb_async((uint32_t)n, reinterpret_cast<const float4*>(d_pos4), d_radius, lo, hi, st);
    if (e == cudaSuccess)
        e = sd::sap_sort_lower_x_async((uint32_t)n, lo, false, keys, vals, keys_tmp, vals_tmp, sort_scratch, &in_tmp,
                                       st);
    if (e == cudaSuccess) {
        sd::project_kernel<<<sd::grid_for(n, sd::kSapThreads), sd::kSapThreads, 0, st>>>((uint32_t)n, lo, hi, upperx, uppery, lowery);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = sd::sap_sweep_ref_async((uint32_t)n, upperx, reinterpret_cast<const float*>(in_tmp ? keys_tmp : keys),
                                    uppery, lowery, in_tmp ? vals_tmp : vals, d_rows, st);
    if (e != cudaSuccess) return sd_cuda_fail(nullptr, e, "sd_sap_process_collisions");
    return SD_OK;
}

}  // extern "C"
