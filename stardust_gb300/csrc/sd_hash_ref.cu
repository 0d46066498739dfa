// sd_hash_ref.cu -- the reference's spatial-hash broad phase, bit-exact.
//
// ref_hash_build_kernel restates constructCollisionListCUDA
// (src/engine/cuda/sh_collision_detection.cu:27-127): nine (cell, sphere)
// slots per sphere, home entry first, then the phantom entries the reference
// emits, then padding.  Keys, padding words and the valid-entry count are
// reproduced exactly, including the reference's parse of its phantom test
// (:95), under which only offsets in {0,+1}^3 are ever emitted.  Unlike the
// reference's 16-CTA grid-stride launch, one thread handles one sphere on a
// grid sized to the input, and the count is warp-reduced before one atomic
// per warp.
//
// The candidate-pair kernels restate the run traversal of
// tranverseCollisionListCUDA (collision_resolution.cu:100-199): within each
// run of equal cell (key >> 1), each of the first h entries (the homes, which
// sort first because their key LSB is 0) pairs with every later entry.  The
// reference walks runs serially per thread; here every entry is independent:
// pass 1 counts each home's pairs, a decoupled-look-back scan turns counts
// into offsets, pass 2 writes the pairs at those offsets -- the same order
// the reference's traversal visits them.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sd_common.cuh"
#include "sd_internal.h"

namespace sd {

__device__ __forceinline__ uint32_t f2u_rz_sat(float q) {
    // cvt.rzi.u32.f32: truncate, saturate to [0, 2^32-1], NaN -> 0
    return __float2uint_rz(q);
}

__global__ void ref_hash_build_kernel(uint32_t n, float cell_dim, uint32_t* __restrict__ cells,
                                      uint32_t* __restrict__ spheres, const float* __restrict__ sizes,
                                      const float4* __restrict__ pos4, uint32_t* __restrict__ d_count) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t count = 0;
    if (i < n) {
        float4 p4 = pos4[i];
        float pos[3] = {p4.x, p4.y, p4.z};
        float a = sizes[i];
        uint32_t hash = 0, sides = 0;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            float x = pos[j];
            float q = __fdiv_rn(x, cell_dim);
            hash = (hash << 8) | f2u_rz_sat(q);
            x = __fmaf_rn(-floorf(q), cell_dim, x);
            sides <<= 2;
            if (x < a) sides |= 3u;
            else if (__fsub_rn(cell_dim, x) < a) sides |= 1u;
        }
        uint32_t c[9], s[9];
        c[0] = hash << 1;
        s[0] = (i << 1) | 1u;
        count = 1;
#pragma unroll
        for (int j = 0; j < 27; ++j) {
            if (j == 13) continue;
            int q = j;
            uint32_t hh = 0;
            bool invalid = false;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                int r = q % 3 - 1;
                float x = pos[k];
                uint32_t side = (sides >> ((3 - k - 1) * 2)) & 3u;
                float shifted = __fadd_rn(x, __fmul_rn((float)r, cell_dim));
                if ((r != 0 && (side ^ (uint32_t)r) != 0u) || shifted < 0.0f || shifted >= 1.0f) {
                    invalid = true;
                    break;
                }
                hh = (hh << 8) | (f2u_rz_sat(__fdiv_rn(x, cell_dim)) + (uint32_t)r);
                q /= 3;
            }
            if (!invalid) {
                c[count] = (hh << 1) | 1u;
                s[count] = i << 1;
                ++count;
            }
        }
        // count <= 8 here: the emittable offsets are {0,1}^3 minus the
        // origin, i.e. seven phantoms at most
        size_t base = 9 * (size_t)i;
#pragma unroll
        for (int m = 0; m < 9; ++m) {
            bool real = (uint32_t)m < count;
            cells[base + m] = real ? c[m] : 0xffffffffu;
            spheres[base + m] = real ? s[m] : (i << 2);
        }
    }
    // warp-aggregate the count, one atomic per warp
    uint32_t v = count;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane_id() == 0 && v) atomicAdd(d_count, v);
}

cudaError_t ref_hash_build_async(uint32_t n, float cell_dim, uint32_t* cells, uint32_t* spheres,
                                 const float* sizes, const float4* pos, uint32_t* d_count,
                                 cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(d_count, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess || n == 0) return e;
    const int threads = 256;
    ref_hash_build_kernel<<<(n + threads - 1) / threads, threads, 0, st>>>(n, cell_dim, cells, spheres,
                                                                           sizes, pos, d_count);
    return cudaGetLastError();
}

// ------------------------------------------------------- candidate pairs
// Per-entry pair count: entry j at run offset o (run of length L with h
// homes) contributes L-1-o pairs when o < h, else 0; same-body partners
// are removed when body_of is given.
constexpr int kPairThreads = 256;
constexpr int kPairItems = 8;
constexpr int kPairTile = kPairThreads * kPairItems;

__device__ __forceinline__ void run_bounds(const uint32_t* cells, uint32_t count, uint32_t j,
                                           uint32_t* start, uint32_t* end) {
    uint32_t key = cells[j] >> 1;
    uint32_t s = j;
    while (s > 0 && (cells[s - 1] >> 1) == key) --s;
    uint32_t e = j + 1;
    while (e < count && (cells[e] >> 1) == key) ++e;
    *start = s;
    *end = e;
}

// Pairs contributed by entry j (0 when j is not among the run's homes).
__device__ __forceinline__ uint32_t entry_pairs(const uint32_t* cells, const uint32_t* spheres,
                                                uint32_t count, const int32_t* body_of, uint32_t j,
                                                uint32_t* rs, uint32_t* re) {
    uint32_t s, e;
    run_bounds(cells, count, j, &s, &e);
    *rs = s;
    *re = e;
    uint32_t h = 0;
    for (uint32_t k = s; k < e; ++k) h += spheres[k] & 1u;
    if (h == 0 || j - s >= h) return 0;  // run without a home, or j is a phantom slot
    if (!body_of) return e - j - 1;
    uint32_t home = spheres[j] >> 1;
    int32_t bh = body_of[home];
    uint32_t c = 0;
    for (uint32_t k = j + 1; k < e; ++k) c += body_of[spheres[k] >> 1] != bh;
    return c;
}

// Single-pass exclusive scan over 64-bit pair counts with decoupled
// look-back.  A tile's status is one 64-bit word: flag in the top two bits
// (1 aggregate, 2 inclusive), count in the low 62, so it is published and
// read atomically.
__device__ __forceinline__ unsigned long long ld_relaxed64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
constexpr unsigned long long kPairAgg = 1ull << 62, kPairInc = 2ull << 62, kPairMask = (1ull << 62) - 1;

__global__ void __launch_bounds__(kPairThreads)
ref_pairs_kernel(const uint32_t* __restrict__ cells, const uint32_t* __restrict__ spheres,
                 const uint32_t* __restrict__ d_count, uint32_t n_entries,
                 const int32_t* __restrict__ body_of, uint32_t* __restrict__ pair_a,
                 uint32_t* __restrict__ pair_b, uint64_t cap, unsigned long long* __restrict__ d_npairs,
                 uint32_t* __restrict__ scratch) {
    __shared__ unsigned long long s_part[kPairThreads / kWarp];
    __shared__ unsigned long long s_excl;
    __shared__ uint32_t s_tile;
    const uint32_t count = min(*d_count, n_entries);
    unsigned long long* tiles = reinterpret_cast<unsigned long long*>(scratch + 16);
    if (threadIdx.x == 0) s_tile = atomicAdd(scratch + 4, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t base = tile * kPairTile + threadIdx.x * kPairItems;

    uint32_t np[kPairItems], re[kPairItems];
    unsigned long long mine = 0;
#pragma unroll
    for (int q = 0; q < kPairItems; ++q) {
        uint32_t j = base + q, rs = 0;
        re[q] = 0;
        np[q] = j < count ? entry_pairs(cells, spheres, count, body_of, j, &rs, &re[q]) : 0u;
        mine += np[q];
    }
    unsigned long long inc = mine;
#pragma unroll
    for (int o = 1; o < kWarp; o <<= 1) {
        unsigned long long t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane_id() >= (uint32_t)o) inc += t;
    }
    const int w = threadIdx.x / kWarp;
    if (lane_id() == kWarp - 1) s_part[w] = inc;
    __syncthreads();
    unsigned long long wpre = 0, tile_total = 0;
    for (int k = 0; k < kPairThreads / kWarp; ++k) {
        if (k < w) wpre += s_part[k];
        tile_total += s_part[k];
    }
    const unsigned long long excl_in_tile = wpre + inc - mine;

    if (threadIdx.x == 0) {
        unsigned long long excl = 0;
        if (tile == 0) {
            st_relaxed64(&tiles[0], kPairInc | tile_total);
        } else {
            st_relaxed64(&tiles[tile], kPairAgg | tile_total);
            int64_t p = (int64_t)tile - 1;
            uint32_t spins = 0;
            while (p >= 0) {
                unsigned long long v = ld_relaxed64(&tiles[p]);
                if ((v & ~kPairMask) == 0) {
                    if (++spins > kSpinLimit) {
                        atomicOr(&scratch[0], kErrLookbackTimeout);
                        break;
                    }
                    if (spins > 64) __nanosleep(32);
                    continue;
                }
                excl += v & kPairMask;
                if (v & kPairInc) break;
                --p;
            }
            st_relaxed64(&tiles[tile], kPairInc | (excl + tile_total));
        }
        s_excl = excl;
    }
    __syncthreads();
    unsigned long long off = s_excl + excl_in_tile;
    // the last tile by index ends at n_entries, so its last thread's
    // inclusive prefix is the grand total
    if (tile == gridDim.x - 1 && threadIdx.x == kPairThreads - 1) {
        *d_npairs = off + mine;
        if (off + mine > cap) atomicOr(&scratch[0], kErrPairOverflow);
    }

#pragma unroll
    for (int q = 0; q < kPairItems; ++q) {
        if (np[q] == 0) continue;
        uint32_t j = base + q;
        uint32_t home = spheres[j] >> 1;
        int32_t bh = body_of ? body_of[home] : 0;
        for (uint32_t k = j + 1; k < re[q]; ++k) {
            uint32_t other = spheres[k] >> 1;
            if (body_of && body_of[other] == bh) continue;
            if (off < cap) {
                pair_a[off] = home;
                pair_b[off] = other;
            }
            ++off;
        }
    }
}

uint64_t ref_pairs_scratch_words(uint64_t n_entries) {
    uint64_t tiles = (n_entries + kPairTile - 1) / kPairTile;
    if (tiles == 0) tiles = 1;
    return 16 + 2 * tiles;
}

cudaError_t ref_candidate_pairs_async(const uint32_t* cells, const uint32_t* spheres,
                                      const uint32_t* d_count, uint32_t n_entries,
                                      const int32_t* body_of, uint32_t* pair_a, uint32_t* pair_b,
                                      uint64_t cap, unsigned long long* d_npairs, uint32_t* scratch,
                                      cudaStream_t st) {
    uint64_t words = ref_pairs_scratch_words(n_entries);
    cudaError_t e = cudaMemsetAsync(scratch + 4, 0, (words - 4) * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(d_npairs, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    if (n_entries == 0) return cudaSuccess;
    uint32_t tiles = (uint32_t)((n_entries + kPairTile - 1) / kPairTile);
    ref_pairs_kernel<<<tiles, kPairThreads, 0, st>>>(cells, spheres, d_count, n_entries, body_of, pair_a,
                                                     pair_b, cap, d_npairs, scratch);
    return cudaGetLastError();
}

}  // namespace sd
