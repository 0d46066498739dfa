// sd_mlp.cu -- the GJK warm-start network on the 5th-generation tensor
// cores: forward (inference) and backward (training) kernels built from
// tcgen05.mma (BF16 operands in shared memory, FP32 accumulators in tensor
// memory), plus the Adam update.
//
// Network: 16 inputs (12 used, see hull_prev_seed_kernel) -> 64 -> ReLU ->
// 64 -> ReLU -> 16 outputs (3 used), added to inputs 8..10 (the pair's
// previous separating direction, zero for a new pair): a residual network
// whose output is a GJK search direction in the body frame of the pair's
// first hull.  With the last layer at zero it reproduces the previous
// direction; training learns the correction.  Weights are kept in FP32 (master copy, Adam
// moments) and re-packed after every update into BF16 operand images in the
// UMMA canonical K-major layout without swizzle, so a CTA copies them to
// shared memory as-is.
//
// Every GEMM is M = 128 rows (one row per thread of a 128-thread CTA, which
// is also the TMEM lane), N in {16, 64}, K in {16, 64, 128}, issued by one
// thread as K/16 tcgen05.mma instructions of kind::f16 and completed through
// tcgen05.commit on an mbarrier.  Weight gradients are GEMMs over the samples
// (K = the 128 rows of a tile) and accumulate in tensor memory across the
// tiles a CTA processes; per-CTA partial sums are reduced in a fixed order.
//
// No counterpart in the reference: the learned warm start is new.
#include "sd_common.cuh"

#include <cuda_bf16.h>

namespace sd {

namespace {

constexpr int kRows = 128;    // tile rows = threads per CTA = TMEM lanes
constexpr int kIn = 16, kHid = 64, kOut = 16;
constexpr uint32_t kMmaSpin = 1u << 22;

// parameter offsets (floats)
constexpr int kW1 = 0, kB1 = kW1 + kHid * kIn, kW2 = kB1 + kHid, kB2 = kW2 + kHid * kHid, kW3 = kB2 + kHid,
              kB3 = kW3 + kOut * kHid, kParams = kB3 + kOut;
static_assert(kParams == 6288, "parameter layout");

// packed BF16 operand images (bytes), canonical K-major layouts
constexpr uint32_t kImgW1 = 0;                       // N 64 x K 16
constexpr uint32_t kImgW2 = kImgW1 + kHid * kIn * 2;  // N 64 x K 64
constexpr uint32_t kImgW3 = kImgW2 + kHid * kHid * 2; // N 16 x K 64
constexpr uint32_t kImgW2T = kImgW3 + kOut * kHid * 2;  // N 64 x K 64 (W2 transposed)
constexpr uint32_t kImgW3T = kImgW2T + kHid * kHid * 2; // N 64 x K 16 (W3 transposed)
constexpr uint32_t kImgBytes = kImgW3T + kHid * kOut * 2;

// Byte offset of element (r, k) of a K-major BF16 operand with K columns:
// 8x8 core matrices of 128 contiguous bytes, K-adjacent cores 128 B apart
// (leading byte offset), 8-row groups (K/8)*128 B apart (stride byte offset).
__host__ __device__ constexpr uint32_t cm_off(uint32_t r, uint32_t k, uint32_t K) {
    return ((r >> 3) * (K >> 3) + (k >> 3)) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor (tcgen05): start >> 4, LBO >> 4, SBO >> 4,
// version 1 at bit 46, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

// Instruction descriptor, kind::f16: D FP32, A and B BF16, both K-major.
__host__ __device__ constexpr uint32_t idesc(uint32_t M, uint32_t N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(id), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
                 : "memory");
}

__device__ __forceinline__ void mbar_init1(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (uint32_t it = 0; it < kMmaSpin; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(ok)
            : "r"(saddr(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
        if (it > 64) __nanosleep(32);
    }
    return false;
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive FP32 columns of this thread's lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ uint16_t bf16_bits(float x) {
    return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}
__device__ __forceinline__ float bf16_val(uint16_t b) { return __bfloat162float(__ushort_as_bfloat16(b)); }

__device__ __forceinline__ void st_bf16(uint8_t* base, uint32_t off, float x) {
    *reinterpret_cast<uint16_t*>(base + off) = bf16_bits(x);
}
__device__ __forceinline__ float ld_bf16(const uint8_t* base, uint32_t off) {
    return bf16_val(*reinterpret_cast<const uint16_t*>(base + off));
}

// D (tmem columns at d) [+]= A (128 x K, K-major) * B (N x K, K-major)^T.
__device__ __forceinline__ void gemm_issue(uint32_t d, const uint8_t* A, const uint8_t* B, uint32_t N, uint32_t K,
                                           bool accumulate) {
    const uint32_t sboA = (K >> 3) * 128u, sboB = sboA;
    const uint32_t id = idesc(kRows, N);
    for (uint32_t s = 0; s < K / 16; ++s) {
        const uint64_t a = sdesc(saddr(A) + s * 256u, 128u, sboA);
        const uint64_t b = sdesc(saddr(B) + s * 256u, 128u, sboB);
        mma_f16(d, a, b, id, (accumulate || s > 0) ? 1u : 0u);
    }
}

// One GEMM step: thread 0 issues and commits, everyone waits for the commit.
// Returns false (and flags) if the wait gave up.
__device__ __forceinline__ bool gemm_sync(uint32_t d, const uint8_t* A, const uint8_t* B, uint32_t N, uint32_t K,
                                          bool accumulate, uint64_t* bar, uint32_t& phase, uint32_t* status) {
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x == 0) {
        gemm_issue(d, A, B, N, K, accumulate);
        mma_commit(bar);
    }
    const bool mine = mbar_wait(bar, phase);
    const bool ok = __syncthreads_and(mine) != 0;  // one verdict for the whole CTA
    if (ok) {
        phase ^= 1u;
    } else {
        atomicOr(status, kErrWaitTimeout);
    }
    tc_fence_after();
    return ok;
}

// After a wait gave up: wait once more (bounded) for the MMAs in flight
// before the caller frees tensor memory.
__device__ __forceinline__ void drain(uint64_t* bar, uint32_t phase) { (void)mbar_wait(bar, phase); }

// The CTA's shared-memory view, aligned to 1 KB (the launch adds 1 KB).
__device__ __forceinline__ uint8_t* aligned_smem(uint8_t* raw) {
    const uint32_t pad = (1024u - (saddr(raw) & 1023u)) & 1023u;
    return raw + pad;
}

__device__ __forceinline__ void copy_img(uint8_t* dst, const uint8_t* src, uint32_t bytes) {
    const uint4* s = reinterpret_cast<const uint4*>(src);
    uint4* d = reinterpret_cast<uint4*>(dst);
    for (uint32_t i = threadIdx.x; i < bytes / 16; i += blockDim.x) d[i] = s[i];
}

struct InferSmem {
    alignas(1024) uint8_t w1[kHid * kIn * 2];
    alignas(1024) uint8_t w2[kHid * kHid * 2];
    alignas(1024) uint8_t w3[kOut * kHid * 2];
    alignas(1024) uint8_t x[kRows * kIn * 2];
    alignas(1024) uint8_t h1[kRows * kHid * 2];
    alignas(1024) uint8_t h2[kRows * kHid * 2];
    float b[kHid + kHid + kOut];
    uint64_t bar;
    uint32_t tmem;
};

// Forward pass over tiles of 128 rows of feat (16 floats per row).
// MODE 0: seeds[e] = (y0, y1, y2, 1) for rows with the previous-contact flag
//         (feat[7] == 1), else zero; rows e < *d_count.
// MODE 1: out[e] = (y0, y1, y2, 0), rows e < n.
template <int MODE>
__global__ void __launch_bounds__(kRows) mlp_forward_kernel(const uint8_t* __restrict__ img,
                                                           const float* __restrict__ params,
                                                           const float* __restrict__ feat, float4* __restrict__ out,
                                                           const uint32_t* __restrict__ d_count, uint64_t n,
                                                           uint32_t* __restrict__ status) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    InferSmem& S = *reinterpret_cast<InferSmem*>(aligned_smem(smem_raw));
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    const uint64_t rows = MODE == 0 ? min((uint64_t)*d_count, n) : n;
    const uint64_t tiles = (rows + kRows - 1) / kRows;
    if ((uint64_t)blockIdx.x >= tiles) return;
    copy_img(S.w1, img + kImgW1, sizeof S.w1);
    copy_img(S.w2, img + kImgW2, sizeof S.w2);
    copy_img(S.w3, img + kImgW3, sizeof S.w3);
    for (uint32_t i = tid; i < kHid; i += kRows) {
        S.b[i] = params[kB1 + i];
        S.b[kHid + i] = params[kB2 + i];
    }
    if (tid < kOut) S.b[2 * kHid + tid] = params[kB3 + tid];
    if (warp == 0) tmem_alloc(&S.tmem, 256);
    if (tid == 0) mbar_init1(&S.bar);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tm = S.tmem;
    const uint32_t lane_base = (warp * 32u) << 16;
    uint32_t phase = 0;
    bool ok = true;
    for (uint64_t t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
        const uint64_t e = t * kRows + tid;
        const bool live = e < rows;
        float f7 = 0.f, skip[3] = {0.f, 0.f, 0.f};
        // layer 1 operand: this thread's row of inputs
        for (int k = 0; k < kIn; ++k) {
            const float v = live ? feat[16 * e + k] : 0.0f;
            if (k == 7) f7 = v;
            if (k >= 8 && k < 11) skip[k - 8] = v;
            st_bf16(S.x, cm_off(tid, k, kIn), v);
        }
        if (!(ok = gemm_sync(tm + 0, S.x, S.w1, kHid, kIn, false, &S.bar, phase, status))) break;
        for (int c = 0; c < kHid; c += 16) {
            float v[16];
            tmem_ld16(tm + lane_base + c, v);
#pragma unroll
            for (int k = 0; k < 16; ++k) st_bf16(S.h1, cm_off(tid, c + k, kHid), fmaxf(v[k] + S.b[c + k], 0.0f));
        }
        if (!(ok = gemm_sync(tm + 64, S.h1, S.w2, kHid, kHid, false, &S.bar, phase, status))) break;
        for (int c = 0; c < kHid; c += 16) {
            float v[16];
            tmem_ld16(tm + lane_base + 64 + c, v);
#pragma unroll
            for (int k = 0; k < 16; ++k)
                st_bf16(S.h2, cm_off(tid, c + k, kHid), fmaxf(v[k] + S.b[kHid + c + k], 0.0f));
        }
        if (!(ok = gemm_sync(tm + 128, S.h2, S.w3, kOut, kHid, false, &S.bar, phase, status))) break;
        float y[16];
        tmem_ld16(tm + lane_base + 128, y);
        if (live) {
            const float y0 = (y[0] + S.b[2 * kHid]) + skip[0], y1 = (y[1] + S.b[2 * kHid + 1]) + skip[1],
                        y2 = (y[2] + S.b[2 * kHid + 2]) + skip[2];
            if (MODE == 0)
                out[e] = f7 == 1.0f ? make_float4(y0, y1, y2, 1.0f) : make_float4(0.f, 0.f, 0.f, 0.f);
            else
                out[e] = make_float4(y0, y1, y2, 0.f);
        }
        tc_fence_before();
        __syncthreads();  // the tile's operands are reused by the next tile
        tc_fence_after();
    }
    if (!ok) drain(&S.bar, phase);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tm, 256);
}

struct TrainSmem {
    alignas(1024) uint8_t w1[kHid * kIn * 2];
    alignas(1024) uint8_t w2[kHid * kHid * 2];
    alignas(1024) uint8_t w3[kOut * kHid * 2];
    alignas(1024) uint8_t w2t[kHid * kHid * 2];
    alignas(1024) uint8_t w3t[kHid * kOut * 2];
    alignas(1024) uint8_t x[kRows * kIn * 2];
    alignas(1024) uint8_t h1[kRows * kHid * 2];
    alignas(1024) uint8_t h2[kRows * kHid * 2];
    alignas(1024) uint8_t dy[kRows * kOut * 2];
    alignas(1024) uint8_t dz2[kRows * kHid * 2];
    alignas(1024) uint8_t dz1[kRows * kHid * 2];
    // transposed operands of the weight gradients: A = 128 x 128 (rows 64..127
    // are the zero block that follows), B = up to 64 x 128
    alignas(1024) uint8_t at[kHid * kRows * 2];
    alignas(1024) uint8_t zero[kHid * kRows * 2];
    alignas(1024) uint8_t bt[kHid * kRows * 2];
    float b[kHid + kHid + kOut];
    float gb[kHid + kHid + kOut];
    uint64_t bar;
    uint32_t tmem;
};

// Forward + backward of the cosine loss 1 - y.t/|y| (mean over valid rows)
// for the tiles of this CTA; per-CTA gradient partials to part[cta][6288].
// tgt rows: (tx, ty, tz, valid).
__global__ void __launch_bounds__(kRows) mlp_train_kernel(const uint8_t* __restrict__ img,
                                                         const float* __restrict__ params,
                                                         const float* __restrict__ feat, const float4* __restrict__ tgt,
                                                         uint32_t n, float inv_batch, float* __restrict__ part,
                                                         uint32_t* __restrict__ status,
                                                         const uint32_t* __restrict__ d_count) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(aligned_smem(smem_raw));
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    if (d_count) n = min(n, *d_count);  // rows: the step's entry count, read on the device
    const uint32_t tiles = (n + kRows - 1) / kRows;
    copy_img(S.w1, img + kImgW1, sizeof S.w1);
    copy_img(S.w2, img + kImgW2, sizeof S.w2);
    copy_img(S.w3, img + kImgW3, sizeof S.w3);
    copy_img(S.w2t, img + kImgW2T, sizeof S.w2t);
    copy_img(S.w3t, img + kImgW3T, sizeof S.w3t);
    for (uint32_t i = tid; i < sizeof S.zero / 16; i += kRows) reinterpret_cast<uint4*>(S.zero)[i] = make_uint4(0, 0, 0, 0);
    for (uint32_t i = tid; i < kHid; i += kRows) {
        S.b[i] = params[kB1 + i];
        S.b[kHid + i] = params[kB2 + i];
    }
    if (tid < kOut) S.b[2 * kHid + tid] = params[kB3 + tid];
    for (uint32_t i = tid; i < 2 * kHid + kOut; i += kRows) S.gb[i] = 0.0f;
    if (warp == 0) tmem_alloc(&S.tmem, 256);
    if (tid == 0) mbar_init1(&S.bar);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tm = S.tmem;
    const uint32_t lane_base = (warp * 32u) << 16;
    // tensor-memory columns: forward and activation gradients reuse [0, 144);
    // the weight gradients accumulate over tiles in [144, 240)
    const uint32_t cL1 = 0, cL2 = 64, cL3 = 128, cG3 = 144, cG2 = 160, cG1 = 224;
    uint32_t phase = 0;
    bool ok = true;
    bool first = true;
    for (uint32_t t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
        const uint32_t e = t * kRows + tid;
        const bool live = e < n;
        float skip[3] = {0.f, 0.f, 0.f};
        for (int k = 0; k < kIn; ++k) {
            const float v = live ? feat[16 * (size_t)e + k] : 0.0f;
            if (k >= 8 && k < 11) skip[k - 8] = v;
            st_bf16(S.x, cm_off(tid, k, kIn), v);
        }
        ok = gemm_sync(tm + cL1, S.x, S.w1, kHid, kIn, false, &S.bar, phase, status);
        if (!ok) break;
        for (int c = 0; c < kHid; c += 16) {
            float v[16];
            tmem_ld16(tm + lane_base + cL1 + c, v);
#pragma unroll
            for (int k = 0; k < 16; ++k) st_bf16(S.h1, cm_off(tid, c + k, kHid), fmaxf(v[k] + S.b[c + k], 0.0f));
        }
        ok = gemm_sync(tm + cL2, S.h1, S.w2, kHid, kHid, false, &S.bar, phase, status);
        if (!ok) break;
        for (int c = 0; c < kHid; c += 16) {
            float v[16];
            tmem_ld16(tm + lane_base + cL2 + c, v);
#pragma unroll
            for (int k = 0; k < 16; ++k)
                st_bf16(S.h2, cm_off(tid, c + k, kHid), fmaxf(v[k] + S.b[kHid + c + k], 0.0f));
        }
        ok = gemm_sync(tm + cL3, S.h2, S.w3, kOut, kHid, false, &S.bar, phase, status);
        if (!ok) break;
        {
            float y[16];
            tmem_ld16(tm + lane_base + cL3, y);
            const float4 g = live ? tgt[e] : make_float4(0.f, 0.f, 0.f, 0.f);
            float d[3] = {0.f, 0.f, 0.f};
            if (g.w != 0.0f) {
                const float y0 = (y[0] + S.b[2 * kHid]) + skip[0], y1 = (y[1] + S.b[2 * kHid + 1]) + skip[1],
                            y2 = (y[2] + S.b[2 * kHid + 2]) + skip[2];
                const float nn = sqrtf(((y0 * y0 + y1 * y1) + y2 * y2) + 1e-8f);
                const float c = ((y0 * g.x + y1 * g.y) + y2 * g.z) / nn;
                const float s = -inv_batch / nn;
                d[0] = s * (g.x - c * y0 / nn);
                d[1] = s * (g.y - c * y1 / nn);
                d[2] = s * (g.z - c * y2 / nn);
            }
            for (int k = 0; k < kOut; ++k) st_bf16(S.dy, cm_off(tid, k, kOut), k < 3 ? d[k] : 0.0f);
        }
        // dH2 = dY W3  (B = W3^T, N 64 x K 16)
        ok = gemm_sync(tm + cL1, S.dy, S.w3t, kHid, kOut, false, &S.bar, phase, status);
        if (!ok) break;
        for (int c = 0; c < kHid; c += 16) {
            float v[16];
            tmem_ld16(tm + lane_base + cL1 + c, v);
#pragma unroll
            for (int k = 0; k < 16; ++k) {
                const uint32_t o = cm_off(tid, c + k, kHid);
                st_bf16(S.dz2, o, ld_bf16(S.h2, o) > 0.0f ? v[k] : 0.0f);
            }
        }
        // dH1 = dZ2 W2  (B = W2^T)
        ok = gemm_sync(tm + cL2, S.dz2, S.w2t, kHid, kHid, false, &S.bar, phase, status);
        if (!ok) break;
        for (int c = 0; c < kHid; c += 16) {
            float v[16];
            tmem_ld16(tm + lane_base + cL2 + c, v);
#pragma unroll
            for (int k = 0; k < 16; ++k) {
                const uint32_t o = cm_off(tid, c + k, kHid);
                st_bf16(S.dz1, o, ld_bf16(S.h1, o) > 0.0f ? v[k] : 0.0f);
            }
        }
        __syncthreads();
        // bias gradients: column sums over the tile's rows, fixed order
        if (tid < kHid) {
            float a1 = 0.f, a2 = 0.f;
            for (uint32_t m = 0; m < kRows; ++m) {
                a1 += ld_bf16(S.dz1, cm_off(m, tid, kHid));
                a2 += ld_bf16(S.dz2, cm_off(m, tid, kHid));
            }
            S.gb[tid] += a1;
            S.gb[kHid + tid] += a2;
        } else if (tid < kHid + 3) {
            const uint32_t o = tid - kHid;
            float a3 = 0.f;
            for (uint32_t m = 0; m < kRows; ++m) a3 += ld_bf16(S.dy, cm_off(m, o, kOut));
            S.gb[2 * kHid + o] += a3;
        }
        // weight gradients, K = the tile's rows.  dW3^T (j, o) = H2^T dY
        for (int j = 0; j < kHid; ++j) {
            const uint16_t hv = *reinterpret_cast<const uint16_t*>(S.h2 + cm_off(tid, j, kHid));
            *reinterpret_cast<uint16_t*>(S.at + cm_off(j, tid, kRows)) = hv;
        }
        for (int o = 0; o < kOut; ++o) {
            const uint16_t dv = *reinterpret_cast<const uint16_t*>(S.dy + cm_off(tid, o, kOut));
            *reinterpret_cast<uint16_t*>(S.bt + cm_off(o, tid, kRows)) = dv;
        }
        ok = gemm_sync(tm + cG3, S.at, S.bt, kOut, kRows, !first, &S.bar, phase, status);
        if (!ok) break;
        // dW2 (k, j) = dZ2^T H1
        for (int j = 0; j < kHid; ++j) {
            const uint16_t a = *reinterpret_cast<const uint16_t*>(S.dz2 + cm_off(tid, j, kHid));
            const uint16_t b = *reinterpret_cast<const uint16_t*>(S.h1 + cm_off(tid, j, kHid));
            *reinterpret_cast<uint16_t*>(S.at + cm_off(j, tid, kRows)) = a;
            *reinterpret_cast<uint16_t*>(S.bt + cm_off(j, tid, kRows)) = b;
        }
        ok = gemm_sync(tm + cG2, S.at, S.bt, kHid, kRows, !first, &S.bar, phase, status);
        if (!ok) break;
        // dW1 (j, i) = dZ1^T X
        for (int j = 0; j < kHid; ++j) {
            const uint16_t a = *reinterpret_cast<const uint16_t*>(S.dz1 + cm_off(tid, j, kHid));
            *reinterpret_cast<uint16_t*>(S.at + cm_off(j, tid, kRows)) = a;
        }
        for (int i = 0; i < kIn; ++i) {
            const uint16_t b = *reinterpret_cast<const uint16_t*>(S.x + cm_off(tid, i, kIn));
            *reinterpret_cast<uint16_t*>(S.bt + cm_off(i, tid, kRows)) = b;
        }
        ok = gemm_sync(tm + cG1, S.at, S.bt, kIn, kRows, !first, &S.bar, phase, status);
        first = false;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    float* P = part + (size_t)blockIdx.x * kParams;
    if (ok && !first) {
        if (warp < 2) {  // lanes 0..63 hold the 64 rows of every weight gradient
            const uint32_t r = tid;
            float v[16];
            tmem_ld16(tm + lane_base + cG3, v);  // dW3^T row j = r
#pragma unroll
            for (int o = 0; o < kOut; ++o) P[kW3 + o * kHid + r] = o < 3 ? v[o] : 0.0f;
            for (int c = 0; c < kHid; c += 16) {
                tmem_ld16(tm + lane_base + cG2 + c, v);
#pragma unroll
                for (int k = 0; k < 16; ++k) P[kW2 + r * kHid + c + k] = v[k];
            }
            tmem_ld16(tm + lane_base + cG1, v);
#pragma unroll
            for (int i = 0; i < kIn; ++i) P[kW1 + r * kIn + i] = v[i];
        }
        for (uint32_t i = tid; i < kHid; i += kRows) {
            P[kB1 + i] = S.gb[i];
            P[kB2 + i] = S.gb[kHid + i];
        }
        if (tid < kOut) P[kB3 + tid] = tid < 3 ? S.gb[2 * kHid + tid] : 0.0f;
    } else {
        for (uint32_t i = tid; i < kParams; i += kRows) P[i] = 0.0f;
    }
    if (!ok) drain(&S.bar, phase);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tm, 256);
}

// grad[p] = sum over CTAs of part[c][p], in CTA order; then (adam != 0) an
// Adam step on the master parameters (W3, b3 rows 3..15 stay zero).
__global__ void mlp_reduce_kernel(const float* __restrict__ part, uint32_t nparts, float* __restrict__ grad,
                                  float* __restrict__ params, float* __restrict__ m1, float* __restrict__ m2,
                                  int adam, float lr, float c1, float c2) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (uint32_t)kParams) return;
    float g = 0.0f;
    for (uint32_t c = 0; c < nparts; ++c) g += part[(size_t)c * kParams + p];
    const bool dead = (p >= (uint32_t)kW3 && p < (uint32_t)kB3 && (p - kW3) / kHid >= 3) || (p >= (uint32_t)kB3 + 3);
    if (dead) g = 0.0f;
    if (grad) grad[p] = g;
    if (!adam || dead) return;
    const float a = 0.9f * m1[p] + 0.1f * g;
    const float b = 0.999f * m2[p] + 0.001f * (g * g);
    m1[p] = a;
    m2[p] = b;
    params[p] -= lr * (a * c1) / (sqrtf(b * c2) + 1e-8f);
}

// BF16 operand images of W1, W2, W3 and the transposes W2^T, W3^T.
__global__ void mlp_pack_kernel(const float* __restrict__ params, uint8_t* __restrict__ img) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < (uint32_t)(kHid * kIn)) {  // W1 [n][k]
        const uint32_t r = i / kIn, k = i % kIn;
        *reinterpret_cast<uint16_t*>(img + kImgW1 + cm_off(r, k, kIn)) = bf16_bits(params[kW1 + i]);
    }
    if (i < (uint32_t)(kHid * kHid)) {  // W2 [n][k] and W2^T [n=k_in][k=k_out]
        const uint32_t r = i / kHid, k = i % kHid;
        const uint16_t b = bf16_bits(params[kW2 + i]);
        *reinterpret_cast<uint16_t*>(img + kImgW2 + cm_off(r, k, kHid)) = b;
        *reinterpret_cast<uint16_t*>(img + kImgW2T + cm_off(k, r, kHid)) = b;
    }
    if (i < (uint32_t)(kOut * kHid)) {  // W3 [o][j] and W3^T [j][o]
        const uint32_t o = i / kHid, j = i % kHid;
        const uint16_t b = bf16_bits(params[kW3 + i]);
        *reinterpret_cast<uint16_t*>(img + kImgW3 + cm_off(o, j, kHid)) = b;
        *reinterpret_cast<uint16_t*>(img + kImgW3T + cm_off(j, o, kOut)) = b;
    }
}

inline uint32_t grid_for(uint64_t n, int threads) { return (uint32_t)((n + threads - 1) / threads); }

constexpr uint32_t kMaxTrainCtas = 148;

}  // namespace

// Device state: params | m1 | m2 | grad | image | partials | status
uint64_t mlp_state_bytes() {
    return 4ull * kParams * 4 + kImgBytes + 4ull * kParams * kMaxTrainCtas + 256;
}
uint32_t mlp_param_count() { return kParams; }

MlpState mlp_carve(void* base) {
    MlpState s;
    char* p = static_cast<char*>(base);
    s.params = reinterpret_cast<float*>(p);
    s.m1 = s.params + kParams;
    s.m2 = s.m1 + kParams;
    s.grad = s.m2 + kParams;
    s.img = reinterpret_cast<uint8_t*>(s.grad + kParams);
    s.part = reinterpret_cast<float*>(s.img + kImgBytes);
    s.status = reinterpret_cast<uint32_t*>(s.part + (size_t)kParams * kMaxTrainCtas);
    return s;
}

cudaError_t mlp_init_kernels() {
    cudaError_t e = cudaFuncSetAttribute(mlp_forward_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(InferSmem) + 1024);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(mlp_forward_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(InferSmem) + 1024);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(TrainSmem) + 1024);
    return e;
}

cudaError_t mlp_set_params_async(MlpState& s, const float* host_params, cudaStream_t st) {
    cudaError_t e = cudaMemcpyAsync(s.params, host_params, 4ull * kParams, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s.m1, 0, 8ull * kParams, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s.img, 0, kImgBytes, st);
    if (e != cudaSuccess) return e;
    mlp_pack_kernel<<<grid_for(kHid * kHid, 256), 256, 0, st>>>(s.params, s.img);
    return cudaGetLastError();
}

// The dynamic shared memory base is only 16-byte aligned by default; the
// launch asks for 1 KB more and the kernel uses an aligned view.  (The
// __align__ on the extern array gives 1024-byte alignment on sm_90+.)
cudaError_t mlp_forward_async(const MlpState& s, const float* feat, float4* out, const uint32_t* d_count, uint64_t n,
                              bool seeds, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const uint32_t tiles = grid_for(n, kRows);
    const uint32_t grid = tiles < 304 ? tiles : 304;
    const size_t sm = sizeof(InferSmem) + 1024;
    if (seeds)
        mlp_forward_kernel<0><<<grid, kRows, sm, st>>>(s.img, s.params, feat, out, d_count, n, s.status);
    else
        mlp_forward_kernel<1><<<grid, kRows, sm, st>>>(s.img, s.params, feat, out, nullptr, n, s.status);
    return cudaGetLastError();
}

cudaError_t mlp_train_async(MlpState& s, const float* feat, const float4* tgt, uint32_t n, uint32_t n_valid, float lr,
                            uint32_t adam_step, bool update, cudaStream_t st, const uint32_t* d_count) {
    if (n == 0) return cudaSuccess;
    const uint32_t tiles = grid_for(n, kRows);
    const uint32_t ctas = tiles < kMaxTrainCtas ? tiles : kMaxTrainCtas;
    const float inv = n_valid ? 1.0f / (float)n_valid : 0.0f;
    mlp_train_kernel<<<ctas, kRows, sizeof(TrainSmem) + 1024, st>>>(s.img, s.params, feat, tgt, n, inv, s.part,
                                                                     s.status, d_count);
    const float c1 = update ? (float)(1.0 / (1.0 - std::pow(0.9, (double)adam_step))) : 0.f;
    const float c2 = update ? (float)(1.0 / (1.0 - std::pow(0.999, (double)adam_step))) : 0.f;
    mlp_reduce_kernel<<<grid_for(kParams, 256), 256, 0, st>>>(s.part, ctas, s.grad, s.params, s.m1, s.m2,
                                                              update ? 1 : 0, lr, c1, c2);
    if (update) mlp_pack_kernel<<<grid_for(kHid * kHid, 256), 256, 0, st>>>(s.params, s.img);
    return cudaGetLastError();
}

}  // namespace sd
