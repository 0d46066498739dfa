// sd_lbvh.cu -- linear BVH broad phase over axis-aligned boxes.
//
// Replaces the LBVH prototype of sandbox/testLBVH.cu (:42-907), which
// builds its tree from Thrust/CUB calls, a depth probe with a device-to-host
// copy (:1148-1149) and depth+1 refit launches.  Here:
//   1. bounds: a two-level min/max reduction of the boxes (the global
//      domain, constructGlobalDomain, testLBVH.cu:82-89);
//   2. Morton codes exactly as computeSpaceFillingCurveCUDA (:113-151):
//      30 bits, centroid relative to the domain centre in units of
//      domain/1024, clamped to [-512, 511];
//   3. this library's onesweep radix sort of (code, index), 30-bit keys;
//   4. Karras (2012) binary radix tree, one thread per internal node, ties
//      between equal codes broken by the leaf index;
//   5. refit in ONE launch: every leaf climbs towards the root and the
//      second thread to reach a node (atomic visit counter) writes its box;
//   6. per-leaf stack traversal, in two passes (count, then write after an
//      exclusive scan) so every body gets a compact, deterministic partner
//      list, sorted by partner id in the writing thread.
// The pair set is the exact set of overlapping closed boxes, independent of
// the tree's shape.
#include "sd_common.cuh"

#include <utility>

namespace sd {

namespace {

constexpr int kLbvhThreads = 256;
constexpr uint32_t kLeaf = 0x80000000u;
constexpr int kStack = 64;  // Karras tree depth <= 32 code bits + 32 index bits

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr uint32_t kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ bool box_overlap(float4 alo, float4 ahi, float4 blo, float4 bhi) {
    return blo.x <= ahi.x && alo.x <= bhi.x && blo.y <= ahi.y && alo.y <= bhi.y && blo.z <= ahi.z &&
           alo.z <= bhi.z;
}

// ---------------------------------------------------------------- scan

__global__ void scan_reduce_kernel(const uint32_t* __restrict__ in, uint32_t n, uint32_t* __restrict__ part) {
    __shared__ uint32_t ws[33];
    const uint32_t base = blockIdx.x * kScanTile;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const uint32_t i = base + k * kScanThreads + threadIdx.x;
        if (i < n) s += in[i];
    }
    uint32_t total;
    block_exclusive_scan(s, ws, &total);
    if (threadIdx.x == 0) part[blockIdx.x] = total;
}

// One block: exclusive scan of the tile sums; part[nt] = grand total.
__global__ void scan_partials_kernel(uint32_t* __restrict__ part, uint32_t nt, uint32_t* __restrict__ total_out) {
    __shared__ uint32_t ws[33];
    uint32_t carry = 0;
    for (uint32_t b = 0; b < nt; b += blockDim.x) {
        const uint32_t i = b + threadIdx.x;
        const uint32_t v = i < nt ? part[i] : 0u;
        uint32_t tot;
        const uint32_t ex = block_exclusive_scan(v, ws, &tot);
        if (i < nt) part[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) *total_out = carry;
}

__global__ void scan_apply_kernel(const uint32_t* __restrict__ in, uint32_t n, const uint32_t* __restrict__ part,
                                  uint32_t* __restrict__ out) {
    __shared__ uint32_t ws[33];
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < n ? in[base + k] : 0u;
        s += v[k];
    }
    uint32_t tot;
    uint32_t run = part[blockIdx.x] + block_exclusive_scan(s, ws, &tot);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
}

// ------------------------------------------------------------ bounds

__global__ void bounds_partial_kernel(const float4* __restrict__ lo, const float4* __restrict__ hi, uint32_t n,
                                      float* __restrict__ part) {
    __shared__ float s[6][kLbvhThreads];
    float m[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = lo[i], b = hi[i];
        m[0] = fminf(m[0], a.x); m[1] = fminf(m[1], a.y); m[2] = fminf(m[2], a.z);
        m[3] = fmaxf(m[3], b.x); m[4] = fmaxf(m[4], b.y); m[5] = fmaxf(m[5], b.z);
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) s[k][threadIdx.x] = m[k];
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                s[k][threadIdx.x] = fminf(s[k][threadIdx.x], s[k][threadIdx.x + o]);
                s[k + 3][threadIdx.x] = fmaxf(s[k + 3][threadIdx.x], s[k + 3][threadIdx.x + o]);
            }
        }
        __syncthreads();
    }
    if (threadIdx.x < 6) part[6 * blockIdx.x + threadIdx.x] = s[threadIdx.x][0];
}

__global__ void bounds_final_kernel(const float* __restrict__ part, uint32_t nb, float* __restrict__ bounds) {
    if (threadIdx.x >= 6) return;
    const int k = threadIdx.x;
    float m = k < 3 ? INFINITY : -INFINITY;
    for (uint32_t b = 0; b < nb; ++b) m = k < 3 ? fminf(m, part[6 * b + k]) : fmaxf(m, part[6 * b + k]);
    bounds[k] = m;
}

// --------------------------------------------------------------- Morton

__device__ __forceinline__ uint32_t spread10(uint32_t x) {
    x &= 0x3ffu;
    x = (x ^ (x << 16)) & 0xff0000ffu;
    x = (x ^ (x << 8)) & 0x0300f00fu;
    x = (x ^ (x << 4)) & 0x030c30c3u;
    x = (x ^ (x << 2)) & 0x09249249u;
    return x;
}

__global__ void morton_kernel(const float4* __restrict__ lo, const float4* __restrict__ hi, uint32_t n,
                              const float* __restrict__ bounds, uint32_t* __restrict__ keys,
                              uint32_t* __restrict__ vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = lo[i], b = hi[i];
    const float c[3] = {(a.x + b.x) * 0.5f, (a.y + b.y) * 0.5f, (a.z + b.z) * 0.5f};
    uint32_t q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float cen = (bounds[k] + bounds[3 + k]) * 0.5f;
        const float cell = (bounds[3 + k] - bounds[k]) / 1024.0f;
        const float p = cell > 0.0f ? (c[k] - cen) / cell : 0.0f;  // all centroids equal: code 512
        int32_t d = p >= 0.0f ? (int32_t)p : (int32_t)floorf(p);
        d = d < -512 ? -512 : (d > 511 ? 511 : d);
        q[k] = (uint32_t)(d + 512);
    }
    keys[i] = spread10(q[0]) | (spread10(q[1]) << 1) | (spread10(q[2]) << 2);
    vals[i] = i;
}

// ------------------------------------------------------------ radix tree

__device__ __forceinline__ int delta(const uint32_t* __restrict__ k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint32_t a = k[i], b = k[j];
    if (a == b) return 32 + __clz((uint32_t)(i ^ j));
    return __clz(a ^ b);
}

// Karras, "Maximizing Parallelism in the Construction of BVHs, Octrees, and
// k-d Trees" (HPG 2012), Figure 4.  parent[] holds internal nodes at
// [0, n-1) and leaves at [n-1, 2n-1).
__global__ void build_kernel(const uint32_t* __restrict__ keys, int n, int2* __restrict__ children,
                             int32_t* __restrict__ parent) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(keys, n, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int g = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    const int left = lo == g ? (int)(g | kLeaf) : g;
    const int right = hi == g + 1 ? (int)((g + 1) | kLeaf) : g + 1;
    children[i] = make_int2(left, right);
    parent[lo == g ? (n - 1) + g : g] = i;
    parent[hi == g + 1 ? (n - 1) + g + 1 : g + 1] = i;
}

__device__ __forceinline__ float4 ldcg4(const float4* p) { return __ldcg(p); }

// A child reference is a leaf below n or an internal node below n - 1.
__device__ __forceinline__ bool child_ok(int c, int n) {
    return (c & kLeaf) ? (c & ~kLeaf) < n : (c >= 0 && c < n - 1);
}

// Bottom-up boxes: the last of a node's two children to finish computes
// the node's box and writes the node's record -- both children's boxes,
// each lower corner's w lane holding the child reference -- which the
// traversal reads in one 64-byte piece instead of the children's indices
// and then their boxes.
__global__ void refit_kernel(int n, const uint32_t* __restrict__ vals, const float4* __restrict__ lo,
                             const float4* __restrict__ hi, float4* leaf_lo, float4* leaf_hi, float4* node_lo,
                             float4* node_hi, const int2* __restrict__ children, const int32_t* __restrict__ parent,
                             uint32_t* visit, float4* __restrict__ rec, uint32_t* __restrict__ status) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t id = vals[k];
    leaf_lo[k] = lo[id];
    leaf_hi[k] = hi[id];
    __threadfence();
    int p = n > 1 ? parent[(n - 1) + k] : -1;
    for (int level = 0; p >= 0; ++level) {
        if (level > 2 * kStack || p >= n - 1) {  // a malformed tree: report, never loop or stray
            atomicOr(status, kErrBadInput);
            return;
        }
        if (atomicAdd(&visit[p], 1u) == 0u) return;  // the sibling subtree is not done yet
        __threadfence();
        const int2 c = children[p];
        if (!child_ok(c.x, n) || !child_ok(c.y, n)) {
            atomicOr(status, kErrBadInput);
            return;
        }
        float4 a0, a1, b0, b1;
        if (c.x & kLeaf) { a0 = ldcg4(leaf_lo + (c.x & ~kLeaf)); a1 = ldcg4(leaf_hi + (c.x & ~kLeaf)); }
        else { a0 = ldcg4(node_lo + c.x); a1 = ldcg4(node_hi + c.x); }
        if (c.y & kLeaf) { b0 = ldcg4(leaf_lo + (c.y & ~kLeaf)); b1 = ldcg4(leaf_hi + (c.y & ~kLeaf)); }
        else { b0 = ldcg4(node_lo + c.y); b1 = ldcg4(node_hi + c.y); }
        node_lo[p] = make_float4(fminf(a0.x, b0.x), fminf(a0.y, b0.y), fminf(a0.z, b0.z), 0.f);
        node_hi[p] = make_float4(fmaxf(a1.x, b1.x), fmaxf(a1.y, b1.y), fmaxf(a1.z, b1.z), 0.f);
        rec[4 * (size_t)p + 0] = make_float4(a0.x, a0.y, a0.z, __int_as_float(c.x));
        rec[4 * (size_t)p + 1] = a1;
        rec[4 * (size_t)p + 2] = make_float4(b0.x, b0.y, b0.z, __int_as_float(c.y));
        rec[4 * (size_t)p + 3] = b1;
        __threadfence();
        p = parent[p];
    }
}

// Traversal of leaf k (sorted position) against the tree.  WRITE == false:
// count[id] = number of partners, and the first kLbvhFirst partners found
// into first[k * kLbvhFirst ...].  WRITE == true: partners of body id at
// [off[id], off[id+1]), ascending, and self[] of each entry -- sorted from
// first[] when the counting pass kept them all, else found by a second
// traversal.
template <bool WRITE>
__global__ void query_kernel(int n, const uint32_t* __restrict__ vals, const float4* __restrict__ leaf_lo,
                             const float4* __restrict__ leaf_hi, const float4* __restrict__ rec,
                             uint32_t* __restrict__ count, const uint32_t* __restrict__ off,
                             uint32_t* __restrict__ partners, uint32_t* __restrict__ self, uint64_t cap,
                             uint32_t* __restrict__ first, uint32_t* __restrict__ status) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t id = vals[k];
    uint32_t c = 0;
    const uint32_t base = WRITE ? off[id] : 0u;
    const uint32_t lim = WRITE ? off[id + 1] : 0u;
    if constexpr (WRITE) {
      if (lim - base <= (uint32_t)kLbvhFirst) {
        if ((uint64_t)lim > cap) {
            atomicOr(status, kErrPairOverflow);
            return;
        }
        // the partners the counting pass kept: sorted in registers (a
        // network over kLbvhFirst values; ids are distinct, so the order
        // is the ascending one)
        uint32_t v[kLbvhFirst];
#pragma unroll
        for (int i = 0; i < kLbvhFirst; ++i) v[i] = (uint32_t)i < lim - base ? first[(size_t)k * kLbvhFirst + i] : 0xffffffffu;
#pragma unroll
        for (int a = 0; a < kLbvhFirst; ++a)
#pragma unroll
            for (int b = (a & 1); b + 1 < kLbvhFirst; b += 2)
                if (v[b] > v[b + 1]) {
                    const uint32_t t = v[b];
                    v[b] = v[b + 1];
                    v[b + 1] = t;
                }
#pragma unroll
        for (int i = 0; i < kLbvhFirst; ++i)
            if ((uint32_t)i < lim - base) {
                partners[base + i] = v[i];
                self[base + i] = id;
            }
        return;
      }
    }
    const float4 qlo = leaf_lo[k], qhi = leaf_hi[k];
    if (n > 1) {
        int stack[kStack];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            const int node = stack[--sp];
            // the node's record: both children's boxes and references
            const float4 r0 = rec[4 * (size_t)node + 0], r1 = rec[4 * (size_t)node + 1];
            const float4 r2 = rec[4 * (size_t)node + 2], r3 = rec[4 * (size_t)node + 3];
            const int cx = __float_as_int(r0.w), cy = __float_as_int(r2.w);
            if (!child_ok(cx, n) || !child_ok(cy, n)) {
                atomicOr(status, kErrBadInput);
                continue;
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int x = h ? cy : cx;
                const float4 blo = h ? r2 : r0, bhi = h ? r3 : r1;
                if (x & kLeaf) {
                    const int j = x & ~kLeaf;
                    if (j == k || !box_overlap(qlo, qhi, blo, bhi)) continue;
                    if constexpr (WRITE) {
                        const uint32_t e = base + c;
                        if (e < lim && (uint64_t)e < cap) partners[e] = vals[j];
                    } else if (c < (uint32_t)kLbvhFirst) {
                        first[(size_t)k * kLbvhFirst + c] = vals[j];
                    }
                    ++c;
                } else if (box_overlap(qlo, qhi, blo, bhi)) {
                    if (sp < kStack) stack[sp++] = x;
                    else atomicOr(status, kErrPairOverflow);
                }
            }
        }
    }
    if constexpr (!WRITE) {
        count[id] = c;
    } else {
        if ((uint64_t)lim > cap) {
            atomicOr(status, kErrPairOverflow);
            return;
        }
        // sort the body's partner list ascending (insertion sort: lists are short)
        for (uint32_t e = base + 1; e < lim; ++e) {
            const uint32_t x = partners[e];
            uint32_t m = e;
            while (m > base && partners[m - 1] > x) {
                partners[m] = partners[m - 1];
                --m;
            }
            partners[m] = x;
        }
        for (uint32_t e = base; e < lim; ++e) self[e] = id;
    }
}

// Unique pairs (i < j) of the partner lists, ascending u64.
__global__ void upper_count_kernel(uint32_t n, const uint32_t* __restrict__ off, const uint32_t* __restrict__ partners,
                                   uint32_t* __restrict__ cnt, uint64_t partners_cap) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t c = 0;
    if ((uint64_t)off[n] > partners_cap) {  // overflowed lists are reported, not read
        cnt[i] = 0;
        return;
    }
    for (uint32_t e = off[i]; e < off[i + 1]; ++e) c += partners[e] > i;
    cnt[i] = c;
}

__global__ void upper_write_kernel(uint32_t n, const uint32_t* __restrict__ off, const uint32_t* __restrict__ partners,
                                   const uint32_t* __restrict__ pos, unsigned long long* __restrict__ out,
                                   uint64_t cap, uint64_t partners_cap) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (uint64_t)off[n] > partners_cap) return;
    uint32_t w = pos[i];
    for (uint32_t e = off[i]; e < off[i + 1]; ++e) {
        const uint32_t j = partners[e];
        if (j > i) {
            if (w < cap) out[w] = ((unsigned long long)i << 32) | j;
            ++w;
        }
    }
}

inline uint32_t grid_for(uint64_t n, int threads) { return (uint32_t)((n + threads - 1) / threads); }

inline uint32_t bounds_blocks(uint32_t n) {
    uint32_t b = grid_for(n, kLbvhThreads);
    return b < 1 ? 1 : (b > 304 ? 304 : b);
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

uint64_t scan_scratch_words(uint32_t n) { return grid_for(n, kScanTile) + 1; }

cudaError_t scan_exclusive_async(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* scratch,
                                 cudaStream_t st) {
    const uint32_t nt = grid_for(n, kScanTile);
    if (n == 0) return cudaMemsetAsync(out, 0, 4, st);
    scan_reduce_kernel<<<nt, kScanThreads, 0, st>>>(in, n, scratch);
    scan_partials_kernel<<<1, 1024, 0, st>>>(scratch, nt, out + n);
    scan_apply_kernel<<<nt, kScanThreads, 0, st>>>(in, n, scratch, out);
    return cudaGetLastError();
}

uint64_t lbvh_scratch_bytes(uint32_t n) {
    const uint64_t m = n ? n : 1;
    size_t b = 0;
    b += 4 * align256(4 * m);                                      // keys, vals, keys_tmp, vals_tmp
    b += align256(4 * sort_scratch_words(m, 30));                  // sort
    b += align256(4 * 8) + align256(4 * 6 * 304);                  // bounds + partials
    b += align256(8 * m) + align256(4 * (2 * m)) + align256(4 * m); // children, parent, visit
    b += 4 * align256(16 * m);                                     // node lo/hi, leaf lo/hi
    b += align256(4 * (m + 1)) + align256(4 * scan_scratch_words((uint32_t)m + 1));
    b += align256(4 * kLbvhFirst * m);                             // first partners per leaf
    b += align256(64 * m);                                         // node records
    b += align256(4 * 4);                                          // status
    return b;
}

void lbvh_carve(void* scratch, uint32_t n, Lbvh* t) {
    const uint64_t m = n ? n : 1;
    char* p = static_cast<char*>(scratch);
    auto take = [&](size_t bytes) {
        char* r = p;
        p += align256(bytes);
        return r;
    };
    t->n = n;
    t->keys = (uint32_t*)take(4 * m);
    t->vals = (uint32_t*)take(4 * m);
    t->keys_tmp = (uint32_t*)take(4 * m);
    t->vals_tmp = (uint32_t*)take(4 * m);
    t->sort_scratch = (uint32_t*)take(4 * sort_scratch_words(m, 30));
    t->bounds = (float*)take(4 * 8);
    t->bound_part = (float*)take(4 * 6 * 304);
    t->children = (int2*)take(8 * m);
    t->parent = (int32_t*)take(4 * 2 * m);
    t->visit = (uint32_t*)take(4 * m);
    t->node_lo = (float4*)take(16 * m);
    t->node_hi = (float4*)take(16 * m);
    t->leaf_lo = (float4*)take(16 * m);
    t->leaf_hi = (float4*)take(16 * m);
    t->counts = (uint32_t*)take(4 * (m + 1));
    t->scan_scratch = (uint32_t*)take(4 * scan_scratch_words((uint32_t)m + 1));
    t->first = (uint32_t*)take(4 * kLbvhFirst * m);
    t->rec = (float4*)take(64 * m);
    t->status = (uint32_t*)take(16);
    t->skeys = t->keys;
    t->svals = t->vals;
}

cudaError_t lbvh_morton_async(Lbvh& t, const float4* lo, const float4* hi, cudaStream_t st) {
    const uint32_t n = t.n;
    if (n == 0) return cudaSuccess;
    const uint32_t nb = bounds_blocks(n);
    bounds_partial_kernel<<<nb, kLbvhThreads, 0, st>>>(lo, hi, n, t.bound_part);
    bounds_final_kernel<<<1, 32, 0, st>>>(t.bound_part, nb, t.bounds);
    morton_kernel<<<grid_for(n, kLbvhThreads), kLbvhThreads, 0, st>>>(lo, hi, n, t.bounds, t.keys, t.vals);
    return cudaGetLastError();
}

cudaError_t lbvh_build_async(Lbvh& t, const float4* lo, const float4* hi, cudaStream_t st) {
    const uint32_t n = t.n;
    cudaError_t e;
    if (n == 0) return cudaSuccess;
    if ((e = lbvh_morton_async(t, lo, hi, st)) != cudaSuccess) return e;
    bool in_tmp = false;
    if ((e = sort_pairs_async(t.keys, t.vals, t.keys_tmp, t.vals_tmp, n, 30, t.sort_scratch, st, &in_tmp)) !=
        cudaSuccess)
        return e;
    t.skeys = in_tmp ? t.keys_tmp : t.keys;
    t.svals = in_tmp ? t.vals_tmp : t.vals;
    if ((e = cudaMemsetAsync(t.parent, 0xff, 4 * (2 * (size_t)n - 1), st)) != cudaSuccess) return e;
    if (n > 1) {
        if ((e = cudaMemsetAsync(t.visit, 0, 4 * ((size_t)n - 1), st)) != cudaSuccess) return e;
        build_kernel<<<grid_for(n - 1, kLbvhThreads), kLbvhThreads, 0, st>>>(t.skeys, (int)n, t.children,
                                                                              t.parent);
    }
    refit_kernel<<<grid_for(n, kLbvhThreads), kLbvhThreads, 0, st>>>((int)n, t.svals, lo, hi, t.leaf_lo, t.leaf_hi,
                                                                       t.node_lo, t.node_hi, t.children, t.parent,
                                                                       t.visit, t.rec, t.status);
    return cudaGetLastError();
}

cudaError_t lbvh_refit_async(Lbvh& t, const float4* lo, const float4* hi, cudaStream_t st) {
    const uint32_t n = t.n;
    if (n == 0) return cudaSuccess;
    cudaError_t e;
    if (n > 1 && (e = cudaMemsetAsync(t.visit, 0, 4 * ((size_t)n - 1), st)) != cudaSuccess) return e;
    refit_kernel<<<grid_for(n, kLbvhThreads), kLbvhThreads, 0, st>>>((int)n, t.svals, lo, hi, t.leaf_lo, t.leaf_hi,
                                                                       t.node_lo, t.node_hi, t.children, t.parent,
                                                                       t.visit, t.rec, t.status);
    return cudaGetLastError();
}

static int g_lbvh_rebuild = 16;
void lbvh_set_rebuild_every(int k) { g_lbvh_rebuild = k < 1 ? 1 : k; }
int lbvh_rebuild_every() { return g_lbvh_rebuild; }

cudaError_t lbvh_partners_async(Lbvh& t, uint32_t* off, uint32_t* partners, uint32_t* self, uint64_t cap,
                                cudaStream_t st) {
    const uint32_t n = t.n;
    if (n == 0) return cudaMemsetAsync(off, 0, 4, st);
    query_kernel<false><<<grid_for(n, kLbvhThreads), kLbvhThreads, 0, st>>>(
        (int)n, t.svals, t.leaf_lo, t.leaf_hi, t.rec, t.counts, nullptr, nullptr, nullptr, 0, t.first, t.status);
    cudaError_t e = scan_exclusive_async(t.counts, off, n, t.scan_scratch, st);
    if (e != cudaSuccess) return e;
    query_kernel<true><<<grid_for(n, kLbvhThreads), kLbvhThreads, 0, st>>>(
        (int)n, t.svals, t.leaf_lo, t.leaf_hi, t.rec, nullptr, off, partners, self, cap, t.first, t.status);
    return cudaGetLastError();
}

cudaError_t csr_unique_pairs_async(uint32_t n, const uint32_t* off, const uint32_t* partners, uint64_t partners_cap,
                                   uint32_t* counts, uint32_t* scan_scratch, uint32_t* pos, unsigned long long* out,
                                   uint64_t cap, cudaStream_t st) {
    if (n == 0) return cudaMemsetAsync(pos, 0, 4, st);
    upper_count_kernel<<<grid_for(n, kLbvhThreads), kLbvhThreads, 0, st>>>(n, off, partners, counts, partners_cap);
    cudaError_t e = scan_exclusive_async(counts, pos, n, scan_scratch, st);
    if (e != cudaSuccess) return e;
    upper_write_kernel<<<grid_for(n, kLbvhThreads), kLbvhThreads, 0, st>>>(n, off, partners, pos, out, cap,
                                                                           partners_cap);
    return cudaGetLastError();
}

cudaError_t lbvh_unique_pairs_async(Lbvh& t, const uint32_t* off, const uint32_t* partners, uint64_t partners_cap,
                                    uint32_t* pos, unsigned long long* out, uint64_t cap, cudaStream_t st) {
    return csr_unique_pairs_async(t.n, off, partners, partners_cap, t.counts, t.scan_scratch, pos, out, cap, st);
}

}  // namespace sd
