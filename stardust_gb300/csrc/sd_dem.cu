// sd_dem.cu -- the per-step DEM pipeline on a cell-sorted sphere state.
//
// One step is three stages (plus the sort between them):
//
//   contact_integrate   for each sorted slot i: gather every sphere in the
//                       3x3 columns of cells z-1..z+1 around i (each column a
//                       contiguous slot range because keys are z-fastest),
//                       accumulate spring-dashpot + Coulomb contact forces and
//                       box-wall forces, integrate (symplectic Euler), write
//                       the next state at slot i and its new cell key, and
//                       count the key digits for the sort.  No atomics on the
//                       physics: every pair is evaluated from both sides, so
//                       the result does not depend on thread timing.
//   sort                (key, slot) onesweep radix sort, sd_sort.cu
//   reorder             gather the next state into sorted order and fill
//                       cell_start (lower-bound of every cell, empty cells
//                       included) block-cooperatively -- no memset needed.
//
// The contact stage has two kernels with identical results (the autotuner
// picks one, knob "contact_mode"):
//   0  one thread per slot, candidates read through L1 from global memory;
//   1  one CTA per (x, y) grid column: the 3x3 neighbour columns -- nine
//      contiguous slot ranges -- are staged into shared memory with TMA bulk
//      copies (cp.async.bulk + mbarrier), and candidates are read from there.
//
// Replaces the reference's step (simulation_kernel.cu:52-153:
// updateSphereData -> cleanBuffers -> broad phase -> reactCollisions ->
// computeForcesAndTorques -> advect) for free spheres.  The reference's
// force law (collision_resolution.cu:79-95: forces multiplied by velocity
// signs, partner force assigned non-atomically) is replaced by the linear
// spring-dashpot law with restitution damping and Coulomb friction, walls
// and gravity.  The operation order here is the specification the CPU
// oracle restates; the file is compiled with -fmad=false so nothing is
// contracted except the explicit __fmaf_rn.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sd_common.cuh"
#include "sd_internal.h"

namespace sd {

constexpr uint32_t kIdMask = 0x7fffffffu;

__device__ __forceinline__ int32_t axis_cell(float x, float lo, float cell, int32_t n) {
    float t = (x - lo) / cell;
    if (!(t >= 0.0f)) return 0;
    if (t >= (float)n) return n - 1;
    return (int32_t)t;
}

// Cells [c0, c1] on one axis that can hold a centre within `reach` of x,
// from one reciprocal instead of two divisions.  The range is widened by a
// margin far above the rounding error of either form, so it contains every
// cell the exact division would give; a wider range only adds candidates
// that fail the distance test, and the contacts keep their visiting order,
// so forces are unchanged bit for bit.
__device__ __forceinline__ void axis_window(float x, float reach, float lo, float ic, int32_t n, int32_t& c0,
                                            int32_t& c1) {
    const float t = (x - lo) * ic, r = reach * ic;
    const float m = 1e-3f + 4e-7f * (float)n;
    const float a = t - r - m, b = t + r + m;
    c0 = a >= 0.0f ? (a < (float)n ? (int32_t)a : n - 1) : 0;
    c1 = b >= 0.0f ? (b < (float)n ? (int32_t)b : n - 1) : 0;
}

// The grid a sphere lives in: the engine's one grid, or its scene's grid in a
// batch (keys offset by the scene's base).
struct Grid {
    float lo[3], hi[3];
    float cell;   // x and y cell edge
    float cellz;  // z cell edge (cell / z_div)
    int32_t nx, ny, nz;
    uint32_t base;
};

__device__ __forceinline__ Grid grid_of(const DemParams& p) {
    Grid g;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        g.lo[a] = p.lo[a];
        g.hi[a] = p.hi[a];
    }
    g.cell = p.cell;
    g.cellz = p.cell_z;
    g.nx = p.nx;
    g.ny = p.ny;
    g.nz = p.nz;
    g.base = 0;
    return g;
}

// Scene of slot i: the last s with scene_first[s] <= i.
__device__ __forceinline__ Grid grid_of_slot(const SceneGrid* __restrict__ scenes,
                                             const uint32_t* __restrict__ first, uint32_t nscenes, uint32_t i) {
    uint32_t a = 0, z = nscenes;  // invariant: first[a] <= i < first[z]
    while (z - a > 1) {
        const uint32_t m = (a + z) >> 1;
        if (__ldg(first + m) <= i) a = m;
        else z = m;
    }
    const SceneGrid* sg = scenes + a;
    Grid g;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        g.lo[k] = __ldg(&sg->lo[k]);
        g.hi[k] = __ldg(&sg->hi[k]);
    }
    g.cell = __ldg(&sg->cell);
    g.cellz = g.cell;  // scenes of a batch keep z_div 1
    g.nx = __ldg(&sg->nx);
    g.ny = __ldg(&sg->ny);
    g.nz = __ldg(&sg->nz);
    g.base = __ldg(&sg->base);
    return g;
}

__device__ __forceinline__ uint32_t cell_key_g(const Grid& g, float x, float y, float z) {
    int32_t ix = axis_cell(x, g.lo[0], g.cell, g.nx);
    int32_t iy = axis_cell(y, g.lo[1], g.cell, g.ny);
    int32_t iz = axis_cell(z, g.lo[2], g.cellz, g.nz);
    return g.base + (uint32_t)((ix * g.ny + iy) * g.nz + iz);
}

struct Batch {
    const SceneGrid* scenes;
    const uint32_t* first;
    uint32_t n;
};

__device__ __forceinline__ uint32_t cell_key(const DemParams& p, float x, float y, float z) {
    int32_t ix = axis_cell(x, p.lo[0], p.cell, p.nx);
    int32_t iy = axis_cell(y, p.lo[1], p.cell, p.ny);
    int32_t iz = axis_cell(z, p.lo[2], p.cell_z, p.nz);
    return (uint32_t)((ix * p.ny + iy) * p.nz + iz);
}

// Linear spring-dashpot normal force with restitution damping
// (gamma_n = damp * sqrt(m_eff), damp = 2*beta*sqrt(kn),
// beta = -ln e / sqrt(pi^2 + ln^2 e)) -- not clipped at zero, so a binary
// collision restores exactly the configured restitution -- and
// viscous-regularised Coulomb friction |Ft| = min(mu*max(Fn,0), gamma_n*|vt|).
// n points from the partner to this sphere; (dv, ws) give the relative
// contact velocity v_rel = dv - ws x n with ws = ri*wi + rj*wj.
__device__ __forceinline__ void contact_response(const DemParams& p, float nx, float ny, float nz,
                                                 float delta, float dvx, float dvy, float dvz,
                                                 float wsx, float wsy, float wsz, float meff, float ri,
                                                 float3& f, float3& t) {
    float cx = wsy * nz - wsz * ny;
    float cy = wsz * nx - wsx * nz;
    float cz = wsx * ny - wsy * nx;
    float vrx = dvx - cx, vry = dvy - cy, vrz = dvz - cz;
    float vn = (vrx * nx + vry * ny) + vrz * nz;
    float gn = p.damp * sqrtf(meff);
    float fn = p.kn * delta - gn * vn;
    const float fc = fn > 0.0f ? fn : 0.0f;
    float vtx = vrx - vn * nx, vty = vry - vn * ny, vtz = vrz - vn * nz;
    float vt2 = (vtx * vtx + vty * vty) + vtz * vtz;
    f.x += fn * nx;
    f.y += fn * ny;
    f.z += fn * nz;
    if (vt2 > 0.0f) {
        float vt = sqrtf(vt2);
        float ftm = fminf(p.mu * fc, gn * vt);
        float s = ftm / vt;
        float ftx = -(s * vtx), fty = -(s * vty), ftz = -(s * vtz);
        f.x += ftx;
        f.y += fty;
        f.z += ftz;
        float qx = ny * ftz - nz * fty;
        float qy = nz * ftx - nx * ftz;
        float qz = nx * fty - ny * ftx;
        t.x -= ri * qx;
        t.y -= ri * qy;
        t.z -= ri * qz;
    }
}

// |d|^2 as specified for the overlap test: dx*dx, then two fused
// multiply-adds (the CPU restatement uses fmaf in the same order).
__device__ __forceinline__ float dist2(float dx, float dy, float dz) {
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, dx * dx));
}

// Sphere-sphere contact of i with slot s: (dx, dy, dz) = x_i - x_j,
// d2 = |x_i - x_j|^2, rs = r_i + r_j.
__device__ __forceinline__ void pair_contact(const DemParams& p, float dx, float dy, float dz, float d2, float rs,
                                             float rj, float ri, float mi, const float4& vi, const float4& wi,
                                             const float4* __restrict__ vel, const float4* __restrict__ omg,
                                             uint32_t s, float3& f, float3& t) {
    const float4 vj = __ldg(&vel[s]);
    const float4 wj = __ldg(&omg[s]);
    const float mj = vj.w;
    const float dist = sqrtf(d2);
    const float inv = 1.0f / dist;
    const float nx = dx * inv, ny = dy * inv, nz = dz * inv;
    const float wsx = ri * wi.x + rj * wj.x;
    const float wsy = ri * wi.y + rj * wj.y;
    const float wsz = ri * wi.z + rj * wj.z;
    const float meff = (mi * mj) / (mi + mj);
    contact_response(p, nx, ny, nz, rs - dist, vi.x - vj.x, vi.y - vj.y, vi.z - vj.z, wsx, wsy, wsz, meff, ri, f,
                     t);
}

// Where a kernel reads candidate positions from: slot s of the neighbour
// column coded c = (dx+1)*3 + (dy+1) relative to the sphere's own column is
// element s + delta_of(c) of the source.
struct GlobalSource {
    static constexpr bool kExactWindow = false;  // any superset of the partner cells will do
    const float4* __restrict__ pos;
    __device__ __forceinline__ uint32_t delta_of(uint32_t, int32_t, int32_t) const { return 0u; }
    __device__ __forceinline__ float4 load(uint32_t k) const { return __ldg(&pos[k]); }
};

// Used only for spheres of the CTA's own column, so the sphere's column and
// the tile's centre column coincide.
struct TileSource {
    static constexpr bool kExactWindow = true;  // columns must lie in the staged 3x3 block
    const float4* tile;     // staged slots of the 3x3 neighbour columns
    const uint32_t* shift;  // per neighbour column: tile offset - first slot (mod 2^32)
    __device__ __forceinline__ uint32_t delta_of(uint32_t c, int32_t, int32_t) const { return shift[c]; }
    __device__ __forceinline__ float4 load(uint32_t k) const { return tile[k]; }
};

// Rigid-clump context of the contact stage (all null without clumps).
struct ClumpCtx {
    const int32_t* __restrict__ body_of;  // per sphere id
    float4* __restrict__ sf;               // per slot: force handed to the body
    float4* __restrict__ st;               // per slot: torque handed to the body
};

// The incremental re-sort's list of moved slots (sd_resort.cu): the step's
// key writers append (key << 32 | slot) for every slot whose new key
// differs from the sorted key it sits under, keys_prev[slot]; entries past
// mmax are counted, not written (the radix fallback sorts then).  A null
// list: the step builds the radix sort's histograms instead.
struct MoveSink {
    const uint32_t* keys_prev;
    unsigned long long* list;
    uint32_t* count;
    uint32_t mmax;
};

// Contact partner lists of the two-kernel contact stage (scenes without
// clumps or meshes): per slot a count and up to kNbrCap partner slots,
// appended in any order by dem_pair_lists_kernel.
struct NbrLists {
    uint32_t* cnt;
    const uint32_t* nbr;
};

// Skin lists of the single-scene free-sphere step, in slot order (the
// in-place reorder moves them with the state): per slot its neighbours'
// ids within r_i + r_j + skin at the last build, the position then, and
// the slot of every id this step.
struct SkinLists {
    uint32_t* cnt;            // per slot; kVlCap + 1 = overflowed (the sphere scans)
    uint32_t* nbr;            // kVlCap rows of n ids: entry q of slot s at nbr[q * n + s]
    float4* ref;              // per slot: position at the build
    const uint32_t* flags;    // [0]: build this step
    uint32_t* next;           // = flags + 1: set when a sphere left its skin
    const uint32_t* slot_of;  // per id: slot this step
    float skin, thr2;         // skin; (0.45 skin)^2, the displacement that forces a build
};

// True when slot s holds a sphere of the same rigid body as the clump sphere
// with id bits `idb` (such pairs are skipped, collision_resolution.cu:69).
__device__ __forceinline__ bool same_body(const ClumpCtx& cc, uint32_t idb, const float4* __restrict__ omg,
                                          uint32_t s) {
    const uint32_t jdb = __float_as_uint(__ldg(reinterpret_cast<const float*>(omg) + 4 * (size_t)s + 3));
    return (jdb & kClumpFlag) && cc.body_of[idb & kIdMask] == cc.body_of[jdb & kIdMask];
}

// ------------------------------------------------------------- mesh walls

__device__ __forceinline__ float3 f3v(float4 a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float3 sub3(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 add3(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 mul3(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }

// Closest point of triangle (a, b, c) to p (Ericson, Real-Time Collision
// Detection, 5.1.5: Voronoi regions of vertices, edges, face).
__device__ __forceinline__ float3 closest_on_triangle(float3 p, float3 a, float3 b, float3 c) {
    const float3 ab = sub3(b, a), ac = sub3(c, a), ap = sub3(p, a);
    const float d1 = dot3(ab, ap), d2 = dot3(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f) return a;
    const float3 bp = sub3(p, b);
    const float d3 = dot3(ab, bp), d4 = dot3(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) return b;
    const float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) return add3(a, mul3(ab, d1 / (d1 - d3)));
    const float3 cp = sub3(p, c);
    const float d5 = dot3(ab, cp), d6 = dot3(ac, cp);
    if (d6 >= 0.0f && d5 <= d6) return c;
    const float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) return add3(a, mul3(ac, d2 / (d2 - d6)));
    const float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f)
        return add3(b, mul3(sub3(c, b), (d4 - d3) / ((d4 - d3) + (d5 - d6))));
    const float den = 1.0f / ((va + vb) + vc);
    return add3(add3(a, mul3(ab, vb * den)), mul3(ac, vc * den));
}

// Contacts of a sphere (centre x, radius ri) with the mesh: the triangles
// listed in its cell of the mesh grid, ascending; per patch the deepest
// contact (the first of equal depth) is kept; each kept contact applies the
// sphere law against the moving wall (velocity omega axis x (q - c)).
// Triangle tr as a contact candidate of the sphere at q (mesh frame):
// updates the deepest contact of its patch (the first of equal depth).
__device__ __forceinline__ void mesh_candidate(const MeshView& m, uint32_t tr, float3 q, float r2, int32_t* pid,
                                               float* pd2, float3* pv, float3* pq, int& np) {
    const float3 a = f3v(__ldg(m.tri + 3 * tr)), b = f3v(__ldg(m.tri + 3 * tr + 1)), cc = f3v(__ldg(m.tri + 3 * tr + 2));
    const float3 cl = closest_on_triangle(q, a, b, cc);
    const float3 v = sub3(q, cl);
    const float d2 = dot3(v, v);
    if (!(d2 < r2) || d2 == 0.0f) return;
    const int32_t pa = __ldg(m.patch + tr);
    int k = 0;
    while (k < np && pid[k] != pa) ++k;
    if (k < np) {
        if (d2 < pd2[k]) {
            pd2[k] = d2;
            pv[k] = v;
            pq[k] = cl;
        }
    } else if (np < kMeshPatches) {
        pid[np] = pa;
        pd2[np] = d2;
        pv[np] = v;
        pq[np] = cl;
        ++np;
    }
}

__device__ __forceinline__ void mesh_contacts(const DemParams& p, const MeshView& m, float4 pi, float4 vi, float4 wi,
                                              float3& f, float3& t, uint32_t* status) {
    const float* S = m.state;
    float R[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) R[k] = __ldg(S + k);
    const float3 c = make_float3(__ldg(S + 9), __ldg(S + 10), __ldg(S + 11));
    const float3 ax = make_float3(__ldg(S + 12), __ldg(S + 13), __ldg(S + 14));
    const float om = __ldg(S + 15);
    const float3 d = sub3(make_float3(pi.x, pi.y, pi.z), c);
    const float3 q = make_float3((R[0] * d.x + R[3] * d.y) + R[6] * d.z, (R[1] * d.x + R[4] * d.y) + R[7] * d.z,
                                 (R[2] * d.x + R[5] * d.y) + R[8] * d.z);  // R^T d: mesh frame
    const float r2 = pi.w * pi.w;
    int32_t pid[kMeshPatches];
    float pd2[kMeshPatches];
    float3 pv[kMeshPatches], pq[kMeshPatches];
    int np = 0;
    if (m.sap_n) {
        // sweep and prune along sap_axis: triangles whose box starts within
        // [x - r - longest extent, x + r] (sorted lower bounds, binary
        // search); those whose box meets the sphere's are tested, the ones in
        // contact are taken in ascending id order -- the grid's order -- so the
        // patch choices, and the force sums, are the same bits
        const float qs[3] = {q.x, q.y, q.z};
        const float xa = qs[m.sap_axis], r = pi.w;
        const float from = (xa - r) - m.sap_len, to = xa + r;
        uint32_t lo = 0, hi = m.sap_n;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldg(m.sap_lo + mid) < from) lo = mid + 1;
            else hi = mid;
        }
        uint32_t hits[kSapHits];
        uint32_t nh = 0;
        for (uint32_t k = lo; k < m.sap_n && __ldg(m.sap_lo + k) <= to; ++k) {
            const float4 bl = __ldg(m.sap_box + 2 * k), bh = __ldg(m.sap_box + 2 * k + 1);
            if (bl.x > q.x + r || bh.x < q.x - r || bl.y > q.y + r || bh.y < q.y - r || bl.z > q.z + r ||
                bh.z < q.z - r)
                continue;
            const uint32_t tr = __float_as_uint(bh.w);
            const float3 a = f3v(__ldg(m.tri + 3 * tr)), b = f3v(__ldg(m.tri + 3 * tr + 1)),
                         cc = f3v(__ldg(m.tri + 3 * tr + 2));
            const float3 v = sub3(q, closest_on_triangle(q, a, b, cc));
            const float d2 = dot3(v, v);
            if (!(d2 < r2) || d2 == 0.0f) continue;
            if (nh == kSapHits) {  // more contacts than the sweep can order
                if (status) atomicOr(status, kErrPairOverflow);
                break;
            }
            uint32_t j = nh++;
            for (; j > 0 && hits[j - 1] > tr; --j) hits[j] = hits[j - 1];
            hits[j] = tr;
        }
        for (uint32_t k = 0; k < nh; ++k) mesh_candidate(m, hits[k], q, r2, pid, pd2, pv, pq, np);
    } else {
        const int32_t ix = axis_cell(q.x, m.lo[0], m.h, m.nx);
        const int32_t iy = axis_cell(q.y, m.lo[1], m.h, m.ny);
        const int32_t iz = axis_cell(q.z, m.lo[2], m.h, m.nz);
        const uint32_t cell = (uint32_t)((ix * m.ny + iy) * m.nz + iz);
        const uint32_t e0 = __ldg(m.cell_off + cell), e1 = __ldg(m.cell_off + cell + 1);
        for (uint32_t e = e0; e < e1; ++e) mesh_candidate(m, __ldg(m.cell_tri + e), q, r2, pid, pd2, pv, pq, np);
    }
    for (int k = 0; k < np; ++k) {
        const float dist = sqrtf(pd2[k]);
        const float inv = 1.0f / dist;
        const float3 nl = mul3(pv[k], inv);
        const float3 n = make_float3((R[0] * nl.x + R[1] * nl.y) + R[2] * nl.z,
                                     (R[3] * nl.x + R[4] * nl.y) + R[5] * nl.z,
                                     (R[6] * nl.x + R[7] * nl.y) + R[8] * nl.z);
        const float3 qw = make_float3((R[0] * pq[k].x + R[1] * pq[k].y) + R[2] * pq[k].z,
                                      (R[3] * pq[k].x + R[4] * pq[k].y) + R[5] * pq[k].z,
                                      (R[6] * pq[k].x + R[7] * pq[k].y) + R[8] * pq[k].z);  // q - c, world
        const float3 vw = mul3(make_float3(ax.y * qw.z - ax.z * qw.y, ax.z * qw.x - ax.x * qw.z,
                                           ax.x * qw.y - ax.y * qw.x), om);
        const float ri = pi.w;
        contact_response(p, n.x, n.y, n.z, ri - dist, vi.x - vw.x, vi.y - vw.y, vi.z - vw.z, ri * wi.x, ri * wi.y,
                         ri * wi.z, vi.w, ri, f, t);
    }
}

// Listed neighbour k of slot i: its slot this step and position, and
// whether it is in contact (|x_i - x_j| < r_i + r_j, centres apart).
template <class SRC>
__device__ __forceinline__ bool listed_hit(const SkinLists* sk, uint32_t n, uint32_t i, uint32_t k, const SRC& src,
                                           const float4& pi, float ri, uint32_t& s, float4& pa) {
    const uint32_t jd = sk->nbr[(size_t)k * n + i];
    if (jd >= n) return false;
    s = sk->slot_of[jd];
    if (s >= n) return false;
    pa = src.load(s);
    const float da = dist2(pi.x - pa.x, pi.y - pa.y, pi.z - pa.z);
    const float ra = ri + pa.w;
    return da < ra * ra && da != 0.0f;
}

// Contacts of slot i over its candidate cells, then walls, integration and
// the next-state write.  Returns the new cell key; a clump sphere hands its
// force and torque to its body instead (the body kernel writes its next
// state and key) and *has_key is false.
template <bool RECORD, bool CLUMPS, class SRC, bool BATCHED = false, bool MESH = false, bool LISTED = false,
          bool SKIN = false>
__device__ __forceinline__ uint32_t particle_step(const DemParams& p, uint32_t n, uint32_t i, const SRC& src,
                                                  const float4* __restrict__ pos, const float4* __restrict__ vel,
                                                  const float4* __restrict__ omg,
                                                  const uint32_t* __restrict__ cell_start,
                                                  float4* __restrict__ pos_n, float4* __restrict__ vel_n,
                                                  float4* __restrict__ omg_n, uint32_t* __restrict__ keys,
                                                  uint32_t* __restrict__ vals, float4* __restrict__ force,
                                                  float4* __restrict__ torque, uint32_t& contacts,
                                                  const ClumpCtx& cc, bool* has_key, const Batch& bt = Batch{},
                                                  const MeshView* mesh = nullptr, const NbrLists* nl = nullptr,
                                                  const SkinLists* sk = nullptr, uint32_t* status = nullptr) {
    const Grid g = BATCHED ? grid_of_slot(bt.scenes, bt.first, bt.n, i) : grid_of(p);
    const float4 pi = pos[i], vi = vel[i], wi = omg[i];
    const float ri = pi.w, mi = vi.w;
    const uint32_t idb = __float_as_uint(wi.w);
    const bool clump_i = CLUMPS && (idb & kClumpFlag);
    float3 f = make_float3(0.f, 0.f, 0.f), t = make_float3(0.f, 0.f, 0.f);
    int32_t cx = 0, cy = 0, x0 = 0, x1 = -1, y0 = 0, y1 = -1, z0 = 0, z1 = -1;
    bool scan = true;  // false once the contacts came from a list
    // the list state of slot i, loaded with the sphere's own state so that
    // the loads overlap (the build flag is one word every thread reads)
    uint32_t sk_cnt = 0;
    float4 sk_ref = make_float4(0.f, 0.f, 0.f, 0.f);
    bool sk_build = false;
    if constexpr (SKIN) {
        sk_build = sk->flags[0] != 0u;
        sk_cnt = sk->cnt[i];
        sk_ref = sk->ref[i];
    }
    if constexpr (SKIN) {
        // A pair in contact now was within r_i + r_j + skin at the build:
        // every sphere has moved less than 0.45 skin since (checked at the
        // end of every step), so the distance changed by less than 0.9
        // skin.  Contacts are applied in ascending slot order, the scan's.
        if (sk_build) {  // build: the scan over the window widened by the skin
            const float reach_b = (ri + p.rmax + sk->skin) * 1.00001f;
            int32_t bx0, bx1, by0, by1, bz0, bz1;
            axis_window(pi.x, reach_b, g.lo[0], 1.0f / g.cell, g.nx, bx0, bx1);
            axis_window(pi.y, reach_b, g.lo[1], 1.0f / g.cell, g.ny, by0, by1);
            axis_window(pi.z, reach_b, g.lo[2], 1.0f / g.cellz, g.nz, bz0, bz1);
            uint32_t c = 0;
            for (int32_t X = bx0; X <= bx1; ++X) {
                for (int32_t Y = by0; Y <= by1; ++Y) {
                    const uint32_t col = g.base + (uint32_t)((X * g.ny + Y) * g.nz);
                    const uint32_t s0 = __ldg(&cell_start[col + (uint32_t)bz0]);
                    const uint32_t s1 = min(__ldg(&cell_start[col + (uint32_t)bz1 + 1]), n);
                    for (uint32_t s = s0; s < s1; ++s) {
                        const float4 pa = src.load(s);
                        const float ax = pi.x - pa.x, ay = pi.y - pa.y, az = pi.z - pa.z;
                        const float da = dist2(ax, ay, az);
                        if (s == i) continue;  // the sphere itself; a coincident partner is listed
                        // a sphere of the same rigid body is never a contact: not listed
                        if (clump_i && same_body(cc, idb, omg, s)) continue;
                        const float rl = ri + pa.w + sk->skin;
                        if (da < rl * rl) {
                            if (c < kVlCap)
                                sk->nbr[(size_t)c * n + i] =
                                    __float_as_uint(__ldg(reinterpret_cast<const float*>(omg) + 4 * (size_t)s + 3)) &
                                    kIdMask;
                            ++c;
                            const float ra = ri + pa.w;
                            if (da < ra * ra && da != 0.0f) {  // coincident centres: no normal, no contact
                                ++contacts;
                                pair_contact(p, ax, ay, az, da, ra, pa.w, ri, mi, vi, wi, vel, omg, s, f, t);
                            }
                        }
                    }
                }
            }
            sk->cnt[i] = min(c, kVlCap + 1);
            sk->ref[i] = pi;
            scan = false;
        } else if (sk_cnt <= kVlCap) {
            // the listed neighbours in contact, applied by ascending slot (the
            // scan's order).  A first pass finds them and whether list order
            // already ascends -- the usual case: the list was written in scan
            // order and few slots cross between builds; otherwise each is
            // picked as the smallest slot above the last one applied.
            const uint32_t c = sk_cnt;
            uint32_t m = 0, last = 0;
            bool asc = true;
            for (uint32_t k = 0; k < c; ++k) {
                uint32_t s;
                float4 pa;
                if (listed_hit(sk, n, i, k, src, pi, ri, s, pa)) {
                    if (m && s < last) asc = false;
                    last = s;
                    ++m;
                }
            }
            uint32_t lo = 0, k0 = 0;  // slots below lo are applied; asc: entries below k0 too
            for (uint32_t r = 0; r < m; ++r) {
                uint32_t best = 0xffffffffu;
                float4 pb = make_float4(0.f, 0.f, 0.f, 0.f);
                for (uint32_t k = asc ? k0 : 0u; k < c; ++k) {
                    uint32_t s;
                    float4 pa;
                    if (listed_hit(sk, n, i, k, src, pi, ri, s, pa) && s >= lo && s < best) {
                        best = s;
                        pb = pa;
                        if (asc) {  // list order ascends: the next hit is the next to apply
                            k0 = k + 1u;
                            break;
                        }
                    }
                }
                if (best >= n) break;  // not reached: m hits were found above
                const float ax = pi.x - pb.x, ay = pi.y - pb.y, az = pi.z - pb.z;
                const float da = dist2(ax, ay, az);
                const float ra = ri + pb.w;
                ++contacts;
                pair_contact(p, ax, ay, az, da, ra, pb.w, ri, mi, vi, wi, vel, omg, best, f, t);
                lo = best + 1u;
            }
            scan = false;
        }
        // else: an overflowed list -- the scan below
    }
    if constexpr (LISTED) {
        // the partners found by the pair kernel, applied in ascending slot
        // order -- the order of the scan below (columns in key order, slots
        // ascending in each) -- unless the list overflowed
        const uint32_t c = nl->cnt[i];
        nl->cnt[i] = 0u;  // cleared for the next step's pair kernel
        if (c <= kNbrCap) {
            scan = false;
            uint32_t js[kNbrCap];
            for (uint32_t k = 0; k < c; ++k) {
                const uint32_t v = nl->nbr[(size_t)i * kNbrCap + k];
                uint32_t m = k;
                for (; m > 0 && js[m - 1] > v; --m) js[m] = js[m - 1];
                js[m] = v;
            }
            for (uint32_t k = 0; k < c; ++k) {
                const uint32_t s = js[k];
                if (s >= n) continue;
                const float4 pa = src.load(s);
                const float ax = pi.x - pa.x, ay = pi.y - pa.y, az = pi.z - pa.z;
                const float da = dist2(ax, ay, az);
                const float ra = ri + pa.w;
                if (da < ra * ra && da != 0.0f) {
                    ++contacts;
                    pair_contact(p, ax, ay, az, da, ra, pa.w, ri, mi, vi, wi, vel, omg, s, f, t);
                }
            }
        }
    }
    if (scan) {
        // The candidate cells: the 3x3x3 block around i's cell, cut per axis
        // to the cells a partner's centre can occupy, |x_j - x_i| < r_i +
        // r_max (padded by 1e-5 against rounding).  Only non-contacts are
        // dropped, and the surviving candidates keep the block's visiting
        // order -- columns (x outer, y inner), slots ascending -- so the
        // force sums are identical to a full 27-cell scan.
        const float reach = (ri + p.rmax) * 1.00001f;
        if constexpr (SRC::kExactWindow) {
            cx = axis_cell(pi.x, g.lo[0], g.cell, g.nx);
            cy = axis_cell(pi.y, g.lo[1], g.cell, g.ny);
            x0 = max(cx - 1, axis_cell(pi.x - reach, g.lo[0], g.cell, g.nx));
            x1 = min(cx + 1, axis_cell(pi.x + reach, g.lo[0], g.cell, g.nx));
            y0 = max(cy - 1, axis_cell(pi.y - reach, g.lo[1], g.cell, g.ny));
            y1 = min(cy + 1, axis_cell(pi.y + reach, g.lo[1], g.cell, g.ny));
            z0 = axis_cell(pi.z - reach, g.lo[2], g.cellz, g.nz);
            z1 = axis_cell(pi.z + reach, g.lo[2], g.cellz, g.nz);
        } else {
            const float ic = 1.0f / g.cell;
            axis_window(pi.x, reach, g.lo[0], ic, g.nx, x0, x1);
            axis_window(pi.y, reach, g.lo[1], ic, g.ny, y0, y1);
            axis_window(pi.z, reach, g.lo[2], 1.0f / g.cellz, g.nz, z0, z1);
        }
    }
    for (int32_t X = x0; X <= x1; ++X) {
        for (int32_t Y = y0; Y <= y1; ++Y) {
            const uint32_t col = g.base + (uint32_t)((X * g.ny + Y) * g.nz);
            const uint32_t s0 = __ldg(&cell_start[col + (uint32_t)z0]);
            const uint32_t s1 = min(__ldg(&cell_start[col + (uint32_t)z1 + 1]), n);
            const uint32_t d = src.delta_of((uint32_t)((X - cx + 1) * 3 + (Y - cy + 1)), cx, cy);
            uint32_t s = s0;
            // two candidates per iteration for load-level parallelism;
            // contacts are applied in slot order.  The sphere itself has
            // d2 == 0 and fails the contact test.
            for (; s + 1 < s1; s += 2) {
                const float4 pa = src.load(s + d);
                const float4 pb = src.load(s + 1 + d);
                const float ax = pi.x - pa.x, ay = pi.y - pa.y, az = pi.z - pa.z;
                const float bx = pi.x - pb.x, by = pi.y - pb.y, bz = pi.z - pb.z;
                const float da = dist2(ax, ay, az), db = dist2(bx, by, bz);
                const float ra = ri + pa.w, rb = ri + pb.w;
                const bool ha = da < ra * ra && da != 0.0f, hb = db < rb * rb && db != 0.0f;
                if constexpr (!CLUMPS && !MESH) {
                    // free spheres in a box: most candidate pairs hold no
                    // contact, and one branch on both tests skips them
                    // together (1,048,576-sphere settling box: 0.204 ->
                    // 0.201 ms per step).  In the dense clump-and-mesh beds
                    // a third of the pairs hold one and the separate tests
                    // below are faster (drum: 0.590 vs 0.531 ms).
                    if (__builtin_expect(ha | hb, 0)) {
                        if (ha) {
                            ++contacts;
                            pair_contact(p, ax, ay, az, da, ra, pa.w, ri, mi, vi, wi, vel, omg, s, f, t);
                        }
                        if (hb) {
                            ++contacts;
                            pair_contact(p, bx, by, bz, db, rb, pb.w, ri, mi, vi, wi, vel, omg, s + 1, f, t);
                        }
                    }
                } else {
                    if (ha && !(clump_i && same_body(cc, idb, omg, s))) {
                        ++contacts;
                        pair_contact(p, ax, ay, az, da, ra, pa.w, ri, mi, vi, wi, vel, omg, s, f, t);
                    }
                    if (hb && !(clump_i && same_body(cc, idb, omg, s + 1))) {
                        ++contacts;
                        pair_contact(p, bx, by, bz, db, rb, pb.w, ri, mi, vi, wi, vel, omg, s + 1, f, t);
                    }
                }
            }
            if (s < s1) {
                const float4 pa = src.load(s + d);
                const float ax = pi.x - pa.x, ay = pi.y - pa.y, az = pi.z - pa.z;
                const float da = dist2(ax, ay, az);
                const float ra = ri + pa.w;
                if (da < ra * ra && da != 0.0f && !(clump_i && same_body(cc, idb, omg, s))) {
                    ++contacts;
                    pair_contact(p, ax, ay, az, da, ra, pa.w, ri, mi, vi, wi, vel, omg, s, f, t);
                }
            }
        }
    }
    if (MESH) mesh_contacts(p, *mesh, pi, vi, wi, f, t, status);
    if (p.walls) {
        const float wsx = ri * wi.x, wsy = ri * wi.y, wsz = ri * wi.z;
        const float xs[3] = {pi.x, pi.y, pi.z};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                if (!(p.walls & (1 << (2 * a + side)))) continue;
                const float gap = side == 0 ? xs[a] - g.lo[a] : g.hi[a] - xs[a];
                if (!(gap < ri)) continue;
                float nn[3] = {0.f, 0.f, 0.f};
                nn[a] = side == 0 ? 1.0f : -1.0f;
                contact_response(p, nn[0], nn[1], nn[2], ri - gap, vi.x, vi.y, vi.z, wsx, wsy, wsz, mi, ri, f, t);
            }
        }
    }
    if (RECORD) {
        // recorded by sphere id: the slot order changes in the reorder that
        // ends the step
        const uint32_t id = __float_as_uint(wi.w) & kIdMask;
        if (id < n) {
            force[id] = make_float4(f.x, f.y, f.z, 0.0f);
            torque[id] = make_float4(t.x, t.y, t.z, 0.0f);
        }
    }
    if (clump_i) {
        cc.sf[i] = make_float4(f.x, f.y, f.z, 0.0f);
        cc.st[i] = make_float4(t.x, t.y, t.z, 0.0f);
        *has_key = false;
        return 0u;
    }
    *has_key = true;
    const float dt = p.dt;
    // force / mass and torque / inertia; a sphere with no contact and no
    // wall has f = t = +0 exactly, and +0 / m = +0 for any mass, so its six
    // divisions are skipped with the same bits
    float ax = 0.0f, ay = 0.0f, az = 0.0f, bx = 0.0f, by = 0.0f, bz = 0.0f;
    if ((__float_as_uint(f.x) | __float_as_uint(f.y) | __float_as_uint(f.z) | __float_as_uint(t.x) |
         __float_as_uint(t.y) | __float_as_uint(t.z)) != 0u) {
        const float inertia = ((0.4f * mi) * ri) * ri;
        ax = f.x / mi;
        ay = f.y / mi;
        az = f.z / mi;
        bx = t.x / inertia;
        by = t.y / inertia;
        bz = t.z / inertia;
    }
    const float nvx = vi.x + dt * (ax + p.g[0]);
    const float nvy = vi.y + dt * (ay + p.g[1]);
    const float nvz = vi.z + dt * (az + p.g[2]);
    const float nxp = pi.x + dt * nvx, nyp = pi.y + dt * nvy, nzp = pi.z + dt * nvz;
    pos_n[i] = make_float4(nxp, nyp, nzp, ri);
    vel_n[i] = make_float4(nvx, nvy, nvz, mi);
    omg_n[i] = make_float4(wi.x + dt * bx, wi.y + dt * by, wi.z + dt * bz, wi.w);
    if constexpr (SKIN) {  // left 0.45 skin of the build position: build next step
        const float4 r = sk_build ? pi : sk_ref;  // a build step recorded pi
        if (dist2(nxp - r.x, nyp - r.y, nzp - r.z) > sk->thr2) atomicOr(sk->next, 1u);
    }
    const uint32_t key = cell_key_g(g, nxp, nyp, nzp);
    keys[i] = key;
    if (vals) vals[i] = i;  // the slot identity, for a radix sort (null: the re-sort step)
    return key;
}

// Passes whose digit histograms the contact kernels can build (keys up to 27
// bits, i.e. grids up to 2^27 cells); larger grids use the sort's own
// histogram kernel.  The plan travels packed in one word: passes in bits
// 0-1, then per pass q a 5-bit shift at 2+9q and a 4-bit width at 7+9q.
constexpr int kFusedPasses = 3;

static uint32_t pack_hist_spec(const SortPlan& plan) {
    uint32_t v = ((uint32_t)plan.passes & 3u) | (plan.stride == 1024 ? 1u << 29 : 0u);
    for (int q = 0; q < plan.passes && q < kFusedPasses; ++q)
        v |= ((uint32_t)plan.shift[q] & 31u) << (2 + 9 * q) | ((uint32_t)plan.bits[q] & 15u) << (7 + 9 * q);
    return v;
}

// Words of a block's shared digit histograms: pass q at q * stride (3 x 512
// or 2 x 1024), the layout of the sort's global histograms.
constexpr int kHistWords = 2048;
__device__ __forceinline__ uint32_t spec_stride(uint32_t spec) { return (spec >> 29) & 1u ? 1024u : 512u; }

// Adds the warp's keys to the block's shared digit histograms (all lanes
// of the warp must call; `valid` marks lanes that hold a key).
__device__ __forceinline__ void hist_add(uint32_t* s_hist, uint32_t spec, uint32_t key, bool valid) {
    const int passes = (int)(spec & 3u);
    const uint32_t stride = spec_stride(spec);
#pragma unroll
    for (int q = 0; q < kFusedPasses; ++q) {
        if (q >= passes) break;
        const uint32_t shift = (spec >> (2 + 9 * q)) & 31u, bits = (spec >> (7 + 9 * q)) & 15u;
        const uint32_t d = (key >> shift) & ((1u << bits) - 1u);
        const uint32_t peers = __match_any_sync(0xffffffffu, valid ? d : 0xffffffffu);
        if (valid && (peers & lanemask_lt()) == 0) atomicAdd(&s_hist[q * stride + d], __popc(peers));
    }
}

// Block's histograms to the global ones: one atomic per non-empty bin.
__device__ __forceinline__ void hist_flush(const uint32_t* s_hist, uint32_t spec, uint32_t* ghist) {
    const int passes = (int)(spec & 3u);
    const uint32_t stride = spec_stride(spec);
    for (int q = 0; q < passes; ++q) {
        const uint32_t bits = (spec >> (7 + 9 * q)) & 15u;
        for (uint32_t d = threadIdx.x; d < (1u << bits); d += blockDim.x)
            if (s_hist[q * stride + d]) atomicAdd(&ghist[q * stride + d], s_hist[q * stride + d]);
    }
}

// Appends the moved slots among a warp's (all 32 lanes call it; kprev =
// keys_prev[slot] where valid): one atomic per warp that holds any.
__device__ __forceinline__ void move_append_warp(const MoveSink& ms, uint32_t slot, uint32_t key, bool valid,
                                                 uint32_t kprev) {
    const bool mv = valid && key != kprev;
    const uint32_t m = __ballot_sync(0xffffffffu, mv);
    if (!m) return;
    const uint32_t leader = (uint32_t)__ffs(m) - 1u;
    uint32_t base = 0;
    if (lane_id() == leader) base = atomicAdd(ms.count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, (int)leader);
    if (mv) {
        const uint32_t r = base + (uint32_t)__popc(m & lanemask_lt());
        if (r < ms.mmax) ms.list[r] = ((unsigned long long)key << 32) | slot;
    }
}

// One slot, from a thread that may be alone in its branch.
__device__ __forceinline__ void move_append_one(const MoveSink& ms, uint32_t slot, uint32_t key) {
    if (key == ms.keys_prev[slot]) return;
    const uint32_t r = atomicAdd(ms.count, 1u);
    if (r < ms.mmax) ms.list[r] = ((unsigned long long)key << 32) | slot;
}

__device__ __forceinline__ void count_contacts(uint32_t* status, uint32_t contacts) {
    uint32_t v = contacts;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane_id() == 0 && v) atomicAdd(reinterpret_cast<unsigned long long*>(status + 2), (unsigned long long)v);
}

// ---------------------------------------------- contact_mode 0: per slot
// The first kernel of the two-kernel contact stage: each candidate pair is
// tested once, by its lower slot, over the upper part of that sphere's
// candidate window (the columns after its own, and its own column above
// it).  The test is symmetric -- x_j - x_i is the exact negation of
// x_i - x_j and r_i + r_j commutes -- so it decides exactly as the
// partner's own scan would, and every pair in contact lies in the lower
// slot's window.  A contact is appended to both spheres' lists.
template <bool BATCHED>
__global__ void __launch_bounds__(256)
dem_pair_lists_kernel(DemParams p, uint32_t n, const float4* __restrict__ pos,
                      const uint32_t* __restrict__ cell_start, uint32_t* __restrict__ cnt,
                      uint32_t* __restrict__ nbr, Batch bt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Grid g = BATCHED ? grid_of_slot(bt.scenes, bt.first, bt.n, i) : grid_of(p);
    const float4 pi = __ldg(&pos[i]);
    const float ri = pi.w;
    const float reach = (ri + p.rmax) * 1.00001f;
    int32_t x0, x1, y0, y1, z0, z1;
    const float ic = 1.0f / g.cell;
    axis_window(pi.x, reach, g.lo[0], ic, g.nx, x0, x1);
    axis_window(pi.y, reach, g.lo[1], ic, g.ny, y0, y1);
    axis_window(pi.z, reach, g.lo[2], 1.0f / g.cellz, g.nz, z0, z1);
    for (int32_t X = x0; X <= x1; ++X) {
        for (int32_t Y = y0; Y <= y1; ++Y) {
            const uint32_t col = g.base + (uint32_t)((X * g.ny + Y) * g.nz);
            const uint32_t s1 = min(__ldg(&cell_start[col + (uint32_t)z1 + 1]), n);
            if (s1 <= i + 1) continue;  // the column holds no slot above i
            uint32_t s = max(__ldg(&cell_start[col + (uint32_t)z0]), i + 1);
            for (; s < s1; ++s) {
                const float4 pa = __ldg(&pos[s]);
                const float ax = pi.x - pa.x, ay = pi.y - pa.y, az = pi.z - pa.z;
                const float da = dist2(ax, ay, az);
                const float ra = ri + pa.w;
                if (__builtin_expect(da < ra * ra && da != 0.0f, 0)) {
                    const uint32_t a = atomicAdd(&cnt[i], 1u);
                    if (a < kNbrCap) nbr[(size_t)i * kNbrCap + a] = s;
                    const uint32_t b = atomicAdd(&cnt[s], 1u);
                    if (b < kNbrCap) nbr[(size_t)s * kNbrCap + b] = i;
                }
            }
        }
    }
}

template <bool RECORD, bool CLUMPS, bool BATCHED = false, bool MESH = false, bool LISTED = false,
          bool SKIN = false>
__global__ void __launch_bounds__(256)
dem_contact_integrate_kernel(DemParams p, uint32_t n, const float4* __restrict__ pos,
                             const float4* __restrict__ vel, const float4* __restrict__ omg,
                             const uint32_t* __restrict__ cell_start, float4* __restrict__ pos_n,
                             float4* __restrict__ vel_n, float4* __restrict__ omg_n,
                             uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                             float4* __restrict__ force, float4* __restrict__ torque,
                             uint32_t* __restrict__ status, uint32_t hist_spec, uint32_t* __restrict__ ghist,
                             ClumpCtx cc, Batch bt = Batch{}, MeshView mesh = MeshView{},
                             NbrLists nl = NbrLists{}, SkinLists sk = SkinLists{}, MoveSink ms = MoveSink{}) {
    __shared__ uint32_t s_hist[kHistWords];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t contacts = 0, key = 0;
    bool has_key = false;
    // the key this slot sits under, loaded up front with the slot's state
    const uint32_t kprev = ms.list && i < n ? __ldg(ms.keys_prev + i) : 0u;
    if (i < n)
        key = particle_step<RECORD, CLUMPS, GlobalSource, BATCHED, MESH, LISTED, SKIN>(
            p, n, i, GlobalSource{pos}, pos, vel, omg, cell_start, pos_n, vel_n, omg_n, keys, vals, force, torque,
            contacts, cc, &has_key, bt, &mesh, &nl, &sk, status);
    if (ghist) {
        for (int q = threadIdx.x; q < kHistWords; q += blockDim.x) s_hist[q] = 0;
        __syncthreads();
        hist_add(s_hist, hist_spec, key, has_key);
        __syncthreads();
        hist_flush(s_hist, hist_spec, ghist);
    }
    if (ms.list) move_append_warp(ms, i, key, has_key, kprev);
    if (RECORD) count_contacts(status, contacts);
}

// The single-scene free-sphere step over contact lists (knob skin_um): one
// thread per slot, the listed neighbours between builds, the widened scan
// at a build.  Its own kernel so that the registers are capped for the
// listed steps' occupancy (they are bound by load latency): MINB resident
// blocks of 256 per SM (4: 64 registers; 5: 48, with spills in the build
// scan; 6: 40; 8: 32; knob "listed_blocks", default 5).  It never builds radix histograms (the lists
// run only with the incremental re-sort).
template <bool RECORD, int MINB, bool BATCHED, bool CLUMPS = false, bool MESH = false>
__global__ void __launch_bounds__(256, MINB)
dem_contact_listed_kernel(DemParams p, uint32_t n, const float4* __restrict__ pos, const float4* __restrict__ vel,
                          const float4* __restrict__ omg, const uint32_t* __restrict__ cell_start,
                          float4* __restrict__ pos_n, float4* __restrict__ vel_n, float4* __restrict__ omg_n,
                          uint32_t* __restrict__ keys, uint32_t* __restrict__ vals, float4* __restrict__ force,
                          float4* __restrict__ torque, uint32_t* __restrict__ status, SkinLists sk, MoveSink ms,
                          Batch bt, ClumpCtx cc = ClumpCtx{}, MeshView mesh = MeshView{}) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t contacts = 0, key = 0;
    bool has_key = false;
    const uint32_t kprev = ms.list && i < n ? __ldg(ms.keys_prev + i) : 0u;
    if (i < n)
        key = particle_step<RECORD, CLUMPS, GlobalSource, BATCHED, MESH, false, true>(
            p, n, i, GlobalSource{pos}, pos, vel, omg, cell_start, pos_n, vel_n, omg_n, keys, vals, force, torque,
            contacts, cc, &has_key, bt, &mesh, nullptr, &sk, status);
    if (ms.list) move_append_warp(ms, i, key, has_key, kprev);
    if (RECORD) count_contacts(status, contacts);
}

// ------------------------------------- contact_mode 1: TMA column tiles
constexpr int kColThreads = 512;
constexpr uint32_t kTileSlots = 4096;  // staged positions per CTA (64 KB)
constexpr uint32_t kTmaSpinLimit = 1u << 24;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned)
// from global to this CTA's shared memory, completing on `bar`.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, uint32_t parity) {
    for (uint32_t it = 0; it < kTmaSpinLimit; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if (it > 64) __nanosleep(64);
    }
    return false;
}

// One CTA per (x, y) grid column.  Its spheres' candidates all lie in the
// 3x3 neighbour columns, nine contiguous slot ranges of the sorted state,
// which one thread stages into shared memory with TMA bulk copies.  A CTA
// whose neighbourhood exceeds kTileSlots reads global memory instead; the
// results are the same either way.
template <bool RECORD, bool CLUMPS>
__global__ void __launch_bounds__(kColThreads, 2)
dem_contact_column_kernel(DemParams p, uint32_t n, const float4* __restrict__ pos,
                          const float4* __restrict__ vel, const float4* __restrict__ omg,
                          const uint32_t* __restrict__ cell_start, float4* __restrict__ pos_n,
                          float4* __restrict__ vel_n, float4* __restrict__ omg_n, uint32_t* __restrict__ keys,
                          uint32_t* __restrict__ vals, float4* __restrict__ force, float4* __restrict__ torque,
                          uint32_t* __restrict__ status, uint32_t hist_spec, uint32_t* __restrict__ ghist,
                          ClumpCtx cc, MoveSink ms) {
    extern __shared__ __align__(128) float4 s_tile[];
    __shared__ uint32_t s_hist[kHistWords];
    __shared__ __align__(8) unsigned long long s_bar;
    __shared__ uint32_t s_beg[9], s_cnt[9], s_shift[9], s_total;

    const int32_t X = (int32_t)blockIdx.x / p.ny, Y = (int32_t)blockIdx.x % p.ny;
    if (threadIdx.x < 9) {
        const int32_t Xn = X + (int32_t)threadIdx.x / 3 - 1, Yn = Y + (int32_t)threadIdx.x % 3 - 1;
        uint32_t b = 0, c = 0;
        if (Xn >= 0 && Xn < p.nx && Yn >= 0 && Yn < p.ny) {
            const uint32_t cb = (uint32_t)(Xn * p.ny + Yn) * (uint32_t)p.nz;
            b = min(cell_start[cb], n);
            const uint32_t e = min(cell_start[cb + (uint32_t)p.nz], n);
            c = e > b ? e - b : 0u;
        }
        s_beg[threadIdx.x] = b;
        s_cnt[threadIdx.x] = c;
    }
    if (ghist)
        for (int q = threadIdx.x; q < kHistWords; q += blockDim.x) s_hist[q] = 0;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t off = 0;
        for (int c = 0; c < 9; ++c) {
            s_shift[c] = off - s_beg[c];
            off += s_cnt[c];
        }
        s_total = off;
        if (s_cnt[4] > 0 && off <= kTileSlots) mbar_init(&s_bar, 1);
    }
    __syncthreads();
    const uint32_t own_beg = s_beg[4], own_cnt = s_cnt[4];
    if (own_cnt == 0) return;  // uniform across the CTA
    const bool staged = s_total <= kTileSlots;
    if (staged && threadIdx.x == 0) {
        mbar_arrive_expect_tx(&s_bar, s_total * 16u);
        for (int c = 0; c < 9; ++c)
            if (s_cnt[c]) bulk_copy_g2s(&s_tile[s_shift[c] + s_beg[c]], pos + s_beg[c], s_cnt[c] * 16u, &s_bar);
    }
    bool use_tile = staged;
    if (staged && !mbar_wait_bounded(&s_bar, 0)) {
        atomicOr(status, kErrWaitTimeout);
        use_tile = false;  // read global memory instead; same results
    }
    const TileSource tile{s_tile, s_shift};
    const GlobalSource glob{pos};
    uint32_t contacts = 0;
    const uint32_t rounds = (own_cnt + blockDim.x - 1) / blockDim.x;
    for (uint32_t r = 0; r < rounds; ++r) {
        const uint32_t k = r * blockDim.x + threadIdx.x;
        const bool valid = k < own_cnt;
        uint32_t key = 0;
        bool has_key = false;
        if (valid) {
            const uint32_t i = own_beg + k;
            // The tile holds the neighbours of column (X, Y) only.  A sphere's
            // cell is recomputed from its position exactly as its sort key
            // was, so it always lies in this column; the check keeps every
            // shared-memory index in bounds regardless.
            const float4 q = pos[i];
            const bool mine = axis_cell(q.x, p.lo[0], p.cell, p.nx) == X && axis_cell(q.y, p.lo[1], p.cell, p.ny) == Y;
            if (!mine) atomicOr(status, kErrBadInput);
            key = (use_tile && mine)
                      ? particle_step<RECORD, CLUMPS>(p, n, i, tile, pos, vel, omg, cell_start, pos_n, vel_n, omg_n, keys,
                                              vals, force, torque, contacts, cc, &has_key)
                      : particle_step<RECORD, CLUMPS>(p, n, i, glob, pos, vel, omg, cell_start, pos_n, vel_n, omg_n, keys,
                                              vals, force, torque, contacts, cc, &has_key);
        }
        if (ghist) hist_add(s_hist, hist_spec, key, has_key);
        if (ms.list) move_append_warp(ms, own_beg + k, key, has_key, has_key ? ms.keys_prev[own_beg + k] : 0u);
    }
    if (ghist) {
        __syncthreads();
        hist_flush(s_hist, hist_spec, ghist);
    }
    if (RECORD) count_contacts(status, contacts);
    // never leave with a bulk copy in flight into this CTA's shared memory
    if (staged && !use_tile && threadIdx.x == 0) mbar_wait_bounded(&s_bar, 0);
}

// Rotation matrix (row-major) of a unit quaternion (s, x, y, z).
__device__ __forceinline__ void quat_rot(float qs, float qx, float qy, float qz, float* R) {
    R[0] = 1.0f - 2.0f * (qy * qy + qz * qz);
    R[1] = 2.0f * (qx * qy - qs * qz);
    R[2] = 2.0f * (qx * qz + qs * qy);
    R[3] = 2.0f * (qx * qy + qs * qz);
    R[4] = 1.0f - 2.0f * (qx * qx + qz * qz);
    R[5] = 2.0f * (qy * qz - qs * qx);
    R[6] = 2.0f * (qx * qz - qs * qy);
    R[7] = 2.0f * (qy * qz + qs * qx);
    R[8] = 1.0f - 2.0f * (qx * qx + qy * qy);
}

// A rigid body's step (replaces computeForcesAndTorquesCUDA +
// advectParticlesCUDA + updateSphereDataCUDA, physics_update.cu:26-310):
// gather the body's sphere forces and torques in sphere-id order (the
// segmented reduction, no atomics), add gravity, integrate momentum and
// angular momentum, w = R I0^-1 R^T L, normalised first-order quaternion
// update, then write every sphere's next state and cell key (and its
// digits to the block's shared sort histograms when s_hist is given).
// One body per quad of lanes (q = lane & 3): lane q loads and writes the
// body's spheres q, q + 4, ...; the sums over the spheres are formed in
// sphere-id order in every lane of the quad from the values the lanes
// exchange, so every lane holds the same body state (the same bits as one
// thread walking the spheres in order) and integrates it.  Loops run to the
// warp's largest sphere count so that every lane takes part in the
// exchanges.
__device__ __forceinline__ void body_step(
    const DemParams& p, uint32_t b, bool valid, uint32_t q, float4* __restrict__ bpos, float4* __restrict__ bvel,
    float4* __restrict__ bquat, float4* __restrict__ bomg, float4* __restrict__ bang,
    const float4* __restrict__ binv, const uint32_t* __restrict__ bfirst, const uint32_t* __restrict__ bcount,
    const float4* __restrict__ r0, const uint32_t* __restrict__ slot_of, const float4* __restrict__ pos,
    const float4* __restrict__ omg, const float4* __restrict__ sf, const float4* __restrict__ st,
    float4* __restrict__ pos_n, float4* __restrict__ vel_n, float4* __restrict__ omg_n,
    uint32_t* __restrict__ keys, uint32_t* __restrict__ vals, uint32_t n, uint32_t hist_spec,
    uint32_t* s_hist, const MoveSink& ms, const SkinLists& sk) {
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 bp = valid ? bpos[b] : z4, bv = valid ? bvel[b] : z4, bq = valid ? bquat[b] : z4,
                 bl = valid ? bang[b] : z4;
    const float x = bp.x, y = bp.y, z = bp.z, m = bp.w;
    const uint32_t first = valid ? bfirst[b] : 0u, cnt = valid ? bcount[b] : 0u;
    const uint32_t kmax = __reduce_max_sync(0xffffffffu, cnt);
    float Fx = 0, Fy = 0, Fz = 0, Tx = 0, Ty = 0, Tz = 0;
    for (uint32_t k0 = 0; k0 < kmax; k0 += 4) {
        const uint32_t k = k0 + q;
        float4 fs = z4, ts = z4;
        float cx = 0.f, cy = 0.f, cz = 0.f;
        bool has = false;
        if (k < cnt) {
            const uint32_t s = slot_of[first + k];
            if (s < n) {  // a consistent slot table never fails this
                const float4 ps = pos[s];
                fs = sf[s];
                ts = st[s];
                const float rx = ps.x - x, ry = ps.y - y, rz = ps.z - z;
                cx = ry * fs.z - rz * fs.y;
                cy = rz * fs.x - rx * fs.z;
                cz = rx * fs.y - ry * fs.x;
                has = true;
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {  // spheres k0 .. k0 + 3, in order
            const float fx = __shfl_sync(0xffffffffu, fs.x, u, 4), fy = __shfl_sync(0xffffffffu, fs.y, u, 4),
                        fz = __shfl_sync(0xffffffffu, fs.z, u, 4);
            const float ux = __shfl_sync(0xffffffffu, cx, u, 4), uy = __shfl_sync(0xffffffffu, cy, u, 4),
                        uz = __shfl_sync(0xffffffffu, cz, u, 4);
            const float tx = __shfl_sync(0xffffffffu, ts.x, u, 4), ty = __shfl_sync(0xffffffffu, ts.y, u, 4),
                        tz = __shfl_sync(0xffffffffu, ts.z, u, 4);
            if (__shfl_sync(0xffffffffu, has ? 1 : 0, u, 4)) {
                Fx = Fx + fx;
                Fy = Fy + fy;
                Fz = Fz + fz;
                Tx = Tx + ux;
                Ty = Ty + uy;
                Tz = Tz + uz;
                Tx = Tx + tx;
                Ty = Ty + ty;
                Tz = Tz + tz;
            }
        }
    }
    if (!valid) return;
    const float dt = p.dt;
    const float vx = bv.x + dt * (Fx / m + p.g[0]);
    const float vy = bv.y + dt * (Fy / m + p.g[1]);
    const float vz = bv.z + dt * (Fz / m + p.g[2]);
    const float nxp = x + dt * vx, nyp = y + dt * vy, nzp = z + dt * vz;
    const float Lx = bl.x + dt * Tx, Ly = bl.y + dt * Ty, Lz = bl.z + dt * Tz;
    const float4 i0 = binv[3 * b], i1 = binv[3 * b + 1], i2 = binv[3 * b + 2];
    const float I[12] = {i0.x, i0.y, i0.z, i0.w, i1.x, i1.y, i1.z, i1.w, i2.x, i2.y, i2.z, i2.w};
    float R[9], A[9], W[9];
    quat_rot(bq.x, bq.y, bq.z, bq.w, R);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) A[3 * r + c] = (R[3 * r] * I[c] + R[3 * r + 1] * I[4 + c]) + R[3 * r + 2] * I[8 + c];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            W[3 * r + c] = (A[3 * r] * R[3 * c] + A[3 * r + 1] * R[3 * c + 1]) + A[3 * r + 2] * R[3 * c + 2];
    const float wx = (W[0] * Lx + W[1] * Ly) + W[2] * Lz;
    const float wy = (W[3] * Lx + W[4] * Ly) + W[5] * Lz;
    const float wz = (W[6] * Lx + W[7] * Ly) + W[8] * Lz;
    const float qs = bq.x, qx = bq.y, qy = bq.z, qz = bq.w;
    const float h = 0.5f * dt;
    const float ds = -((wx * qx + wy * qy) + wz * qz);
    const float dx = qs * wx + (wy * qz - wz * qy);
    const float dy = qs * wy + (wz * qx - wx * qz);
    const float dz = qs * wz + (wx * qy - wy * qx);
    const float ns = qs + h * ds, nx = qx + h * dx, ny = qy + h * dy, nz = qz + h * dz;
    const float nrm = sqrtf((ns * ns + nx * nx) + (ny * ny + nz * nz));
    const float q0 = ns / nrm, q1 = nx / nrm, q2 = ny / nrm, q3 = nz / nrm;
    quat_rot(q0, q1, q2, q3, R);
    for (uint32_t k = q; k < cnt; k += 4) {
        const uint32_t id = first + k, s = slot_of[id];
        if (s >= n) continue;
        const float4 o = r0[id];
        const float rx = (R[0] * o.x + R[1] * o.y) + R[2] * o.z;
        const float ry = (R[3] * o.x + R[4] * o.y) + R[5] * o.z;
        const float rz = (R[6] * o.x + R[7] * o.y) + R[8] * o.z;
        const float4 po = make_float4(nxp + rx, nyp + ry, nzp + rz, pos[s].w);
        pos_n[s] = po;
        if (sk.ref) {  // contact lists: a clump sphere that left 0.45 skin of its build position
            const float4 r = sk.ref[s];
            if (dist2(po.x - r.x, po.y - r.y, po.z - r.z) > sk.thr2) atomicOr(sk.next, 1u);
        }
        vel_n[s] = make_float4(vx + (wy * rz - wz * ry), vy + (wz * rx - wx * rz), vz + (wx * ry - wy * rx), m);
        omg_n[s] = make_float4(wx, wy, wz, omg[s].w);
        const uint32_t key = cell_key(p, po.x, po.y, po.z);
        keys[s] = key;
        if (vals) vals[s] = s;
        if (ms.list) move_append_one(ms, s, key);
        if (s_hist) {
            const int passes = (int)(hist_spec & 3u);
            const uint32_t stride = spec_stride(hist_spec);
            for (int pq = 0; pq < passes; ++pq) {
                const uint32_t shift = (hist_spec >> (2 + 9 * pq)) & 31u, bits = (hist_spec >> (7 + 9 * pq)) & 15u;
                atomicAdd(&s_hist[pq * stride + ((key >> shift) & ((1u << bits) - 1u))], 1u);
            }
        }
    }
    if (q == 0) {
        bpos[b] = make_float4(nxp, nyp, nzp, m);
        bvel[b] = make_float4(vx, vy, vz, bv.w);
        bang[b] = make_float4(Lx, Ly, Lz, bl.w);
        bquat[b] = make_float4(q0, q1, q2, q3);
        bomg[b] = make_float4(wx, wy, wz, 0.0f);
    }
}

// Four lanes per body (see body_step).  The clump spheres' key digits are
// counted in shared memory and added to the global histograms once per
// block: a global atomic per sphere piles onto the few bins of the high
// digits (one L2 slice) and stalls the whole kernel behind it.
__global__ void __launch_bounds__(128)
dem_body_kernel(DemParams p, uint32_t nb, float4* __restrict__ bpos, float4* __restrict__ bvel,
                float4* __restrict__ bquat, float4* __restrict__ bomg, float4* __restrict__ bang,
                const float4* __restrict__ binv, const uint32_t* __restrict__ bfirst,
                const uint32_t* __restrict__ bcount, const float4* __restrict__ r0, const uint32_t* __restrict__ slot_of,
                const float4* __restrict__ pos, const float4* __restrict__ omg, const float4* __restrict__ sf,
                const float4* __restrict__ st, float4* __restrict__ pos_n, float4* __restrict__ vel_n,
                float4* __restrict__ omg_n, uint32_t* __restrict__ keys, uint32_t* __restrict__ vals, uint32_t n,
                uint32_t hist_spec, uint32_t* __restrict__ ghist, MoveSink ms, SkinLists sk) {
    __shared__ uint32_t s_hist[kHistWords];
    if (ghist) {
        for (int q = threadIdx.x; q < kHistWords; q += blockDim.x) s_hist[q] = 0;
        __syncthreads();
    }
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t b = t >> 2;
    body_step(p, b, b < nb, t & 3u, bpos, bvel, bquat, bomg, bang, binv, bfirst, bcount, r0, slot_of, pos, omg, sf,
              st, pos_n, vel_n, omg_n, keys, vals, n, hist_spec, ghist ? s_hist : nullptr, ms, sk);
    if (ghist) {
        __syncthreads();
        hist_flush(s_hist, hist_spec, ghist);
    }
}

__global__ void dem_keys_kernel(DemParams p, uint32_t n, const float4* __restrict__ pos,
                                uint32_t* __restrict__ keys, uint32_t* __restrict__ vals, Batch bt) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 q = pos[i];
    const Grid g = bt.n > 1 ? grid_of_slot(bt.scenes, bt.first, bt.n, i) : grid_of(p);
    keys[i] = cell_key_g(g, q.x, q.y, q.z);
    vals[i] = i;
}

constexpr int kReorderThreads = 256;

// Writes cell_start for the cells block [b0, b1) owns, (s_keys[0],
// s_keys[cnt]] (the first block starts at cell 0, the last ends at ncells),
// by binary search over the block's sorted keys s_keys[1..cnt] in shared
// memory, so that every cell's lower bound is written exactly once.  Cells
// at or before the block's first key take b0 and cells after its last key
// (only the last block has them: the tail up to ncells) take b1 without a
// search -- an empty region past the last sphere can be tens of thousands
// of cells, all in that one block.
__device__ __forceinline__ void block_cell_starts(const uint32_t* s_keys, uint32_t b0, uint32_t b1, uint32_t n,
                                                  uint32_t ncells, uint32_t* __restrict__ cell_start) {
    const int64_t lo = b0 == 0 ? -1 : (int64_t)s_keys[0];
    const int64_t hi = b1 == n ? (int64_t)ncells : min((int64_t)s_keys[b1 - b0], (int64_t)ncells);
    const uint32_t cnt = b1 - b0;
    const int64_t kfirst = cnt ? (int64_t)s_keys[1] : hi, klast = cnt ? (int64_t)s_keys[cnt] : lo;
    for (int64_t c = lo + 1 + threadIdx.x; c <= hi; c += blockDim.x) {
        if (c <= kfirst || c > klast) {
            cell_start[c] = c <= kfirst ? b0 : b1;
            continue;
        }
        uint32_t a = 0, z = cnt;  // first index in [0, cnt) with key >= c, else cnt
        while (a < z) {
            uint32_t m = (a + z) >> 1;
            if ((int64_t)s_keys[m + 1] < c) a = m + 1;
            else z = m;
        }
        cell_start[c] = b0 + a;
    }
}

// Gather the next state into sorted order and write cell_start.
__global__ void __launch_bounds__(kReorderThreads)
dem_reorder_kernel(uint32_t n, uint32_t ncells, const uint32_t* __restrict__ keys,
                   const uint32_t* __restrict__ vals, const float4* __restrict__ pos_n,
                   const float4* __restrict__ vel_n, const float4* __restrict__ omg_n,
                   float4* __restrict__ pos, float4* __restrict__ vel, float4* __restrict__ omg,
                   uint32_t* __restrict__ cell_start, uint32_t* __restrict__ slot_of,
                   uint32_t* __restrict__ keys_prev, bool slot_all) {
    __shared__ uint32_t s_keys[kReorderThreads + 1];
    const uint32_t b0 = blockIdx.x * kReorderThreads;
    const uint32_t b1 = min(b0 + kReorderThreads, n);
    const uint32_t k = b0 + threadIdx.x;
    if (k < n) {
        const uint32_t src = vals[k];
        if (src < n) {  // always true for a valid permutation
            pos[k] = pos_n[src];
            vel[k] = vel_n[src];
            const float4 o = omg_n[src];
            omg[k] = o;
            // clump spheres: where their body finds them next step
            const uint32_t idb = __float_as_uint(o.w);
            if (slot_of && (slot_all || (idb & kClumpFlag)) && (idb & kIdMask) < n) slot_of[idb & kIdMask] = k;
        }
        const uint32_t key = keys[k];
        s_keys[threadIdx.x + 1] = key;
        keys_prev[k] = key;  // what the next step's incremental re-sort compares against
    }
    if (threadIdx.x == 0) s_keys[0] = b0 == 0 ? 0u : keys[b0 - 1];
    __syncthreads();
    block_cell_starts(s_keys, b0, b1, n, ncells, cell_start);
}

// The order the incremental re-sort found: the new keys, and the M moved
// entries in (key, slot) order with their sorted positions and, per moved
// slot in ascending order, slot - rank.
struct ResortView {
    const uint32_t* keys_new;
    const uint32_t* pos;
    const uint32_t* q;
    const unsigned long long* list;
    const uint32_t* scratch;  // [1] = M, [3] = T
    uint32_t mmax;
    const uint32_t* iv_lo;    // per moved entry: first position of the interval its move shifts
    const uint32_t* iv_pre;   // exclusive prefix sums of the intervals' lengths (T = iv_pre[M])
};

// First index in [0, m) of ascending a with a[i] >= x (m if none).
__device__ __forceinline__ uint32_t lower_idx(const uint32_t* a, uint32_t m, uint32_t x) {
    uint32_t lo = 0, hi = m;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// First index in [0, m) of ascending a with a[i] > x (m if none).
__device__ __forceinline__ uint32_t upper_idx(const uint32_t* a, uint32_t m, uint32_t x) {
    uint32_t lo = 0, hi = m;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a[mid] <= x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Copies the re-sort's positions and slot - rank lists (M <= kResortMaxCap)
// into the block's shared memory; every thread calls it.
__device__ __forceinline__ void load_resort_lists(const ResortView& rv, uint32_t M, uint32_t* s_pos, uint32_t* s_q) {
    for (uint32_t i = threadIdx.x; i < M; i += blockDim.x) {
        s_pos[i] = rv.pos[i];
        s_q[i] = rv.q[i];
    }
    __syncthreads();
}

// Source slot and key of sorted position k: a moved entry where one was
// placed (returns true), else the unmoved slot of rank u = k - (moved
// entries placed before k), which is u + #{moved slots s_j with s_j - j <=
// u}.  An unmoved slot's new key is its previous one.
template <bool KEY>
__device__ __forceinline__ bool sorted_entry(uint32_t k, uint32_t M, const uint32_t* s_pos, const uint32_t* s_q,
                                             const ResortView& rv, uint32_t n, uint32_t& src, uint32_t& key) {
    const uint32_t lo = lower_idx(s_pos, M, k);
    if (lo < M && s_pos[lo] == k) {
        const unsigned long long c = rv.list[lo];
        src = (uint32_t)c;
        if (KEY) key = (uint32_t)(c >> 32);
        return true;
    }
    const uint32_t u = k - lo;
    src = u + upper_idx(s_q, M, u);
    if (KEY) key = src < n ? rv.keys_new[src] : 0u;
    return false;
}

// The contact lists the in-place reorder moves with the state (all null
// when the step uses none): per slot count, build position and kVlCap rows
// of neighbour ids, and same-sized buffers for the gathered entries.
struct ListView {
    uint32_t* cnt;
    float4* ref;
    uint32_t* nbr;
    uint32_t* cnt_t;
    float4* ref_t;
    uint32_t* nbr_t;
};

// The in-place reorder of a step whose next state stays where the contact
// kernel wrote it (S, the *_n buffers, in the previous slot order).  Sorted
// position k needs the entry of slot src(k); where src(k) == k -- every
// slot but those shifted by the moved keys -- nothing moves.  Only
// positions between a moved entry's old slot and its new position can
// change hands, so with the re-sort's order the kernels visit those
// intervals (T positions in all; a position in several is visited by each,
// writing the same values) rather than all n, unless T is above n / 4.
// Phase 1 gathers the positions that change hands into the free buffer T
// (the step's input state, no longer read) and, with the re-sort's order,
// shifts the cell table: cell_start[c] counts the entries with key < c, so
// an entry moving from key a to key b takes one from the cells (a, b] when
// b > a and adds one to (b, a] when b < a (atomic adds: several entries may
// share cells).  Phase 2 copies the gathered entries back and records
// their keys; for the radix passes' order (more moves than the re-sort
// takes) every position is visited and the cell table is rebuilt as the
// plain reorder does.  Both kernels run on a fixed grid (grid-stride).

// Position visited by work item t: in interval mode the position of item t
// among the intervals' concatenation, else t itself.
__device__ __forceinline__ uint32_t visit_position(uint32_t t, bool iv, uint32_t M, const uint32_t* s_ivlo,
                                                   const uint32_t* s_ivpre) {
    if (!iv) return t;
    const uint32_t r = upper_idx(s_ivpre, M, t) - 1u;  // s_ivpre[0] = 0 <= t
    return s_ivlo[r] + (t - s_ivpre[r]);
}

// Loads the re-sort's lists (and the intervals when iv) into shared memory.
__device__ __forceinline__ void load_fix_lists(const ResortView& rv, uint32_t M, bool iv, uint32_t* s_pos,
                                               uint32_t* s_q, uint32_t* s_ivlo, uint32_t* s_ivpre) {
    for (uint32_t i = threadIdx.x; i < M; i += blockDim.x) {
        s_pos[i] = rv.pos[i];
        s_q[i] = rv.q[i];
        if (iv) {
            s_ivlo[i] = rv.iv_lo[i];
            s_ivpre[i] = rv.iv_pre[i];
        }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kReorderThreads)
dem_fix_gather_kernel(uint32_t n, uint32_t ncells, const uint32_t* __restrict__ vals,
                      const float4* __restrict__ s_pos4, const float4* __restrict__ s_vel,
                      const float4* __restrict__ s_omg, float4* __restrict__ t_pos, float4* __restrict__ t_vel,
                      float4* __restrict__ t_omg, uint32_t* __restrict__ cell_start,
                      const uint32_t* __restrict__ keys_prev, ResortView rv, ListView lv) {
    __shared__ uint32_t s_pos[kResortMaxCap], s_q[kResortMaxCap], s_ivlo[kResortMaxCap], s_ivpre[kResortMaxCap];
    const uint32_t M = rv.scratch[1];
    const bool inc = M <= rv.mmax;
    const uint32_t T = inc ? (M ? rv.scratch[3] : 0u) : n;
    const bool iv = inc && T <= n / 4;
    const uint32_t total = iv ? T : n;
    // a block with neither positions nor a moved entry (cell shifts) to take
    if (blockIdx.x * kReorderThreads >= total && !(inc && blockIdx.x < M)) return;
    if (inc) load_fix_lists(rv, M, iv, s_pos, s_q, s_ivlo, s_ivpre);
    for (uint32_t t = blockIdx.x * kReorderThreads + threadIdx.x; t < total; t += gridDim.x * kReorderThreads) {
        const uint32_t k = visit_position(t, iv, M, s_ivlo, s_ivpre);
        if (k >= n) continue;
        uint32_t src, key;
        if (inc) sorted_entry<false>(k, M, s_pos, s_q, rv, n, src, key);
        else src = vals[k];
        if (src != k && src < n) {
            t_pos[k] = s_pos4[src];
            t_vel[k] = s_vel[src];
            t_omg[k] = s_omg[src];
            if (lv.cnt) {
                const uint32_t c = lv.cnt[src];
                lv.cnt_t[k] = c;
                lv.ref_t[k] = lv.ref[src];
                for (uint32_t q = 0; q < min(c, kVlCap); ++q) lv.nbr_t[(size_t)q * n + k] = lv.nbr[(size_t)q * n + src];
            }
        }
    }
    if (!inc) return;
    for (uint32_t r = blockIdx.x; r < M; r += gridDim.x) {  // one moved entry per block
        const unsigned long long c = rv.list[r];
        const uint32_t b = min((uint32_t)(c >> 32), ncells), slot = (uint32_t)c;
        const uint32_t a = slot < n ? min(keys_prev[slot], ncells) : b;
        const uint32_t lo = min(a, b) + 1, hi = max(a, b);  // cells [lo, hi]
        const uint32_t d = b > a ? 0xffffffffu : 1u;          // -1 or +1
        for (uint32_t cc = lo + threadIdx.x; cc <= hi; cc += kReorderThreads) atomicAdd(&cell_start[cc], d);
    }
}

__global__ void __launch_bounds__(kReorderThreads)
dem_fix_place_kernel(uint32_t n, uint32_t ncells, const uint32_t* __restrict__ keys,
                     const uint32_t* __restrict__ vals, const float4* __restrict__ t_pos,
                     const float4* __restrict__ t_vel, const float4* __restrict__ t_omg, float4* __restrict__ s_pos4,
                     float4* __restrict__ s_vel, float4* __restrict__ s_omg, uint32_t* __restrict__ cell_start,
                     uint32_t* __restrict__ slot_of, uint32_t* __restrict__ keys_prev, ResortView rv,
                     bool slot_all, ListView lv) {
    __shared__ uint32_t s_keys[kReorderThreads + 1];
    __shared__ uint32_t s_pos[kResortMaxCap], s_q[kResortMaxCap], s_ivlo[kResortMaxCap], s_ivpre[kResortMaxCap];
    const uint32_t M = rv.scratch[1];
    const bool inc = M <= rv.mmax;
    const uint32_t T = inc ? (M ? rv.scratch[3] : 0u) : n;
    const bool iv = inc && T <= n / 4;
    // the radix order: chunks of kReorderThreads consecutive positions per
    // block iteration, so that each chunk rebuilds its part of the cell table
    const uint32_t total = inc ? (iv ? T : n) : (n + kReorderThreads - 1) / kReorderThreads * kReorderThreads;
    if (blockIdx.x * kReorderThreads >= total) return;  // no positions for this block
    if (inc) load_fix_lists(rv, M, iv, s_pos, s_q, s_ivlo, s_ivpre);
    for (uint32_t t0 = blockIdx.x * kReorderThreads; t0 < total; t0 += gridDim.x * kReorderThreads) {
        const uint32_t t = t0 + threadIdx.x;
        const uint32_t k = t < total ? visit_position(t, iv, M, s_ivlo, s_ivpre) : n;
        if (k < n) {
            uint32_t src, key = 0;
            bool write = true;
            if (inc) {
                // a position that keeps its unmoved entry keeps its key too:
                // nothing to write there
                const bool moved = sorted_entry<false>(k, M, s_pos, s_q, rv, n, src, key);
                if (src == k && !moved) write = false;
                else key = moved ? (uint32_t)(rv.list[lower_idx(s_pos, M, k)] >> 32)
                                 : (src < n ? rv.keys_new[src] : 0u);
            } else {
                src = vals[k];
                key = keys[k];
            }
            if (write) {
                if (src != k && src < n) {
                    s_pos4[k] = t_pos[k];
                    s_vel[k] = t_vel[k];
                    const float4 o = t_omg[k];
                    s_omg[k] = o;
                    const uint32_t idb = __float_as_uint(o.w);
                    if (slot_of && (slot_all || (idb & kClumpFlag)) && (idb & kIdMask) < n)
                        slot_of[idb & kIdMask] = k;
                    if (lv.cnt) {
                        const uint32_t c = lv.cnt_t[k];
                        lv.cnt[k] = c;
                        lv.ref[k] = lv.ref_t[k];
                        for (uint32_t q = 0; q < min(c, kVlCap); ++q)
                            lv.nbr[(size_t)q * n + k] = lv.nbr_t[(size_t)q * n + k];
                    }
                }
                keys_prev[k] = key;
            }
            if (!inc) s_keys[threadIdx.x + 1] = key;
        }
        if (!inc) {  // uniform: the radix order rebuilds the cell table chunk by chunk
            const uint32_t b0 = t0, b1 = min(t0 + kReorderThreads, n);
            if (threadIdx.x == 0) s_keys[0] = b0 == 0 ? 0u : keys[b0 - 1];
            __syncthreads();
            block_cell_starts(s_keys, b0, b1, n, ncells, cell_start);
            __syncthreads();
        }
    }
}

__global__ void dem_pairs_kernel(DemParams p, uint32_t n, const float4* __restrict__ pos,
                                 const float4* __restrict__ omg, const uint32_t* __restrict__ cell_start,
                                 unsigned long long* __restrict__ pairs, unsigned long long* __restrict__ npairs,
                                 uint64_t cap, uint32_t* __restrict__ status, const int32_t* __restrict__ body_of,
                                 Batch bt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Grid g = bt.n > 1 ? grid_of_slot(bt.scenes, bt.first, bt.n, i) : grid_of(p);
    const float4 pi = pos[i];
    const uint32_t idbi = __float_as_uint(omg[i].w);
    const uint32_t idi = idbi & kIdMask;
    const int32_t bi = (body_of && (idbi & kClumpFlag)) ? body_of[idi] : -1;
    const int32_t cx = axis_cell(pi.x, g.lo[0], g.cell, g.nx);
    const int32_t cy = axis_cell(pi.y, g.lo[1], g.cell, g.ny);
    // every partner centre is within one cell edge (a contact needs
    // |dz| < r_i + r_j <= cell); truncation of the rounded quotient is
    // monotone, so these z cells contain all of them
    const int32_t z0 = axis_cell(pi.z - g.cell * 1.00001f, g.lo[2], g.cellz, g.nz);
    const int32_t z1 = axis_cell(pi.z + g.cell * 1.00001f, g.lo[2], g.cellz, g.nz);
    for (int32_t ddx = -1; ddx <= 1; ++ddx) {
        const int32_t X = cx + ddx;
        if (X < 0 || X >= g.nx) continue;
        for (int32_t ddy = -1; ddy <= 1; ++ddy) {
            const int32_t Y = cy + ddy;
            if (Y < 0 || Y >= g.ny) continue;
            const uint32_t col = g.base + (uint32_t)((X * g.ny + Y) * g.nz);
            const uint32_t s1 = min(cell_start[col + (uint32_t)z1 + 1], n);
            for (uint32_t s = cell_start[col + (uint32_t)z0]; s < s1; ++s) {
                if (s == i) continue;
                const float4 pj = pos[s];
                const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                const float d2 = dist2(dx, dy, dz);
                const float rs = pi.w + pj.w;
                if (!(d2 < rs * rs) || d2 == 0.0f) continue;
                const uint32_t idbj = __float_as_uint(omg[s].w);
                const uint32_t idj = idbj & kIdMask;
                if (bi >= 0 && (idbj & kClumpFlag) && body_of[idj] == bi) continue;  // same rigid body
                if (idi < idj) {
                    unsigned long long slot = atomicAdd(npairs, 1ull);
                    if (slot < cap) pairs[slot] = ((unsigned long long)idi << 32) | idj;
                    else atomicOr(status, kErrPairOverflow);
                }
            }
        }
    }
}

// dst[id] = src[slot]: back to the order spheres were added.
__global__ void dem_unsort_kernel(const float4* __restrict__ src, const float4* __restrict__ omg,
                                  float4* __restrict__ dst, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t id = __float_as_uint(omg[i].w) & kIdMask;
    if (id < n) dst[id] = src[i];
}

// dst[slot] = src_by_id[id], keeping the w lane of dst when keep_w (the id
// lane of the omega array).
__global__ void dem_scatter_in_kernel(const float4* __restrict__ src, const float4* __restrict__ omg,
                                      float4* __restrict__ dst, uint32_t n, bool keep_w) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t id = __float_as_uint(omg[i].w) & kIdMask;
    if (id >= n) return;
    float4 v = src[id];
    if (keep_w) v.w = dst[i].w;
    dst[i] = v;
}

// slot_of_id[id] = slot for every sphere (ids in the omega w lane).
__global__ void dem_slot_of_id_kernel(const float4* __restrict__ omg, uint32_t* __restrict__ slot_of_id, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = __float_as_uint(omg[i].w) & kIdMask;
    if (id < n) slot_of_id[id] = i;
}

// Id-ordered host buffer <-> slot-ordered state, one thread per id: the
// host side is read or written in order (one pass over the host link); the
// slot side is the random one, in device memory.
__global__ void dem_by_id_in_kernel(const float4* __restrict__ host_src, const uint32_t* __restrict__ slot_of_id,
                                    float4* __restrict__ dst, uint32_t n, bool keep_w) {
    const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const uint32_t s = slot_of_id[id];
    if (s >= n) return;
    float4 v = host_src[id];
    if (keep_w) v.w = dst[s].w;
    dst[s] = v;
}

__global__ void dem_by_id_out_kernel(const float4* __restrict__ src, const uint32_t* __restrict__ slot_of_id,
                                     float4* __restrict__ host_dst, uint32_t n) {
    const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= n) return;
    const uint32_t s = slot_of_id[id];
    if (s < n) host_dst[id] = src[s];
}

// Kinetic energy (translational + rotational, solid spheres) and linear
// momentum, accumulated in double.
__global__ void dem_energy_kernel(uint32_t n, const float4* __restrict__ pos, const float4* __restrict__ vel,
                                  const float4* __restrict__ omg, double* __restrict__ out) {
    double e = 0, px = 0, py = 0, pz = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 v = vel[i], w = omg[i], q = pos[i];
        if (__float_as_uint(w.w) & kClumpFlag) continue;  // counted with its body
        double m = v.w, r = q.w;
        double I = 0.4 * m * r * r;
        e += 0.5 * m * ((double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z) +
             0.5 * I * ((double)w.x * w.x + (double)w.y * w.y + (double)w.z * w.z);
        px += m * v.x;
        py += m * v.y;
        pz += m * v.z;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        e += __shfl_down_sync(0xffffffffu, e, o);
        px += __shfl_down_sync(0xffffffffu, px, o);
        py += __shfl_down_sync(0xffffffffu, py, o);
        pz += __shfl_down_sync(0xffffffffu, pz, o);
    }
    if (lane_id() == 0) {
        atomicAdd(&out[0], e);
        atomicAdd(&out[1], px);
        atomicAdd(&out[2], py);
        atomicAdd(&out[3], pz);
    }
}

// The mesh pose of the next step: q <- normalize(dq (x) q) (Hamilton
// product), then the rotation matrix of q (the expression of the rigid
// bodies).
__global__ void mesh_advance_kernel(float* __restrict__ S, int advance) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float qs = S[16], qx = S[17], qy = S[18], qz = S[19];
    if (advance) {
        const float ds = S[20], dx = S[21], dy = S[22], dz = S[23];
        const float ns = ds * qs - ((dx * qx + dy * qy) + dz * qz);
        const float nx = (ds * qx + qs * dx) + (dy * qz - dz * qy);
        const float ny = (ds * qy + qs * dy) + (dz * qx - dx * qz);
        const float nz = (ds * qz + qs * dz) + (dx * qy - dy * qx);
        const float nrm = sqrtf((ns * ns + nx * nx) + (ny * ny + nz * nz));
        qs = ns / nrm;
        qx = nx / nrm;
        qy = ny / nrm;
        qz = nz / nrm;
        S[16] = qs;
        S[17] = qx;
        S[18] = qy;
        S[19] = qz;
    }
    S[0] = 1.0f - 2.0f * (qy * qy + qz * qz);
    S[1] = 2.0f * (qx * qy - qs * qz);
    S[2] = 2.0f * (qx * qz + qs * qy);
    S[3] = 2.0f * (qx * qy + qs * qz);
    S[4] = 1.0f - 2.0f * (qx * qx + qz * qz);
    S[5] = 2.0f * (qy * qz - qs * qx);
    S[6] = 2.0f * (qx * qz - qs * qy);
    S[7] = 2.0f * (qy * qz + qs * qx);
    S[8] = 1.0f - 2.0f * (qx * qx + qy * qy);
}

static inline unsigned grid_for(uint32_t n, unsigned threads) { return (n + threads - 1) / threads; }

cudaError_t mesh_advance_async(const MeshView& m, int advance, cudaStream_t st) {
    if (m.ntri == 0) return cudaSuccess;
    mesh_advance_kernel<<<1, 32, 0, st>>>(m.state, advance);
    return cudaGetLastError();
}

cudaError_t dem_init_kernels() {
    const int sm = (int)(kTileSlots * sizeof(float4));
    const void* kernels[] = {(const void*)dem_contact_column_kernel<false, false>,
                             (const void*)dem_contact_column_kernel<true, false>,
                             (const void*)dem_contact_column_kernel<false, true>,
                             (const void*)dem_contact_column_kernel<true, true>};
    for (const void* k : kernels) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Counts the slots whose sphere's cell key, from its current position,
// differs from the sorted key it is placed under.
__global__ void dem_keys_changed_kernel(DemParams p, uint32_t n, const float4* __restrict__ pos,
                                        const uint32_t* __restrict__ sorted_keys, Batch bt,
                                        uint32_t* __restrict__ count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool changed = false;
    if (i < n) {
        const float4 q = pos[i];
        const Grid g = bt.n > 1 ? grid_of_slot(bt.scenes, bt.first, bt.n, i) : grid_of(p);
        changed = cell_key_g(g, q.x, q.y, q.z) != sorted_keys[i];
    }
    const uint32_t m = __ballot_sync(0xffffffffu, changed);
    if (lane_id() == 0 && m) atomicAdd(count, __popc(m));
}

// Positions written by the host: a sphere now more than 0.45 skin from its
// position at the last list build makes the next step build the lists (the
// steps' own check runs only after integration).
__global__ void dem_skin_check_kernel(uint32_t n, const float4* __restrict__ pos, const float4* __restrict__ ref,
                                      float thr2, uint32_t* __restrict__ flags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool far = false;
    if (i < n) {
        const float4 q = pos[i], r = ref[i];
        far = dist2(q.x - r.x, q.y - r.y, q.z - r.z) > thr2;
    }
    if (__ballot_sync(0xffffffffu, far) && lane_id() == 0) flags[0] = 1u;
}

cudaError_t dem_skin_check_async(const DemBuffers& b, cudaStream_t st) {
    if (b.n == 0 || !b.vl_flags || !(b.vl_skin > 0.0f)) return cudaSuccess;
    const float thr = 0.45f * b.vl_skin;
    dem_skin_check_kernel<<<grid_for(b.n, 256), 256, 0, st>>>(b.n, b.pos, b.vl_ref, thr * thr, b.vl_flags);
    return cudaGetLastError();
}

cudaError_t dem_keys_changed_async(const DemParams& p, const DemBuffers& b, uint32_t* count, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess || b.n == 0) return e;
    dem_keys_changed_kernel<<<grid_for(b.n, 256), 256, 0, st>>>(p, b.n, b.pos, b.keys_prev,
                                                                Batch{b.scenes, b.scene_first, b.nscenes}, count);
    return cudaGetLastError();
}

cudaError_t dem_keys_from_state_async(const DemParams& p, DemBuffers& b, cudaStream_t st) {
    if (b.n == 0) return cudaSuccess;
    dem_keys_kernel<<<grid_for(b.n, 256), 256, 0, st>>>(p, b.n, b.pos_n, b.keys, b.vals,
                                                        Batch{b.scenes, b.scene_first, b.nscenes});
    return cudaGetLastError();
}

int dem_key_bits(uint32_t ncells) {
    int bits = 1;
    while (bits < 32 && (1ull << bits) < (unsigned long long)ncells) ++bits;
    return bits;
}

cudaError_t dem_sort_async(DemBuffers& b, cudaStream_t st) {
    b.sorted_in_tmp = false;
    if (b.n == 0) return cudaSuccess;
    return sort_pairs_async(b.keys, b.vals, b.keys_tmp, b.vals_tmp, b.n, dem_key_bits(b.ncells), b.sort_scratch,
                            st, &b.sorted_in_tmp);
}

// The slot table covers every sphere when the skin lists use it, else only
// clump spheres (null without clumps or lists).
static bool slot_all_of(const DemBuffers& b) { return b.vl_skin > 0.0f && b.vl_cnt; }

cudaError_t dem_reorder_async(DemBuffers& b, cudaStream_t st) {
    if (b.n == 0) return cudaMemsetAsync(b.cell_start, 0, sizeof(uint32_t) * (b.ncells + 1), st);
    const uint32_t* k = b.sorted_in_tmp ? b.keys_tmp : b.keys;
    const uint32_t* v = b.sorted_in_tmp ? b.vals_tmp : b.vals;
    dem_reorder_kernel<<<grid_for(b.n, kReorderThreads), kReorderThreads, 0, st>>>(
        b.n, b.ncells, k, v, b.pos_n, b.vel_n, b.omg_n, b.pos, b.vel, b.omg, b.cell_start,
        b.slot_of, b.keys_prev, slot_all_of(b));
    return cudaGetLastError();
}

cudaError_t dem_sort_reorder_async(const DemParams& p, DemBuffers& b, cudaStream_t st) {
    (void)p;
    cudaError_t e = dem_sort_async(b, st);
    if (e != cudaSuccess) return e;
    return dem_reorder_async(b, st);
}

static int g_contact_mode = 0;  // 0: per slot (default), 1: TMA column tiles
// The two-kernel contact stage (pair kernel + listed contacts) for scenes
// without clumps or meshes: 0 never, 1 always, 2 for batches of scenes only.
// Measured: 512-scene batch 0.381 -> 0.365 ms per step with it; the
// 1,048,576-sphere box 0.158 -> 0.179 ms (the second pass over the state
// and the per-column setup cost more than the halved candidate tests).
static int g_pair_lists = 2;

void dem_set_pair_lists(int mode) { g_pair_lists = mode; }

// launch shapes (knobs "contact_block", "fix_blocks"): threads per block of
// the per-slot contact kernels (64, 128 or 256) and blocks per SM of the
// in-place reorder's fixed grid (2, 4 or 8)
static int g_contact_block = 256;
static int g_fix_blocks = 8;
void dem_set_contact_block(int t) { g_contact_block = t; }
int dem_contact_block() { return g_contact_block; }
void dem_set_fix_blocks(int b) { g_fix_blocks = b; }
int dem_fix_blocks() { return g_fix_blocks; }

// resident blocks per SM the listed kernel is compiled for: 4 or 5.  Five
// (48 registers, spills only in the build scan) measured 0.0632 ms per
// step at 1,048,576 spheres against 0.0668 ms with four (64 registers)
static int g_listed_blocks = 5;
void dem_set_listed_blocks(int b) { g_listed_blocks = (b == 5 || b == 6 || b == 8) ? b : 4; }
int dem_listed_blocks() { return g_listed_blocks; }
int dem_pair_lists() { return g_pair_lists; }

void dem_set_contact_mode(int mode) { g_contact_mode = mode == 0 ? 0 : 1; }
int dem_contact_mode() { return g_contact_mode; }

template <bool RECORD>
static void launch_contact_t(const DemParams& p, DemBuffers& b, uint32_t spec, uint32_t* ghist, cudaStream_t st,
                             bool skin, const MoveSink& ms) {
    float4* f = RECORD ? b.force : nullptr;
    float4* t = RECORD ? b.torque : nullptr;
    const ClumpCtx cc{b.nb ? b.body_of : nullptr, b.sf, b.st};
    const unsigned cols = (unsigned)p.nx * (unsigned)p.ny;
    const size_t tile = kTileSlots * sizeof(float4);
    const unsigned cb = (unsigned)g_contact_block;  // threads per block of the per-slot kernels
    const unsigned grid = grid_for(b.n, cb);
    // the re-sort step needs no slot identity (its radix fallback writes it)
    uint32_t* const vals = ms.list ? nullptr : b.vals;
    if (skin) {  // one scene or a batch, contact lists (clumps and meshes: one scene)
        const float thr = 0.45f * b.vl_skin;
        const SkinLists sk{b.vl_cnt, b.vl_nbr, b.vl_ref, b.vl_flags, b.vl_flags + 1, b.slot_of, b.vl_skin, thr * thr};
        const Batch bt{b.scenes, b.scene_first, b.nscenes};
        if (b.nscenes > 1) {
            if (g_listed_blocks == 5)
                dem_contact_listed_kernel<RECORD, 5, true><<<grid, cb, 0, st>>>(
                    p, b.n, b.pos, b.vel, b.omg, b.cell_start, b.pos_n, b.vel_n, b.omg_n, b.keys, vals, f, t,
                    b.dev_status, sk, ms, bt);
            else
                dem_contact_listed_kernel<RECORD, 4, true><<<grid, cb, 0, st>>>(
                    p, b.n, b.pos, b.vel, b.omg, b.cell_start, b.pos_n, b.vel_n, b.omg_n, b.keys, vals, f, t,
                    b.dev_status, sk, ms, bt);
        } else if (b.nb && b.mesh.ntri) {
            dem_contact_listed_kernel<RECORD, 5, false, true, true><<<grid, cb, 0, st>>>(
                p, b.n, b.pos, b.vel, b.omg, b.cell_start, b.pos_n, b.vel_n, b.omg_n, b.keys, vals, f, t,
                b.dev_status, sk, ms, Batch{}, cc, b.mesh);
        } else if (b.nb) {
            dem_contact_listed_kernel<RECORD, 5, false, true, false><<<grid, cb, 0, st>>>(
                p, b.n, b.pos, b.vel, b.omg, b.cell_start, b.pos_n, b.vel_n, b.omg_n, b.keys, vals, f, t,
                b.dev_status, sk, ms, Batch{}, cc);
        } else if (b.mesh.ntri) {
            dem_contact_listed_kernel<RECORD, 5, false, false, true><<<grid, cb, 0, st>>>(
                p, b.n, b.pos, b.vel, b.omg, b.cell_start, b.pos_n, b.vel_n, b.omg_n, b.keys, vals, f, t,
                b.dev_status, sk, ms, Batch{}, ClumpCtx{}, b.mesh);
        } else if (g_listed_blocks == 6) {
            dem_contact_listed_kernel<RECORD, 6, false><<<grid, cb, 0, st>>>(
                p, b.n, b.pos, b.vel, b.omg, b.cell_start, b.pos_n, b.vel_n, b.omg_n, b.keys, vals, f, t,
                b.dev_status, sk, ms, Batch{});
        } else if (g_listed_blocks == 8) {
            dem_contact_listed_kernel<RECORD, 8, false><<<grid, cb, 0, st>>>(
                p, b.n, b.pos, b.vel, b.omg, b.cell_start, b.pos_n, b.vel_n, b.omg_n, b.keys, vals, f, t,
                b.dev_status, sk, ms, Batch{});
        } else if (g_listed_blocks == 5) {
            dem_contact_listed_kernel<RECORD, 5, false><<<grid, cb, 0, st>>>(
                p, b.n, b.pos, b.vel, b.omg, b.cell_start, b.pos_n, b.vel_n, b.omg_n, b.keys, vals, f, t,
                b.dev_status, sk, ms, Batch{});
        } else {
            dem_contact_listed_kernel<RECORD, 4, false><<<grid, cb, 0, st>>>(
                p, b.n, b.pos, b.vel, b.omg, b.cell_start, b.pos_n, b.vel_n, b.omg_n, b.keys, vals, f, t,
                b.dev_status, sk, ms, Batch{});
        }
    } else if (b.mesh.ntri) {  // mesh walls (one scene; clumps allowed; per-slot kernel)
        if (b.nb)
            dem_contact_integrate_kernel<RECORD, true, false, true><<<grid, cb, 0, st>>>(
                p, b.n, b.pos, b.vel, b.omg, b.cell_start, b.pos_n, b.vel_n, b.omg_n, b.keys, vals, f, t,
                b.dev_status, spec, ghist, cc, Batch{}, b.mesh, NbrLists{}, SkinLists{}, ms);
        else
            dem_contact_integrate_kernel<RECORD, false, false, true><<<grid, cb, 0, st>>>(
                p, b.n, b.pos, b.vel, b.omg, b.cell_start, b.pos_n, b.vel_n, b.omg_n, b.keys, vals, f, t,
                b.dev_status, spec, ghist, cc, Batch{}, b.mesh, NbrLists{}, SkinLists{}, ms);
    } else if (b.nscenes > 1) {  // a batch: scene grids per slot (clumps are not batched)
        const Batch bt{b.scenes, b.scene_first, b.nscenes};
        if (g_pair_lists != 0 && b.nbr_cnt) {
            dem_pair_lists_kernel<true><<<grid, cb, 0, st>>>(p, b.n, b.pos, b.cell_start, b.nbr_cnt, b.nbr, bt);
            dem_contact_integrate_kernel<RECORD, false, true, false, true><<<grid, cb, 0, st>>>(
                p, b.n, b.pos, b.vel, b.omg, b.cell_start, b.pos_n, b.vel_n, b.omg_n, b.keys, vals, f, t,
                b.dev_status, spec, ghist, cc, bt, MeshView{}, NbrLists{b.nbr_cnt, b.nbr}, SkinLists{}, ms);
        } else {
            dem_contact_integrate_kernel<RECORD, false, true><<<grid, cb, 0, st>>>(
                p, b.n, b.pos, b.vel, b.omg, b.cell_start, b.pos_n, b.vel_n, b.omg_n, b.keys, vals, f, t,
                b.dev_status, spec, ghist, cc, bt, MeshView{}, NbrLists{}, SkinLists{}, ms);
        }
    } else if (g_contact_mode == 0 && !b.nb && g_pair_lists == 1 && b.nbr_cnt) {
        dem_pair_lists_kernel<false><<<grid, cb, 0, st>>>(p, b.n, b.pos, b.cell_start, b.nbr_cnt, b.nbr, Batch{});
        dem_contact_integrate_kernel<RECORD, false, false, false, true><<<grid, cb, 0, st>>>(
            p, b.n, b.pos, b.vel, b.omg, b.cell_start, b.pos_n, b.vel_n, b.omg_n, b.keys, vals, f, t,
            b.dev_status, spec, ghist, cc, Batch{}, MeshView{}, NbrLists{b.nbr_cnt, b.nbr}, SkinLists{}, ms);
    } else if (g_contact_mode == 0) {
        if (b.nb)
            dem_contact_integrate_kernel<RECORD, true><<<grid, cb, 0, st>>>(
                p, b.n, b.pos, b.vel, b.omg, b.cell_start, b.pos_n, b.vel_n, b.omg_n, b.keys, vals, f, t,
                b.dev_status, spec, ghist, cc, Batch{}, MeshView{}, NbrLists{}, SkinLists{}, ms);
        else
            dem_contact_integrate_kernel<RECORD, false><<<grid, cb, 0, st>>>(
                p, b.n, b.pos, b.vel, b.omg, b.cell_start, b.pos_n, b.vel_n, b.omg_n, b.keys, vals, f, t,
                b.dev_status, spec, ghist, cc, Batch{}, MeshView{}, NbrLists{}, SkinLists{}, ms);
    } else {
        if (b.nb)
            dem_contact_column_kernel<RECORD, true><<<cols, kColThreads, tile, st>>>(
                p, b.n, b.pos, b.vel, b.omg, b.cell_start, b.pos_n, b.vel_n, b.omg_n, b.keys, vals, f, t,
                b.dev_status, spec, ghist, cc, ms);
        else
            dem_contact_column_kernel<RECORD, false><<<cols, kColThreads, tile, st>>>(
                p, b.n, b.pos, b.vel, b.omg, b.cell_start, b.pos_n, b.vel_n, b.omg_n, b.keys, vals, f, t,
                b.dev_status, spec, ghist, cc, ms);
    }
}

// Contact + integration of free spheres, then (with clumps) the body
// kernel, which completes the next state and keys of the clump spheres.
// The new keys feed either the radix sort's histograms (ghist) or the
// incremental re-sort's list of moved slots (ms.list).
static cudaError_t launch_contact(const DemParams& p, DemBuffers& b, bool record, const SortPlan& plan,
                                  uint32_t* ghist, cudaStream_t st, bool skin = false,
                                  const MoveSink& ms = MoveSink{}) {
    if (b.n == 0) return cudaSuccess;
    const uint32_t spec = pack_hist_spec(plan);
    if (record) {
        cudaError_t e = cudaMemsetAsync(b.dev_status + 2, 0, sizeof(unsigned long long), st);
        if (e != cudaSuccess) return e;
        launch_contact_t<true>(p, b, spec, ghist, st, skin, ms);
    } else {
        launch_contact_t<false>(p, b, spec, ghist, st, skin, ms);
    }
    if (b.nb) {
        dem_body_kernel<<<grid_for(4u * b.nb, 128), 128, 0, st>>>(
            p, b.nb, b.bpos, b.bvel, b.bquat, b.bomg, b.bang, b.binv, b.bfirst, b.bcount, b.r0, b.slot_of, b.pos,
            b.omg, b.sf, b.st, b.pos_n, b.vel_n, b.omg_n, b.keys, ms.list ? nullptr : b.vals, b.n, spec, ghist, ms,
            skin ? SkinLists{b.vl_cnt, b.vl_nbr, b.vl_ref, b.vl_flags, b.vl_flags + 1, b.slot_of, b.vl_skin,
                             (0.45f * b.vl_skin) * (0.45f * b.vl_skin)}
                 : SkinLists{});
    }
    return cudaGetLastError();
}

cudaError_t dem_contact_integrate_async(const DemParams& p, DemBuffers& b, bool record, cudaStream_t st) {
    // the step's own variant: with contact lists on, the listed kernel (or
    // the build scan when a build is due)
    return launch_contact(p, b, record, SortPlan{}, nullptr, st, dem_step_skin(b));
}

// Fixed grid of the in-place reorder's kernels (grid-stride loops): most
// steps touch a few thousand positions, the radix fallback all of them.
static unsigned fix_grid(uint32_t n) {
    const unsigned g = grid_for(n, kReorderThreads), cap = 152u * (unsigned)g_fix_blocks;
    return g < cap ? g : cap;
}

// One whole step.  With the incremental re-sort (dem_step_swaps): contact +
// integrate (which lists the slots whose key changed), the re-sort's plan,
// the radix fallback (histogram + passes, returning at once when the plan
// placed the moves), the in-place reorder.  Otherwise: clear the sort's
// scratch, contact + integrate (which builds the key histograms), the
// digit passes, the reorder.
cudaError_t dem_step_async(const DemParams& p, DemBuffers& b, bool record, cudaStream_t st) {
    if (b.n == 0) return cudaSuccess;
    const SortPlan plan = sort_plan(dem_key_bits(b.ncells));
    if (plan.passes > kFusedPasses) {
        cudaError_t e = dem_contact_integrate_async(p, b, record, st);
        if (e != cudaSuccess) return e;
        if ((e = dem_sort_reorder_async(p, b, st)) != cudaSuccess) return e;
        return mesh_advance_async(b.mesh, 1, st);
    }
    cudaError_t e;
    if (!dem_step_swaps(b)) {
        if ((e = sort_clear_async(b.n, plan, b.sort_scratch, st)) != cudaSuccess) return e;
        if ((e = launch_contact(p, b, record, plan, sort_hist_ptr(b.sort_scratch), st)) != cudaSuccess) return e;
        if ((e = sort_passes_async(b.keys, b.vals, b.keys_tmp, b.vals_tmp, b.n, plan, b.sort_scratch, st,
                                   &b.sorted_in_tmp, nullptr, 0)) != cudaSuccess)
            return e;
        if ((e = dem_reorder_async(b, st)) != cudaSuccess) return e;
        return mesh_advance_async(b.mesh, 1, st);
    }
    const bool skin = dem_step_skin(b);
    const MoveSink ms{b.keys_prev, b.rs_list, b.rs_scratch, b.rs_max};
    if ((e = launch_contact(p, b, record, plan, nullptr, st, skin, ms)) != cudaSuccess) return e;
    if ((e = resort_plan_async(b, st, skin ? b.vl_flags : nullptr)) != cudaSuccess) return e;
    if ((e = sort_fallback_async(b.keys, b.vals, b.keys_tmp, b.vals_tmp, b.n, plan, b.sort_scratch, st,
                                 &b.sorted_in_tmp, b.rs_scratch, b.rs_max)) != cudaSuccess)
        return e;
    // sorted in place: the next state stays in the *_n buffers
    const uint32_t* k = b.sorted_in_tmp ? b.keys_tmp : b.keys;
    const uint32_t* v = b.sorted_in_tmp ? b.vals_tmp : b.vals;
    const ResortView rv{b.keys, b.rs_pos, b.rs_q, b.rs_list, b.rs_scratch, b.rs_max, b.rs_iv_lo, b.rs_iv_pre};
    const ListView lv = skin ? ListView{b.vl_cnt, b.vl_ref, b.vl_nbr, b.vl_cnt_t, b.vl_ref_t, b.vl_nbr_t}
                             : ListView{};
    const unsigned grid = fix_grid(b.n);
    dem_fix_gather_kernel<<<grid, kReorderThreads, 0, st>>>(b.n, b.ncells, v, b.pos_n, b.vel_n, b.omg_n, b.pos,
                                                            b.vel, b.omg, b.cell_start, b.keys_prev, rv, lv);
    dem_fix_place_kernel<<<grid, kReorderThreads, 0, st>>>(b.n, b.ncells, k, v, b.pos, b.vel, b.omg, b.pos_n,
                                                           b.vel_n, b.omg_n, b.cell_start, b.slot_of, b.keys_prev,
                                                           rv, slot_all_of(b), lv);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return mesh_advance_async(b.mesh, 1, st);
}

bool dem_step_skin(const DemBuffers& b) {
    return b.vl_skin > 0.0f && b.vl_cnt && b.slot_of &&
           g_contact_mode == 0 && dem_step_swaps(b);
}

bool dem_step_swaps(const DemBuffers& b) {
    return b.n > 0 && b.rs_max > 0 && b.rs_max <= kResortMaxCap && (b.rs_max & (b.rs_max - 1)) == 0 &&
           sort_plan(dem_key_bits(b.ncells)).passes <= kFusedPasses;
}

cudaError_t dem_pairs_async(const DemParams& p, DemBuffers& b, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(b.npairs, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess || b.n == 0) return e;
    dem_pairs_kernel<<<grid_for(b.n, 256), 256, 0, st>>>(p, b.n, b.pos, b.omg, b.cell_start, b.pairs, b.npairs,
                                                         b.pair_cap, b.dev_status, b.nb ? b.body_of : nullptr,
                                                         Batch{b.scenes, b.scene_first, b.nscenes});
    return cudaGetLastError();
}

cudaError_t dem_unsort_async(const float4* src, const float4* omg, float4* dst, uint32_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    dem_unsort_kernel<<<grid_for(n, 256), 256, 0, st>>>(src, omg, dst, n);
    return cudaGetLastError();
}

cudaError_t dem_slot_of_all_async(const float4* omg, uint32_t* slot_of, uint32_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    dem_slot_of_id_kernel<<<grid_for(n, 256), 256, 0, st>>>(omg, slot_of, n);
    return cudaGetLastError();
}

cudaError_t dem_host_in_async(const float4* host_src, const float4* omg, float4* dst, uint32_t* slot_of_id,
                              uint32_t n, bool keep_w, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    dem_slot_of_id_kernel<<<grid_for(n, 256), 256, 0, st>>>(omg, slot_of_id, n);
    dem_by_id_in_kernel<<<grid_for(n, 256), 256, 0, st>>>(host_src, slot_of_id, dst, n, keep_w);
    return cudaGetLastError();
}

cudaError_t dem_host_out_async(const float4* src, const float4* omg, float4* host_dst, uint32_t* slot_of_id,
                               uint32_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    dem_slot_of_id_kernel<<<grid_for(n, 256), 256, 0, st>>>(omg, slot_of_id, n);
    dem_by_id_out_kernel<<<grid_for(n, 256), 256, 0, st>>>(src, slot_of_id, host_dst, n);
    return cudaGetLastError();
}

cudaError_t dem_scatter_in_async(const float4* src_by_id, const float4* omg, float4* dst, uint32_t n, bool keep_w,
                                 cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    dem_scatter_in_kernel<<<grid_for(n, 256), 256, 0, st>>>(src_by_id, omg, dst, n, keep_w);
    return cudaGetLastError();
}

cudaError_t dem_energy_async(const DemBuffers& b, double* d_out, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(d_out, 0, 4 * sizeof(double), st);
    if (e != cudaSuccess || b.n == 0) return e;
    unsigned g = grid_for(b.n, 256);
    if (g > 152 * 4) g = 152 * 4;
    dem_energy_kernel<<<g, 256, 0, st>>>(b.n, b.pos, b.vel, b.omg, d_out);
    return cudaGetLastError();
}

}  // namespace sd
