// sd_hull.cu -- convex-hull rigid bodies: world AABBs, GJK/EPA narrow
// phase with atomic-free force reduction, quaternion integration.
//
// Narrow phase: sandbox/testGJK.cu:52-315 (support mapping of a vertex soup,
// Minkowski difference B - A, simplex cases, termination dot(w, d) < 0,
// at most 64 support evaluations) in the standard GJK formulation
// (Gilbert, Johnson, Keerthi 1988) with the full line/triangle/tetrahedron
// case analysis; EPA (van den Bergen 2001) for the penetration depth,
// normal and witness points, which the reference lacks.
//
// Work split: one thread per candidate ENTRY (self, other) of the per-body
// partner lists built by the LBVH; each entry evaluates its pair as
// (A, B) = (min, max), so the two entries of a pair compute identical
// numbers and take opposite signs -- exact action = reaction with no
// atomics.  One thread per body then sums its entries in list order (the
// segmented reduction), adds walls and gravity and integrates.
//
// Every float operation follows oracle/sd_oracle_hull.c in order
// (-fmad=false), so results are bit-identical to the CPU restatement.
#include "sd_common.cuh"

namespace sd {

namespace {

constexpr int kHullThreads = 128;
constexpr int kEpaWarps = 4;  // warps per block of the EPA kernel
constexpr int kGjkMaxIt = 64;
// support evaluations a seeded GJK run gets to certify separation before the
// plain run takes over
constexpr int kSeedMaxIt = 2;
constexpr int kEpaMaxV = 48;
constexpr int kEpaMaxF = 96;
constexpr int kEpaMaxIt = 48;
enum : int { kSep = 0, kHit = 1, kTouch = 2, kNoConv = 3 };

struct v3 {
    float x, y, z;
};
__device__ __forceinline__ v3 mk(float x, float y, float z) { return v3{x, y, z}; }
__device__ __forceinline__ v3 vadd(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ v3 vsub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ v3 vneg(v3 a) { return mk(-a.x, -a.y, -a.z); }
__device__ __forceinline__ v3 vscale(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float vdot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ v3 vcross(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ bool vzero(v3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
__device__ __forceinline__ v3 f3(float4 a) { return mk(a.x, a.y, a.z); }

struct Mat {
    float r[9];
};

__device__ __forceinline__ Mat qrot(float4 q) {
    const float qs = q.x, qx = q.y, qy = q.z, qz = q.w;
    Mat R;
    R.r[0] = 1.0f - 2.0f * (qy * qy + qz * qz);
    R.r[1] = 2.0f * (qx * qy - qs * qz);
    R.r[2] = 2.0f * (qx * qz + qs * qy);
    R.r[3] = 2.0f * (qx * qy + qs * qz);
    R.r[4] = 1.0f - 2.0f * (qx * qx + qz * qz);
    R.r[5] = 2.0f * (qy * qz - qs * qx);
    R.r[6] = 2.0f * (qx * qz - qs * qy);
    R.r[7] = 2.0f * (qy * qz + qs * qx);
    R.r[8] = 1.0f - 2.0f * (qx * qx + qy * qy);
    return R;
}
__device__ __forceinline__ v3 rot(const Mat& R, v3 v) {
    return mk((R.r[0] * v.x + R.r[1] * v.y) + R.r[2] * v.z, (R.r[3] * v.x + R.r[4] * v.y) + R.r[5] * v.z,
              (R.r[6] * v.x + R.r[7] * v.y) + R.r[8] * v.z);
}
__device__ __forceinline__ v3 rotT(const Mat& R, v3 d) {
    return mk((R.r[0] * d.x + R.r[3] * d.y) + R.r[6] * d.z, (R.r[1] * d.x + R.r[4] * d.y) + R.r[7] * d.z,
              (R.r[2] * d.x + R.r[5] * d.y) + R.r[8] * d.z);
}

struct HBody {
    Mat R;
    const float4* V;
    uint32_t nv;
};

struct Cso {
    v3 w, a, b;
    uint32_t key;
};

struct HPair {
    HBody A, B;
    v3 off;  // x_B - x_A
};

__device__ __forceinline__ uint32_t support(const HBody& h, v3 d, v3* out) {
    const v3 db = rotT(h.R, d);
    uint32_t best = 0;
    float bd = vdot(db, f3(__ldg(h.V)));
    for (uint32_t k = 1; k < h.nv; ++k) {
        const float t = vdot(db, f3(__ldg(h.V + k)));
        if (t > bd) {
            bd = t;
            best = k;
        }
    }
    *out = rot(h.R, f3(__ldg(h.V + best)));
    return best;
}

__device__ __forceinline__ Cso cso(const HPair& P, v3 d) {
    Cso r;
    const uint32_t ia = support(P.A, vneg(d), &r.a);
    v3 bb;
    const uint32_t ib = support(P.B, d, &bb);
    r.b = vadd(bb, P.off);
    r.w = vsub(r.b, r.a);
    r.key = ia * 1024u + ib;
    return r;
}

struct Simplex {
    Cso s[4];
    int n;
    v3 d;
    float pad;  // 45 words: one thread's simplex per bank offset when kept in shared memory
};

// A support key (ia * 1024 + ib, both indices below 256) in 16 bits.
__device__ __forceinline__ uint16_t key16(uint32_t key) { return (uint16_t)(((key >> 10) << 8) | (key & 1023u)); }

/* Closest point to the origin of the simplex S->s[0..n) (Ericson, Real-Time
 * Collision Detection, 5.1.2, 5.1.5, 5.1.6: Voronoi-region tests of the
 * segment, triangle and tetrahedron).  Reduces the simplex to the vertices of
 * the closest feature (kept in their order) and returns the point in *v; for
 * a tetrahedron that contains the origin returns 1 and leaves S whole. */
__device__ void closest_tri(const Cso* A, const Cso* B, const Cso* C, v3* v, int* mask) {
    const v3 ab = vsub(B->w, A->w), ac = vsub(C->w, A->w), ap = vneg(A->w);
    const float d1 = vdot(ab, ap), d2 = vdot(ac, ap);
    if (d1 <= 0.0f && d2 <= 0.0f) { *v = A->w; *mask = 1; return; }
    const v3 bp = vneg(B->w);
    const float d3 = vdot(ab, bp), d4 = vdot(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) { *v = B->w; *mask = 2; return; }
    const float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
        const float t = d1 / (d1 - d3);
        *v = vadd(A->w, vscale(ab, t));
        *mask = 3;
        return;
    }
    const v3 cp = vneg(C->w);
    const float d5 = vdot(ab, cp), d6 = vdot(ac, cp);
    if (d6 >= 0.0f && d5 <= d6) { *v = C->w; *mask = 4; return; }
    const float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
        const float t = d2 / (d2 - d6);
        *v = vadd(A->w, vscale(ac, t));
        *mask = 5;
        return;
    }
    const float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
        const float t = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        *v = vadd(B->w, vscale(vsub(C->w, B->w), t));
        *mask = 6;
        return;
    }
    const float den = 1.0f / ((va + vb) + vc);
    const float s = vb * den, t = vc * den;
    *v = vadd(vadd(A->w, vscale(ab, s)), vscale(ac, t));
    *mask = 7;
}

__device__ void keep(Simplex* S, const int* idx, int m) {
    Cso t[4];
    for (int k = 0; k < m; ++k) t[k] = S->s[idx[k]];
    for (int k = 0; k < m; ++k) S->s[k] = t[k];
    S->n = m;
}

__device__ void keep_mask(Simplex* S, const int* tri, int mask) {
    int idx[3], m = 0;
    for (int k = 0; k < 3; ++k)
        if (mask & (1 << k)) idx[m++] = tri[k];
    keep(S, idx, m);
}

__device__ int closest_simplex(Simplex* S, v3* v) {
    if (S->n == 1) {
        *v = S->s[0].w;
        return 0;
    }
    if (S->n == 2) {
        const v3 A = S->s[0].w, ab = vsub(S->s[1].w, A);
        const float t = vdot(vneg(A), ab);
        if (t <= 0.0f) {
            S->n = 1;
            *v = A;
            return 0;
        }
        const float den = vdot(ab, ab);
        if (t >= den) {
            S->s[0] = S->s[1];
            S->n = 1;
            *v = S->s[0].w;
            return 0;
        }
        *v = vadd(A, vscale(ab, t / den));
        return 0;
    }
    if (S->n == 3) {
        const int tri[3] = {0, 1, 2};
        int mask;
        closest_tri(&S->s[0], &S->s[1], &S->s[2], v, &mask);
        keep_mask(S, tri, mask);
        return 0;
    }
    /* tetrahedron: faces with the opposite vertex */
    const int face[4][4] = {{0, 1, 2, 3}, {0, 2, 3, 1}, {0, 3, 1, 2}, {1, 3, 2, 0}};
    int best = -1, best_mask = 0;
    float best_d = 0.0f;
    v3 best_v = mk(0.0f, 0.0f, 0.0f);
    for (int f = 0; f < 4; ++f) {
        const v3 p = S->s[face[f][0]].w, q = S->s[face[f][1]].w, r = S->s[face[f][2]].w, o = S->s[face[f][3]].w;
        const v3 nrm = vcross(vsub(q, p), vsub(r, p));
        const float sp = vdot(vneg(p), nrm), so = vdot(vsub(o, p), nrm);
        const bool outside = (sp > 0.0f && so < 0.0f) || (sp < 0.0f && so > 0.0f) || so == 0.0f;
        if (!outside) continue;
        v3 cv;
        int mask;
        closest_tri(&S->s[face[f][0]], &S->s[face[f][1]], &S->s[face[f][2]], &cv, &mask);
        const float dd = vdot(cv, cv);
        if (best < 0 || dd < best_d) {
            best = f;
            best_d = dd;
            best_v = cv;
            best_mask = mask;
        }
    }
    if (best < 0) return 1;
    keep_mask(S, face[best], best_mask);
    *v = best_v;
    return 0;
}

/* GJK (distance form) on B - A from a seed direction d0: v is the closest
 * point of the current simplex to the origin, the next support is taken in
 * -v, and the reference's test dot(w, d) < 0 ends it as separated; a
 * support point seen before in the run ends it as touching (no further
 * progress is possible: the origin is on the boundary of B - A within
 * rounding); a simplex that encloses the origin ends it as a hit; a zero
 * |v| as touching; max_it supports without an end as not converged.
 *
 * Run over a sequence of attempts: attempt a starts from d0[a] and may take
 * max_it[a] supports; the first attempt that certifies separation, or the
 * last attempt, decides.  Each attempt is a whole GJK run from its seed
 * (its own simplex and seen supports), but all attempts run in one loop
 * with one support call per pass, so the threads of a warp in different
 * attempts still share that call.  Returns the status; *iters =
 * supports over all attempts run, *which = the deciding attempt, *dir and
 * *S of the deciding attempt. */
struct GjkAttempts {
    v3 d0[3];
    int max_it[3];
    int n;
    // selects, not indexing, so that the attempts stay in registers
    __device__ __forceinline__ v3 seed(int a) const { return a == 0 ? d0[0] : (a == 1 ? d0[1] : d0[2]); }
    __device__ __forceinline__ int limit(int a) const {
        return a == 0 ? max_it[0] : (a == 1 ? max_it[1] : max_it[2]);
    }
};

__device__ int gjk_attempts(const HPair& P, const GjkAttempts& at, Simplex* S, int* iters, v3* dir, int* which,
                            uint16_t* seen, uint32_t seen_stride) {
    int a = 0, it = 0, total = 0;
    bool first = true;
    v3 v = mk(0.f, 0.f, 0.f);
    float vv = 0.0f;
    for (;;) {
        v3 d;
        if (first) {
            d = at.seed(a);
            if (vzero(d)) d = mk(1.0f, 0.0f, 0.0f);
            it = 0;
        } else {
            d = vneg(v);
        }
        *dir = d;
        const Cso p = cso(P, d);
        ++it;
        int st = -1;
        if (vdot(p.w, d) < 0.0f) {
            st = kSep;
        } else if (first) {
            S->s[0] = p;
            S->n = 1;
            seen[0] = key16(p.key);
            v = p.w;
            vv = vdot(v, v);
            first = false;
        } else {
            for (int k = 0; k < it - 1; ++k)
                if (seen[(size_t)k * seen_stride] == key16(p.key)) st = kTouch;
            if (st < 0) {
                seen[(size_t)(it - 1) * seen_stride] = key16(p.key);
                for (int k = S->n; k > 0; --k) S->s[k] = S->s[k - 1];
                S->s[0] = p;
                S->n += 1;
                if (closest_simplex(S, &v)) st = kHit;
                else vv = vdot(v, v);
            }
        }
        if (st < 0) {  // the tests made before the next support
            if (vv == 0.0f) st = kTouch;
            else if (it >= at.limit(a)) st = kNoConv;
        }
        if (st >= 0) {
            total += it;
            if (st == kSep || a + 1 >= at.n) {
                *iters = total;
                *which = a;
                return st;
            }
            ++a;
            first = true;
        }
    }
}

/* The separating direction of largest margin, for training the warm-start
 * network: distance-form GJK run to convergence (|v|^2 - v.w <= 1e-5 |v|^2,
 * at most kGjkMaxIt supports) from d0; returns false when the pair is not
 * cleanly separated.  *out = -v / |v|, the direction of the closest points. */
__device__ bool gjk_margin_dir(const HPair& P, v3 d0, v3* out) {
    Simplex S;
    v3 d = vzero(d0) ? mk(1.0f, 0.0f, 0.0f) : d0;
    Cso p = cso(P, d);
    S.s[0] = p;
    S.n = 1;
    v3 v = p.w;
    for (int it = 1; it < kGjkMaxIt; ++it) {
        const float vv = vdot(v, v);
        if (!(vv > 0.0f)) return false;
        d = vneg(v);
        p = cso(P, d);
        if (vv - vdot(v, p.w) <= 1e-5f * vv) break;  // converged: v is (nearly) the closest point
        if (S.n >= 4) return false;  // (closest_simplex keeps at most 3 points unless it reports a hit)
        for (int k = S.n; k > 0; --k) S.s[k] = S.s[k - 1];
        S.s[0] = p;
        S.n += 1;
        if (closest_simplex(&S, &v)) return false;
    }
    const float vv = vdot(v, v);
    if (!(vv > 0.0f)) return false;
    const float inv = 1.0f / sqrtf(vv);
    *out = mk(-v.x * inv, -v.y * inv, -v.z * inv);
    return true;
}

struct Face {
    uint8_t i[3];
    v3 n;
    float dist;
};

__device__ __forceinline__ bool face_make(const Cso* V, uint8_t a, uint8_t b, uint8_t c, Face* f) {
    const v3 nn = vcross(vsub(V[b].w, V[a].w), vsub(V[c].w, V[a].w));
    const float len = sqrtf(vdot(nn, nn));
    if (!(len > 0.0f)) return false;
    f->i[0] = a;
    f->i[1] = b;
    f->i[2] = c;
    f->n = mk(nn.x / len, nn.y / len, nn.z / len);
    f->dist = vdot(f->n, V[a].w);
    return true;
}

struct Contact {
    float depth;
    v3 n, c;
    int epa_iters;
    bool ok;
};

// ---------------------------------------------------------------- EPA
// One warp per intersecting pair; the polytope lives in shared memory.  The
// warp splits the scans (faces, vertices of the support calls, duplicate
// keys, face visibility, new faces) and keeps the sequential algorithm's
// choices exactly: the first face of least distance, the first vertex of
// largest dot product, kept faces and new faces in list order; lane 0 alone
// builds the horizon edge list (its order decides the new faces' order).

constexpr uint32_t kFull = 0xffffffffu;

struct EpaShared {
    Cso V[kEpaMaxV];
    Face F[kEpaMaxF];
    uint8_t E[3 * kEpaMaxF][2];
};

// support() by a warp: the first vertex (lowest index) of largest dot
// product, as the sequential scan's strict '>' from vertex 0 picks (a NaN
// product never wins, and a NaN at vertex 0 keeps vertex 0).
__device__ __forceinline__ uint32_t support_warp(const HBody& h, v3 d, v3* out) {
    const uint32_t lane = threadIdx.x & 31;
    const v3 db = rotT(h.R, d);
    float bd = 0.0f;
    uint32_t best = 0xffffffffu;
    for (uint32_t k = lane; k < h.nv; k += 32) {
        const float t = vdot(db, f3(__ldg(h.V + k)));
        if (t != t) continue;
        if (best == 0xffffffffu || t > bd) {
            bd = t;
            best = k;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float ob = __shfl_xor_sync(kFull, bd, o);
        const uint32_t oi = __shfl_xor_sync(kFull, best, o);
        if (oi != 0xffffffffu && (best == 0xffffffffu || ob > bd || (ob == bd && oi < best))) {
            bd = ob;
            best = oi;
        }
    }
    const float t0 = vdot(db, f3(__ldg(h.V)));
    if (t0 != t0 || best == 0xffffffffu) best = 0;
    *out = rot(h.R, f3(__ldg(h.V + best)));
    return best;
}

__device__ __forceinline__ Cso cso_warp(const HPair& P, v3 d) {
    Cso r;
    const uint32_t ia = support_warp(P.A, vneg(d), &r.a);
    v3 bb;
    const uint32_t ib = support_warp(P.B, d, &bb);
    r.b = vadd(bb, P.off);
    r.w = vsub(r.b, r.a);
    r.key = ia * 1024u + ib;
    return r;
}

// The support point a key names (key = ia * 1024 + ib): the same arithmetic
// as cso(), so the same bits.
__device__ __forceinline__ Cso cso_of_key(const HPair& P, uint32_t key) {
    Cso r;
    r.a = rot(P.A.R, f3(__ldg(P.A.V + (key >> 10))));
    const v3 bb = rot(P.B.R, f3(__ldg(P.B.V + (key & 1023u))));
    r.b = vadd(bb, P.off);
    r.w = vsub(r.b, r.a);
    r.key = key;
    return r;
}

// The sequential "best = 0; if (F[k].dist < F[best].dist) best = k" by a
// warp: the first face of least distance (NaN never wins; NaN at face 0
// keeps face 0).
__device__ __forceinline__ int closest_face_warp(const Face* F, int nf) {
    const int lane = threadIdx.x & 31;
    float bd = 0.0f;
    int best = -1;
    for (int k = lane; k < nf; k += 32) {
        const float t = F[k].dist;
        if (t != t) continue;
        if (best < 0 || t < bd) {
            bd = t;
            best = k;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float ob = __shfl_xor_sync(kFull, bd, o);
        const int oi = __shfl_xor_sync(kFull, best, o);
        if (oi >= 0 && (best < 0 || ob < bd || (ob == bd && oi < best))) {
            bd = ob;
            best = oi;
        }
    }
    const float d0 = F[0].dist;
    return (d0 != d0 || best < 0) ? 0 : best;
}

/* EPA from GJK's enclosing tetrahedron s[0..3] (every lane holds it):
 * expands the polytope of B - A towards the origin's closest face until the
 * support gains at most tol (or repeats a vertex, or a capacity is reached);
 * the contact is that face's plane (normal -n, depth) and the midpoint of
 * the witness points at the origin's projection.  Every lane returns the
 * same *out. */
__device__ void epa_warp(const HPair& P, const Cso* s, float tol, EpaShared& sh, Contact* out) {
    const int lane = threadIdx.x & 31;
    const uint32_t lt = (1u << lane) - 1u;
    int nv = 4, nf = 0;
    __syncwarp();  // the previous pair's reads of the polytope are done
    if (lane < 4) sh.V[lane] = s[lane];
    __syncwarp();
    const uint8_t init[4][3] = {{0, 1, 2}, {0, 2, 3}, {0, 3, 1}, {1, 3, 2}};
    for (int k = 0; k < 4; ++k) {
        Face f;
        if (!face_make(sh.V, init[k][0], init[k][1], init[k][2], &f)) continue;
        if (f.dist < 0.0f) {
            const uint8_t t = f.i[1];
            f.i[1] = f.i[2];
            f.i[2] = t;
            f.n = vneg(f.n);
            f.dist = -f.dist;
        }
        if (lane == 0) sh.F[nf] = f;
        ++nf;
    }
    out->ok = false;
    out->epa_iters = 0;
    __syncwarp();
    if (nf == 0) return;
    int best = 0;
    for (int it = 0;; ++it) {
        best = closest_face_warp(sh.F, nf);
        out->epa_iters = it + 1;
        if (it >= kEpaMaxIt || nv >= kEpaMaxV) break;
        const Face fb = sh.F[best];
        const Cso p = cso_warp(P, fb.n);
        bool dup = false;
        for (int k = lane; k < nv; k += 32) dup |= sh.V[k].key == p.key;
        if (__any_sync(kFull, dup) || vdot(p.w, fb.n) - fb.dist <= tol) break;
        const uint8_t q = (uint8_t)nv;
        // faces that see p (before any face moves)
        uint32_t vis[(kEpaMaxF + 31) / 32];
        for (int c = 0; c < (kEpaMaxF + 31) / 32; ++c) {
            const int k = 32 * c + lane;
            bool v = false;
            if (k < nf) v = vdot(sh.F[k].n, vsub(p.w, sh.V[sh.F[k].i[0]].w)) > 0.0f;
            vis[c] = __ballot_sync(kFull, v);
        }
        __syncwarp();
        if (lane == 0) sh.V[nv] = p;
        ++nv;
        // horizon: edges of the visible faces in face order, an edge met
        // again reversed cancels (the last edge moves into its place)
        int ne = 0;
        if (lane == 0) {
            for (int k = 0; k < nf; ++k) {
                if (!((vis[k >> 5] >> (k & 31)) & 1u)) continue;
                for (int e = 0; e < 3; ++e) {
                    const uint8_t a = sh.F[k].i[e], b = sh.F[k].i[(e + 1) % 3];
                    int found = -1;
                    for (int m = 0; m < ne; ++m)
                        if (sh.E[m][0] == b && sh.E[m][1] == a) {
                            found = m;
                            break;
                        }
                    if (found >= 0) {
                        sh.E[found][0] = sh.E[ne - 1][0];
                        sh.E[found][1] = sh.E[ne - 1][1];
                        --ne;
                    } else {
                        sh.E[ne][0] = a;
                        sh.E[ne][1] = b;
                        ++ne;
                    }
                }
            }
        }
        ne = __shfl_sync(kFull, ne, 0);
        __syncwarp();
        // the faces that do not see p, compacted in order (a face moves to
        // an index at or below its own: read a chunk, then write it)
        int keep = 0;
        for (int c = 0; 32 * c < nf; ++c) {
            const int k = 32 * c + lane;
            const bool kept = k < nf && !((vis[c] >> lane) & 1u);
            Face f;
            if (kept) f = sh.F[k];
            const uint32_t m = __ballot_sync(kFull, kept);
            __syncwarp();
            if (kept) sh.F[keep + __popc(m & lt)] = f;
            keep += __popc(m);
            __syncwarp();
        }
        nf = keep;
        if (nf + ne > kEpaMaxF) break;
        // new faces (edge, p) in edge order; degenerate ones are dropped
        for (int c = 0; 32 * c < ne; ++c) {
            const int m = 32 * c + lane;
            Face f;
            const bool ok = m < ne && face_make(sh.V, sh.E[m][0], sh.E[m][1], q, &f);
            const uint32_t mk_ = __ballot_sync(kFull, ok);
            if (ok) sh.F[nf + __popc(mk_ & lt)] = f;
            nf += __popc(mk_);
        }
        __syncwarp();
        if (nf == 0) return;
    }
    Cso t[3] = {sh.V[sh.F[best].i[0]], sh.V[sh.F[best].i[1]], sh.V[sh.F[best].i[2]]};
    __syncwarp();  // the polytope is read: the next pair may overwrite it
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2 - a; ++b)
            if (t[b].key > t[b + 1].key) {
                const Cso s2 = t[b];
                t[b] = t[b + 1];
                t[b + 1] = s2;
            }
    const v3 e0 = vsub(t[1].w, t[0].w), e1 = vsub(t[2].w, t[0].w);
    const v3 nn = vcross(e0, e1);
    const float len = sqrtf(vdot(nn, nn));
    if (!(len > 0.0f)) return;
    v3 n = mk(nn.x / len, nn.y / len, nn.z / len);
    float depth = vdot(n, t[0].w);
    if (depth < 0.0f) {
        n = vneg(n);
        depth = -depth;
    }
    const v3 pp = vscale(n, depth);
    const v3 e2 = vsub(pp, t[0].w);
    const float d00 = vdot(e0, e0), d01 = vdot(e0, e1), d11 = vdot(e1, e1);
    const float d20 = vdot(e2, e0), d21 = vdot(e2, e1);
    const float den = d00 * d11 - d01 * d01;
    float l1 = 0.0f, l2 = 0.0f;
    if (den != 0.0f) {
        l1 = (d11 * d20 - d01 * d21) / den;
        l2 = (d00 * d21 - d01 * d20) / den;
    }
    const float l0 = (1.0f - l1) - l2;
    const v3 a = vadd(vadd(vscale(t[0].a, l0), vscale(t[1].a, l1)), vscale(t[2].a, l2));
    const v3 b = vadd(vadd(vscale(t[0].b, l0), vscale(t[1].b, l1)), vscale(t[2].b, l2));
    out->depth = depth;
    out->n = vneg(n);
    out->c = vscale(vadd(a, b), 0.5f);
    out->ok = true;
}

__device__ __forceinline__ void make_pair(const HullBuffers& H, uint32_t A, uint32_t B, HPair* P) {
    P->A.R = qrot(H.quat[A]);
    P->B.R = qrot(H.quat[B]);
    P->A.V = H.verts + H.vstart[A];
    P->A.nv = H.vcount[A];
    P->B.V = H.verts + H.vstart[B];
    P->B.nv = H.vcount[B];
    P->off = vsub(f3(H.pos[B]), f3(H.pos[A]));
}

__device__ __forceinline__ v3 contact_force(const HullParams& p, float delta, v3 m, v3 vr, float meff) {
    const float vn = vdot(vr, m);
    const float gn = p.damp * sqrtf(meff);
    const float fn = p.kn * delta - gn * vn;
    const float fc = fn > 0.0f ? fn : 0.0f;
    const v3 vt = mk(vr.x - vn * m.x, vr.y - vn * m.y, vr.z - vn * m.z);
    const float vt2 = vdot(vt, vt);
    v3 f = mk(fn * m.x, fn * m.y, fn * m.z);
    if (vt2 > 0.0f) {
        const float vtm = sqrtf(vt2);
        const float ftm = fminf(p.mu * fc, gn * vtm);
        const float s = ftm / vtm;
        f.x += -(s * vt.x);
        f.y += -(s * vt.y);
        f.z += -(s * vt.z);
    }
    return f;
}

// ------------------------------------------------------------- kernels

__global__ void hull_aabb_kernel(HullBuffers H) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= H.nb) return;
    const Mat R = qrot(H.quat[b]);
    const float4* V = H.verts + H.vstart[b];
    const uint32_t nv = H.vcount[b];
    v3 w = rot(R, f3(V[0]));
    float mn[3] = {w.x, w.y, w.z}, mx[3] = {w.x, w.y, w.z};
    uint32_t imn[3] = {0, 0, 0}, imx[3] = {0, 0, 0};
    for (uint32_t k = 1; k < nv; ++k) {
        w = rot(R, f3(V[k]));
        const float c[3] = {w.x, w.y, w.z};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (c[a] < mn[a]) {
                mn[a] = c[a];
                imn[a] = k;
            }
            if (c[a] > mx[a]) {
                mx[a] = c[a];
                imx[a] = k;
            }
        }
    }
    const float4 x = H.pos[b];
    H.lo[b] = make_float4(x.x + mn[0], x.y + mn[1], x.z + mn[2], 0.f);
    H.hi[b] = make_float4(x.x + mx[0], x.y + mx[1], x.z + mx[2], 0.f);
    H.ext[2 * b] = imn[0] | (imn[1] << 8) | (imn[2] << 16);
    H.ext[2 * b + 1] = imx[0] | (imx[1] << 8) | (imx[2] << 16);
}

// Seeds from the previous step's final directions (seed mode 2): the pair's
// entry in the previous partner list of A (binary search) carries the
// direction in A's body frame.  feat (may be null) receives the 12 MLP
// inputs and w of seeds the previous-contact flag.
__global__ void hull_prev_seed_kernel(HullBuffers H, uint32_t mode) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= H.cap) return;
    const uint32_t total = H.off[H.nb];
    if (e >= total || (uint64_t)total > H.cap) return;  // an overflowed step is reported, not evaluated
    const uint32_t self = H.self[e], other = H.partners[e];
    const uint32_t A = min(self, other), B = max(self, other);
    // previous entry of (A, B); a previous list that overflowed is ignored
    float4 prev = make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t lo = H.prev_off[A];
    const uint32_t end = (uint64_t)H.prev_off[H.nb] > H.cap ? lo : H.prev_off[A + 1];
    uint32_t hi = end;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        const uint32_t v = H.prev_partners[mid];
        if (v < B) lo = mid + 1;
        else hi = mid;
    }
    const bool found = lo < end && H.prev_partners[lo] == B;
    if (found) prev = H.prev_dir[lo];
    const bool have = found && prev.w != 0.0f;
    // mode 2 seeds from the previous direction; mode 1's seeds are written by
    // the network afterwards; mode 0 runs plain GJK (the inputs are still
    // recorded, for training)
    H.seeds[e] = (mode == 2u && have) ? make_float4(prev.x, prev.y, prev.z, 1.0f) : make_float4(0.f, 0.f, 0.f, 0.f);
    if (H.feat) {
        // 12 inputs in A's body frame: relative quaternion conj(qA) (x) qB,
        // centre offset / (rhoA + rhoB), previous-contact flag, previous
        // direction (unit), |offset| / (rhoA + rhoB)
        const float4 qa = H.quat[A], qb = H.quat[B];
        const float as = qa.x, ax = -qa.y, ay = -qa.z, az = -qa.w;
        const float rs = as * qb.x - ((ax * qb.y + ay * qb.z) + az * qb.w);
        const float rx = as * qb.y + qb.x * ax + (ay * qb.w - az * qb.z);
        const float ry = as * qb.z + qb.x * ay + (az * qb.y - ax * qb.w);
        const float rz = as * qb.w + qb.x * az + (ax * qb.z - ay * qb.y);
        const Mat R = qrot(qa);
        const float scale = 1.0f / (H.iinv[A].w + H.iinv[B].w);
        const v3 o = vscale(rotT(R, vsub(f3(H.pos[B]), f3(H.pos[A]))), scale);
        float* f = H.feat + 16 * (size_t)e;
        f[0] = rs; f[1] = rx; f[2] = ry; f[3] = rz;
        f[4] = o.x; f[5] = o.y; f[6] = o.z;
        f[7] = have ? 1.0f : 0.0f;
        const float pn = sqrtf((prev.x * prev.x + prev.y * prev.y) + prev.z * prev.z);
        const float pi = (have && pn > 0.0f) ? 1.0f / pn : 0.0f;
        f[8] = prev.x * pi; f[9] = prev.y * pi; f[10] = prev.z * pi;
        f[11] = sqrtf(vdot(o, o));
        f[12] = 0.0f; f[13] = 0.0f; f[14] = 0.0f; f[15] = 0.0f;
    }
}

// Unique pairs: per body the number of its entries with a larger partner,
// then the list of those entries (body order, partner order).
__global__ void hull_unique_count_kernel(HullBuffers H) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= H.nb) return;
    uint32_t c = 0;
    if ((uint64_t)H.off[H.nb] <= H.cap)
        for (uint32_t e = H.off[b]; e < H.off[b + 1]; ++e) c += H.partners[e] > b;
    H.ucount[b] = c;
}

__global__ void hull_unique_fill_kernel(HullBuffers H) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= H.nb || (uint64_t)H.off[H.nb] > H.cap) return;
    uint32_t w = H.upos[b];
    for (uint32_t e = H.off[b]; e < H.off[b + 1]; ++e)
        if (H.partners[e] > b) H.ulist[w++] = e;
}

// The mirror entry (B, A) of the unique entry e = (A, B): binary search in
// B's ascending partner list.
__device__ __forceinline__ uint32_t mirror_entry(const HullBuffers& H, uint32_t A, uint32_t B) {
    uint32_t lo = H.off[B], hi = H.off[B + 1];
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (H.partners[mid] < A) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Narrow phase, part 1, one thread per unique pair (A, B), A < B, from its
// entry in A's list: GJK (seeded or plain).  A separated or touching pair is
// finished here -- its entry and its mirror in B's list get the status, the
// direction and zero force; a pair GJK found intersecting goes to the hit
// list for hull_epa_kernel.  Split so that GJK, which every pair runs, does
// not carry EPA's registers and polytope (the hits are a few per cent).
// MINB: resident blocks per SM it is compiled for (knob "hull_blocks").
template <int MINB>
__global__ void __launch_bounds__(kHullThreads, MINB) hull_gjk_kernel(HullBuffers H) {
    const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t total = H.off[H.nb];
    if ((uint64_t)total > H.cap || u >= H.upos[H.nb]) return;  // an overflowed step is reported, not evaluated
    const uint32_t e = H.ulist[u];
    const uint32_t A = H.self[e], B = H.partners[e];
    const uint32_t em = mirror_entry(H, A, B);
    HPair P;
    make_pair(H, A, B, &P);
    v3 d0 = vneg(P.off);
    const float4 sd = H.seeds ? H.seeds[e] : make_float4(0.f, 0.f, 0.f, 0.f);
    const bool seeded = sd.w == 1.0f;
    if (seeded) d0 = rot(P.A.R, f3(sd));
    // the simplex and the supports seen, per thread in shared memory (in
    // local memory they missed L1 at this occupancy)
    __shared__ Simplex s_simplex[kHullThreads];
    __shared__ uint16_t s_seen[kGjkMaxIt * kHullThreads];
    Simplex& S = s_simplex[threadIdx.x];
    int iters = 0;
    v3 dir;
    // a seeded run gets kSeedMaxIt support evaluations to certify separation;
    // only that certificate is taken from it -- any other outcome is the
    // plain run's, so contact sets, forces and states do not depend on seeds.
    // Learned seeds (keep_anchor): the pair's anchor direction (its last
    // certificate, inputs 8..10) is tried first with one support, and the
    // network's direction -- trained on the pairs whose anchor failed -- with
    // one more only when the anchor fails.
    const bool learned = seeded && H.keep_anchor && H.feat;
    // the plain run decides whenever no seed certifies
    GjkAttempts at;
    if (learned) {
        at = {{rot(P.A.R, mk(H.feat[16 * (size_t)e + 8], H.feat[16 * (size_t)e + 9], H.feat[16 * (size_t)e + 10])),
               d0, vneg(P.off)},
              {1, 1, kGjkMaxIt},
              3};
    } else if (seeded) {
        at = {{d0, vneg(P.off), vneg(P.off)}, {kSeedMaxIt, kGjkMaxIt, kGjkMaxIt}, 2};
    } else {
        at = {{vneg(P.off), vneg(P.off), vneg(P.off)}, {kGjkMaxIt, kGjkMaxIt, kGjkMaxIt}, 1};
    }
    int which = 0;
    const int st = gjk_attempts(P, at, &S, &iters, &dir, &which, s_seen + threadIdx.x, kHullThreads);
    const bool certified_by_anchor = learned && which == 0;
    const bool anchor_failed = learned && which > 0;
    // final direction in A's frame (seed of the next step); with learned
    // seeds a seed's certificate keeps the anchor it was predicted from
    const v3 dA = certified_by_anchor
                      ? mk(H.feat[16 * (size_t)e + 8], H.feat[16 * (size_t)e + 9], H.feat[16 * (size_t)e + 10])
                      : rotT(P.A.R, dir);
    const float4 d4 = make_float4(dA.x, dA.y, dA.z, st == kSep ? 1.0f : 0.0f);
    const bool mirror = em < H.off[B + 1];  // always true for consistent lists
    H.dir[e] = d4;
    if (mirror) H.dir[em] = d4;
    if (H.teach && *H.teach_on) {
        // a training step: the max-margin direction of a separated pair
        // whose anchor failed (the cases the network's seed is tried on)
        v3 m;
        const bool ok = st == kSep && anchor_failed && gjk_margin_dir(P, dir, &m);
        const v3 mA = rotT(P.A.R, m);
        H.teach[e] = ok ? make_float4(mA.x, mA.y, mA.z, 1.0f) : make_float4(0.f, 0.f, 0.f, 0.f);
        if (mirror) H.teach[em] = make_float4(0.f, 0.f, 0.f, 0.f);  // one sample per pair
    }
    if (st == kHit) {  // EPA and the contact force in hull_epa_kernel
        const uint32_t k = atomicAdd(H.hit_count, 1u);  // k < unique pairs <= cap / 2 + 1
        H.hits[k] = make_uint2(u, (uint32_t)iters);
        H.hit_keys[k] = make_uint4(S.s[0].key, S.s[1].key, S.s[2].key, S.s[3].key);
        return;
    }
    const uint32_t info = (uint32_t)st | ((uint32_t)iters << 8);
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    H.ef[e] = z;
    H.et[e] = z;
    H.info[e] = info;
    if (mirror) {
        H.ef[em] = z;
        H.et[em] = z;
        H.info[em] = info;
    }
}

// Narrow phase, part 2, one warp per pair GJK found intersecting: EPA from
// GJK's enclosing tetrahedron (rebuilt from its support keys), the contact
// force at the EPA point; A's entry and B's mirror get forces of opposite
// sign -- exact action = reaction, no atomics.  Warps stride over the hit
// count.
__global__ void __launch_bounds__(kEpaWarps * 32) hull_epa_kernel(HullParams p, HullBuffers H) {
    __shared__ EpaShared polytope[kEpaWarps];
    EpaShared& sh = polytope[threadIdx.x >> 5];
    const uint32_t n_hits = *H.hit_count;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < n_hits; k += nwarps) {
        const uint2 hit = H.hits[k];
        const uint4 keys = H.hit_keys[k];
        const uint32_t e = H.ulist[hit.x];
        const uint32_t A = H.self[e], B = H.partners[e];
        const uint32_t em = mirror_entry(H, A, B);
        HPair P;
        make_pair(H, A, B, &P);
        const Cso s[4] = {cso_of_key(P, keys.x), cso_of_key(P, keys.y), cso_of_key(P, keys.z), cso_of_key(P, keys.w)};
        int st = kHit;
        v3 fa = mk(0.f, 0.f, 0.f), ta = mk(0.f, 0.f, 0.f), fbv = mk(0.f, 0.f, 0.f), tb = mk(0.f, 0.f, 0.f);
        Contact c;
        epa_warp(P, s, (H.iinv[A].w + H.iinv[B].w) * 1e-7f, sh, &c);
        // contact skin: overlaps within it (float GJK cannot resolve them
        // reliably) carry no force and the spring acts on depth - skin
        const float skin = (H.iinv[A].w + H.iinv[B].w) * 1e-4f;
        if (!c.ok || !(c.depth > skin)) {
            st = kTouch;
        } else {
            const float4 pa = H.pos[A], pb = H.pos[B];
            const float mA = pa.w, mB = pb.w;
            const v3 rA = c.c, rB = vsub(c.c, P.off);
            const v3 vA = vadd(f3(H.vel[A]), vcross(f3(H.omg[A]), rA));
            const v3 vB = vadd(f3(H.vel[B]), vcross(f3(H.omg[B]), rB));
            const float meff = (mA * mB) / (mA + mB);
            fbv = contact_force(p, c.depth - skin, c.n, vsub(vB, vA), meff);
            tb = vcross(rB, fbv);
            fa = vneg(fbv);
            ta = vcross(rA, fa);
        }
        if (lane == 0) {
            const uint32_t info = (uint32_t)st | (hit.y << 8) | ((uint32_t)c.epa_iters << 16);
            H.ef[e] = make_float4(fa.x, fa.y, fa.z, 0.f);
            H.et[e] = make_float4(ta.x, ta.y, ta.z, 0.f);
            H.info[e] = info;
            if (em < H.off[B + 1]) {
                H.ef[em] = make_float4(fbv.x, fbv.y, fbv.z, 0.f);
                H.et[em] = make_float4(tb.x, tb.y, tb.z, 0.f);
                H.info[em] = info;
            }
        }
    }
}

// Per body: segmented sum of its entries (list order), walls, integration.
__global__ void hull_integrate_kernel(HullParams p, HullBuffers H) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= H.nb) return;
    v3 f = mk(0.f, 0.f, 0.f), t = mk(0.f, 0.f, 0.f);
    const uint32_t e0 = H.off[b], e1 = H.off[b + 1];
    if ((uint64_t)H.off[H.nb] <= H.cap) {
        for (uint32_t e = e0; e < e1; ++e) {
            f = vadd(f, f3(H.ef[e]));
            t = vadd(t, f3(H.et[e]));
        }
    }
    const float4 x4 = H.pos[b], v4 = H.vel[b], w4 = H.omg[b], q4 = H.quat[b];
    const Mat R = qrot(q4);
    if (p.walls) {
        const float4* V = H.verts + H.vstart[b];
        const uint32_t ex[2] = {H.ext[2 * b], H.ext[2 * b + 1]};
        const float xs[3] = {x4.x, x4.y, x4.z};
        for (int a = 0; a < 3; ++a) {
            for (int side = 0; side < 2; ++side) {
                if (!(p.walls & (1 << (2 * a + side)))) continue;
                const uint32_t k = (ex[side] >> (8 * a)) & 0xffu;
                const v3 r = rot(R, f3(V[k]));
                const float rc[3] = {r.x, r.y, r.z};
                const float xa = xs[a] + rc[a];
                const float gap = side == 0 ? xa - p.lo[a] : p.hi[a] - xa;
                if (!(gap < 0.0f)) continue;
                float nn[3] = {0.0f, 0.0f, 0.0f};
                nn[a] = side == 0 ? 1.0f : -1.0f;
                const v3 vc = vadd(f3(v4), vcross(f3(w4), r));
                const v3 fw = contact_force(p, -gap, mk(nn[0], nn[1], nn[2]), vc, x4.w);
                f = vadd(f, fw);
                t = vadd(t, vcross(r, fw));
            }
        }
    }
    if (H.force) H.force[b] = make_float4(f.x, f.y, f.z, 0.f);
    if (H.torque) H.torque[b] = make_float4(t.x, t.y, t.z, 0.f);
    const float dt = p.dt, m = x4.w;
    const float vx = v4.x + dt * (f.x / m + p.g[0]);
    const float vy = v4.y + dt * (f.y / m + p.g[1]);
    const float vz = v4.z + dt * (f.z / m + p.g[2]);
    const float px = x4.x + dt * vx, py = x4.y + dt * vy, pz = x4.z + dt * vz;
    const float4 L4 = H.ang[b];
    const float Lx = L4.x + dt * t.x, Ly = L4.y + dt * t.y, Lz = L4.z + dt * t.z;
    const float4 ii = H.iinv[b];
    v3 lb = rotT(R, mk(Lx, Ly, Lz));
    lb = mk(lb.x * ii.x, lb.y * ii.y, lb.z * ii.z);
    const v3 om = rot(R, lb);
    const float wx = om.x, wy = om.y, wz = om.z;
    const float qs = q4.x, qx = q4.y, qy = q4.z, qz = q4.w;
    const float h = 0.5f * dt;
    const float ds = -((wx * qx + wy * qy) + wz * qz);
    const float dx = qs * wx + (wy * qz - wz * qy);
    const float dy = qs * wy + (wz * qx - wx * qz);
    const float dz = qs * wz + (wx * qy - wy * qx);
    const float ns = qs + h * ds, nx = qx + h * dx, ny = qy + h * dy, nz = qz + h * dz;
    const float nrm = sqrtf((ns * ns + nx * nx) + (ny * ny + nz * nz));
    H.pos[b] = make_float4(px, py, pz, m);
    H.vel[b] = make_float4(vx, vy, vz, 0.f);
    H.ang[b] = make_float4(Lx, Ly, Lz, 0.f);
    H.quat[b] = make_float4(ns / nrm, nx / nrm, ny / nrm, nz / nrm);
    H.omg[b] = make_float4(wx, wy, wz, 0.f);
}

// Step statistics over the unique pairs (entries with self < other):
// [0] pairs, [1] GJK support evaluations, [2] intersecting pairs,
// [3] EPA iterations.
__global__ void hull_stats_kernel(HullBuffers H, unsigned long long* __restrict__ out) {
    __shared__ unsigned long long s[4];
    if (threadIdx.x < 4) s[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t total = min((uint64_t)H.off[H.nb], H.cap);
    unsigned long long c[4] = {0, 0, 0, 0};
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        if (H.self[e] > H.partners[e]) continue;
        const uint32_t inf = H.info[e];
        c[0] += 1;
        c[1] += (inf >> 8) & 0xffu;
        c[2] += (inf & 0xffu) == (uint32_t)kHit;
        c[3] += (inf >> 16) & 0xffu;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        for (int o = 16; o > 0; o >>= 1) c[k] += __shfl_down_sync(0xffffffffu, c[k], o);
        if (lane_id() == 0) atomicAdd(&s[k], c[k]);
    }
    __syncthreads();
    if (threadIdx.x < 4) atomicAdd(out + threadIdx.x, s[threadIdx.x]);
}

inline uint32_t grid_for(uint64_t n, int threads) { return (uint32_t)((n + threads - 1) / threads); }

}  // namespace

cudaError_t hull_aabb_async(HullBuffers& H, cudaStream_t st) {
    if (H.nb == 0) return cudaSuccess;
    hull_aabb_kernel<<<grid_for(H.nb, 128), 128, 0, st>>>(H);
    return cudaGetLastError();
}

cudaError_t hull_seed_async(HullBuffers& H, uint32_t mode, cudaStream_t st) {
    if (H.nb == 0 || H.cap == 0) return cudaSuccess;
    hull_prev_seed_kernel<<<grid_for(H.cap, 256), 256, 0, st>>>(H, mode);
    return cudaGetLastError();
}

// Each pair is evaluated once, by one thread, into both of its entries.
// The grid covers the largest possible pair count (cap / 2); threads past
// the step's count return at once.
__global__ void hull_teach_flags_kernel(const float4* __restrict__ teach, const uint32_t* __restrict__ d_count,
                                        uint32_t cap, uint32_t* __restrict__ flags) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= cap) return;
    const uint32_t n = min(*d_count, cap);
    flags[e] = e < n && teach[e].w == 1.0f ? 1u : 0u;
}

__global__ void hull_teach_gather_kernel(const float* __restrict__ feat, const float4* __restrict__ teach,
                                         const uint32_t* __restrict__ flags, const uint32_t* __restrict__ pos,
                                         uint32_t cap, uint32_t rows_cap, float* __restrict__ feat_c,
                                         float4* __restrict__ teach_c, uint32_t* __restrict__ d_total) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= cap) return;
    if (e == cap - 1) *d_total = min(pos[e] + flags[e], rows_cap);
    if (!flags[e]) return;
    const uint32_t r = pos[e];
    if (r >= rows_cap) return;  // one sample per unique pair fits; inconsistent lists could exceed it
    const float4* src = reinterpret_cast<const float4*>(feat + 16 * (size_t)e);
    float4* dst = reinterpret_cast<float4*>(feat_c + 16 * (size_t)r);
#pragma unroll
    for (int k = 0; k < 4; ++k) dst[k] = src[k];
    teach_c[r] = teach[e];
}

static int g_hull_blocks = 4;
void hull_set_blocks(int b) { g_hull_blocks = b == 3 ? 3 : 4; }
int hull_blocks() { return g_hull_blocks; }

cudaError_t hull_teach_compact_async(const HullBuffers& H, const uint32_t* d_count, float* feat_c, float4* teach_c,
                                     uint32_t* flags, uint32_t* pos, uint32_t* scan, uint32_t* d_total,
                                     cudaStream_t st) {
    const uint32_t cap = (uint32_t)H.cap;
    if (cap == 0) return cudaMemsetAsync(d_total, 0, 4, st);
    hull_teach_flags_kernel<<<grid_for(cap, 256), 256, 0, st>>>(H.teach, d_count, cap, flags);
    cudaError_t e = scan_exclusive_async(flags, pos, cap, scan, st);
    if (e != cudaSuccess) return e;
    hull_teach_gather_kernel<<<grid_for(cap, 256), 256, 0, st>>>(H.feat, H.teach, flags, pos, cap, cap / 2 + 1,
                                                                 feat_c, teach_c, d_total);
    return cudaGetLastError();
}

cudaError_t hull_narrow_async(const HullParams& p, HullBuffers& H, cudaStream_t st) {
    if (H.nb == 0 || H.cap == 0) return cudaSuccess;
    hull_unique_count_kernel<<<grid_for(H.nb, 256), 256, 0, st>>>(H);
    cudaError_t e = scan_exclusive_async(H.ucount, H.upos, H.nb, H.uscan, st);
    if (e != cudaSuccess) return e;
    hull_unique_fill_kernel<<<grid_for(H.nb, 256), 256, 0, st>>>(H);
    if ((e = cudaMemsetAsync(H.hit_count, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
    if (g_hull_blocks == 3)
        hull_gjk_kernel<3><<<grid_for(H.cap / 2 + 1, kHullThreads), kHullThreads, 0, st>>>(H);
    else
        hull_gjk_kernel<4><<<grid_for(H.cap / 2 + 1, kHullThreads), kHullThreads, 0, st>>>(H);
    hull_epa_kernel<<<152 * 4, kEpaWarps * 32, 0, st>>>(p, H);
    return cudaGetLastError();
}

cudaError_t hull_integrate_async(const HullParams& p, HullBuffers& H, cudaStream_t st) {
    if (H.nb == 0) return cudaSuccess;
    hull_integrate_kernel<<<grid_for(H.nb, 128), 128, 0, st>>>(p, H);
    return cudaGetLastError();
}

cudaError_t hull_stats_async(HullBuffers& H, unsigned long long* out, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(out, 0, 4 * sizeof(unsigned long long), st);
    if (e != cudaSuccess || H.nb == 0 || H.cap == 0) return e;
    hull_stats_kernel<<<152, 256, 0, st>>>(H, out);
    return cudaGetLastError();
}

}  // namespace sd
