/*
 * sd_oracle_hull.c -- CPU oracle for the convex-hull path (test
 * infrastructure only; see sd_oracle.h for who may use it).
 *
 * Restates, in plain C with -ffp-contract=off and the operation order the
 * CUDA kernels follow:
 *   - the reference's 30-bit Morton code of an AABB centroid
 *     (computeSpaceFillingCurveCUDA, sandbox/testLBVH.cu:91-151);
 *   - the exact AABB-overlap pair set of a box list by sort-and-sweep on x
 *     (the set an LBVH or SAP broad phase must return);
 *   - world AABBs of rotated hulls;
 *   - GJK (Gilbert, Johnson, Keerthi 1988) in the boolean form of
 *     sandbox/testGJK.cu:52-315: support mapping of a vertex soup, the
 *     Minkowski difference B - A, the line/triangle/tetrahedron simplex
 *     cases and the termination test dot(w, d) < 0, at most 64 support
 *     evaluations;
 *   - EPA (expanding polytope, van den Bergen 2001) for the penetration
 *     depth, normal and witness points of intersecting pairs (absent in the
 *     reference);
 *   - the hull contact law (the sphere law of sd_oracle.c applied at the EPA
 *     contact point) and quaternion integration with a diagonal body-frame
 *     inertia.
 */
#include "sd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct { float x, y, z; } v3;

static inline v3 mk(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vneg(v3 a) { return mk(-a.x, -a.y, -a.z); }
static inline v3 vscale(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline float vdot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline v3 vcross(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline v3 vtriple(v3 a, v3 b, v3 c) { return vcross(vcross(a, b), c); }
static inline int vzero(v3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
static inline v3 ld3(const float* p) { return mk(p[0], p[1], p[2]); }

/* Rotation matrix (row-major) of a unit quaternion (s, x, y, z); the same
 * expression as the rigid-clump integrator. */
static void hq_rot(const float* q, float* R) {
    const float qs = q[0], qx = q[1], qy = q[2], qz = q[3];
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
static inline v3 rot(const float* R, v3 v) {
    return mk((R[0] * v.x + R[1] * v.y) + R[2] * v.z, (R[3] * v.x + R[4] * v.y) + R[5] * v.z,
              (R[6] * v.x + R[7] * v.y) + R[8] * v.z);
}
static inline v3 rotT(const float* R, v3 d) {
    return mk((R[0] * d.x + R[3] * d.y) + R[6] * d.z, (R[1] * d.x + R[4] * d.y) + R[7] * d.z,
              (R[2] * d.x + R[5] * d.y) + R[8] * d.z);
}

/* ------------------------------------------------------------ Morton codes */

static uint32_t spread10(uint32_t x) {
    x &= 0x3ffu;
    x = (x ^ (x << 16)) & 0xff0000ffu;
    x = (x ^ (x << 8)) & 0x0300f00fu;
    x = (x ^ (x << 4)) & 0x030c30c3u;
    x = (x ^ (x << 2)) & 0x09249249u;
    return x;
}

/* computeSpaceFillingCurveCUDA (testLBVH.cu:113-151): centroid relative to
 * the domain centre in units of domain/1024, floored toward -inf, clamped
 * to [-512, 511], offset by 512, bits interleaved x | y<<1 | z<<2. */
void sdo_morton_ref(uint32_t n, const float* lo4, const float* hi4, const float* glo, const float* ghi,
                    uint32_t* codes) {
    float cen[3], cell[3];
    for (int a = 0; a < 3; ++a) {
        cen[a] = (glo[a] + ghi[a]) * 0.5f;
        cell[a] = (ghi[a] - glo[a]) / 1024.0f;
    }
    for (uint32_t i = 0; i < n; ++i) {
        int32_t q[3];
        for (int a = 0; a < 3; ++a) {
            const float c = (lo4[4 * (size_t)i + a] + hi4[4 * (size_t)i + a]) * 0.5f;
            const float p = cell[a] > 0.0f ? (c - cen[a]) / cell[a] : 0.0f;
            int32_t d = p >= 0.0f ? (int32_t)p : (int32_t)floorf(p);
            d = d < -512 ? -512 : (d > 511 ? 511 : d);
            q[a] = d + 512;
        }
        codes[i] = spread10((uint32_t)q[0]) | (spread10((uint32_t)q[1]) << 1) | (spread10((uint32_t)q[2]) << 2);
    }
}

/* ------------------------------------------------------- AABB pair sets */

static const float* g_sort_lo;  /* qsort context (single-threaded use) */
static int cmp_lo_x(const void* a, const void* b) {
    const uint32_t i = *(const uint32_t*)a, j = *(const uint32_t*)b;
    const float x = g_sort_lo[4 * (size_t)i], y = g_sort_lo[4 * (size_t)j];
    if (x < y) return -1;
    if (x > y) return 1;
    return i < j ? -1 : (i > j);
}
static int cmp_u64h(const void* a, const void* b) {
    const uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : (x > y);
}

static inline int overlap_yz(const float* lo4, const float* hi4, uint32_t i, uint32_t j) {
    return lo4[4 * (size_t)j + 1] <= hi4[4 * (size_t)i + 1] && lo4[4 * (size_t)i + 1] <= hi4[4 * (size_t)j + 1] &&
           lo4[4 * (size_t)j + 2] <= hi4[4 * (size_t)i + 2] && lo4[4 * (size_t)i + 2] <= hi4[4 * (size_t)j + 2];
}

/* Every pair (i < j) whose closed boxes overlap on all three axes, as
 * u64 (i << 32 | j), ascending.  Sort by lower x, then sweep forward while
 * the next lower x is <= this box's upper x.  Returns the count (only cap
 * are written). */
uint64_t sdo_aabb_pairs(uint32_t n, const float* lo4, const float* hi4, uint64_t* out, uint64_t cap) {
    uint32_t* idx = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
    if (!idx) return 0;
    for (uint32_t i = 0; i < n; ++i) idx[i] = i;
    g_sort_lo = lo4;
    qsort(idx, n, sizeof(uint32_t), cmp_lo_x);
    uint64_t cnt = 0;
    for (uint32_t k = 0; k < n; ++k) {
        const uint32_t i = idx[k];
        const float hx = hi4[4 * (size_t)i];
        for (uint32_t m = k + 1; m < n; ++m) {
            const uint32_t j = idx[m];
            if (!(lo4[4 * (size_t)j] <= hx)) break;
            if (!overlap_yz(lo4, hi4, i, j)) continue;
            if (cnt < cap) out[cnt] = i < j ? ((uint64_t)i << 32 | j) : ((uint64_t)j << 32 | i);
            ++cnt;
        }
    }
    free(idx);
    if (out && cnt <= cap) qsort(out, (size_t)cnt, sizeof(uint64_t), cmp_u64h);
    return cnt;
}

/* ----------------------------------------------------------- hull AABBs */

void sdo_hull_aabbs(uint32_t nb, const float* pos4, const float* quat4, const uint32_t* vstart,
                    const uint32_t* vcount, const float* verts4, float* lo4, float* hi4, uint32_t* ext6) {
    for (uint32_t b = 0; b < nb; ++b) {
        float R[9];
        hq_rot(quat4 + 4 * (size_t)b, R);
        const float* V = verts4 + 4 * (size_t)vstart[b];
        float mn[3], mx[3];
        uint32_t imn[3] = {0, 0, 0}, imx[3] = {0, 0, 0};
        v3 w = rot(R, ld3(V));
        mn[0] = mx[0] = w.x; mn[1] = mx[1] = w.y; mn[2] = mx[2] = w.z;
        for (uint32_t k = 1; k < vcount[b]; ++k) {
            w = rot(R, ld3(V + 4 * (size_t)k));
            const float c[3] = {w.x, w.y, w.z};
            for (int a = 0; a < 3; ++a) {
                if (c[a] < mn[a]) { mn[a] = c[a]; imn[a] = k; }
                if (c[a] > mx[a]) { mx[a] = c[a]; imx[a] = k; }
            }
        }
        const float* x = pos4 + 4 * (size_t)b;
        for (int a = 0; a < 3; ++a) {
            lo4[4 * (size_t)b + a] = x[a] + mn[a];
            hi4[4 * (size_t)b + a] = x[a] + mx[a];
            if (ext6) {
                ext6[6 * (size_t)b + a] = imn[a];
                ext6[6 * (size_t)b + 3 + a] = imx[a];
            }
        }
        lo4[4 * (size_t)b + 3] = 0.0f;
        hi4[4 * (size_t)b + 3] = 0.0f;
    }
}

/* ------------------------------------------------------------ GJK + EPA */

typedef struct {
    float R[9];
    const float* V;  /* body-frame vertices (float4 rows) */
    uint32_t nv;
} hbody;

typedef struct {
    v3 w, a, b;  /* w = b - a, a on A (relative to A's centre), b on B (same origin) */
    uint32_t key;
} csop;

typedef struct {
    hbody A, B;
    v3 off;  /* x_B - x_A */
} hpair;

static inline uint32_t support(const hbody* h, v3 d, v3* out) {
    const v3 db = rotT(h->R, d);
    uint32_t best = 0;
    float bd = vdot(db, ld3(h->V));
    for (uint32_t k = 1; k < h->nv; ++k) {
        const float t = vdot(db, ld3(h->V + 4 * (size_t)k));
        if (t > bd) { bd = t; best = k; }
    }
    *out = rot(h->R, ld3(h->V + 4 * (size_t)best));
    return best;
}

static inline csop cso(const hpair* P, v3 d) {
    csop r;
    const uint32_t ia = support(&P->A, vneg(d), &r.a);
    v3 bb;
    const uint32_t ib = support(&P->B, d, &bb);
    r.b = vadd(bb, P->off);
    r.w = vsub(r.b, r.a);
    r.key = ia * 1024u + ib;
    return r;
}

enum { GJK_SEP = 0, GJK_HIT = 1, GJK_TOUCH = 2, GJK_NOCONV = 3 };
#define GJK_MAX_IT 64
/* support evaluations a seeded run gets to certify separation before the
 * plain run takes over */
#define GJK_SEED_MAX_IT 2
#define EPA_MAXV 48
#define EPA_MAXF 96
#define EPA_MAX_IT 48

typedef struct {
    csop s[4];
    int n;
    v3 d;
} simplex_t;

/* Closest point to the origin of the simplex S->s[0..n) (Ericson, Real-Time
 * Collision Detection, 5.1.2, 5.1.5, 5.1.6: Voronoi-region tests of the
 * segment, triangle and tetrahedron).  Reduces the simplex to the vertices of
 * the closest feature (kept in their order) and returns the point in *v; for
 * a tetrahedron that contains the origin returns 1 and leaves S whole. */
static void closest_tri(const csop* A, const csop* B, const csop* C, v3* v, int* mask) {
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

static void keep(simplex_t* S, const int* idx, int m) {
    csop t[4];
    for (int k = 0; k < m; ++k) t[k] = S->s[idx[k]];
    for (int k = 0; k < m; ++k) S->s[k] = t[k];
    S->n = m;
}

static void keep_mask(simplex_t* S, const int* tri, int mask) {
    int idx[3], m = 0;
    for (int k = 0; k < 3; ++k)
        if (mask & (1 << k)) idx[m++] = tri[k];
    keep(S, idx, m);
}

static int closest_simplex(simplex_t* S, v3* v) {
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
        static const int tri[3] = {0, 1, 2};
        int mask;
        closest_tri(&S->s[0], &S->s[1], &S->s[2], v, &mask);
        keep_mask(S, tri, mask);
        return 0;
    }
    /* tetrahedron: faces with the opposite vertex */
    static const int face[4][4] = {{0, 1, 2, 3}, {0, 2, 3, 1}, {0, 3, 1, 2}, {1, 3, 2, 0}};
    int best = -1, best_mask = 0;
    float best_d = 0.0f;
    v3 best_v = mk(0.0f, 0.0f, 0.0f);
    for (int f = 0; f < 4; ++f) {
        const v3 p = S->s[face[f][0]].w, q = S->s[face[f][1]].w, r = S->s[face[f][2]].w, o = S->s[face[f][3]].w;
        const v3 nrm = vcross(vsub(q, p), vsub(r, p));
        const float sp = vdot(vneg(p), nrm), so = vdot(vsub(o, p), nrm);
        const int outside = (sp > 0.0f && so < 0.0f) || (sp < 0.0f && so > 0.0f) || so == 0.0f;
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

/* GJK (distance form) on B - A from seed direction d0: v is the closest
 * point of the current simplex to the origin, the next support is taken in
 * -v, and the reference's test dot(w, d) < 0 ends it as separated.  Returns
 * the status, the number of support evaluations in *iters and, for a
 * separated pair, the separating search direction in *dir. */
static int gjk(const hpair* P, v3 d0, simplex_t* S, int* iters, v3* dir, int max_it) {
    v3 d = d0;
    if (vzero(d)) d = mk(1.0f, 0.0f, 0.0f);
    csop p = cso(P, d);
    int it = 1;
    *dir = d;
    if (vdot(p.w, d) < 0.0f) {
        *iters = it;
        return GJK_SEP;
    }
    S->s[0] = p;
    S->n = 1;
    uint32_t seen[GJK_MAX_IT];
    seen[0] = p.key;
    v3 v = p.w;
    float vv = vdot(v, v);
    for (;;) {
        if (vv == 0.0f) {
            *iters = it;
            return GJK_TOUCH;
        }
        if (it >= max_it) {
            *iters = it;
            return GJK_NOCONV;
        }
        d = vneg(v);
        *dir = d;
        p = cso(P, d);
        ++it;
        if (vdot(p.w, d) < 0.0f) {
            *iters = it;
            return GJK_SEP;
        }
        /* a support point seen before in this run: no further progress is
         * possible (the origin is on the boundary of B - A within rounding) */
        for (int k = 0; k < it - 1; ++k) {
            if (seen[k] == p.key) {
                *iters = it;
                return GJK_TOUCH;
            }
        }
        seen[it - 1] = p.key;
        for (int k = S->n; k > 0; --k) S->s[k] = S->s[k - 1];
        S->s[0] = p;
        S->n += 1;
        if (closest_simplex(S, &v)) {
            *iters = it;
            return GJK_HIT;
        }
        vv = vdot(v, v);
    }
}

typedef struct {
    uint8_t i[3];
    v3 n;
    float dist;
} epa_face;

static int epa_face_make(const csop* V, uint8_t a, uint8_t b, uint8_t c, epa_face* f) {
    const v3 nn = vcross(vsub(V[b].w, V[a].w), vsub(V[c].w, V[a].w));
    const float len = sqrtf(vdot(nn, nn));
    if (!(len > 0.0f)) return 0;
    f->i[0] = a;
    f->i[1] = b;
    f->i[2] = c;
    f->n = mk(nn.x / len, nn.y / len, nn.z / len);
    f->dist = vdot(f->n, V[a].w);
    return 1;
}

typedef struct {
    float depth;
    v3 n;      /* unit contact normal from A to B */
    v3 c;      /* contact point relative to A's centre */
    int epa_iters;
    int ok;
} contact_t;

/* EPA from GJK's enclosing tetrahedron; the result is recomputed from the
 * final face with its vertices in canonical (support-index) order, so two
 * runs that end on the same face of B - A agree bit for bit. */
static void epa(const hpair* P, const simplex_t* S, float tol, contact_t* out) {
    csop V[EPA_MAXV];
    epa_face F[EPA_MAXF];
    uint8_t E[3 * EPA_MAXF][2];
    int nv = 4, nf = 0;
    for (int k = 0; k < 4; ++k) V[k] = S->s[k];
    static const uint8_t init[4][3] = {{0, 1, 2}, {0, 2, 3}, {0, 3, 1}, {1, 3, 2}};
    for (int k = 0; k < 4; ++k) {
        epa_face f;
        if (!epa_face_make(V, init[k][0], init[k][1], init[k][2], &f)) continue;
        if (f.dist < 0.0f) {
            const uint8_t t = f.i[1];
            f.i[1] = f.i[2];
            f.i[2] = t;
            f.n = vneg(f.n);
            f.dist = -f.dist;
        }
        F[nf++] = f;
    }
    out->ok = 0;
    out->epa_iters = 0;
    if (nf == 0) return;
    int best = 0;
    for (int it = 0;; ++it) {
        best = 0;
        for (int k = 1; k < nf; ++k)
            if (F[k].dist < F[best].dist) best = k;
        out->epa_iters = it + 1;
        if (it >= EPA_MAX_IT || nv >= EPA_MAXV) break;
        const csop p = cso(P, F[best].n);
        int dup = 0;
        for (int k = 0; k < nv; ++k) dup |= V[k].key == p.key;
        if (dup || vdot(p.w, F[best].n) - F[best].dist <= tol) break;
        const uint8_t q = (uint8_t)nv;
        V[nv++] = p;
        int ne = 0, keep = 0;
        for (int k = 0; k < nf; ++k) {
            if (vdot(F[k].n, vsub(p.w, V[F[k].i[0]].w)) > 0.0f) {
                for (int e = 0; e < 3; ++e) {
                    const uint8_t a = F[k].i[e], b = F[k].i[(e + 1) % 3];
                    int found = -1;
                    for (int m = 0; m < ne; ++m)
                        if (E[m][0] == b && E[m][1] == a) { found = m; break; }
                    if (found >= 0) {
                        E[found][0] = E[ne - 1][0];
                        E[found][1] = E[ne - 1][1];
                        --ne;
                    } else {
                        E[ne][0] = a;
                        E[ne][1] = b;
                        ++ne;
                    }
                }
            } else {
                F[keep++] = F[k];
            }
        }
        nf = keep;
        if (nf + ne > EPA_MAXF) break;
        for (int m = 0; m < ne; ++m) {
            epa_face f;
            if (epa_face_make(V, E[m][0], E[m][1], q, &f)) F[nf++] = f;
        }
        if (nf == 0) return;
    }
    /* canonical recomputation on the final face */
    csop t[3] = {V[F[best].i[0]], V[F[best].i[1]], V[F[best].i[2]]};
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2 - a; ++b)
            if (t[b].key > t[b + 1].key) { const csop s = t[b]; t[b] = t[b + 1]; t[b + 1] = s; }
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
    const v3 p = vscale(n, depth);
    const v3 e2 = vsub(p, t[0].w);
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
    out->ok = 1;
}

static void make_pair(hpair* P, const float* pos4, const float* quat4, const uint32_t* vstart,
                      const uint32_t* vcount, const float* verts4, uint32_t A, uint32_t B) {
    hq_rot(quat4 + 4 * (size_t)A, P->A.R);
    hq_rot(quat4 + 4 * (size_t)B, P->B.R);
    P->A.V = verts4 + 4 * (size_t)vstart[A];
    P->A.nv = vcount[A];
    P->B.V = verts4 + 4 * (size_t)vstart[B];
    P->B.nv = vcount[B];
    P->off = vsub(ld3(pos4 + 4 * (size_t)B), ld3(pos4 + 4 * (size_t)A));
}

/* The contact skin of a pair: 1e-4 of the summed bounding radii. */
static inline float hull_skin(const float* iinv4, uint32_t A, uint32_t B) {
    return (iinv4[4 * (size_t)A + 3] + iinv4[4 * (size_t)B + 3]) * 1e-4f;
}

/* The EPA stopping tolerance of a pair: 1e-7 of the summed bounding radii. */
static inline float epa_tol(const float* iinv4, uint32_t A, uint32_t B) {
    return (iinv4[4 * (size_t)A + 3] + iinv4[4 * (size_t)B + 3]) * 1e-7f;
}

/* One narrow-phase query of the pair (A, B), A < B, seeded with seed
 * (world; NULL -> the reference seed x_A - x_B, testGJK.cu:266).  out8:
 * status, gjk iterations, epa iterations, depth, normal xyz (A to B),
 * contact point xyz (world), final search direction xyz. */
void sdo_gjk_epa(const float* pos4, const float* quat4, const float* iinv4, const uint32_t* vstart,
                 const uint32_t* vcount, const float* verts4, uint32_t A, uint32_t B, const float* seed,
                 int32_t* status_iters3, float* res10) {
    hpair P;
    make_pair(&P, pos4, quat4, vstart, vcount, verts4, A, B);
    const v3 d0 = seed ? ld3(seed) : vneg(P.off);
    simplex_t S;
    int iters = 0;
    v3 dir;
    const int st = gjk(&P, d0, &S, &iters, &dir, GJK_MAX_IT);
    contact_t c;
    memset(&c, 0, sizeof c);
    if (st == GJK_HIT) epa(&P, &S, epa_tol(iinv4, A, B), &c);
    status_iters3[0] = st;
    status_iters3[1] = iters;
    status_iters3[2] = c.epa_iters;
    const float* xa = pos4 + 4 * (size_t)A;
    res10[0] = c.ok ? c.depth : 0.0f;
    res10[1] = c.n.x; res10[2] = c.n.y; res10[3] = c.n.z;
    res10[4] = xa[0] + c.c.x; res10[5] = xa[1] + c.c.y; res10[6] = xa[2] + c.c.z;
    res10[7] = dir.x; res10[8] = dir.y; res10[9] = dir.z;
}

/* ---------------------------------------------------------- hull dynamics */

/* Linear spring-dashpot + Coulomb friction at a contact point; the force on
 * B (fb) along m (unit, A to B) for overlap delta and the velocity of B
 * relative to A at the contact point vr. */
static void hull_contact_force(const sdo_hull_params* p, float delta, v3 m, v3 vr, float meff, v3* fb) {
    const float vn = vdot(vr, m);
    const float gn = p->damp * sqrtf(meff);
    const float fn = p->kn * delta - gn * vn;
    const float fc = fn > 0.0f ? fn : 0.0f;
    const v3 vt = mk(vr.x - vn * m.x, vr.y - vn * m.y, vr.z - vn * m.z);
    const float vt2 = vdot(vt, vt);
    v3 f = mk(fn * m.x, fn * m.y, fn * m.z);
    if (vt2 > 0.0f) {
        const float vtm = sqrtf(vt2);
        const float ftm = fminf(p->mu * fc, gn * vtm);
        const float s = ftm / vtm;
        f.x += -(s * vt.x);
        f.y += -(s * vt.y);
        f.z += -(s * vt.z);
    }
    *fb = f;
}

/* Narrow phase + contact force of one directed entry (self, other).  The
 * pair is always evaluated as (A, B) = (min, max) so both directions give
 * the same numbers with opposite sign.  seed4: the seed of the pair in A's
 * body frame (w = 1 -> use xyz, else the reference seed x_A - x_B).
 * Returns the GJK status; *f, *t receive the force and torque on self (zero
 * without contact) and *dirA the final search direction in A's frame. */
static int hull_entry(const sdo_hull_params* p, const float* pos4, const float* vel4, const float* quat4,
                      const float* omg4, const float* iinv4, const uint32_t* vstart, const uint32_t* vcount,
                      const float* verts4, uint32_t self, uint32_t other, const float* seed4, int* iters,
                      int* epa_iters, v3* dirA, v3* f, v3* t) {
    const uint32_t A = self < other ? self : other, B = self < other ? other : self;
    hpair P;
    make_pair(&P, pos4, quat4, vstart, vcount, verts4, A, B);
    v3 d0 = vneg(P.off);
    const int seeded = seed4 && seed4[3] == 1.0f;
    if (seeded) d0 = rot(P.A.R, ld3(seed4));
    simplex_t S;
    v3 dir;
    /* a seeded run has GJK_SEED_MAX_IT supports to certify separation; only
     * that certificate is taken from it, any other outcome is the plain run's */
    int st = gjk(&P, d0, &S, iters, &dir, seeded ? GJK_SEED_MAX_IT : GJK_MAX_IT);
    if (seeded && st != GJK_SEP) {
        int it2 = 0;
        st = gjk(&P, vneg(P.off), &S, &it2, &dir, GJK_MAX_IT);
        *iters += it2;
    }
    *f = mk(0.0f, 0.0f, 0.0f);
    *t = mk(0.0f, 0.0f, 0.0f);
    *epa_iters = 0;
    *dirA = rotT(P.A.R, dir);
    if (st != GJK_HIT) return st;
    contact_t c;
    memset(&c, 0, sizeof c);
    epa(&P, &S, epa_tol(iinv4, A, B), &c);
    *epa_iters = c.epa_iters;
    if (!c.ok) return GJK_TOUCH;
    /* contact skin: overlaps within it (float GJK cannot resolve them
     * reliably) carry no force and the spring acts on depth - skin */
    const float skin = hull_skin(iinv4, A, B);
    if (!(c.depth > skin)) return GJK_TOUCH;
    const float mA = pos4[4 * (size_t)A + 3], mB = pos4[4 * (size_t)B + 3];
    const v3 rA = c.c, rB = vsub(c.c, P.off);
    const v3 vA = vadd(ld3(vel4 + 4 * (size_t)A), vcross(ld3(omg4 + 4 * (size_t)A), rA));
    const v3 vB = vadd(ld3(vel4 + 4 * (size_t)B), vcross(ld3(omg4 + 4 * (size_t)B), rB));
    const float meff = (mA * mB) / (mA + mB);
    v3 fb;
    hull_contact_force(p, c.depth - skin, c.n, vsub(vB, vA), meff, &fb);
    if (self == B) {
        *f = fb;
        *t = vcross(rB, fb);
    } else {
        *f = vneg(fb);
        *t = vcross(rA, *f);
    }
    return st;
}

/* Box walls: per wall, the hull's extreme vertex along the wall normal. */
static void hull_walls(const sdo_hull_params* p, const float* x, const float* v, const float* w, float m,
                       const float* R, const float* V, const uint32_t* ext6, v3* f, v3* t) {
    for (int a = 0; a < 3; ++a) {
        for (int side = 0; side < 2; ++side) {
            if (!(p->walls & (1 << (2 * a + side)))) continue;
            const v3 r = rot(R, ld3(V + 4 * (size_t)ext6[3 * side + a]));
            const float rc[3] = {r.x, r.y, r.z};
            const float xa = x[a] + rc[a];
            const float gap = side == 0 ? xa - p->lo[a] : p->hi[a] - xa;
            if (!(gap < 0.0f)) continue;
            float nn[3] = {0.0f, 0.0f, 0.0f};
            nn[a] = side == 0 ? 1.0f : -1.0f;
            /* the wall is body A (at rest, infinite mass), the hull body B */
            const v3 vc = vadd(ld3(v), vcross(ld3(w), r));
            v3 fw;
            hull_contact_force(p, -gap, ld3(nn), vc, m, &fw);
            *f = vadd(*f, fw);
            *t = vadd(*t, vcross(r, fw));
        }
    }
}

/* Integration of one hull body: symplectic Euler on momentum and angular
 * momentum, w = R diag(I0^-1) R^T L with the pre-step rotation, and the
 * normalised first-order quaternion step of the rigid clumps. */
static void hull_integrate(const sdo_hull_params* p, float* x, float* v, float* q, float* w, float* L,
                           const float* iinv, v3 f, v3 t) {
    const float dt = p->dt, m = x[3];
    const float vx = v[0] + dt * (f.x / m + p->g[0]);
    const float vy = v[1] + dt * (f.y / m + p->g[1]);
    const float vz = v[2] + dt * (f.z / m + p->g[2]);
    const float px = x[0] + dt * vx, py = x[1] + dt * vy, pz = x[2] + dt * vz;
    const float Lx = L[0] + dt * t.x, Ly = L[1] + dt * t.y, Lz = L[2] + dt * t.z;
    float R[9];
    hq_rot(q, R);
    v3 lb = rotT(R, mk(Lx, Ly, Lz));
    lb = mk(lb.x * iinv[0], lb.y * iinv[1], lb.z * iinv[2]);
    const v3 om = rot(R, lb);
    const float wx = om.x, wy = om.y, wz = om.z;
    const float qs = q[0], qx = q[1], qy = q[2], qz = q[3];
    const float h = 0.5f * dt;
    const float ds = -((wx * qx + wy * qy) + wz * qz);
    const float dx = qs * wx + (wy * qz - wz * qy);
    const float dy = qs * wy + (wz * qx - wx * qz);
    const float dz = qs * wz + (wx * qy - wy * qx);
    const float ns = qs + h * ds, nx = qx + h * dx, ny = qy + h * dy, nz = qz + h * dz;
    const float nrm = sqrtf((ns * ns + nx * nx) + (ny * ny + nz * nz));
    x[0] = px; x[1] = py; x[2] = pz;
    v[0] = vx; v[1] = vy; v[2] = vz;
    L[0] = Lx; L[1] = Ly; L[2] = Lz;
    q[0] = ns / nrm; q[1] = nx / nrm; q[2] = ny / nrm; q[3] = nz / nrm;
    w[0] = wx; w[1] = wy; w[2] = wz;
}

/* Candidate partners of every body from the AABB pair set: CSR (off[nb+1],
 * partners sorted ascending per body, both directions).  Returns the number
 * of entries, or -1 when cap is too small. */
int64_t sdo_hull_partners(uint32_t nb, const float* lo4, const float* hi4, uint32_t* off, uint32_t* partners,
                          uint64_t cap) {
    uint64_t np = sdo_aabb_pairs(nb, lo4, hi4, NULL, 0);
    uint64_t* pairs = (uint64_t*)malloc(sizeof(uint64_t) * (np ? np : 1));
    if (!pairs) return -1;
    sdo_aabb_pairs(nb, lo4, hi4, pairs, np);
    if (2 * np > cap) {
        free(pairs);
        return -1;
    }
    memset(off, 0, sizeof(uint32_t) * ((size_t)nb + 1));
    for (uint64_t k = 0; k < np; ++k) {
        off[(pairs[k] >> 32) + 1]++;
        off[(pairs[k] & 0xffffffffu) + 1]++;
    }
    for (uint32_t b = 0; b < nb; ++b) off[b + 1] += off[b];
    uint32_t* fill = (uint32_t*)malloc(sizeof(uint32_t) * (nb ? nb : 1));
    memcpy(fill, off, sizeof(uint32_t) * nb);
    /* pairs ascend by (i, j): for body i the partners j arrive ascending;
     * for body j the partners i arrive ascending as well */
    for (uint64_t k = 0; k < np; ++k) {
        const uint32_t i = (uint32_t)(pairs[k] >> 32), j = (uint32_t)(pairs[k] & 0xffffffffu);
        partners[fill[i]++] = j;
        partners[fill[j]++] = i;
    }
    /* body j's list mixes partners < j (from pairs (i, j)) and > j (from
     * (j, k)); both runs ascend, so one insertion pass sorts it */
    for (uint32_t b = 0; b < nb; ++b) {
        for (uint32_t e = off[b] + 1; e < off[b + 1]; ++e) {
            const uint32_t x = partners[e];
            uint32_t m = e;
            while (m > off[b] && partners[m - 1] > x) {
                partners[m] = partners[m - 1];
                --m;
            }
            partners[m] = x;
        }
    }
    free(fill);
    free(pairs);
    return (int64_t)(2 * np);
}

/* One hull step over given candidate lists (CSR, partners ascending).
 * seeds4 (per entry, may be NULL): GJK seeds, w = 1 marks a seed.
 * Per entry, status/iters (may be NULL) and the final search direction
 * dir4 (may be NULL).  force4/torque4 (may be NULL): the total force and
 * torque on each body.  State arrays are updated in place. */
void sdo_hull_step(const sdo_hull_params* p, uint32_t nb, float* pos4, float* vel4, float* quat4, float* omg4,
                   float* ang4, const float* iinv4, const uint32_t* vstart, const uint32_t* vcount,
                   const float* verts4, const uint32_t* off, const uint32_t* partners, const float* seeds4,
                   int32_t* status, int32_t* iters, float* dir4, float* force4, float* torque4) {
    float* lo = (float*)malloc(sizeof(float) * 8 * (size_t)(nb ? nb : 1));
    uint32_t* ext = (uint32_t*)malloc(sizeof(uint32_t) * 6 * (size_t)(nb ? nb : 1));
    float* F = (float*)malloc(sizeof(float) * 8 * (size_t)(nb ? nb : 1));
    if (!lo || !ext || !F) {
        free(lo); free(ext); free(F);
        return;
    }
    float* hi = lo + 4 * (size_t)nb;
    sdo_hull_aabbs(nb, pos4, quat4, vstart, vcount, verts4, lo, hi, ext);
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t bi = 0; bi < (int64_t)nb; ++bi) {
        const uint32_t b = (uint32_t)bi;
        v3 f = mk(0.0f, 0.0f, 0.0f), t = mk(0.0f, 0.0f, 0.0f);
        for (uint32_t e = off[b]; e < off[b + 1]; ++e) {
            int it = 0, eit = 0;
            v3 dir, fe, te;
            const int st = hull_entry(p, pos4, vel4, quat4, omg4, iinv4, vstart, vcount, verts4, b, partners[e],
                                      seeds4 ? seeds4 + 4 * (size_t)e : NULL, &it, &eit, &dir, &fe, &te);
            f = vadd(f, fe);
            t = vadd(t, te);
            if (status) status[e] = st;
            if (iters) iters[e] = it;
            if (dir4) {
                dir4[4 * (size_t)e] = dir.x; dir4[4 * (size_t)e + 1] = dir.y; dir4[4 * (size_t)e + 2] = dir.z;
                dir4[4 * (size_t)e + 3] = st == GJK_SEP ? 1.0f : 0.0f;
            }
        }
        float R[9];
        hq_rot(quat4 + 4 * (size_t)b, R);
        hull_walls(p, pos4 + 4 * (size_t)b, vel4 + 4 * (size_t)b, omg4 + 4 * (size_t)b, pos4[4 * (size_t)b + 3], R,
                   verts4 + 4 * (size_t)vstart[b], ext + 6 * (size_t)b, &f, &t);
        F[8 * (size_t)b] = f.x; F[8 * (size_t)b + 1] = f.y; F[8 * (size_t)b + 2] = f.z;
        F[8 * (size_t)b + 4] = t.x; F[8 * (size_t)b + 5] = t.y; F[8 * (size_t)b + 6] = t.z;
    }
    for (uint32_t b = 0; b < nb; ++b) {
        const v3 f = ld3(F + 8 * (size_t)b), t = ld3(F + 8 * (size_t)b + 4);
        if (force4) { memcpy(force4 + 4 * (size_t)b, &f, 12); force4[4 * (size_t)b + 3] = 0.0f; }
        if (torque4) { memcpy(torque4 + 4 * (size_t)b, &t, 12); torque4[4 * (size_t)b + 3] = 0.0f; }
        hull_integrate(p, pos4 + 4 * (size_t)b, vel4 + 4 * (size_t)b, quat4 + 4 * (size_t)b, omg4 + 4 * (size_t)b,
                       ang4 + 4 * (size_t)b, iinv4 + 4 * (size_t)b, f, t);
    }
    free(lo); free(ext); free(F);
}

/* ------------------------------------------------ sweep and prune (ref) */

/* sweepAndPruneCUDA (src/engine/cuda/collisions/SAP/sap_detection.cu:
 * 385-440) with populateCollisions (:293-323): per sorted position tid,
 * partners among the next 64 sorted positions; the x test compares the
 * phantom's lower x with the home upper x, which the kernel overwrites with
 * the home upper y (:413) once an x test passes, and the y test compares
 * the phantom's lower y with it; a partner is kept when it is not in the
 * row yet, fewer than 10 are kept and its id differs from tid.  Rows are
 * 16 int32, cleared to -1 first. */
void sdo_sap_sweep_ref(uint32_t n, const float* upperx, const float* lowerx_sorted, const float* uppery,
                       const float* lowery, const uint32_t* idx_sorted, int32_t* rows) {
    for (uint32_t tid = 0; tid < n; ++tid) {
        int32_t* row = rows + 16 * (size_t)tid;
        for (int k = 0; k < 16; ++k) row[k] = -1;
        int len = 0;
        const uint32_t home = idx_sorted[tid];
        float home_upper = upperx[home];
        const uint32_t end = tid + 64 < n ? tid + 64 : n;
        for (uint32_t i = tid + 1; i < end; ++i) {
            const float pl = lowerx_sorted[i];
            const uint32_t ph = idx_sorted[i];
            if (!(pl <= home_upper)) continue;
            home_upper = uppery[home];
            if (!(lowery[ph] <= home_upper)) continue;
            int unique = 1;
            for (int k = 0; k < 16; ++k) unique &= row[k] != (int32_t)ph;
            if (unique && len <= 8 && ph != tid) row[len++] = (int32_t)ph;
        }
    }
}

static inline uint32_t f32_bits(float v) {
    uint32_t b;
    memcpy(&b, &v, 4);
    return b;
}

/* SAPCollision::processCollisions (sap_detection.cu:668-706): AABB = centre
 * -/+ radius (radius4 NULL: pos.w), stable radix sort of the lower x
 * extents' float bits (sortLowestExtents :278-290, the sort's intended
 * semantics), projections, the sweep above. */
void sdo_sap_process(uint32_t n, const float* pos4, const float* radius, int32_t* rows) {
    const size_t m = n ? n : 1;
    uint32_t* keys = (uint32_t*)malloc(4 * m * 4);
    float* proj = (float*)malloc(4 * m * 4);
    if (!keys || !proj) {
        free(keys); free(proj);
        return;
    }
    uint32_t *vals = keys + m, *tk = vals + m, *tv = tk + m;
    float *upperx = proj, *uppery = proj + m, *lowery = proj + 2 * m, *lowerx_sorted = proj + 3 * m;
    for (uint32_t i = 0; i < n; ++i) {
        const float* p = pos4 + 4 * (size_t)i;
        const float r = radius ? radius[i] : p[3];
        upperx[i] = p[0] + r;
        uppery[i] = p[1] + r;
        lowery[i] = p[1] - r;
        keys[i] = f32_bits(p[0] - r);
        vals[i] = i;
    }
    sdo_radix_sort_pairs(keys, vals, n, 32, tk, tv);
    for (uint32_t i = 0; i < n; ++i) memcpy(&lowerx_sorted[i], &keys[i], 4);
    sdo_sap_sweep_ref(n, upperx, lowerx_sorted, uppery, lowery, vals, rows);
    free(keys);
    free(proj);
}
