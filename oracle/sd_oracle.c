/*
 * sd_oracle.c -- CPU oracle for the stardust-gb300 DEM step (test
 * infrastructure only; see sd_oracle.h for who may use it).
 *
 * Build: gcc -O2 -std=c11 -ffp-contract=off -fopenmp -shared -fPIC
 * (oracle/build.py).  -ffp-contract=off matters: every float operation must
 * round on its own, exactly as the -fmad=false CUDA kernels do.
 */
#include "sd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int sdo_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void sdo_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ======================================================== ref_compat ===== */

/* (uint32_t)(float) as the GPU converts it (cvt.rzi.u32.f32): truncation
 * toward zero, saturating to [0, 2^32-1], NaN -> 0. */
static inline uint32_t f2u_rz_sat(float q) {
    if (!(q > 0.0f)) return 0u;
    if (q >= 4294967296.0f) return 0xffffffffu;
    return (uint32_t)q;
}

/* Restates constructCollisionListCUDA, sh_collision_detection.cu:44-123.
 * - hash = x<<16 | y<<8 | z of (uint32)(coord / cell_dim), OR-ed per axis,
 *   so an axis index above 255 spills into the next field as it does there;
 * - the in-cell offset `x -= floor(x/cell)*cell` (:66) is one fused
 *   multiply-add, which is what nvcc emits for that line by default;
 * - side flags (:68-76): 3 when offset < size, else 1 when cell-offset < size;
 * - the phantom test (:95) parses as ((sides >> s) & 3) ^ r, which is never
 *   zero for r = -1, so only offsets in {0,+1}^3 \ {0} can be emitted;
 * - the domain test (:96) is 0 <= coord + r*cell < 1 and is applied only to
 *   phantom entries. */
uint32_t sdo_ref_hash_build(uint32_t n, float cell_dim, const float* pos4,
                            const float* sizes, uint32_t* cells, uint32_t* spheres) {
    uint32_t count = 0;
    for (uint32_t i = 0; i < n; ++i) {
        float pos[3] = {pos4[4 * (size_t)i + 0], pos4[4 * (size_t)i + 1], pos4[4 * (size_t)i + 2]};
        uint32_t hash = 0, sides = 0;
        for (int j = 0; j < 3; ++j) {
            float x = pos[j];
            float q = x / cell_dim;
            hash = (hash << 8) | f2u_rz_sat(q);
            x = fmaf(-floorf(q), cell_dim, x);
            float a = sizes[i];
            sides <<= 2;
            if (x < a) sides |= 3u;
            else if (cell_dim - x < a) sides |= 1u;
        }
        size_t h = 9 * (size_t)i;
        cells[h] = hash << 1;
        spheres[h] = (i << 1) | 1u;
        ++count;
        int m = 1;
        for (int j = 0; j < 27; ++j) {
            if (j == 13) continue;
            int q = j;
            uint32_t hh = 0;
            int invalid = 0;
            for (int k = 0; k < 3; ++k) {
                int r = q % 3 - 1;
                float x = pos[k];
                uint32_t side = (sides >> ((3 - k - 1) * 2)) & 3u;
                float shifted = x + (float)r * cell_dim;
                if ((r != 0 && (side ^ (uint32_t)r) != 0u) || shifted < 0.0f || shifted >= 1.0f) {
                    invalid = 1;
                    break;
                }
                hh = (hh << 8) | (f2u_rz_sat(x / cell_dim) + (uint32_t)r);
                q /= 3;
            }
            if (!invalid) {
                ++count;
                ++h;
                cells[h] = (hh << 1) | 1u;
                spheres[h] = i << 1;
                ++m;
            }
        }
        while (m < 9) {
            ++h;
            cells[h] = 0xffffffffu;
            spheres[h] = i << 2;
            ++m;
        }
    }
    return count;
}

/* Stable LSD radix sort, 8-bit digits (the intended semantics of
 * sh_collision_detection.cu:129-360; parallel over contiguous chunks, each
 * chunk scattered in order, so the result is the unique stable order). */
void sdo_radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t n, int nbits,
                          uint32_t* tmp_k, uint32_t* tmp_v) {
    if (n == 0 || nbits <= 0) return;
    int passes = (nbits + 7) / 8;
    int nt = 1;
#ifdef _OPENMP
    nt = n >= (1u << 16) ? omp_get_max_threads() : 1;
#endif
    size_t* hist = (size_t*)malloc(sizeof(size_t) * 256 * (size_t)nt);
    uint32_t *src_k = keys, *src_v = vals, *dst_k = tmp_k, *dst_v = tmp_v;
    for (int p = 0; p < passes; ++p) {
        int shift = 8 * p;
        memset(hist, 0, sizeof(size_t) * 256 * (size_t)nt);
#pragma omp parallel num_threads(nt)
        {
            int t = 0;
#ifdef _OPENMP
            t = omp_get_thread_num();
#endif
            size_t lo = (size_t)n * t / nt, hi = (size_t)n * (t + 1) / nt;
            size_t* hst = hist + 256 * (size_t)t;
            for (size_t i = lo; i < hi; ++i) hst[(src_k[i] >> shift) & 255u]++;
#pragma omp barrier
#pragma omp single
            {
                size_t run = 0;
                for (int d = 0; d < 256; ++d)
                    for (int tt = 0; tt < nt; ++tt) {
                        size_t c = hist[256 * (size_t)tt + d];
                        hist[256 * (size_t)tt + d] = run;
                        run += c;
                    }
            }
            for (size_t i = lo; i < hi; ++i) {
                uint32_t d = (src_k[i] >> shift) & 255u;
                size_t o = hst[d]++;
                dst_k[o] = src_k[i];
                dst_v[o] = src_v[i];
            }
        }
        uint32_t* t;
        t = src_k; src_k = dst_k; dst_k = t;
        t = src_v; src_v = dst_v; dst_v = t;
    }
    if (src_k != keys) {
        memcpy(keys, src_k, sizeof(uint32_t) * n);
        memcpy(vals, src_v, sizeof(uint32_t) * n);
    }
    free(hist);
}

/* Runs of tranverseCollisionListCUDA (collision_resolution.cu:145-190):
 * a run is a maximal range of equal cells[i] >> 1 among the first `count`
 * entries; h counts entries whose sphere word has bit 0 set (home). */
typedef void (*run_visitor)(void* ctx, uint32_t start, uint32_t end, uint32_t h);

static void visit_runs(const uint32_t* cells, const uint32_t* spheres, uint32_t count,
                       run_visitor fn, void* ctx) {
    uint32_t start = 0;
    while (start < count) {
        uint32_t key = cells[start] >> 1, end = start, h = 0;
        while (end < count && (cells[end] >> 1) == key) {
            if (spheres[end] & 1u) ++h;
            ++end;
        }
        uint32_t p = (end - start) - h;
        if (h >= 1 && h + p >= 2) fn(ctx, start, end, h);
        start = end;
    }
}

typedef struct {
    const uint32_t* spheres;
    const int32_t* body_of;
    uint32_t *a, *b;
    uint64_t cap, n;
} pair_ctx;

/* resolveCollisionsCUDA's loop nest (collision_resolution.cu:56-70):
 * j over the first h entries of the run, k over (j, end). */
static void emit_pairs(void* vctx, uint32_t start, uint32_t end, uint32_t h) {
    pair_ctx* c = (pair_ctx*)vctx;
    for (uint32_t j = start; j < start + h; ++j) {
        uint32_t home = c->spheres[j] >> 1;
        for (uint32_t k = j + 1; k < end; ++k) {
            uint32_t other = c->spheres[k] >> 1;
            if (c->body_of && c->body_of[home] == c->body_of[other]) continue;
            if (c->n < c->cap) {
                c->a[c->n] = home;
                c->b[c->n] = other;
            }
            c->n++;
        }
    }
}

uint64_t sdo_ref_candidate_pairs(const uint32_t* cells, const uint32_t* spheres,
                                 uint32_t count, const int32_t* body_of,
                                 uint32_t* pair_a, uint32_t* pair_b, uint64_t cap) {
    pair_ctx c = {spheres, body_of, pair_a, pair_b, cap, 0};
    visit_runs(cells, spheres, count, emit_pairs, &c);
    return c.n;
}

typedef struct {
    const uint32_t* spheres;
    const int32_t* body_of;
    const float *pos4, *vel4;
    float* force4;
} ref_force_ctx;

static inline float sign_ref(float v) { return v > 0.0f ? 1.0f : (v == 0.0f ? 1.0f : -1.0f); }

/* resolveCollisionsCUDA (collision_resolution.cu:30-98) with helper_math
 * float4 semantics: length() includes w (helper_math.hpp:1279-1282),
 * float4*float4 is component-wise (:863), float4/float divides each
 * component (:1007-1010).  The three force terms keep their value from an
 * earlier partner when a later partner is out of range (they are declared
 * outside the k loop), and the partner's force is assigned, not added. */
static void ref_forces(void* vctx, uint32_t start, uint32_t end, uint32_t h) {
    ref_force_ctx* c = (ref_force_ctx*)vctx;
    const float diameter = 0.2f, kn = 2e6f, kt = 200.0f, damping = 200.0f;
    for (uint32_t j = start; j < start + h; ++j) {
        float nf[4] = {0, 0, 0, 0}, df[4] = {0, 0, 0, 0}, tf[4] = {0, 0, 0, 0};
        uint32_t home = c->spheres[j] >> 1;
        for (uint32_t k = j + 1; k < end; ++k) {
            uint32_t ph = c->spheres[k] >> 1;
            if (c->body_of && c->body_of[home] == c->body_of[ph]) continue;
            float rp[4], rv[4];
            for (int q = 0; q < 4; ++q) {
                rp[q] = c->pos4[4 * (size_t)home + q] - c->pos4[4 * (size_t)ph + q];
                rv[q] = c->vel4[4 * (size_t)home + q] - c->vel4[4 * (size_t)ph + q];
            }
            float dist = sqrtf(rp[0] * rp[0] + rp[1] * rp[1] + rp[2] * rp[2] + rp[3] * rp[3]);
            if (dist <= diameter) {
                float np[4], s = -kn * (diameter - dist);
                for (int q = 0; q < 4; ++q) np[q] = rp[q] / dist;
                for (int q = 0; q < 4; ++q) {
                    float tv = rv[q] - (rv[q] * np[q]) * np[q];
                    nf[q] = s * np[q];
                    df[q] = damping * rv[q];
                    tf[q] = kt * tv;
                }
            }
            for (int q = 0; q < 4; ++q) {
                float sv = sign_ref(rv[q]);
                float total = nf[q] + df[q] + tf[q];
                c->force4[4 * (size_t)home + q] += (-sv) * total;
                c->force4[4 * (size_t)ph + q] = sv * total;
            }
        }
    }
}

void sdo_ref_resolve_forces(const uint32_t* cells, const uint32_t* spheres,
                            uint32_t count, const int32_t* body_of,
                            const float* pos4, const float* vel4, float* force4) {
    ref_force_ctx c = {spheres, body_of, pos4, vel4, force4};
    visit_runs(cells, spheres, count, ref_forces, &c);
}

/* ---- rigid-body kernels of physics_update.cu (one body / sphere at a time) */

/* Quaternion (s, vx, vy, vz) in (x, y, z, w) of a float4, cuda_helpers.cuh:130-145. */
static void qmul(const float a[4], const float b[4], float out[4]) {
    float s0 = a[0], s1 = b[0];
    float v0[3] = {a[1], a[2], a[3]}, v1[3] = {b[1], b[2], b[3]};
    float d = v0[0] * v1[0] + v0[1] * v1[1] + v0[2] * v1[2];
    float cr[3] = {v0[1] * v1[2] - v0[2] * v1[1], v0[2] * v1[0] - v0[0] * v1[2],
                   v0[0] * v1[1] - v0[1] * v1[0]};
    out[0] = s0 * s1 - d;
    for (int q = 0; q < 3; ++q) out[q + 1] = (s0 * v1[q] + s1 * v0[q]) + cr[q];
}

/* multiplyQuaternionByVectorCUDA, cuda_helpers.cuh:147-171: q v q*. */
static void qrot(const float q[4], const float v[4], float out[4]) {
    float vq[4] = {0.0f, v[0], v[1], v[2]};
    float qc[4] = {q[0], -q[1], -q[2], -q[3]};
    float t[4], r[4];
    qmul(q, vq, t);
    qmul(t, qc, r);
    out[0] = r[1]; out[1] = r[2]; out[2] = r[3]; out[3] = 0.0f;
}

/* updateSphereDataCUDA, physics_update.cu:26-107. */
void sdo_ref_update_spheres(int n_spheres, const float* init_rel4, const int32_t* body_of,
                            const float* body_pos4, const float* body_vel4,
                            const float* body_quat4, const float* body_omega4,
                            float* pos4, float* rel4, float* vel4) {
    for (int i = 0; i < n_spheres; ++i) {
        int b = body_of[i];
        float rr[4];
        qrot(body_quat4 + 4 * (size_t)b, init_rel4 + 4 * (size_t)i, rr);
        for (int q = 0; q < 4; ++q) {
            rel4[4 * (size_t)i + q] = rr[q];
            pos4[4 * (size_t)i + q] = rr[q] + body_pos4[4 * (size_t)b + q];
        }
        const float* w = body_omega4 + 4 * (size_t)b;
        float c[3] = {w[1] * rr[2] - w[2] * rr[1], w[2] * rr[0] - w[0] * rr[2], w[0] * rr[1] - w[1] * rr[0]};
        for (int q = 0; q < 3; ++q) vel4[4 * (size_t)i + q] = body_vel4[4 * (size_t)b + q] + c[q];
        vel4[4 * (size_t)i + 3] = body_vel4[4 * (size_t)b + 3] + 0.0f;
    }
}

/* computeForcesAndTorquesCUDA, physics_update.cu:144-195: serial per-body sum,
 * gravity (0,0,-9.81) times mass, bodies with mass >= 10 held fixed. */
void sdo_ref_body_forces(int n_bodies, const int32_t* start, const int32_t* length,
                         const float* body_mass, const float* rel4, const float* sphere_force4,
                         float* body_force4, float* body_torque4) {
    for (int b = 0; b < n_bodies; ++b) {
        float fs[4] = {0, 0, 0, 0}, ts[4] = {0, 0, 0, 0};
        float m = body_mass[b];
        for (int i = start[b]; i < start[b] + length[b]; ++i) {
            const float* f = sphere_force4 + 4 * (size_t)i;
            const float* r = rel4 + 4 * (size_t)i;
            for (int q = 0; q < 4; ++q) fs[q] += f[q];
            float t[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]};
            ts[0] += t[0]; ts[1] += t[1]; ts[2] += t[2]; ts[3] += 0.0f;
        }
        if (m >= 10.0f) {
            for (int q = 0; q < 4; ++q) fs[q] = ts[q] = 0.0f;
        } else {
            const float g[4] = {0.0f, 0.0f, -9.81f, 0.0f};
            for (int q = 0; q < 4; ++q) fs[q] += m * g[q];
        }
        for (int q = 0; q < 4; ++q) {
            body_force4[4 * (size_t)b + q] = fs[q];
            body_torque4[4 * (size_t)b + q] = ts[q];
        }
    }
}

/* compute3x3Inverse, cuda_helpers.cuh:65-78 (returns the input when the
 * determinant is below 1e-4). */
static void inv3_ref(const float* m, float* o) {
    float c11 = m[4] * m[8] - m[7] * m[5], c12 = m[7] * m[2] - m[1] * m[8], c13 = m[1] * m[5] - m[4] * m[2];
    float det = m[0] * c11 + m[3] * c12 + m[6] * c13;
    if (1e-4 > det) {
        memcpy(o, m, sizeof(float) * 9);
        return;
    }
    float s = 1 / det;
    o[0] = s * c11; o[1] = s * c12; o[2] = s * c13;
    o[3] = s * m[6] * m[5] - s * m[3] * m[8]; o[4] = s * m[0] * m[8] - s * m[6] * m[2];
    o[5] = s * m[3] * m[2] - s * m[0] * m[5];
    o[6] = s * m[3] * m[7] - s * m[6] * m[4]; o[7] = s * m[6] * m[1] - s * m[0] * m[7];
    o[8] = s * m[0] * m[4] - s * m[3] * m[1];
}

/* computeMatrixMultiplication, cuda_helpers.cuh:89-102 (column-major). */
static void mmul_ref(const float* a, const float* b, float* o) {
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r)
            o[3 * c + r] = a[r] * b[3 * c] + a[3 + r] * b[3 * c + 1] + a[6 + r] * b[3 * c + 2];
}

/* advectParticlesCUDA, physics_update.cu:232-310. */
void sdo_ref_advect(int n_bodies, float dt, const float* body_mass, const float* inertia9,
                    const float* body_force4, const float* body_torque4,
                    float* body_pos4, float* body_vel4, float* body_omega4,
                    float* body_quat4, float* lin_mom4, float* ang_mom4) {
    for (int b = 0; b < n_bodies; ++b) {
        float m = body_mass[b];
        float* L = lin_mom4 + 4 * (size_t)b;
        float* H = ang_mom4 + 4 * (size_t)b;
        float* x = body_pos4 + 4 * (size_t)b;
        float* q = body_quat4 + 4 * (size_t)b;
        for (int k = 0; k < 4; ++k) {
            L[k] += body_force4[4 * (size_t)b + k] * dt;
            H[k] += body_torque4[4 * (size_t)b + k] * dt;
        }
        float v[4];
        float invm = 1 / m;
        for (int k = 0; k < 4; ++k) v[k] = L[k] * invm;
        for (int k = 0; k < 4; ++k) x[k] += v[k] * dt;
        float I0inv[9], R[9], RT[9], tmp[9], Iinv[9];
        inv3_ref(inertia9 + 9 * (size_t)b, I0inv);
        /* quatToRotationCUDA, cuda_helpers.cuh:114-128, quat = (s, x, y, z) in (x, y, z, w) */
        float qs = q[0], qx = q[1], qy = q[2], qz = q[3];
        R[0] = 1 - 2 * (qy * qy) - 2 * (qz * qz);
        R[1] = 2 * qx * qy - 2 * qs * qz;
        R[2] = 2 * qx * qz + 2 * qs * qy;
        R[3] = 2 * qx * qy + 2 * qs * qz;
        R[4] = 1 - 2 * (qx * qx) - 2 * (qz * qz);
        R[5] = 2 * qy * qz - 2 * qs * qx;
        R[6] = 2 * qx * qz - 2 * qs * qy;
        R[7] = 2 * qy * qz + 2 * qs * qx;
        R[8] = 1 - 2 * (qx * qx) - 2 * (qy * qy);
        mmul_ref(R, I0inv, tmp);
        RT[0] = R[0]; RT[1] = R[3]; RT[2] = R[6];
        RT[3] = R[1]; RT[4] = R[4]; RT[5] = R[7];
        RT[6] = R[2]; RT[7] = R[5]; RT[8] = R[8];
        mmul_ref(tmp, RT, Iinv);
        float w[4];
        w[0] = Iinv[0] * H[0] + Iinv[3] * H[1] + Iinv[6] * H[2];
        w[1] = Iinv[1] * H[0] + Iinv[4] * H[1] + Iinv[7] * H[2];
        w[2] = Iinv[2] * H[0] + Iinv[5] * H[1] + Iinv[8] * H[2];
        w[3] = 0.0f;
        float ad[4];
        for (int k = 0; k < 4; ++k) ad[k] = w[k] * dt;
        float adm = sqrtf(ad[0] * ad[0] + ad[1] * ad[1] + ad[2] * ad[2] + ad[3] * ad[3]);
        float wm = sqrtf(w[0] * w[0] + w[1] * w[1] + w[2] * w[2] + w[3] * w[3]);
        float wn[4] = {0, 0, 0, 0};
        if (!(wm == 0.0f)) {
            /* normalize() uses rsqrtf (helper_math.hpp:1298-1302); the host
             * restatement uses the correctly rounded 1/sqrtf, so this term
             * can differ from the GPU's approximate rsqrt by an ulp. */
            float inv = 1.0f / sqrtf(w[0] * w[0] + w[1] * w[1] + w[2] * w[2] + w[3] * w[3]);
            for (int k = 0; k < 4; ++k) wn[k] = w[k] * inv;
        }
        float s = cosf(adm / 2), sn = sinf(adm / 2);
        float dq[4] = {s, wn[0] * sn, wn[1] * sn, wn[2] * sn};
        float nq[4];
        qmul(dq, q, nq);
        memcpy(q, nq, sizeof nq);
        memcpy(body_vel4 + 4 * (size_t)b, v, sizeof v);
        memcpy(body_omega4 + 4 * (size_t)b, w, sizeof w);
    }
}

/* =========================================================== physics ===== */

static inline int32_t axis_cell(float x, float lo, float cell, int32_t n) {
    float t = (x - lo) / cell;
    if (!(t >= 0.0f)) return 0;
    if (t >= (float)n) return n - 1;
    return (int32_t)t;
}

/* z cell edge: the engine splits z z_div times finer than x and y */
static inline float cell_z_of(const sdo_params* p) { return p->cell_z > 0.0f ? p->cell_z : p->cell; }

uint32_t sdo_cell_key(const sdo_params* p, float x, float y, float z) {
    int32_t ix = axis_cell(x, p->lo[0], p->cell, p->nx);
    int32_t iy = axis_cell(y, p->lo[1], p->cell, p->ny);
    int32_t iz = axis_cell(z, p->lo[2], cell_z_of(p), p->nz);
    return (uint32_t)((ix * p->ny + iy) * p->nz + iz);
}

void sdo_cell_keys(const sdo_params* p, uint32_t n, const float* pos4, uint32_t* keys) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i)
        keys[i] = sdo_cell_key(p, pos4[4 * i], pos4[4 * i + 1], pos4[4 * i + 2]);
}

static int key_bits(const sdo_params* p) {
    uint64_t nc = (uint64_t)p->nx * p->ny * p->nz;
    int b = 0;
    while (b < 32 && ((uint64_t)1 << b) < nc) ++b;
    return b < 1 ? 1 : b;
}

void sdo_sort_reorder(const sdo_params* p, uint32_t n,
                      const float* pos_n, const float* vel_n, const float* omg_n,
                      const uint32_t* keys, uint32_t* keys_out,
                      float* pos, float* vel, float* omg, uint32_t* cell_start) {
    uint32_t* k = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1) * 4);
    uint32_t *v = k + n, *tk = v + n, *tv = tk + n;
    memcpy(k, keys, sizeof(uint32_t) * n);
    for (uint32_t i = 0; i < n; ++i) v[i] = i;
    sdo_radix_sort_pairs(k, v, n, key_bits(p), tk, tv);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        uint32_t s = v[i];
        memcpy(pos + 4 * i, pos_n + 4 * (size_t)s, 16);
        memcpy(vel + 4 * i, vel_n + 4 * (size_t)s, 16);
        memcpy(omg + 4 * i, omg_n + 4 * (size_t)s, 16);
    }
    uint32_t nc = (uint32_t)(p->nx * p->ny * p->nz);
    uint32_t s = 0;
    for (uint32_t c = 0; c <= nc; ++c) {
        while (s < n && k[s] < c) ++s;
        cell_start[c] = s;
    }
    if (keys_out) memcpy(keys_out, k, sizeof(uint32_t) * n);
    free(k);
}

static inline uint32_t bits_f32(float v) {
    uint32_t b;
    memcpy(&b, &v, 4);
    return b;
}
/* the FP64 twin carries no sphere ids (no clumps in the error statement) */
static inline uint32_t bits_f64(double v) {
    (void)v;
    return 0u;
}

/* The engine's contact law and integrator.  The operation order below is
 * the specification the CUDA kernels follow; it is written once as a macro
 * template and instantiated for float (the parity oracle) and double (the
 * error statement). */
#define SDO_DEFINE_STEP(REAL, SQRT, FMIN, FMA, BITS, SUFFIX)                                           \
static inline void contact_response##SUFFIX(                                                 \
    const sdo_params* p, REAL nx, REAL ny, REAL nz, REAL delta,                              \
    REAL dvx, REAL dvy, REAL dvz, REAL wsx, REAL wsy, REAL wsz, REAL meff, REAL ri,          \
    REAL* f, REAL* t) {                                                                      \
    REAL cx = wsy * nz - wsz * ny;                                                           \
    REAL cy = wsz * nx - wsx * nz;                                                           \
    REAL cz = wsx * ny - wsy * nx;                                                           \
    REAL vrx = dvx - cx, vry = dvy - cy, vrz = dvz - cz;                                     \
    REAL vn = (vrx * nx + vry * ny) + vrz * nz;                                              \
    REAL gn = (REAL)p->damp * SQRT(meff);                                                    \
    REAL fn = (REAL)p->kn * delta - gn * vn;                                                 \
    REAL fc = fn > (REAL)0 ? fn : (REAL)0;                                                   \
    REAL vtx = vrx - vn * nx, vty = vry - vn * ny, vtz = vrz - vn * nz;                      \
    REAL vt2 = (vtx * vtx + vty * vty) + vtz * vtz;                                          \
    f[0] += fn * nx; f[1] += fn * ny; f[2] += fn * nz;                                       \
    if (vt2 > (REAL)0) {                                                                     \
        REAL vt = SQRT(vt2);                                                                 \
        REAL ftm = FMIN((REAL)p->mu * fc, gn * vt);                                          \
        REAL s = ftm / vt;                                                                   \
        REAL ftx = -(s * vtx), fty = -(s * vty), ftz = -(s * vtz);                           \
        f[0] += ftx; f[1] += fty; f[2] += ftz;                                               \
        REAL qx = ny * ftz - nz * fty;                                                       \
        REAL qy = nz * ftx - nx * ftz;                                                       \
        REAL qz = nx * fty - ny * ftx;                                                       \
        t[0] -= ri * qx; t[1] -= ri * qy; t[2] -= ri * qz;                                   \
    }                                                                                        \
}                                                                                            \
                                                                                             \
/* mesh walls: closest point of each triangle (Ericson 5.1.5), all        \
 * triangles in ascending order, deepest contact per patch kept */         \
static inline void closest_tri##SUFFIX(const REAL* p, const REAL* a, const REAL* b,         \
    const REAL* c, REAL* q) {                                                                \
    REAL ab[3], ac[3], ap[3], bp[3], cp[3];                                                  \
    for (int k = 0; k < 3; ++k) { ab[k] = b[k] - a[k]; ac[k] = c[k] - a[k]; ap[k] = p[k] - a[k]; } \
    REAL d1 = (ab[0] * ap[0] + ab[1] * ap[1]) + ab[2] * ap[2];                               \
    REAL d2 = (ac[0] * ap[0] + ac[1] * ap[1]) + ac[2] * ap[2];                               \
    if (d1 <= 0 && d2 <= 0) { for (int k = 0; k < 3; ++k) q[k] = a[k]; return; }            \
    for (int k = 0; k < 3; ++k) bp[k] = p[k] - b[k];                                         \
    REAL d3 = (ab[0] * bp[0] + ab[1] * bp[1]) + ab[2] * bp[2];                               \
    REAL d4 = (ac[0] * bp[0] + ac[1] * bp[1]) + ac[2] * bp[2];                               \
    if (d3 >= 0 && d4 <= d3) { for (int k = 0; k < 3; ++k) q[k] = b[k]; return; }           \
    REAL vc = d1 * d4 - d3 * d2;                                                             \
    if (vc <= 0 && d1 >= 0 && d3 <= 0) {                                                     \
        REAL v = d1 / (d1 - d3);                                                             \
        for (int k = 0; k < 3; ++k) q[k] = a[k] + ab[k] * v;                                 \
        return;                                                                              \
    }                                                                                        \
    for (int k = 0; k < 3; ++k) cp[k] = p[k] - c[k];                                         \
    REAL d5 = (ab[0] * cp[0] + ab[1] * cp[1]) + ab[2] * cp[2];                               \
    REAL d6 = (ac[0] * cp[0] + ac[1] * cp[1]) + ac[2] * cp[2];                               \
    if (d6 >= 0 && d5 <= d6) { for (int k = 0; k < 3; ++k) q[k] = c[k]; return; }           \
    REAL vb = d5 * d2 - d1 * d6;                                                             \
    if (vb <= 0 && d2 >= 0 && d6 <= 0) {                                                     \
        REAL w = d2 / (d2 - d6);                                                             \
        for (int k = 0; k < 3; ++k) q[k] = a[k] + ac[k] * w;                                 \
        return;                                                                              \
    }                                                                                        \
    REAL va = d3 * d6 - d5 * d4;                                                             \
    if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {                                      \
        REAL w = (d4 - d3) / ((d4 - d3) + (d5 - d6));                                        \
        for (int k = 0; k < 3; ++k) q[k] = b[k] + (c[k] - b[k]) * w;                         \
        return;                                                                              \
    }                                                                                        \
    REAL den = (REAL)1 / ((va + vb) + vc);                                                   \
    REAL v = vb * den, w = vc * den;                                                         \
    for (int k = 0; k < 3; ++k) q[k] = (a[k] + ab[k] * v) + ac[k] * w;                       \
}                                                                                            \
                                                                                             \
static void mesh_contacts##SUFFIX(const sdo_params* p, const sdo_mesh* m, const REAL* pi,   \
    const REAL* vi, const REAL* wi, REAL* f, REAL* t) {                                      \
    const float* S = m->state;                                                               \
    REAL R[9];                                                                               \
    for (int k = 0; k < 9; ++k) R[k] = (REAL)S[k];                                           \
    REAL d[3] = {pi[0] - (REAL)S[9], pi[1] - (REAL)S[10], pi[2] - (REAL)S[11]};              \
    REAL q[3] = {(R[0] * d[0] + R[3] * d[1]) + R[6] * d[2],                                  \
                 (R[1] * d[0] + R[4] * d[1]) + R[7] * d[2],                                  \
                 (R[2] * d[0] + R[5] * d[1]) + R[8] * d[2]};                                 \
    REAL r2 = pi[3] * pi[3];                                                                 \
    int32_t pid[4]; REAL pd2[4], pv[4][3], pq[4][3]; int np = 0;                             \
    for (uint32_t tr = 0; tr < m->ntri; ++tr) {                                              \
        REAL a[3], b[3], c[3], cl[3], v[3];                                                  \
        for (int k = 0; k < 3; ++k) {                                                        \
            a[k] = (REAL)m->tri[12 * (size_t)tr + k];                                        \
            b[k] = (REAL)m->tri[12 * (size_t)tr + 4 + k];                                    \
            c[k] = (REAL)m->tri[12 * (size_t)tr + 8 + k];                                    \
        }                                                                                    \
        closest_tri##SUFFIX(q, a, b, c, cl);                                                 \
        for (int k = 0; k < 3; ++k) v[k] = q[k] - cl[k];                                     \
        REAL d2 = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];                                 \
        if (!(d2 < r2) || d2 == (REAL)0) continue;                                           \
        int32_t pa = m->patch[tr];                                                           \
        int k = 0;                                                                           \
        while (k < np && pid[k] != pa) ++k;                                                  \
        if (k < np) {                                                                        \
            if (d2 < pd2[k]) { pd2[k] = d2; for (int j = 0; j < 3; ++j) { pv[k][j] = v[j]; pq[k][j] = cl[j]; } } \
        } else if (np < 4) {                                                                 \
            pid[np] = pa; pd2[np] = d2;                                                      \
            for (int j = 0; j < 3; ++j) { pv[np][j] = v[j]; pq[np][j] = cl[j]; }             \
            ++np;                                                                            \
        }                                                                                    \
    }                                                                                        \
    REAL ax[3] = {(REAL)S[12], (REAL)S[13], (REAL)S[14]}, om = (REAL)S[15];                  \
    for (int k = 0; k < np; ++k) {                                                           \
        REAL dist = SQRT(pd2[k]);                                                            \
        REAL inv = (REAL)1 / dist;                                                           \
        REAL nl[3] = {pv[k][0] * inv, pv[k][1] * inv, pv[k][2] * inv};                       \
        REAL nn[3], qw[3];                                                                   \
        for (int r = 0; r < 3; ++r) {                                                        \
            nn[r] = (R[3 * r] * nl[0] + R[3 * r + 1] * nl[1]) + R[3 * r + 2] * nl[2];        \
            qw[r] = (R[3 * r] * pq[k][0] + R[3 * r + 1] * pq[k][1]) + R[3 * r + 2] * pq[k][2]; \
        }                                                                                    \
        REAL vw[3] = {(ax[1] * qw[2] - ax[2] * qw[1]) * om, (ax[2] * qw[0] - ax[0] * qw[2]) * om, \
                      (ax[0] * qw[1] - ax[1] * qw[0]) * om};                                 \
        REAL ri = pi[3];                                                                     \
        contact_response##SUFFIX(p, nn[0], nn[1], nn[2], ri - dist, vi[0] - vw[0],           \
            vi[1] - vw[1], vi[2] - vw[2], ri * wi[0], ri * wi[1], ri * wi[2], vi[3], ri, f, t); \
    }                                                                                        \
}                                                                                            \
                                                                                             \
static uint64_t contact_integrate##SUFFIX(const sdo_params* p, uint32_t n,                   \
    const REAL* pos, const REAL* vel, const REAL* omg, const uint32_t* cell_start,           \
    REAL* pos_n, REAL* vel_n, REAL* omg_n, uint32_t* keys_n, REAL* force4, REAL* torque4,    \
    const int32_t* body_of, REAL* sf4, REAL* st4, const sdo_mesh* mesh) {                    \
    uint64_t contacts = 0;                                                                   \
    _Pragma("omp parallel for schedule(dynamic, 1024) reduction(+:contacts)")               \
    for (int64_t i = 0; i < (int64_t)n; ++i) {                                               \
        const REAL* pi = pos + 4 * i;                                                        \
        const REAL* vi = vel + 4 * i;                                                        \
        const REAL* wi = omg + 4 * i;                                                        \
        REAL xi = pi[0], yi = pi[1], zi = pi[2], ri = pi[3], mi = vi[3];                     \
        REAL f[3] = {0, 0, 0}, t[3] = {0, 0, 0};                                             \
        const uint32_t idb = BITS(wi[3]);                                                    \
        const int clump_i = body_of && (idb & 0x80000000u);                                  \
        int32_t cx = axis_cell((float)xi, p->lo[0], p->cell, p->nx);                         \
        int32_t cy = axis_cell((float)yi, p->lo[1], p->cell, p->ny);                         \
        /* z cells of every centre within one cell edge (r_i + r_j <= cell), padded */     \
        int32_t z0 = axis_cell((float)zi - p->cell * 1.00001f, p->lo[2], cell_z_of(p), p->nz); \
        int32_t z1 = axis_cell((float)zi + p->cell * 1.00001f, p->lo[2], cell_z_of(p), p->nz); \
        for (int32_t ddx = -1; ddx <= 1; ++ddx) {                                            \
            int32_t X = cx + ddx;                                                            \
            if (X < 0 || X >= p->nx) continue;                                               \
            for (int32_t ddy = -1; ddy <= 1; ++ddy) {                                        \
                int32_t Y = cy + ddy;                                                        \
                if (Y < 0 || Y >= p->ny) continue;                                           \
                uint32_t col = (uint32_t)((X * p->ny + Y) * p->nz);                          \
                uint32_t s0 = cell_start[col + (uint32_t)z0];                                \
                uint32_t s1 = cell_start[col + (uint32_t)z1 + 1];                            \
                for (uint32_t s = s0; s < s1; ++s) {                                         \
                    if ((int64_t)s == i) continue;                                           \
                    const REAL* pj = pos + 4 * (size_t)s;                                    \
                    REAL dx = xi - pj[0], dy = yi - pj[1], dz = zi - pj[2];                  \
                    REAL d2 = FMA(dz, dz, FMA(dy, dy, dx * dx));                             \
                    REAL rs = ri + pj[3];                                                    \
                    if (!(d2 < rs * rs) || d2 == (REAL)0) continue;                          \
                    const REAL* vj = vel + 4 * (size_t)s;                                    \
                    const REAL* wj = omg + 4 * (size_t)s;                                    \
                    if (clump_i) {                                                           \
                        const uint32_t jdb = BITS(wj[3]);                                    \
                        if ((jdb & 0x80000000u) &&                                           \
                            body_of[idb & 0x7fffffffu] == body_of[jdb & 0x7fffffffu])        \
                            continue;                                                        \
                    }                                                                        \
                    ++contacts;                                                              \
                    REAL rj = pj[3], mj = vj[3];                                             \
                    REAL dist = SQRT(d2);                                                    \
                    REAL inv = (REAL)1 / dist;                                               \
                    REAL nx = dx * inv, ny = dy * inv, nz = dz * inv;                        \
                    REAL wsx = ri * wi[0] + rj * wj[0];                                      \
                    REAL wsy = ri * wi[1] + rj * wj[1];                                      \
                    REAL wsz = ri * wi[2] + rj * wj[2];                                      \
                    REAL meff = (mi * mj) / (mi + mj);                                       \
                    contact_response##SUFFIX(p, nx, ny, nz, rs - dist,                       \
                        vi[0] - vj[0], vi[1] - vj[1], vi[2] - vj[2], wsx, wsy, wsz,          \
                        meff, ri, f, t);                                                     \
                }                                                                            \
            }                                                                                \
        }                                                                                    \
        if (mesh && mesh->ntri) mesh_contacts##SUFFIX(p, mesh, pi, vi, wi, f, t);            \
        if (p->walls) {                                                                      \
            REAL wsx = ri * wi[0], wsy = ri * wi[1], wsz = ri * wi[2];                       \
            REAL xs[3] = {xi, yi, zi};                                                       \
            for (int a = 0; a < 3; ++a) {                                                    \
                for (int side = 0; side < 2; ++side) {                                       \
                    if (!(p->walls & (1 << (2 * a + side)))) continue;                       \
                    REAL gap = side == 0 ? xs[a] - (REAL)p->lo[a] : (REAL)p->hi[a] - xs[a];  \
                    if (!(gap < ri)) continue;                                               \
                    REAL nn[3] = {0, 0, 0};                                                  \
                    nn[a] = side == 0 ? (REAL)1 : (REAL)-1;                                  \
                    contact_response##SUFFIX(p, nn[0], nn[1], nn[2], ri - gap,               \
                        vi[0], vi[1], vi[2], wsx, wsy, wsz, mi, ri, f, t);                   \
                }                                                                            \
            }                                                                                \
        }                                                                                    \
        if (force4) { force4[4*i] = f[0]; force4[4*i+1] = f[1]; force4[4*i+2] = f[2];        \
                      force4[4*i+3] = 0; }                                                   \
        if (torque4) { torque4[4*i] = t[0]; torque4[4*i+1] = t[1]; torque4[4*i+2] = t[2];    \
                       torque4[4*i+3] = 0; }                                                 \
        if (clump_i) {                                                                       \
            /* a clump sphere hands its contact force and torque to its body */              \
            sf4[4*i] = f[0]; sf4[4*i+1] = f[1]; sf4[4*i+2] = f[2]; sf4[4*i+3] = 0;           \
            st4[4*i] = t[0]; st4[4*i+1] = t[1]; st4[4*i+2] = t[2]; st4[4*i+3] = 0;           \
            continue;                                                                        \
        }                                                                                    \
        REAL dt = (REAL)p->dt;                                                               \
        REAL nvx = vi[0] + dt * (f[0] / mi + (REAL)p->g[0]);                                 \
        REAL nvy = vi[1] + dt * (f[1] / mi + (REAL)p->g[1]);                                 \
        REAL nvz = vi[2] + dt * (f[2] / mi + (REAL)p->g[2]);                                 \
        REAL nxp = xi + dt * nvx, nyp = yi + dt * nvy, nzp = zi + dt * nvz;                  \
        REAL inertia = (((REAL)0.4f * mi) * ri) * ri;                                        \
        REAL* po = pos_n + 4 * i; REAL* vo = vel_n + 4 * i; REAL* wo = omg_n + 4 * i;        \
        po[0] = nxp; po[1] = nyp; po[2] = nzp; po[3] = ri;                                   \
        vo[0] = nvx; vo[1] = nvy; vo[2] = nvz; vo[3] = mi;                                   \
        wo[0] = wi[0] + dt * (t[0] / inertia);                                               \
        wo[1] = wi[1] + dt * (t[1] / inertia);                                               \
        wo[2] = wi[2] + dt * (t[2] / inertia);                                               \
        wo[3] = wi[3];                                                                       \
        if (keys_n) keys_n[i] = sdo_cell_key(p, (float)nxp, (float)nyp, (float)nzp);         \
    }                                                                                        \
    return contacts;                                                                         \
}

SDO_DEFINE_STEP(float, sqrtf, fminf, fmaf, bits_f32, _f32)
SDO_DEFINE_STEP(double, sqrt, fmin, fma, bits_f64, _f64)

uint64_t sdo_contact_integrate(const sdo_params* p, uint32_t n,
                               const float* pos, const float* vel, const float* omg,
                               const uint32_t* cell_start,
                               float* pos_n, float* vel_n, float* omg_n, uint32_t* keys_n,
                               float* force4, float* torque4) {
    return contact_integrate_f32(p, n, pos, vel, omg, cell_start, pos_n, vel_n, omg_n,
                                 keys_n, force4, torque4, NULL, NULL, NULL, NULL);
}

uint64_t sdo_contact_integrate_f64(const sdo_params* p, uint32_t n,
                                   const double* pos, const double* vel, const double* omg,
                                   const uint32_t* cell_start,
                                   double* pos_n, double* vel_n, double* omg_n, uint32_t* keys_n,
                                   double* force4, double* torque4) {
    return contact_integrate_f64(p, n, pos, vel, omg, cell_start, pos_n, vel_n, omg_n,
                                 keys_n, force4, torque4, NULL, NULL, NULL, NULL);
}

static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : x > y;
}

uint64_t sdo_contact_pairs(const sdo_params* p, uint32_t n, const float* pos,
                           const float* omg, const uint32_t* cell_start,
                           uint64_t* out, uint64_t cap) {
    uint64_t cnt = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const float* pi = pos + 4 * (size_t)i;
        uint32_t idi;
        memcpy(&idi, omg + 4 * (size_t)i + 3, 4);
        int32_t cx = axis_cell(pi[0], p->lo[0], p->cell, p->nx);
        int32_t cy = axis_cell(pi[1], p->lo[1], p->cell, p->ny);
        int32_t z0 = axis_cell(pi[2] - p->cell * 1.00001f, p->lo[2], cell_z_of(p), p->nz);
        int32_t z1 = axis_cell(pi[2] + p->cell * 1.00001f, p->lo[2], cell_z_of(p), p->nz);
        for (int32_t ddx = -1; ddx <= 1; ++ddx) {
            int32_t X = cx + ddx;
            if (X < 0 || X >= p->nx) continue;
            for (int32_t ddy = -1; ddy <= 1; ++ddy) {
                int32_t Y = cy + ddy;
                if (Y < 0 || Y >= p->ny) continue;
                uint32_t col = (uint32_t)((X * p->ny + Y) * p->nz);
                for (uint32_t s = cell_start[col + (uint32_t)z0]; s < cell_start[col + (uint32_t)z1 + 1]; ++s) {
                    if (s == i) continue;
                    const float* pj = pos + 4 * (size_t)s;
                    float dx = pi[0] - pj[0], dy = pi[1] - pj[1], dz = pi[2] - pj[2];
                    float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                    float rs = pi[3] + pj[3];
                    if (!(d2 < rs * rs) || d2 == 0.0f) continue;
                    uint32_t idj;
                    memcpy(&idj, omg + 4 * (size_t)s + 3, 4);
                    if (idi < idj) {
                        if (cnt < cap) out[cnt] = ((uint64_t)idi << 32) | idj;
                        ++cnt;
                    }
                }
            }
        }
    }
    if (out && cnt <= cap) qsort(out, (size_t)cnt, sizeof(uint64_t), cmp_u64);
    return cnt;
}

int sdo_run(const sdo_params* p, uint32_t n, float* pos, float* vel, float* omg,
            int steps, int prepare) {
    size_t nc = (size_t)p->nx * p->ny * p->nz;
    float* pn = (float*)malloc(sizeof(float) * 12 * (size_t)(n ? n : 1));
    float *vn = pn + 4 * (size_t)n, *wn = vn + 4 * (size_t)n;
    uint32_t* keys = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
    uint32_t* cs = (uint32_t*)malloc(sizeof(uint32_t) * (nc + 1));
    if (!pn || !keys || !cs) {
        free(pn); free(keys); free(cs);
        return -1;
    }
    memcpy(pn, pos, 16 * (size_t)n);
    memcpy(vn, vel, 16 * (size_t)n);
    memcpy(wn, omg, 16 * (size_t)n);
    if (prepare) {
        for (uint32_t i = 0; i < n; ++i) keys[i] = sdo_cell_key(p, pn[4 * i], pn[4 * i + 1], pn[4 * i + 2]);
    }
    /* without `prepare` the caller's state is already cell-sorted; rebuild
     * its cell_start with an identity sort */
    else {
        for (uint32_t i = 0; i < n; ++i) keys[i] = sdo_cell_key(p, pos[4 * i], pos[4 * i + 1], pos[4 * i + 2]);
    }
    sdo_sort_reorder(p, n, pn, vn, wn, keys, NULL, pos, vel, omg, cs);
    for (int s = 0; s < steps; ++s) {
        sdo_contact_integrate(p, n, pos, vel, omg, cs, pn, vn, wn, keys, NULL, NULL);
        sdo_sort_reorder(p, n, pn, vn, wn, keys, NULL, pos, vel, omg, cs);
    }
    free(pn); free(keys); free(cs);
    return 0;
}

/* The FP64 twin of sdo_run, for the error statement of long runs: the same
 * contact law, walls and integrator in double (SDO_DEFINE_STEP), the cell
 * order taken from the float-rounded positions (the order only fixes the
 * summation order).  pos/vel/omg: n x 4 doubles in any order, ids[i] the
 * sphere id of row i; on return the state is cell-sorted and ids permuted
 * with it.  contacts (may be NULL) receives per step s < steps the
 * contact pairs of state s (the one that step integrates from). */
int sdo_run_f64(const sdo_params* p, uint32_t n, double* pos, double* vel, double* omg, uint32_t* ids, int steps,
                uint64_t* contacts) {
    /* contacts (may be NULL): steps entries, [s] = contact pairs of state s */
    size_t nc = (size_t)p->nx * p->ny * p->nz;
    double* pn = (double*)malloc(sizeof(double) * 12 * (size_t)(n ? n : 1));
    double *vn = pn + 4 * (size_t)n, *wn = vn + 4 * (size_t)n;
    uint32_t* k = (uint32_t*)malloc(sizeof(uint32_t) * 5 * (size_t)(n ? n : 1));
    uint32_t* cs = (uint32_t*)malloc(sizeof(uint32_t) * (nc + 1));
    if (!pn || !k || !cs) {
        free(pn); free(k); free(cs);
        return -1;
    }
    uint32_t *v = k + n, *tk = v + n, *tv = tk + n, *idn = tv + n;
    memcpy(pn, pos, 32 * (size_t)n);
    memcpy(vn, vel, 32 * (size_t)n);
    memcpy(wn, omg, 32 * (size_t)n);
    memcpy(idn, ids, 4 * (size_t)n);
    for (int s = 0; s <= steps; ++s) {
        /* sort the (next) state into cell order */
        for (uint32_t i = 0; i < n; ++i) {
            k[i] = sdo_cell_key(p, (float)pn[4 * i], (float)pn[4 * i + 1], (float)pn[4 * i + 2]);
            v[i] = i;
        }
        sdo_radix_sort_pairs(k, v, n, key_bits(p), tk, tv);
        for (uint32_t i = 0; i < n; ++i) {
            memcpy(pos + 4 * (size_t)i, pn + 4 * (size_t)v[i], 32);
            memcpy(vel + 4 * (size_t)i, vn + 4 * (size_t)v[i], 32);
            memcpy(omg + 4 * (size_t)i, wn + 4 * (size_t)v[i], 32);
            ids[i] = idn[v[i]];
        }
        memcpy(idn, ids, 4 * (size_t)n);
        uint32_t q = 0;
        for (uint32_t cc = 0; cc <= (uint32_t)nc; ++cc) {
            while (q < n && k[q] < cc) ++q;
            cs[cc] = q;
        }
        if (s == steps) break;
        uint64_t c = contact_integrate_f64(p, n, pos, vel, omg, cs, pn, vn, wn, NULL, NULL, NULL, NULL, NULL, NULL,
                                           NULL);
        if (contacts) contacts[s] = c / 2;
    }
    free(pn); free(k); free(cs);
    return 0;
}

/* ------------------------------------------------------ rigid clumps ----- */

uint64_t sdo_contact_integrate_bodies(const sdo_params* p, uint32_t n, const float* pos, const float* vel,
                                      const float* omg, const uint32_t* cell_start, const int32_t* body_of,
                                      float* pos_n, float* vel_n, float* omg_n, uint32_t* keys_n,
                                      float* force4, float* torque4, float* sf4, float* st4) {
    return contact_integrate_f32(p, n, pos, vel, omg, cell_start, pos_n, vel_n, omg_n, keys_n, force4, torque4,
                                 body_of, sf4, st4, NULL);
}

void sdo_slot_of(uint32_t n, const float* omg, uint32_t* slot_of) {
    for (uint32_t k = 0; k < n; ++k) slot_of[bits_f32(omg[4 * (size_t)k + 3]) & 0x7fffffffu] = k;
}

/* Rotation matrix (row-major) of a unit quaternion (s, x, y, z). */
static void quat_rot(float qs, float qx, float qy, float qz, float* R) {
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

/* One step of every rigid body: gather its spheres' contact forces and
 * torques (sphere-id order), gravity, symplectic Euler on momentum and
 * angular momentum, w = R I0^-1 R^T L (physics_update.cu:264-279 with a
 * proper inverse), normalised first-order quaternion update
 * q' = normalize(q + dt/2 (0, w) (x) q), then the spheres' next state and
 * cell keys.  binv12 holds I0^-1 as three rows of four floats. */
void sdo_body_step(const sdo_params* p, uint32_t nb, float* bpos4, float* bvel4, float* bquat4, float* bomg4,
                   float* bang4, const float* binv12, const uint32_t* first, const uint32_t* count,
                   const float* r0_4, const uint32_t* slot_of, const float* pos, const float* omg,
                   const float* sf4, const float* st4, float* pos_n, float* vel_n, float* omg_n,
                   uint32_t* keys_n) {
    for (uint32_t b = 0; b < nb; ++b) {
        float* bp = bpos4 + 4 * (size_t)b;
        float* bv = bvel4 + 4 * (size_t)b;
        float* bq = bquat4 + 4 * (size_t)b;
        float* bw = bomg4 + 4 * (size_t)b;
        float* bl = bang4 + 4 * (size_t)b;
        const float* I = binv12 + 12 * (size_t)b;
        const float x = bp[0], y = bp[1], z = bp[2], m = bp[3];
        float Fx = 0, Fy = 0, Fz = 0, Tx = 0, Ty = 0, Tz = 0;
        for (uint32_t k = 0; k < count[b]; ++k) {
            const uint32_t s = slot_of[first[b] + k];
            const float* ps = pos + 4 * (size_t)s;
            const float* fs = sf4 + 4 * (size_t)s;
            const float* ts = st4 + 4 * (size_t)s;
            const float rx = ps[0] - x, ry = ps[1] - y, rz = ps[2] - z;
            Fx = Fx + fs[0];
            Fy = Fy + fs[1];
            Fz = Fz + fs[2];
            Tx = Tx + (ry * fs[2] - rz * fs[1]);
            Ty = Ty + (rz * fs[0] - rx * fs[2]);
            Tz = Tz + (rx * fs[1] - ry * fs[0]);
            Tx = Tx + ts[0];
            Ty = Ty + ts[1];
            Tz = Tz + ts[2];
        }
        const float dt = p->dt;
        const float vx = bv[0] + dt * (Fx / m + p->g[0]);
        const float vy = bv[1] + dt * (Fy / m + p->g[1]);
        const float vz = bv[2] + dt * (Fz / m + p->g[2]);
        const float nxp = x + dt * vx, nyp = y + dt * vy, nzp = z + dt * vz;
        const float Lx = bl[0] + dt * Tx, Ly = bl[1] + dt * Ty, Lz = bl[2] + dt * Tz;
        float R[9], A[9], W[9];
        quat_rot(bq[0], bq[1], bq[2], bq[3], R);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c)
                A[3 * r + c] = (R[3 * r] * I[c] + R[3 * r + 1] * I[4 + c]) + R[3 * r + 2] * I[8 + c];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c)
                W[3 * r + c] = (A[3 * r] * R[3 * c] + A[3 * r + 1] * R[3 * c + 1]) + A[3 * r + 2] * R[3 * c + 2];
        const float wx = (W[0] * Lx + W[1] * Ly) + W[2] * Lz;
        const float wy = (W[3] * Lx + W[4] * Ly) + W[5] * Lz;
        const float wz = (W[6] * Lx + W[7] * Ly) + W[8] * Lz;
        const float qs = bq[0], qx = bq[1], qy = bq[2], qz = bq[3];
        const float h = 0.5f * dt;
        const float ds = -((wx * qx + wy * qy) + wz * qz);
        const float dx = qs * wx + (wy * qz - wz * qy);
        const float dy = qs * wy + (wz * qx - wx * qz);
        const float dz = qs * wz + (wx * qy - wy * qx);
        const float ns = qs + h * ds, nx = qx + h * dx, ny = qy + h * dy, nz = qz + h * dz;
        const float nrm = sqrtf((ns * ns + nx * nx) + (ny * ny + nz * nz));
        const float q0 = ns / nrm, q1 = nx / nrm, q2 = ny / nrm, q3 = nz / nrm;
        quat_rot(q0, q1, q2, q3, R);
        for (uint32_t k = 0; k < count[b]; ++k) {
            const uint32_t id = first[b] + k, s = slot_of[id];
            const float* r0 = r0_4 + 4 * (size_t)id;
            const float rx = (R[0] * r0[0] + R[1] * r0[1]) + R[2] * r0[2];
            const float ry = (R[3] * r0[0] + R[4] * r0[1]) + R[5] * r0[2];
            const float rz = (R[6] * r0[0] + R[7] * r0[1]) + R[8] * r0[2];
            float* po = pos_n + 4 * (size_t)s;
            float* vo = vel_n + 4 * (size_t)s;
            float* wo = omg_n + 4 * (size_t)s;
            po[0] = nxp + rx;
            po[1] = nyp + ry;
            po[2] = nzp + rz;
            po[3] = pos[4 * (size_t)s + 3];
            vo[0] = vx + (wy * rz - wz * ry);
            vo[1] = vy + (wz * rx - wx * rz);
            vo[2] = vz + (wx * ry - wy * rx);
            vo[3] = m;
            wo[0] = wx;
            wo[1] = wy;
            wo[2] = wz;
            wo[3] = omg[4 * (size_t)s + 3];
            keys_n[s] = sdo_cell_key(p, po[0], po[1], po[2]);
        }
        bp[0] = nxp; bp[1] = nyp; bp[2] = nzp;
        bv[0] = vx; bv[1] = vy; bv[2] = vz;
        bl[0] = Lx; bl[1] = Ly; bl[2] = Lz;
        bq[0] = q0; bq[1] = q1; bq[2] = q2; bq[3] = q3;
        bw[0] = wx; bw[1] = wy; bw[2] = wz;
    }
}

int sdo_run_full(const sdo_params* p, uint32_t n, float* pos, float* vel, float* omg, int steps,
                 uint32_t nb, float* bpos4, float* bvel4, float* bquat4, float* bomg4, float* bang4,
                 const float* binv12, const uint32_t* first, const uint32_t* count, const float* r0_4,
                 const int32_t* body_of, sdo_mesh* mesh) {
    size_t nc = (size_t)p->nx * p->ny * p->nz;
    float* buf = (float*)malloc(sizeof(float) * 20 * (size_t)(n ? n : 1));
    uint32_t* keys = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
    uint32_t* slot = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
    uint32_t* cs = (uint32_t*)malloc(sizeof(uint32_t) * (nc + 1));
    if (!buf || !keys || !slot || !cs) {
        free(buf); free(keys); free(slot); free(cs);
        return -1;
    }
    float *pn = buf, *vn = pn + 4 * (size_t)n, *wn = vn + 4 * (size_t)n, *sf = wn + 4 * (size_t)n,
          *st = sf + 4 * (size_t)n;
    memcpy(pn, pos, 16 * (size_t)n);
    memcpy(vn, vel, 16 * (size_t)n);
    memcpy(wn, omg, 16 * (size_t)n);
    sdo_cell_keys(p, n, pos, keys);
    sdo_sort_reorder(p, n, pn, vn, wn, keys, NULL, pos, vel, omg, cs);
    sdo_slot_of(n, omg, slot);
    for (int s = 0; s < steps; ++s) {
        contact_integrate_f32(p, n, pos, vel, omg, cs, pn, vn, wn, keys, NULL, NULL, body_of, sf, st, mesh);
        if (nb)
            sdo_body_step(p, nb, bpos4, bvel4, bquat4, bomg4, bang4, binv12, first, count, r0_4, slot, pos, omg, sf,
                          st, pn, vn, wn, keys);
        sdo_sort_reorder(p, n, pn, vn, wn, keys, NULL, pos, vel, omg, cs);
        sdo_slot_of(n, omg, slot);
        if (mesh && mesh->ntri) sdo_mesh_advance(mesh->state, 1);
    }
    free(buf); free(keys); free(slot); free(cs);
    return 0;
}


int sdo_run_bodies(const sdo_params* p, uint32_t n, float* pos, float* vel, float* omg, int steps,
                   uint32_t nb, float* bpos4, float* bvel4, float* bquat4, float* bomg4, float* bang4,
                   const float* binv12, const uint32_t* first, const uint32_t* count, const float* r0_4,
                   const int32_t* body_of) {
    return sdo_run_full(p, n, pos, vel, omg, steps, nb, bpos4, bvel4, bquat4, bomg4, bang4, binv12, first, count,
                        r0_4, body_of, NULL);
}

/* The mesh pose of the next step (advance != 0): q <- normalize(dq (x) q),
 * then R <- R(q); the kernel mesh_advance_kernel's expressions. */
void sdo_mesh_advance(float* S, int advance) {
    float qs = S[16], qx = S[17], qy = S[18], qz = S[19];
    if (advance) {
        const float ds = S[20], dx = S[21], dy = S[22], dz = S[23];
        const float ns = ds * qs - ((dx * qx + dy * qy) + dz * qz);
        const float nx = (ds * qx + qs * dx) + (dy * qz - dz * qy);
        const float ny = (ds * qy + qs * dy) + (dz * qx - dx * qz);
        const float nz = (ds * qz + qs * dz) + (dx * qy - dy * qx);
        const float nrm = sqrtf((ns * ns + nx * nx) + (ny * ny + nz * nz));
        qs = ns / nrm; qx = nx / nrm; qy = ny / nrm; qz = nz / nrm;
        S[16] = qs; S[17] = qx; S[18] = qy; S[19] = qz;
    }
    quat_rot(qs, qx, qy, qz, S);
}
