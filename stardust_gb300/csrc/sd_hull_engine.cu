// sd_hull_engine.cu -- convex-hull scenes behind the engine handle.
//
// A hull body is the convex hull of a point set (the reference's Hull
// primitive, sandbox/primitives.hpp:37-57, and its prototype narrow phase,
// sandbox/testGJK.cu).  At add time the points are reduced to a principal
// frame: centre = mean of the points, inertia of the points as equal masses
// diagonalised by Jacobi rotations (double), vertices stored in that frame,
// so the integrator needs only a diagonal inverse inertia.
//
// The step, captured as one CUDA graph per step parity (the partner lists of
// consecutive steps alternate between two buffers, so the previous step's
// GJK directions can seed the next step):
//   world AABBs -> LBVH build -> partner lists -> [seeds] -> GJK/EPA per
//   entry -> segmented force sum + integration per body -> step counters.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/stardust.h"
#include "sd_engine_impl.h"
#include "sd_internal.h"

namespace {

#define HULL_CUDA(h, call)                                           \
    do {                                                             \
        cudaError_t _e = (call);                                     \
        if (_e != cudaSuccess) return sd_cuda_fail((h), _e, #call);  \
    } while (0)

template <typename T>
sd_status halloc(sd_engine* h, T** p, size_t count) {
    void* q = nullptr;
    sd_status s = sd_alloc_bytes(h, &q, std::max<size_t>(count, 1) * sizeof(T));
    *p = static_cast<T*>(q);
    return s;
}

// Cyclic Jacobi eigen-decomposition of a symmetric 3x3 matrix (row-major):
// A = V diag(w) V^T, V's columns the eigenvectors.
void jacobi3(const double* Ain, double* w, double* V) {
    double A[9];
    std::memcpy(A, Ain, sizeof A);
    for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 50; ++sweep) {
        const double off = A[1] * A[1] + A[2] * A[2] + A[5] * A[5];
        const double dia = A[0] * A[0] + A[4] * A[4] + A[8] * A[8];
        if (off <= 1e-30 * dia || off == 0.0) break;
        for (int p = 0; p < 2; ++p) {
            for (int q = p + 1; q < 3; ++q) {
                const double apq = A[3 * p + q];
                if (apq == 0.0) continue;
                const double theta = (A[3 * q + q] - A[3 * p + p]) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                // A <- J^T A J with J the rotation in the (p, q) plane
                for (int k = 0; k < 3; ++k) {
                    const double akp = A[3 * k + p], akq = A[3 * k + q];
                    A[3 * k + p] = c * akp - s * akq;
                    A[3 * k + q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; ++k) {
                    const double apk = A[3 * p + k], aqk = A[3 * q + k];
                    A[3 * p + k] = c * apk - s * aqk;
                    A[3 * q + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; ++k) {
                    const double vkp = V[3 * k + p], vkq = V[3 * k + q];
                    V[3 * k + p] = c * vkp - s * vkq;
                    V[3 * k + q] = s * vkp + c * vkq;
                }
            }
        }
    }
    w[0] = A[0];
    w[1] = A[4];
    w[2] = A[8];
}

void quat_to_mat(const double* q, double* R) {
    const double s = q[0], x = q[1], y = q[2], z = q[3];
    R[0] = 1 - 2 * (y * y + z * z); R[1] = 2 * (x * y - s * z); R[2] = 2 * (x * z + s * y);
    R[3] = 2 * (x * y + s * z); R[4] = 1 - 2 * (x * x + z * z); R[5] = 2 * (y * z - s * x);
    R[6] = 2 * (x * z - s * y); R[7] = 2 * (y * z + s * x); R[8] = 1 - 2 * (x * x + y * y);
}

// Shepperd's method; returns (s, x, y, z) with s >= 0.
void mat_to_quat(const double* R, double* q) {
    const double t = R[0] + R[4] + R[8];
    if (t > 0) {
        const double s = std::sqrt(t + 1.0) * 2;
        q[0] = 0.25 * s; q[1] = (R[7] - R[5]) / s; q[2] = (R[2] - R[6]) / s; q[3] = (R[3] - R[1]) / s;
    } else if (R[0] > R[4] && R[0] > R[8]) {
        const double s = std::sqrt(1.0 + R[0] - R[4] - R[8]) * 2;
        q[0] = (R[7] - R[5]) / s; q[1] = 0.25 * s; q[2] = (R[1] + R[3]) / s; q[3] = (R[2] + R[6]) / s;
    } else if (R[4] > R[8]) {
        const double s = std::sqrt(1.0 + R[4] - R[0] - R[8]) * 2;
        q[0] = (R[2] - R[6]) / s; q[1] = (R[1] + R[3]) / s; q[2] = 0.25 * s; q[3] = (R[5] + R[7]) / s;
    } else {
        const double s = std::sqrt(1.0 + R[8] - R[0] - R[4]) * 2;
        q[0] = (R[3] - R[1]) / s; q[1] = (R[2] + R[6]) / s; q[2] = (R[5] + R[7]) / s; q[3] = 0.25 * s;
    }
    const double n = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    for (int k = 0; k < 4; ++k) q[k] /= (q[0] < 0 ? -n : n);
}

sd_status build_hull_graphs(sd_engine* h, float dt) {
    HullScene& S = h->hull;
    for (int k = 0; k < 2; ++k) {
        if (S.graph[k]) {
            cudaGraphExecDestroy(S.graph[k]);
            S.graph[k] = nullptr;
        }
        if (S.graph_refit[k]) {
            cudaGraphExecDestroy(S.graph_refit[k]);
            S.graph_refit[k] = nullptr;
        }
    }
    S.P.dt = dt;
    for (int g2 = 0; g2 < 4; ++g2) {
        const int par = g2 & 1;
        const bool full = g2 < 2;
        sd::HullBuffers H = S.H;
        H.off = S.off[par];
        H.partners = S.partners[par];
        H.dir = S.dir[par];
        H.prev_off = S.off[par ^ 1];
        H.prev_partners = S.partners[par ^ 1];
        H.prev_dir = S.dir[par ^ 1];
        H.keep_anchor = S.seed_mode == SD_GJK_SEED_LEARNED;
        cudaGraph_t g = nullptr;
        HULL_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = sd::hull_aabb_async(H, h->stream);
        if (e == cudaSuccess)
            e = full ? sd::lbvh_build_async(S.tree, H.lo, H.hi, h->stream)
                     : sd::lbvh_refit_async(S.tree, H.lo, H.hi, h->stream);
        if (e == cudaSuccess) e = sd::lbvh_partners_async(S.tree, H.off, H.partners, H.self, H.cap, h->stream);
        if (e == cudaSuccess) e = sd::hull_seed_async(H, (uint32_t)S.seed_mode, h->stream);
        if (e == cudaSuccess && S.seed_mode == SD_GJK_SEED_LEARNED)
            e = sd::mlp_forward_async(S.mlp, H.feat, H.seeds, H.off + H.nb, H.cap, true, h->stream);
        if (e == cudaSuccess) e = sd::hull_narrow_async(S.P, H, h->stream);
        if (e == cudaSuccess) e = sd::hull_integrate_async(S.P, H, h->stream);
        if (e == cudaSuccess) e = sd::hull_stats_async(H, S.stats, h->stream);
        cudaError_t e2 = cudaStreamEndCapture(h->stream, &g);
        if (e != cudaSuccess) return sd_cuda_fail(h, e, "capturing the hull step");
        if (e2 != cudaSuccess) return sd_cuda_fail(h, e2, "cudaStreamEndCapture");
        cudaError_t e3 = cudaGraphInstantiate(full ? &S.graph[par] : &S.graph_refit[par], g, 0);
        if (full) S.graph_kernels = graph_kernel_nodes(g);
        cudaGraphDestroy(g);
        if (e3 != cudaSuccess) return sd_cuda_fail(h, e3, "cudaGraphInstantiate");
    }
    S.graph_dt = dt;
    S.graph_valid = true;
    S.graph_epoch = sd_tune_epoch();
    return SD_OK;
}

}  // namespace

void hull_release(sd_engine* h) {
    HullScene& S = h->hull;
    for (int k = 0; k < 2; ++k) {
        if (S.graph[k]) cudaGraphExecDestroy(S.graph[k]);
        S.graph[k] = nullptr;
        if (S.graph_refit[k]) cudaGraphExecDestroy(S.graph_refit[k]);
        S.graph_refit[k] = nullptr;
    }
    S.graph_valid = false;
    S.tree_built = false;
    S.H = sd::HullBuffers{};
    S.tree = sd::Lbvh{};
    for (int k = 0; k < 2; ++k) {
        S.off[k] = S.partners[k] = nullptr;
        S.dir[k] = nullptr;
    }
    S.stats = nullptr;
    S.mlp = sd::MlpState{};
}

sd_status hull_prepare(sd_engine* h) {
    HullScene& S = h->hull;
    const sd_config& c = h->cfg;
    const uint32_t nb = (uint32_t)S.pos.size();
    // box: as the sphere engine derives it (explicit box, else [0, domain]^3)
    const bool box_given = c.box_hi[0] != 0.f || c.box_hi[1] != 0.f || c.box_hi[2] != 0.f;
    for (int a = 0; a < 3; ++a) {
        S.P.lo[a] = box_given ? c.box_lo[a] : 0.f;
        S.P.hi[a] = box_given ? c.box_hi[a] : c.domain;
        S.P.g[a] = c.gravity[a];
    }
    S.P.kn = c.kn;
    S.P.damp = sd_damp_from(c.kn, c.restitution);
    S.P.mu = c.mu;
    S.P.walls = c.walls;
    int ndev = 0;
    cudaError_t ce = cudaGetDeviceCount(&ndev);
    if (ce != cudaSuccess || ndev == 0)
        return sd_fail(h, SD_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(ce));
    if (h->device >= ndev) return sd_fail(h, SD_ERR_INVALID_ARG, "cuda_device out of range");
    HULL_CUDA(h, cudaSetDevice(h->device));
    HULL_CUDA(h, cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    sd::HullBuffers& H = S.H;
    H.nb = nb;
    const uint64_t cap = std::max<uint64_t>(c.pair_capacity, 40ull * nb);
    H.cap = cap;
    const size_t nv = S.verts.size();
    sd_status s;
    if ((s = halloc(h, &H.pos, nb)) || (s = halloc(h, &H.vel, nb)) || (s = halloc(h, &H.quat, nb)) ||
        (s = halloc(h, &H.omg, nb)) || (s = halloc(h, &H.ang, nb)) || (s = halloc(h, &H.iinv, nb)) ||
        (s = halloc(h, &H.vstart, nb)) || (s = halloc(h, &H.vcount, nb)) || (s = halloc(h, &H.verts, nv)) ||
        (s = halloc(h, &H.lo, nb)) || (s = halloc(h, &H.hi, nb)) || (s = halloc(h, &H.ext, 2 * (size_t)nb)) ||
        (s = halloc(h, &H.self, cap)) || (s = halloc(h, &H.ef, cap)) || (s = halloc(h, &H.et, cap)) ||
        (s = halloc(h, &H.info, cap)) || (s = halloc(h, &H.seeds, cap)) || (s = halloc(h, &H.feat, 16 * cap)) ||
        (s = halloc(h, &S.stats, 4)) || (s = halloc(h, &H.ucount, nb)) || (s = halloc(h, &H.upos, (size_t)nb + 1)) ||
        (s = halloc(h, &H.ulist, cap / 2 + 1)) || (s = halloc(h, &H.uscan, sd::scan_scratch_words(nb) + 1)) ||
        (s = halloc(h, &H.teach, cap)) || (s = halloc(h, &S.teach_flag, 4)) ||
        (s = halloc(h, &S.teach_feat, 16 * (cap / 2 + 1))) || (s = halloc(h, &S.teach_tgt, cap / 2 + 1)) ||
        (s = halloc(h, &S.teach_flags, cap)) || (s = halloc(h, &S.teach_pos, cap)) ||
        (s = halloc(h, &S.teach_scan, sd::scan_scratch_words((uint32_t)cap) + 1)) ||
        (s = halloc(h, &S.teach_total, 1)) ||
        (s = halloc(h, &H.hit_count, 1)) || (s = halloc(h, &H.hits, cap / 2 + 1)) ||
        (s = halloc(h, &H.hit_keys, cap / 2 + 1)))
        return s;
    H.teach_on = S.teach_flag;
    for (int k = 0; k < 2; ++k)
        if ((s = halloc(h, &S.off[k], (size_t)nb + 1)) || (s = halloc(h, &S.partners[k], cap)) ||
            (s = halloc(h, &S.dir[k], cap)))
            return s;
    if (h->cfg.flags & SD_FLAG_RECORD)
        if ((s = halloc(h, &H.force, nb)) || (s = halloc(h, &H.torque, nb))) return s;
    void* tm = nullptr;
    if ((s = sd_alloc_bytes(h, &tm, sd::lbvh_scratch_bytes(nb)))) return s;
    sd::lbvh_carve(tm, nb, &S.tree);
    void* mm = nullptr;
    if ((s = sd_alloc_bytes(h, &mm, sd::mlp_state_bytes()))) return s;
    S.mlp = sd::mlp_carve(mm);
    HULL_CUDA(h, sd::mlp_init_kernels());
    cudaStream_t st = h->stream;
    HULL_CUDA(h, cudaMemcpyAsync(H.pos, S.pos.data(), 16 * (size_t)nb, cudaMemcpyHostToDevice, st));
    HULL_CUDA(h, cudaMemcpyAsync(H.vel, S.vel.data(), 16 * (size_t)nb, cudaMemcpyHostToDevice, st));
    HULL_CUDA(h, cudaMemcpyAsync(H.quat, S.quat.data(), 16 * (size_t)nb, cudaMemcpyHostToDevice, st));
    HULL_CUDA(h, cudaMemcpyAsync(H.omg, S.omg.data(), 16 * (size_t)nb, cudaMemcpyHostToDevice, st));
    HULL_CUDA(h, cudaMemcpyAsync(H.ang, S.ang.data(), 16 * (size_t)nb, cudaMemcpyHostToDevice, st));
    HULL_CUDA(h, cudaMemcpyAsync(H.iinv, S.iinv.data(), 16 * (size_t)nb, cudaMemcpyHostToDevice, st));
    HULL_CUDA(h, cudaMemcpyAsync(H.vstart, S.vstart.data(), 4 * (size_t)nb, cudaMemcpyHostToDevice, st));
    HULL_CUDA(h, cudaMemcpyAsync(H.vcount, S.vcount.data(), 4 * (size_t)nb, cudaMemcpyHostToDevice, st));
    HULL_CUDA(h, cudaMemcpyAsync(H.verts, S.verts.data(), 16 * nv, cudaMemcpyHostToDevice, st));
    for (int k = 0; k < 2; ++k) HULL_CUDA(h, cudaMemsetAsync(S.off[k], 0, 4 * ((size_t)nb + 1), st));
    HULL_CUDA(h, cudaMemsetAsync(S.tree.status, 0, 16, st));
    HULL_CUDA(h, cudaMemsetAsync(S.stats, 0, 32, st));
    HULL_CUDA(h, cudaMemsetAsync(S.mlp.status, 0, 16, st));
    {
        const uint32_t flags[4] = {0u, 0u, 1u, 0u};  // training off; the constants 0 and 1 to copy from
        HULL_CUDA(h, cudaMemcpyAsync(S.teach_flag, flags, sizeof flags, cudaMemcpyHostToDevice, st));
    }
    {
        // network initialisation: uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) for
        // the hidden layers from a fixed SplitMix64 stream; the last layer
        // starts at zero, so the untrained residual network returns the
        // previous direction
        std::vector<float> w(sd::mlp_param_count(), 0.0f);
        uint64_t z = 0x5eed5eedull;
        auto u01 = [&z]() {
            uint64_t x = (z += 0x9e3779b97f4a7c15ull);
            x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
            x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
            x ^= x >> 31;
            return (double)(x >> 11) * (1.0 / 9007199254740992.0);
        };
        const int in = 16, hid = 64;
        for (int i = 0; i < hid * in; ++i) w[i] = (float)((2 * u01() - 1) / std::sqrt(12.0));
        const int w2 = hid * in + hid;
        for (int i = 0; i < hid * hid; ++i) w[w2 + i] = (float)((2 * u01() - 1) / std::sqrt((double)hid));
        HULL_CUDA(h, sd::mlp_set_params_async(S.mlp, w.data(), st));
        S.mlp_step = 0;
        HULL_CUDA(h, cudaStreamSynchronize(st));
    }
    S.parity = 0;
    S.graph_valid = false;
    S.tree_built = false;
    h->prepared = true;
    h->steps = 0;
    return SD_OK;
}

sd_status hull_step(sd_engine* h, float dt, int32_t n_steps) {
    HullScene& S = h->hull;
    HULL_CUDA(h, cudaSetDevice(h->device));
    if (!S.graph_valid || S.graph_dt != dt || S.graph_epoch != sd_tune_epoch()) {
        sd_status s = build_hull_graphs(h, dt);
        if (s) return s;
    }
    const bool online = S.train_every > 0 && S.seed_mode == SD_GJK_SEED_LEARNED;
    for (int32_t k = 0; k < n_steps; ++k) {
        const uint64_t step = h->steps + (uint64_t)k;
        const bool train = online && step % (uint64_t)S.train_every == 0;
        if (train)  // this step logs the max-margin targets of its separated pairs
            HULL_CUDA(h, cudaMemcpyAsync(S.teach_flag, S.teach_flag + 2, 4, cudaMemcpyDeviceToDevice, h->stream));
        // the tree is built again every lbvh_rebuild steps and refitted in
        // between: the pair sets are exact either way
        const bool full = !S.tree_built || step % (uint64_t)sd::lbvh_rebuild_every() == 0;
        HULL_CUDA(h, cudaGraphLaunch(full ? S.graph[S.parity] : S.graph_refit[S.parity], h->stream));
        S.tree_built = true;
        if (train) {
            HULL_CUDA(h, cudaMemcpyAsync(S.teach_flag, S.teach_flag + 1, 4, cudaMemcpyDeviceToDevice, h->stream));
            // Adam on the step's samples (features, targets) gathered in entry
            // order, on the GPU between steps; their count stays on the
            // device.  Adam is invariant to the loss scale, so the mean's
            // divisor is nominal
            HULL_CUDA(h, sd::hull_teach_compact_async(S.H, S.off[S.parity] + S.H.nb, S.teach_feat, S.teach_tgt,
                                                      S.teach_flags, S.teach_pos, S.teach_scan, S.teach_total,
                                                      h->stream));
            for (int32_t it = 0; it < S.train_iters; ++it) {
                S.mlp_step += 1;
                HULL_CUDA(h, sd::mlp_train_async(S.mlp, S.teach_feat, S.teach_tgt, (uint32_t)(S.H.cap / 2 + 1),
                                                 S.H.nb, S.train_lr, S.mlp_step, true, h->stream, S.teach_total));
            }
        }
        S.parity ^= 1;
    }
    h->steps += (uint64_t)n_steps;
    return SD_OK;
}

// The narrow phase alone, for timing between steps: GJK, EPA and the
// contact forces of the last step's candidate lists at the current bodies,
// into the entry buffers.  No body changes; the entry results it rewrites
// (status, forces, directions) are rewritten by the next step, and its
// directions only seed that step's GJK where seeding is on (seeds move
// iteration counts, never the state).
sd_status hull_launch_narrow(sd_engine* h) {
    HullScene& S = h->hull;
    if (!S.graph_valid || h->steps == 0) return sd_fail(h, SD_ERR_STATE, "step the hull scene once first");
    HULL_CUDA(h, cudaSetDevice(h->device));
    const int par = S.parity ^ 1;  // the buffers of the last step
    sd::HullBuffers H = S.H;
    H.off = S.off[par];
    H.partners = S.partners[par];
    H.dir = S.dir[par];
    H.prev_off = S.off[par ^ 1];
    H.prev_partners = S.partners[par ^ 1];
    H.prev_dir = S.dir[par ^ 1];
    H.keep_anchor = S.seed_mode == SD_GJK_SEED_LEARNED;
    HULL_CUDA(h, sd::hull_narrow_async(S.P, H, h->stream));
    return SD_OK;
}

sd_status hull_stats(sd_engine* h, sd_stats* out) {
    HullScene& S = h->hull;
    const uint32_t nb = (uint32_t)S.pos.size();
    out->n_bodies = nb;
    out->n_spheres = 0;
    out->steps = h->steps;
    out->step_kernels = S.graph_valid ? S.graph_kernels : 0;
    if (!h->prepared) return SD_OK;
    std::vector<float4> x(nb), v(nb), w(nb), L(nb);
    unsigned long long c[4] = {0, 0, 0, 0};
    uint32_t err[2] = {0, 0};
    cudaStream_t st = h->stream;
    HULL_CUDA(h, cudaMemcpyAsync(x.data(), S.H.pos, 16 * (size_t)nb, cudaMemcpyDeviceToHost, st));
    HULL_CUDA(h, cudaMemcpyAsync(v.data(), S.H.vel, 16 * (size_t)nb, cudaMemcpyDeviceToHost, st));
    HULL_CUDA(h, cudaMemcpyAsync(w.data(), S.H.omg, 16 * (size_t)nb, cudaMemcpyDeviceToHost, st));
    HULL_CUDA(h, cudaMemcpyAsync(L.data(), S.H.ang, 16 * (size_t)nb, cudaMemcpyDeviceToHost, st));
    HULL_CUDA(h, cudaMemcpyAsync(c, S.stats, sizeof c, cudaMemcpyDeviceToHost, st));
    HULL_CUDA(h, cudaMemcpyAsync(err, S.tree.status, 4, cudaMemcpyDeviceToHost, st));
    HULL_CUDA(h, cudaStreamSynchronize(st));
    double ke = 0, p[3] = {0, 0, 0};
    for (uint32_t b = 0; b < nb; ++b) {
        const double m = x[b].w;
        ke += 0.5 * m * ((double)v[b].x * v[b].x + (double)v[b].y * v[b].y + (double)v[b].z * v[b].z);
        ke += 0.5 * ((double)w[b].x * L[b].x + (double)w[b].y * L[b].y + (double)w[b].z * L[b].z);
        p[0] += m * v[b].x;
        p[1] += m * v[b].y;
        p[2] += m * v[b].z;
    }
    out->kinetic_energy = ke;
    for (int a = 0; a < 3; ++a) out->momentum[a] = p[a];
    out->contacts = c[2];
    out->gjk_pairs = c[0];
    out->gjk_iters = c[1];
    out->epa_iters = c[3];
    out->device_errors = err[0];
    return SD_OK;
}

sd_status hull_get_bodies(sd_engine* h, int32_t field, void* host_dst, size_t bytes) {
    HullScene& S = h->hull;
    const size_t nb = S.pos.size();
    if (bytes != 16 * nb) return sd_fail(h, SD_ERR_INVALID_ARG, "bytes must be n_bodies * 16");
    const float4* src = nullptr;
    switch (field) {
        case SD_BODY_POSITION: src = S.H.pos; break;
        case SD_BODY_VELOCITY: src = S.H.vel; break;
        case SD_BODY_QUATERNION: src = S.H.quat; break;
        case SD_BODY_OMEGA: src = S.H.omg; break;
        case SD_BODY_ANGMOM: src = S.H.ang; break;
        case SD_BODY_HULL_INV_INERTIA: src = S.H.iinv; break;
        case SD_BODY_FORCE: src = S.H.force; break;
        case SD_BODY_TORQUE: src = S.H.torque; break;
        default: return sd_fail(h, SD_ERR_INVALID_ARG, "unknown body field for a hull scene");
    }
    if (!src) return sd_fail(h, SD_ERR_STATE, "forces and torques need SD_FLAG_RECORD");
    HULL_CUDA(h, cudaMemcpyAsync(host_dst, src, bytes, cudaMemcpyDeviceToHost, h->stream));
    HULL_CUDA(h, cudaStreamSynchronize(h->stream));
    return SD_OK;
}

extern "C" {

sd_status sd_engine_add_hull(sd_engine* h, uint32_t n_points, const float* pts4, float mass, const float pos[3],
                             const float quat[4], const float vel[3], const float omega[3]) {
    if (!h || !pts4 || !pos || !vel) return sd_fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (h->prepared) return sd_fail(h, SD_ERR_STATE, "hulls cannot be added after prepare");
    if (n_points < 1 || n_points > 255) return sd_fail(h, SD_ERR_INVALID_ARG, "a hull needs 1..255 points");
    if (!(mass > 0.0f) || !std::isfinite(mass)) return sd_fail(h, SD_ERR_INVALID_ARG, "hull mass must be > 0");
    HullScene& S = h->hull;
    if (S.verts.size() + n_points >= 0x7fffffffull) return sd_fail(h, SD_ERR_CAPACITY, "too many hull vertices");
    double c[3] = {0, 0, 0};
    for (uint32_t k = 0; k < n_points; ++k)
        for (int a = 0; a < 3; ++a) {
            const float x = pts4[4 * k + a];
            if (!std::isfinite(x)) return sd_fail(h, SD_ERR_INVALID_ARG, "hull point not finite");
            c[a] += x;
        }
    for (int a = 0; a < 3; ++a) c[a] /= n_points;
    const double ms = (double)mass / n_points;
    double I[9] = {0};
    for (uint32_t k = 0; k < n_points; ++k) {
        const double r[3] = {pts4[4 * k] - c[0], pts4[4 * k + 1] - c[1], pts4[4 * k + 2] - c[2]};
        const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) I[3 * a + b] += ms * ((a == b ? r2 : 0.0) - r[a] * r[b]);
    }
    double lam[3], E[9];
    jacobi3(I, lam, E);
    const double det = E[0] * (E[4] * E[8] - E[5] * E[7]) - E[1] * (E[3] * E[8] - E[5] * E[6]) +
                       E[2] * (E[3] * E[7] - E[4] * E[6]);
    if (det < 0)
        for (int k = 0; k < 3; ++k) E[3 * k + 2] = -E[3 * k + 2];
    const double lmax = std::max(lam[0], std::max(lam[1], lam[2]));
    if (!(lmax > 0.0)) {
        // a single point: give it the inertia of a small ball
        lam[0] = lam[1] = lam[2] = 1e-12 * mass;
    }
    for (int k = 0; k < 3; ++k) lam[k] = std::max(lam[k], 1e-3 * std::max(lmax, 1e-30));
    double qu[4] = {1, 0, 0, 0};
    if (quat) {
        const double n = std::sqrt((double)quat[0] * quat[0] + (double)quat[1] * quat[1] +
                                   (double)quat[2] * quat[2] + (double)quat[3] * quat[3]);
        if (!(n > 0)) return sd_fail(h, SD_ERR_INVALID_ARG, "hull quaternion is zero");
        for (int k = 0; k < 4; ++k) qu[k] = quat[k] / n;
    }
    double Ru[9], Rw[9];
    quat_to_mat(qu, Ru);
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) Rw[3 * a + b] = Ru[3 * a] * E[b] + Ru[3 * a + 1] * E[3 + b] + Ru[3 * a + 2] * E[6 + b];
    double qw[4];
    mat_to_quat(Rw, qw);
    quat_to_mat(qw, Rw);  // the rotation the device will rebuild from q
    const uint32_t vs = (uint32_t)S.verts.size();
    double rho = 0;
    for (uint32_t k = 0; k < n_points; ++k) {
        const double r[3] = {pts4[4 * k] - c[0], pts4[4 * k + 1] - c[1], pts4[4 * k + 2] - c[2]};
        double v[3];
        for (int b = 0; b < 3; ++b) v[b] = E[b] * r[0] + E[3 + b] * r[1] + E[6 + b] * r[2];  // E^T r
        rho = std::max(rho, std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]));
        S.verts.push_back(make_float4((float)v[0], (float)v[1], (float)v[2], 0.f));
    }
    double com[3];
    for (int a = 0; a < 3; ++a) com[a] = pos[a] + Ru[3 * a] * c[0] + Ru[3 * a + 1] * c[1] + Ru[3 * a + 2] * c[2];
    const double w[3] = {omega ? omega[0] : 0.0, omega ? omega[1] : 0.0, omega ? omega[2] : 0.0};
    double wb[3], Lb[3], L[3];
    for (int b = 0; b < 3; ++b) wb[b] = Rw[b] * w[0] + Rw[3 + b] * w[1] + Rw[6 + b] * w[2];  // Rw^T w
    for (int b = 0; b < 3; ++b) Lb[b] = lam[b] * wb[b];
    for (int a = 0; a < 3; ++a) L[a] = Rw[3 * a] * Lb[0] + Rw[3 * a + 1] * Lb[1] + Rw[3 * a + 2] * Lb[2];
    S.pos.push_back(make_float4((float)com[0], (float)com[1], (float)com[2], mass));
    S.vel.push_back(make_float4(vel[0], vel[1], vel[2], 0.f));
    S.quat.push_back(make_float4((float)qw[0], (float)qw[1], (float)qw[2], (float)qw[3]));
    S.omg.push_back(make_float4((float)w[0], (float)w[1], (float)w[2], 0.f));
    S.ang.push_back(make_float4((float)L[0], (float)L[1], (float)L[2], 0.f));
    S.iinv.push_back(make_float4((float)(1.0 / lam[0]), (float)(1.0 / lam[1]), (float)(1.0 / lam[2]), (float)rho));
    S.vstart.push_back(vs);
    S.vcount.push_back(n_points);
    return SD_OK;
}

sd_status sd_engine_get_hull_shapes(sd_engine* h, uint32_t* vstart, uint32_t* vcount, float* verts4,
                                    uint64_t verts_cap, uint64_t* n_verts) {
    if (!h || !n_verts) return sd_fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    HullScene& S = h->hull;
    *n_verts = S.verts.size();
    if (vstart) std::memcpy(vstart, S.vstart.data(), 4 * S.vstart.size());
    if (vcount) std::memcpy(vcount, S.vcount.data(), 4 * S.vcount.size());
    if (verts4) {
        if (verts_cap < S.verts.size()) return sd_fail(h, SD_ERR_CAPACITY, "verts_cap smaller than the vertex count");
        std::memcpy(verts4, S.verts.data(), 16 * S.verts.size());
    }
    return SD_OK;
}

sd_status sd_engine_set_gjk_seed(sd_engine* h, int32_t mode) {
    if (!h) return sd_fail(nullptr, SD_ERR_INVALID_ARG, "NULL engine");
    if (mode != SD_GJK_SEED_PLAIN && mode != SD_GJK_SEED_LEARNED && mode != SD_GJK_SEED_PREVIOUS)
        return sd_fail(h, SD_ERR_INVALID_ARG, "unknown GJK seed mode");
    h->hull.seed_mode = mode;
    h->hull.graph_valid = false;
    return SD_OK;
}

sd_status sd_engine_set_gjk_training(sd_engine* h, int32_t every, int32_t iters, float lr) {
    if (!h) return sd_fail(nullptr, SD_ERR_INVALID_ARG, "NULL engine");
    if (every < 0 || iters < 0 || !(lr >= 0.0f) || !std::isfinite(lr))
        return sd_fail(h, SD_ERR_INVALID_ARG, "every >= 0, iters >= 0 and a finite lr >= 0");
    h->hull.train_every = every;
    h->hull.train_iters = iters;
    h->hull.train_lr = lr;
    return SD_OK;
}

sd_status sd_engine_hull_entries(sd_engine* h, uint32_t* off, uint32_t* partners, uint32_t* info, float* dir4,
                                 float* seed4, float* feat16, uint64_t cap, uint64_t* n_entries) {
    if (!h || !n_entries) return sd_fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (!h->prepared || !h->hull_mode()) return sd_fail(h, SD_ERR_STATE, "no prepared hull scene");
    HullScene& S = h->hull;
    const uint32_t nb = S.H.nb;
    const int par = S.parity ^ 1;  // the lists of the last step
    std::vector<uint32_t> o(nb + 1);
    HULL_CUDA(h, cudaMemcpyAsync(o.data(), S.off[par], 4 * ((size_t)nb + 1), cudaMemcpyDeviceToHost, h->stream));
    HULL_CUDA(h, cudaStreamSynchronize(h->stream));
    const uint64_t m = o[nb];
    *n_entries = m;
    if (off) std::memcpy(off, o.data(), 4 * ((size_t)nb + 1));
    if (!partners && !info && !dir4 && !seed4 && !feat16) return SD_OK;  // a count query
    if (m > cap) return sd_fail(h, SD_ERR_CAPACITY, "cap smaller than the entry count");
    if (m > S.H.cap) return sd_fail(h, SD_ERR_CAPACITY, "the step's entry buffer overflowed");
    cudaStream_t st = h->stream;
    if (partners) HULL_CUDA(h, cudaMemcpyAsync(partners, S.partners[par], 4 * m, cudaMemcpyDeviceToHost, st));
    if (info) HULL_CUDA(h, cudaMemcpyAsync(info, S.H.info, 4 * m, cudaMemcpyDeviceToHost, st));
    if (dir4) HULL_CUDA(h, cudaMemcpyAsync(dir4, S.dir[par], 16 * m, cudaMemcpyDeviceToHost, st));
    if (seed4) HULL_CUDA(h, cudaMemcpyAsync(seed4, S.H.seeds, 16 * m, cudaMemcpyDeviceToHost, st));
    if (feat16) HULL_CUDA(h, cudaMemcpyAsync(feat16, S.H.feat, 64 * m, cudaMemcpyDeviceToHost, st));
    HULL_CUDA(h, cudaStreamSynchronize(st));
    return SD_OK;
}

// ------------------------------------------------ warm-start network
sd_status sd_engine_mlp_params(sd_engine* h, float* host, uint64_t n, int32_t set) {
    if (!h || !host) return sd_fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (!h->prepared || !h->hull_mode()) return sd_fail(h, SD_ERR_STATE, "no prepared hull scene");
    if (n != sd::mlp_param_count()) return sd_fail(h, SD_ERR_INVALID_ARG, "n must be the parameter count (6288)");
    HullScene& S = h->hull;
    HULL_CUDA(h, cudaSetDevice(h->device));
    if (set) {
        HULL_CUDA(h, sd::mlp_set_params_async(S.mlp, host, h->stream));
        S.mlp_step = 0;
    } else {
        HULL_CUDA(h, cudaMemcpyAsync(host, S.mlp.params, 4 * n, cudaMemcpyDeviceToHost, h->stream));
    }
    HULL_CUDA(h, cudaStreamSynchronize(h->stream));
    return SD_OK;
}

sd_status sd_engine_mlp_forward(sd_engine* h, const float* d_feat16, float* d_out4, uint64_t n) {
    if (!h || (n && (!d_feat16 || !d_out4))) return sd_fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (!h->prepared || !h->hull_mode()) return sd_fail(h, SD_ERR_STATE, "no prepared hull scene");
    if ((reinterpret_cast<uintptr_t>(d_feat16) | reinterpret_cast<uintptr_t>(d_out4)) & 15u)
        return sd_fail(h, SD_ERR_INVALID_ARG, "buffers must be 16-byte aligned");
    HULL_CUDA(h, cudaSetDevice(h->device));
    HULL_CUDA(h, sd::mlp_forward_async(h->hull.mlp, d_feat16, reinterpret_cast<float4*>(d_out4), nullptr, n, false,
                                       h->stream));
    HULL_CUDA(h, cudaStreamSynchronize(h->stream));
    uint32_t st = 0;
    HULL_CUDA(h, cudaMemcpy(&st, h->hull.mlp.status, 4, cudaMemcpyDeviceToHost));
    if (st) return sd_fail(h, SD_ERR_ITER_LIMIT, "device: a tensor-core completion wait gave up");
    return SD_OK;
}

sd_status sd_engine_mlp_train(sd_engine* h, const float* d_feat16, const float* d_tgt4, uint64_t n, int32_t iters,
                              float lr, float* host_grad) {
    if (!h || (n && (!d_feat16 || !d_tgt4))) return sd_fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (!h->prepared || !h->hull_mode()) return sd_fail(h, SD_ERR_STATE, "no prepared hull scene");
    if (n >= (1ull << 31)) return sd_fail(h, SD_ERR_CAPACITY, "n must be < 2^31");
    if (iters < 0 || !(lr >= 0.0f)) return sd_fail(h, SD_ERR_INVALID_ARG, "iters >= 0 and lr >= 0");
    HullScene& S = h->hull;
    HULL_CUDA(h, cudaSetDevice(h->device));
    const float4* t4 = reinterpret_cast<const float4*>(d_tgt4);
    if (iters == 0) {
        HULL_CUDA(h, sd::mlp_train_async(S.mlp, d_feat16, t4, (uint32_t)n, (uint32_t)n, 0.0f, 1, false, h->stream));
    }
    for (int32_t k = 0; k < iters; ++k) {
        S.mlp_step += 1;
        HULL_CUDA(h, sd::mlp_train_async(S.mlp, d_feat16, t4, (uint32_t)n, (uint32_t)n, lr, S.mlp_step, true,
                                         h->stream));
    }
    if (host_grad)
        HULL_CUDA(h, cudaMemcpyAsync(host_grad, S.mlp.grad, 4ull * sd::mlp_param_count(), cudaMemcpyDeviceToHost,
                                     h->stream));
    HULL_CUDA(h, cudaStreamSynchronize(h->stream));
    uint32_t st = 0;
    HULL_CUDA(h, cudaMemcpy(&st, S.mlp.status, 4, cudaMemcpyDeviceToHost));
    if (st) return sd_fail(h, SD_ERR_ITER_LIMIT, "device: a tensor-core completion wait gave up");
    S.graph_valid = false;
    return SD_OK;
}

// ----------------------------------------------------- raw LBVH operators
sd_status sd_lbvh_scratch_bytes(uint64_t n, uint64_t pair_cap, uint64_t* bytes) {
    if (!bytes) return sd_fail(nullptr, SD_ERR_INVALID_ARG, "bytes NULL");
    if (n >= (1ull << 30)) return sd_fail(nullptr, SD_ERR_CAPACITY, "n must be < 2^30");
    auto al = [](uint64_t x) { return (x + 255) & ~255ull; };
    *bytes = al(sd::lbvh_scratch_bytes((uint32_t)n)) + 2 * al(4 * (n + 1)) + 2 * al(4 * (2 * pair_cap + 1));
    return SD_OK;
}

sd_status sd_lbvh_pairs(uint64_t n, const float* d_lo4, const float* d_hi4, uint64_t* d_pairs, uint64_t cap,
                        uint32_t* d_count, void* d_scratch, uint64_t scratch_bytes, void* stream) {
    if (n && (!d_lo4 || !d_hi4 || !d_scratch)) return sd_fail(nullptr, SD_ERR_INVALID_ARG, "NULL pointer");
    if (!d_count) return sd_fail(nullptr, SD_ERR_INVALID_ARG, "d_count NULL");
    uint64_t need = 0;
    sd_status s = sd_lbvh_scratch_bytes(n, cap, &need);
    if (s) return s;
    if (scratch_bytes < need) return sd_fail(nullptr, SD_ERR_CAPACITY, "scratch smaller than sd_lbvh_scratch_bytes");
    if ((reinterpret_cast<uintptr_t>(d_lo4) | reinterpret_cast<uintptr_t>(d_hi4)) & 15u)
        return sd_fail(nullptr, SD_ERR_INVALID_ARG, "boxes must be 16-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto al = [](uint64_t x) { return (x + 255) & ~255ull; };
    char* p = static_cast<char*>(d_scratch);
    sd::Lbvh t;
    sd::lbvh_carve(p, (uint32_t)n, &t);
    p += al(sd::lbvh_scratch_bytes((uint32_t)n));
    uint32_t* off = reinterpret_cast<uint32_t*>(p);
    p += al(4 * (n + 1));
    uint32_t* pos = reinterpret_cast<uint32_t*>(p);
    p += al(4 * (n + 1));
    uint32_t* partners = reinterpret_cast<uint32_t*>(p);
    p += al(4 * (2 * cap + 1));
    uint32_t* self = reinterpret_cast<uint32_t*>(p);
    const float4* lo = reinterpret_cast<const float4*>(d_lo4);
    const float4* hi = reinterpret_cast<const float4*>(d_hi4);
    cudaError_t e = cudaMemsetAsync(t.status, 0, 16, st);
    if (e == cudaSuccess) e = sd::lbvh_build_async(t, lo, hi, st);
    if (e == cudaSuccess) e = sd::lbvh_partners_async(t, off, partners, self, 2 * cap, st);
    if (e == cudaSuccess)
        e = sd::lbvh_unique_pairs_async(t, off, partners, 2 * cap, pos, reinterpret_cast<unsigned long long*>(d_pairs),
                                        cap, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_count, pos + n, 4, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_count + 1, t.status, 4, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return sd_cuda_fail(nullptr, e, "sd_lbvh_pairs");
    return SD_OK;
}

sd_status sd_lbvh_morton(uint64_t n, const float* d_lo4, const float* d_hi4, uint32_t* d_codes, void* d_scratch,
                         uint64_t scratch_bytes, void* stream) {
    if (n && (!d_lo4 || !d_hi4 || !d_codes || !d_scratch)) return sd_fail(nullptr, SD_ERR_INVALID_ARG, "NULL pointer");
    if (n >= (1ull << 30)) return sd_fail(nullptr, SD_ERR_CAPACITY, "n must be < 2^30");
    if (scratch_bytes < sd::lbvh_scratch_bytes((uint32_t)n))
        return sd_fail(nullptr, SD_ERR_CAPACITY, "scratch smaller than sd_lbvh_scratch_bytes");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    sd::Lbvh t;
    sd::lbvh_carve(d_scratch, (uint32_t)n, &t);
    cudaError_t e = sd::lbvh_morton_async(t, reinterpret_cast<const float4*>(d_lo4),
                                          reinterpret_cast<const float4*>(d_hi4), st);
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(d_codes, t.keys, 4 * n, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return sd_cuda_fail(nullptr, e, "sd_lbvh_morton");
    return SD_OK;
}

}  // extern "C"
