// sd_engine.cu -- host side of stardust-gb300: the C ABI of include/stardust.h.
//
// The engine replaces STARDUST::DEMEngine + EntityHandler
// (src/engine/engine.hpp:37-447, src/engine/entities/entity_handler.cpp) for
// the per-step DEM path.  Design differences from the reference, each for a
// GB300 reason:
//   * one structure-of-float4 sphere state kept in cell-sorted order on the
//     device (x,y,z,r | vx,vy,vz,m | wx,wy,wz,id) and re-sorted every step,
//     instead of ~30 separately cudaMalloc'd SoA arrays (engine.cpp:243-599);
//   * the whole step is captured once as a CUDA graph and replayed, instead
//     of a host loop of launches with a device-wide sync (simulation_kernel.cu:31);
//   * errors are status codes plus a per-handle message, not exit();
//   * all device memory is owned by the handle and freed by sd_engine_destroy.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstddef>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/stardust.h"
#include "sd_engine_impl.h"
#include "sd_internal.h"
#include "sd_json.h"

namespace {

thread_local std::string g_last_error;

// Bumped by sd_tune_set: engines whose graph was captured under an older
// epoch re-capture before their next step.
std::atomic<uint64_t> g_tune_epoch{0};

struct CudaBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

}  // namespace

namespace {

sd_status fail(sd_engine* h, sd_status code, const std::string& msg) {
    if (h) h->err = msg;
    g_last_error = msg;
    return code;
}

sd_status cuda_fail(sd_engine* h, cudaError_t e, const char* where) {
    return fail(h, SD_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define SD_CUDA(h, call)                                          \
    do {                                                          \
        cudaError_t _e = (call);                                  \
        if (_e != cudaSuccess) return cuda_fail((h), _e, #call);  \
    } while (0)

inline float4 f4(const float* p) { return make_float4(p[0], p[1], p[2], p[3]); }

uint32_t id_bits(uint32_t id) { return id & 0x7fffffffu; }

float id_as_float(uint32_t id) {
    float f;
    uint32_t b = id_bits(id);
    std::memcpy(&f, &b, 4);
    return f;
}

// damping coefficient prefactor: gamma_n = damp * sqrt(m_eff) with
// damp = 2 * beta * sqrt(kn), beta = -ln(e) / sqrt(pi^2 + ln^2(e))
float damp_from(float kn, float e) {
    double le = std::log((double)e);
    double beta = -le / std::sqrt(M_PI * M_PI + le * le);
    return (float)(2.0 * beta * std::sqrt((double)kn));
}

template <typename T>
sd_status dev_alloc(sd_engine* h, T** p, size_t count) {
    void* q = nullptr;
    size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) return fail(h, SD_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    h->allocations.push_back(q);
    *p = static_cast<T*>(q);
    return SD_OK;
}

void release_device(sd_engine* h) {
    hull_release(h);
    if (h->graph) cudaGraphExecDestroy(h->graph);
    if (h->graph_alt) cudaGraphExecDestroy(h->graph_alt);
    h->graph = nullptr;
    h->graph_alt = nullptr;
    h->graph_valid = false;
    for (void* p : h->allocations) cudaFree(p);
    h->allocations.clear();
    h->B = sd::DemBuffers{};
    h->d_energy = nullptr;
    h->d_tmp = nullptr;
    if (h->stream) cudaStreamDestroy(h->stream);
    h->stream = nullptr;
    h->prepared = false;
}

// Grid dims of a box edge over a float cell: the edge over the cell is an
// integer up to the cell's rounding (1 / 0.02f = 50.000001), which must not
// add a cell layer.
static sd_status grid_dims(sd_engine* h, const float* lo, const float* hi, float cell, int32_t* dims,
                           uint64_t* ncells) {
    *ncells = 1;
    for (int a = 0; a < 3; ++a) {
        if (!(hi[a] > lo[a])) return fail(h, SD_ERR_INVALID_ARG, "box: hi must exceed lo on every axis");
        double nd = std::ceil(((double)hi[a] - (double)lo[a]) / (double)cell * (1.0 - 1e-6));
        if (nd < 1) nd = 1;
        if (nd > (1 << 20)) return fail(h, SD_ERR_INVALID_ARG, "grid too fine (> 2^20 cells per axis)");
        dims[a] = (int32_t)nd;
        *ncells *= (uint64_t)nd;
    }
    return SD_OK;
}

// z cells per cell edge (knob "z_div"; 0 = automatic): automatically the
// largest of 4 and 2 whose finer grid keeps keys within 20 bits and sorts in
// as many passes as the plain one (a 50 x 50 x 100 grid: 18-bit keys -> 20
// bits at 4, 2 passes either way), else 1.  Measured on 1,048,576 spheres
// with the incremental re-sort, per step: z_div 1 0.190 ms, 2 0.174 ms,
// 4 0.169 ms, 8 0.171 ms; on the 2.1M-sphere drum (23-bit keys) any split
// was slower (1 0.477 ms, 2 0.495 ms, 4 0.541 ms).
static int32_t g_z_div = 0;
// skin of the contact lists in micrometres (0: no lists), applied at the
// next step-graph build.  Default 50: on the 1,048,576-sphere settling box
// at step 1,000 the step takes 0.099 ms with it against 0.169 ms without
// (20 um 0.099, 100 um 0.106, 500 um 0.116 ms)
static int32_t g_skin_um = 50;
static int key_bits_of(uint64_t ncells) {
    int b = 1;
    while (b < 32 && (1ull << b) < ncells) ++b;
    return b;
}
static int32_t z_div_for(uint64_t ncells) {
    if (g_z_div > 0) return ncells * (uint64_t)g_z_div <= (1ull << 30) ? g_z_div : 1;
    const int p0 = sd::sort_num_passes(key_bits_of(ncells));
    for (int32_t zd = 4; zd >= 2; zd /= 2) {
        const int bits = key_bits_of(ncells * (uint64_t)zd);
        if (bits <= 20 && sd::sort_num_passes(bits) == p0) return zd;
    }
    return 1;
}

// A batch: per scene its grid (cell = given or 2 x its largest radius) at
// consecutive key ranges, and its slot range.
static sd_status derive_batch(sd_engine* h) {
    h->scene_grids.clear();
    h->scene_first.clear();
    uint64_t base = 0;
    uint32_t first = 0;
    for (size_t k = 0; k < h->scenes.size(); ++k) {
        const auto& sc = h->scenes[k];
        if (sc.first != first) return fail(h, SD_ERR_STATE, "every sphere of a batch must belong to a scene");
        float rmax = 0.0f;
        for (uint32_t i = 0; i < sc.count; ++i) rmax = std::max(rmax, h->h_pos[sc.first + i].w);
        const float cell = sc.cell > 0.0f ? sc.cell : (rmax > 0.0f ? 2.0f * rmax : sc.hi[0] - sc.lo[0]);
        if (cell < 2.0f * rmax)
            return fail(h, SD_ERR_INVALID_ARG, "scene " + std::to_string(k) + ": cell must be >= 2 * largest radius");
        sd::SceneGrid g{};
        int32_t dims[3];
        uint64_t nc = 0;
        sd_status s = grid_dims(h, sc.lo, sc.hi, cell, dims, &nc);
        if (s) return s;
        for (int a = 0; a < 3; ++a) {
            g.lo[a] = sc.lo[a];
            g.hi[a] = sc.hi[a];
        }
        g.cell = cell;
        g.nx = dims[0];
        g.ny = dims[1];
        g.nz = dims[2];
        g.base = (uint32_t)base;
        base += nc;
        if (base > (1ull << 30)) return fail(h, SD_ERR_INVALID_ARG, "the batch's grids exceed 2^30 cells");
        h->scene_grids.push_back(g);
        h->scene_first.push_back(first);
        first += sc.count;
    }
    if (first != h->h_pos.size()) return fail(h, SD_ERR_STATE, "every sphere of a batch must belong to a scene");
    h->scene_first.push_back(first);
    return SD_OK;
}

sd_status derive_params(sd_engine* h) {
    const sd_config& c = h->cfg;
    sd::DemParams& P = h->P;
    float rmax = 0.0f;
    for (auto& p : h->h_pos) rmax = std::max(rmax, p.w);
    if (h->scenes.size() > 1) {
        // a batch: the configured box and cell are not used
        if (!h->hb_pos.empty()) return fail(h, SD_ERR_UNSUPPORTED, "rigid clumps are not supported in a batch");
        if (!h->mesh.tri.empty()) return fail(h, SD_ERR_UNSUPPORTED, "meshes are not supported in a batch");
        sd_status s = derive_batch(h);
        if (s) return s;
        const sd::SceneGrid& g0 = h->scene_grids[0];
        for (int a = 0; a < 3; ++a) {  // sd_engine_params reports the first scene
            P.lo[a] = g0.lo[a];
            P.hi[a] = g0.hi[a];
        }
        P.cell = g0.cell;
        P.nx = g0.nx;
        P.ny = g0.ny;
        P.nz = g0.nz;
        P.cell_z = g0.cell;
        P.z_div = 1;
    } else {
        bool box_given = c.box_hi[0] != 0.f || c.box_hi[1] != 0.f || c.box_hi[2] != 0.f;
        const bool one_scene = h->scenes.size() == 1;
        for (int a = 0; a < 3; ++a) {
            P.lo[a] = one_scene ? h->scenes[0].lo[a] : (box_given ? c.box_lo[a] : 0.0f);
            P.hi[a] = one_scene ? h->scenes[0].hi[a] : (box_given ? c.box_hi[a] : c.domain);
            if (!(P.hi[a] > P.lo[a])) return fail(h, SD_ERR_INVALID_ARG, "box: hi must exceed lo on every axis");
        }
        const float cfg_cell = one_scene ? h->scenes[0].cell : c.cell;
        float cell = cfg_cell > 0.0f ? cfg_cell : 2.0f * rmax;
        if (!(cell > 0.0f)) cell = (P.hi[0] - P.lo[0]);
        // a sphere must fit within the 3x3x3 cell neighbourhood: every contact
        // partner is then found in the adjacent cells
        if (cell < 2.0f * rmax) return fail(h, SD_ERR_INVALID_ARG, "cell must be >= 2 * largest radius");
        P.cell = cell;
        int32_t dims[3];
        uint64_t ncells = 0;
        sd_status s = grid_dims(h, P.lo, P.hi, cell, dims, &ncells);
        if (s) return s;
        P.nx = dims[0];
        P.ny = dims[1];
        if (ncells > (1ull << 30)) return fail(h, SD_ERR_INVALID_ARG, "grid has more than 2^30 cells");
        const int32_t zd = h->z_div_fixed > 0 ? h->z_div_fixed : z_div_for(ncells);
        P.nz = dims[2] * zd;
        P.z_div = zd;
        P.cell_z = cell / (float)zd;
    }
    if (!(c.restitution > 0.0f && c.restitution <= 1.0f))
        return fail(h, SD_ERR_INVALID_ARG, "restitution must be in (0, 1]");
    if (!(c.kn > 0.0f)) return fail(h, SD_ERR_INVALID_ARG, "kn must be > 0");
    if (!(c.mu >= 0.0f)) return fail(h, SD_ERR_INVALID_ARG, "mu must be >= 0");
    P.kn = c.kn;
    P.damp = damp_from(c.kn, c.restitution);
    P.mu = c.mu;
    for (int a = 0; a < 3; ++a) P.g[a] = c.gravity[a];
    P.walls = c.walls;
    P.rmax = rmax;
    P.dt = 0.0f;
    return SD_OK;
}

// Uploads `n` spheres (device order given by the host arrays) into the
// next-state buffers and sorts them into cell order.
sd_status upload_and_sort(sd_engine* h, const float4* pos, const float4* vel, const float4* omg, uint32_t n) {
    sd::DemBuffers& B = h->B;
    if (n) {
        SD_CUDA(h, cudaMemcpyAsync(B.pos_n, pos, sizeof(float4) * n, cudaMemcpyHostToDevice, h->stream));
        SD_CUDA(h, cudaMemcpyAsync(B.vel_n, vel, sizeof(float4) * n, cudaMemcpyHostToDevice, h->stream));
        SD_CUDA(h, cudaMemcpyAsync(B.omg_n, omg, sizeof(float4) * n, cudaMemcpyHostToDevice, h->stream));
    }
    SD_CUDA(h, sd::dem_keys_from_state_async(h->P, B, h->stream));
    SD_CUDA(h, sd::dem_sort_reorder_async(h->P, B, h->stream));
    SD_CUDA(h, cudaStreamSynchronize(h->stream));
    return SD_OK;
}

// The mesh's static grid (mesh frame): cell edge 2 x the largest sphere
// radius (grown until the grid has at most 2^25 cells), every triangle
// listed in every cell its box, grown by that radius, touches -- so a
// sphere's own cell lists every triangle it can reach -- in ascending order.
sd_status build_mesh(sd_engine* h) {
    auto& M = h->mesh;
    sd::MeshView& V = h->B.mesh;
    const uint32_t nt = (uint32_t)(M.tri.size() / 3);
    float rmax = 0.0f;
    for (auto& p : h->h_pos) rmax = std::max(rmax, p.w);
    if (!(rmax > 0.0f)) rmax = 1e-3f;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (const float4& v : M.tri) {
        const float c[3] = {v.x, v.y, v.z};
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], c[a]);
            hi[a] = std::max(hi[a], c[a]);
        }
    }
    float hcell = 2.0f * rmax;
    int32_t dims[3];
    uint64_t nc = 0;
    for (;;) {
        nc = 1;
        for (int a = 0; a < 3; ++a) {
            const double ext = (double)hi[a] - lo[a] + 2.0 * rmax;
            dims[a] = (int32_t)std::max(1.0, std::ceil(ext / hcell));
            nc *= (uint64_t)dims[a];
        }
        if (nc <= (1ull << 25)) break;
        hcell *= 1.5f;
    }
    for (int a = 0; a < 3; ++a) V.lo[a] = lo[a] - rmax;
    V.h = hcell;
    V.nx = dims[0];
    V.ny = dims[1];
    V.nz = dims[2];
    auto cell_of = [&](float x, int a) {
        float t = (x - V.lo[a]) / V.h;
        if (!(t >= 0.0f)) return 0;
        if (t >= (float)dims[a]) return dims[a] - 1;
        return (int)t;
    };
    std::vector<uint32_t> off(nc + 1, 0);
    std::vector<uint32_t> list;
    for (int pass = 0; pass < 2; ++pass) {
        std::vector<uint32_t> fill;
        if (pass == 1) {
            for (uint64_t c = 0; c < nc; ++c) off[c + 1] += off[c];
            list.assign(off[nc], 0u);
            fill.assign(off.begin(), off.end() - 1);
        }
        for (uint32_t t = 0; t < nt; ++t) {
            float tl[3] = {INFINITY, INFINITY, INFINITY}, th[3] = {-INFINITY, -INFINITY, -INFINITY};
            for (int k = 0; k < 3; ++k) {
                const float4 v = M.tri[3 * (size_t)t + k];
                const float c[3] = {v.x, v.y, v.z};
                for (int a = 0; a < 3; ++a) {
                    tl[a] = std::min(tl[a], c[a]);
                    th[a] = std::max(th[a], c[a]);
                }
            }
            int c0[3], c1[3];
            for (int a = 0; a < 3; ++a) {
                c0[a] = cell_of(tl[a] - rmax, a);
                c1[a] = cell_of(th[a] + rmax, a);
            }
            for (int x = c0[0]; x <= c1[0]; ++x)
                for (int y = c0[1]; y <= c1[1]; ++y)
                    for (int z = c0[2]; z <= c1[2]; ++z) {
                        const uint64_t c = ((uint64_t)x * dims[1] + y) * dims[2] + z;
                        if (pass == 0) off[c + 1]++;
                        else list[fill[c]++] = t;
                    }
        }
        if (pass == 0 && off.size() > 1) {
            uint64_t tot = 0;
            for (uint64_t c = 1; c <= nc; ++c) tot += off[c];
            if (tot >= 0xffffffffull) return fail(h, SD_ERR_CAPACITY, "mesh grid lists exceed 2^32 entries");
        }
    }
    sd_status s;
    float4* tri = nullptr;
    int32_t* patch = nullptr;
    uint32_t *coff = nullptr, *ctri = nullptr;
    float* state = nullptr;
    if ((s = dev_alloc(h, &tri, M.tri.size())) || (s = dev_alloc(h, &patch, nt)) ||
        (s = dev_alloc(h, &coff, nc + 1)) || (s = dev_alloc(h, &ctri, std::max<size_t>(list.size(), 1))) ||
        (s = dev_alloc(h, &state, 24)))
        return s;
    SD_CUDA(h, cudaMemcpyAsync(tri, M.tri.data(), 16 * M.tri.size(), cudaMemcpyHostToDevice, h->stream));
    SD_CUDA(h, cudaMemcpyAsync(patch, M.patch.data(), 4 * (size_t)nt, cudaMemcpyHostToDevice, h->stream));
    SD_CUDA(h, cudaMemcpyAsync(coff, off.data(), 4 * (nc + 1), cudaMemcpyHostToDevice, h->stream));
    if (!list.empty())
        SD_CUDA(h, cudaMemcpyAsync(ctri, list.data(), 4 * list.size(), cudaMemcpyHostToDevice, h->stream));
    // pose: R (set by the first mesh_advance with advance = 0), centre, axis,
    // omega, q = identity, dq set when the step's time step is known
    float* S = M.state;
    std::memset(S, 0, sizeof M.state);
    for (int a = 0; a < 3; ++a) {
        S[9 + a] = M.centre[a];
        S[12 + a] = M.axis[a];
    }
    S[15] = M.omega;
    S[16] = 1.0f;
    S[20] = 1.0f;
    SD_CUDA(h, cudaMemcpyAsync(state, S, sizeof M.state, cudaMemcpyHostToDevice, h->stream));
    V.ntri = nt;
    V.tri = tri;
    V.patch = patch;
    V.cell_off = coff;
    V.cell_tri = ctri;
    V.state = state;
    V.sap_n = 0;
    if (h->cfg.collision_engine == SD_ENGINE_SAP && nt) {
        // sweep and prune of the triangles: along the rotation axis of a
        // rotating mesh (its triangles' extents along it never change), else
        // along the mesh's longest extent; boxes sorted by lower bound (ties
        // by triangle id)
        int axis = 0;
        if (M.omega != 0.0f) {
            for (int a = 1; a < 3; ++a)
                if (std::fabs(M.axis[a]) > std::fabs(M.axis[axis])) axis = a;
        } else {
            for (int a = 1; a < 3; ++a)
                if (hi[a] - lo[a] > hi[axis] - lo[axis]) axis = a;
        }
        std::vector<float4> box(2 * (size_t)nt);
        std::vector<uint32_t> order(nt);
        float len = 0.0f;
        for (uint32_t t = 0; t < nt; ++t) {
            float tl[3] = {INFINITY, INFINITY, INFINITY}, th[3] = {-INFINITY, -INFINITY, -INFINITY};
            for (int k = 0; k < 3; ++k) {
                const float4 v = M.tri[3 * (size_t)t + k];
                const float cc[3] = {v.x, v.y, v.z};
                for (int a = 0; a < 3; ++a) {
                    tl[a] = std::min(tl[a], cc[a]);
                    th[a] = std::max(th[a], cc[a]);
                }
            }
            uint32_t id_bits = t;
            float id_f;
            std::memcpy(&id_f, &id_bits, 4);
            box[2 * (size_t)t] = make_float4(tl[0], tl[1], tl[2], tl[axis]);
            box[2 * (size_t)t + 1] = make_float4(th[0], th[1], th[2], id_f);
            len = std::max(len, th[axis] - tl[axis]);
            order[t] = t;
        }
        std::stable_sort(order.begin(), order.end(),
                         [&](uint32_t a, uint32_t b) { return box[2 * (size_t)a].w < box[2 * (size_t)b].w; });
        std::vector<float4> sbox(2 * (size_t)nt);
        std::vector<float> slo(nt);
        for (uint32_t k = 0; k < nt; ++k) {
            sbox[2 * (size_t)k] = box[2 * (size_t)order[k]];
            sbox[2 * (size_t)k + 1] = box[2 * (size_t)order[k] + 1];
            slo[k] = box[2 * (size_t)order[k]].w;
        }
        float4* dbox = nullptr;
        float* dlo = nullptr;
        if ((s = dev_alloc(h, &dbox, 2 * (size_t)nt)) || (s = dev_alloc(h, &dlo, nt))) return s;
        SD_CUDA(h, cudaMemcpyAsync(dbox, sbox.data(), 32 * (size_t)nt, cudaMemcpyHostToDevice, h->stream));
        SD_CUDA(h, cudaMemcpyAsync(dlo, slo.data(), 4 * (size_t)nt, cudaMemcpyHostToDevice, h->stream));
        SD_CUDA(h, cudaStreamSynchronize(h->stream));
        V.sap_n = nt;
        V.sap_box = dbox;
        V.sap_lo = dlo;
        V.sap_axis = axis;
        V.sap_len = len;
    }
    M.dt = 0.0f;
    SD_CUDA(h, sd::mesh_advance_async(V, 0, h->stream));
    return SD_OK;
}

sd_status allocate(sd_engine* h, uint32_t n) {
    sd::DemBuffers& B = h->B;
    B.n = n;
    B.ncells = h->scenes.size() > 1 ? h->scene_first.empty() ? 0u
                                                             : (uint32_t)((uint64_t)h->scene_grids.back().base +
                                                                          (uint64_t)h->scene_grids.back().nx *
                                                                              h->scene_grids.back().ny *
                                                                              h->scene_grids.back().nz)
                                    : (uint32_t)((uint64_t)h->P.nx * h->P.ny * h->P.nz);
    int bits = 1;
    while (bits < 32 && (1ull << bits) < (unsigned long long)B.ncells) ++bits;
    sd_status s;
    if ((s = dev_alloc(h, &B.pos, n)) || (s = dev_alloc(h, &B.vel, n)) || (s = dev_alloc(h, &B.omg, n)) ||
        (s = dev_alloc(h, &B.pos_n, n)) || (s = dev_alloc(h, &B.vel_n, n)) || (s = dev_alloc(h, &B.omg_n, n)) ||
        (s = dev_alloc(h, &B.keys, n)) || (s = dev_alloc(h, &B.vals, n)) || (s = dev_alloc(h, &B.keys_tmp, n)) ||
        (s = dev_alloc(h, &B.vals_tmp, n)) || (s = dev_alloc(h, &B.cell_start, (size_t)B.ncells + 1)) ||
        (s = dev_alloc(h, &B.sort_scratch, sd::sort_scratch_words(n, bits))) ||
        (s = dev_alloc(h, &B.dev_status, 8)) || (s = dev_alloc(h, &h->d_energy, 4)) ||
        (s = dev_alloc(h, &h->d_tmp, n)) || (s = dev_alloc(h, &B.keys_prev, n)) ||
        (s = dev_alloc(h, &B.rs_list, (size_t)sd::kResortMaxCap)) ||
        (s = dev_alloc(h, &B.rs_pos, (size_t)sd::kResortMaxCap)) || (s = dev_alloc(h, &B.rs_q, (size_t)sd::kResortMaxCap)) ||
        (s = dev_alloc(h, &B.rs_iv_lo, (size_t)sd::kResortMaxCap)) ||
        (s = dev_alloc(h, &B.rs_iv_pre, (size_t)sd::kResortMaxCap + 1)) ||
        (s = dev_alloc(h, &B.rs_scratch, sd::resort_scratch_words(n))))
        return s;
    if (h->hb_pos.empty() && h->mesh.tri.empty() && n) {  // the two-kernel contact stage's partner lists
        if ((s = dev_alloc(h, &B.nbr_cnt, n)) || (s = dev_alloc(h, &B.nbr, (size_t)n * sd::kNbrCap))) return s;
        SD_CUDA(h, cudaMemsetAsync(B.nbr_cnt, 0, sizeof(uint32_t) * n, h->stream));
    }
    if (h->cfg.flags & SD_FLAG_RECORD) {
        if ((s = dev_alloc(h, &B.force, n)) || (s = dev_alloc(h, &B.torque, n))) return s;
        SD_CUDA(h, cudaMemsetAsync(B.force, 0, sizeof(float4) * std::max<uint32_t>(n, 1), h->stream));
        SD_CUDA(h, cudaMemsetAsync(B.torque, 0, sizeof(float4) * std::max<uint32_t>(n, 1), h->stream));
    }
    B.pair_cap = h->cfg.pair_capacity;
    if ((s = dev_alloc(h, &B.pairs, (size_t)B.pair_cap)) || (s = dev_alloc(h, &B.npairs, 1))) return s;
    SD_CUDA(h, cudaMemsetAsync(B.dev_status, 0, 8 * sizeof(uint32_t), h->stream));
    SD_CUDA(h, cudaMemsetAsync(B.sort_scratch, 0, 16 * sizeof(uint32_t), h->stream));
    SD_CUDA(h, cudaMemsetAsync(B.rs_scratch, 0, sd::resort_scratch_words(n) * sizeof(uint32_t), h->stream));
    if (!h->mesh.tri.empty()) {
        if ((s = build_mesh(h))) return s;
    }
    B.nscenes = h->scenes.size() > 1 ? (uint32_t)h->scenes.size() : 0u;
    if (B.nscenes) {
        sd::SceneGrid* g = nullptr;
        uint32_t* f = nullptr;
        if ((s = dev_alloc(h, &g, B.nscenes)) || (s = dev_alloc(h, &f, (size_t)B.nscenes + 1))) return s;
        SD_CUDA(h, cudaMemcpyAsync(g, h->scene_grids.data(), sizeof(sd::SceneGrid) * B.nscenes, cudaMemcpyHostToDevice,
                                   h->stream));
        SD_CUDA(h, cudaMemcpyAsync(f, h->scene_first.data(), 4 * ((size_t)B.nscenes + 1), cudaMemcpyHostToDevice,
                                   h->stream));
        B.scenes = g;
        B.scene_first = f;
    }
    // skin lists (knob skin_um): allocated by the first step graph that uses them
    B.vl_skin = 0.0f;
    const uint32_t nb = (uint32_t)h->hb_pos.size();
    B.nb = nb;
    if (nb) {
        if ((s = dev_alloc(h, &B.body_of, n)) || (s = dev_alloc(h, &B.r0, n)) || (s = dev_alloc(h, &B.slot_of, n)) ||
            (s = dev_alloc(h, &B.sf, n)) || (s = dev_alloc(h, &B.st, n)) || (s = dev_alloc(h, &B.bpos, nb)) ||
            (s = dev_alloc(h, &B.bvel, nb)) || (s = dev_alloc(h, &B.bquat, nb)) || (s = dev_alloc(h, &B.bomg, nb)) ||
            (s = dev_alloc(h, &B.bang, nb)) || (s = dev_alloc(h, &B.binv, 3 * (size_t)nb)) ||
            (s = dev_alloc(h, &B.bfirst, nb)) || (s = dev_alloc(h, &B.bcount, nb)))
            return s;
        SD_CUDA(h, cudaMemcpyAsync(B.body_of, h->h_body_of.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, h->stream));
        SD_CUDA(h, cudaMemcpyAsync(B.r0, h->h_r0.data(), 16 * (size_t)n, cudaMemcpyHostToDevice, h->stream));
        SD_CUDA(h, cudaMemsetAsync(B.sf, 0, 16 * (size_t)n, h->stream));
        SD_CUDA(h, cudaMemsetAsync(B.st, 0, 16 * (size_t)n, h->stream));
        SD_CUDA(h, cudaMemsetAsync(B.slot_of, 0xff, 4 * (size_t)n, h->stream));
        SD_CUDA(h, cudaMemcpyAsync(B.bpos, h->hb_pos.data(), 16 * (size_t)nb, cudaMemcpyHostToDevice, h->stream));
        SD_CUDA(h, cudaMemcpyAsync(B.bvel, h->hb_vel.data(), 16 * (size_t)nb, cudaMemcpyHostToDevice, h->stream));
        SD_CUDA(h, cudaMemcpyAsync(B.bquat, h->hb_quat.data(), 16 * (size_t)nb, cudaMemcpyHostToDevice, h->stream));
        SD_CUDA(h, cudaMemcpyAsync(B.bomg, h->hb_omg.data(), 16 * (size_t)nb, cudaMemcpyHostToDevice, h->stream));
        SD_CUDA(h, cudaMemcpyAsync(B.bang, h->hb_ang.data(), 16 * (size_t)nb, cudaMemcpyHostToDevice, h->stream));
        SD_CUDA(h, cudaMemcpyAsync(B.binv, h->hb_inv.data(), 48 * (size_t)nb, cudaMemcpyHostToDevice, h->stream));
        SD_CUDA(h, cudaMemcpyAsync(B.bfirst, h->hb_first.data(), 4 * (size_t)nb, cudaMemcpyHostToDevice, h->stream));
        SD_CUDA(h, cudaMemcpyAsync(B.bcount, h->hb_count.data(), 4 * (size_t)nb, cudaMemcpyHostToDevice, h->stream));
    }
    return SD_OK;
}

sd_status prepare_with(sd_engine* h, const float4* pos, const float4* vel, const float4* omg, uint32_t n) {
    sd_status s = derive_params(h);
    if (s) return s;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(h, SD_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (h->device >= ndev) return fail(h, SD_ERR_INVALID_ARG, "cuda_device out of range");
    SD_CUDA(h, cudaSetDevice(h->device));
    SD_CUDA(h, cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    SD_CUDA(h, sd::dem_init_kernels());
    if ((s = allocate(h, n))) {
        release_device(h);
        return s;
    }
    if ((s = upload_and_sort(h, pos, vel, omg, n))) {
        release_device(h);
        return s;
    }
    h->prepared = true;
    h->keys_current = true;
    h->steps = 0;
    return SD_OK;
}

static void swap_state(sd::DemBuffers& B) {
    std::swap(B.pos, B.pos_n);
    std::swap(B.vel, B.vel_n);
    std::swap(B.omg, B.omg_n);
}

// Contact lists with a skin (knob skin_um) for scenes of free spheres (one
// or a batch): allocated when a step graph first uses them, then kept; the skin
// follows the knob at every graph build (0: no lists).  The slot table
// covers every sphere while the lists are on and is rebuilt here, since
// steps without lists keep it for clump spheres only.
static sd_status ensure_contact_lists(sd_engine* h) {
    sd::DemBuffers& B = h->B;
    const uint32_t n = B.n;
    if (!(g_skin_um > 0 && n)) {
        B.vl_skin = 0.0f;
        return SD_OK;
    }
    sd_status s;
    if (!B.vl_cnt) {
        if ((s = dev_alloc(h, &B.vl_cnt, n)) || (s = dev_alloc(h, &B.vl_nbr, (size_t)n * sd::kVlCap)) ||
            (s = dev_alloc(h, &B.vl_ref, n)) || (s = dev_alloc(h, &B.vl_flags, 4)) ||
            (s = dev_alloc(h, &B.vl_cnt_t, n)) || (s = dev_alloc(h, &B.vl_nbr_t, (size_t)n * sd::kVlCap)) ||
            (s = dev_alloc(h, &B.vl_ref_t, n)))
            return s;
        SD_CUDA(h, cudaMemsetAsync(B.vl_flags, 0, 4 * sizeof(uint32_t), h->stream));
    }
    if (!B.slot_of && (s = dev_alloc(h, &B.slot_of, n))) return s;
    SD_CUDA(h, sd::dem_slot_of_all_async(B.omg, B.slot_of, n, h->stream));
    B.vl_skin = 1e-6f * (float)g_skin_um;
    return SD_OK;
}

// Makes the next step build the contact lists (knob skin_um) from a scan
// over the widened window, whatever the lists' state.
static sd_status force_list_build(sd_engine* h) {
    if (!h->B.vl_flags) return SD_OK;
    const uint32_t build[2] = {1u, 0u};
    SD_CUDA(h, cudaMemcpyAsync(h->B.vl_flags, build, sizeof build, cudaMemcpyHostToDevice, h->stream));
    return SD_OK;
}

sd_status build_graph(sd_engine* h, float dt) {
    if (h->graph) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    if (h->graph_alt) {
        cudaGraphExecDestroy(h->graph_alt);
        h->graph_alt = nullptr;
    }
    h->P.dt = dt;
    bool record = (h->cfg.flags & SD_FLAG_RECORD) != 0;
    if (h->B.mesh.ntri && h->mesh.dt != dt) {
        // the rotation of one step, in double: angle omega dt about the axis
        const double half = 0.5 * (double)h->mesh.omega * (double)dt;
        float dq[4] = {(float)std::cos(half), (float)(std::sin(half) * h->mesh.axis[0]),
                       (float)(std::sin(half) * h->mesh.axis[1]), (float)(std::sin(half) * h->mesh.axis[2])};
        SD_CUDA(h, cudaMemcpyAsync(h->B.mesh.state + 20, dq, sizeof dq, cudaMemcpyHostToDevice, h->stream));
        SD_CUDA(h, cudaStreamSynchronize(h->stream));
        h->mesh.dt = dt;
    }
    h->B.rs_max = sd::dem_resort_max();
    {  // the contact lists follow the skin knob
        sd_status s = ensure_contact_lists(h);
        if (s) return s;
    }
    h->graph_swaps = sd::dem_step_swaps(h->B);
    h->graph_parity = 0;
    // with swaps: the graph on the current buffers, then the one on the
    // swapped buffers (the state after one step); the second swap restores B
    for (int par = 0; par < (h->graph_swaps ? 2 : 1); ++par) {
        cudaGraph_t g = nullptr;
        SD_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e2 = sd::dem_step_async(h->P, h->B, record, h->stream);
        cudaError_t e3 = cudaStreamEndCapture(h->stream, &g);
        if (h->graph_swaps) swap_state(h->B);
        if (e2 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            if (h->graph_swaps && par == 0) swap_state(h->B);
            return cuda_fail(h, e2, "capturing the step");
        }
        if (e3 != cudaSuccess) {
            if (h->graph_swaps && par == 0) swap_state(h->B);
            return cuda_fail(h, e3, "cudaStreamEndCapture");
        }
        cudaError_t e4 = cudaGraphInstantiate(par == 0 ? &h->graph : &h->graph_alt, g, 0);
        h->graph_kernels = graph_kernel_nodes(g);
        cudaGraphDestroy(g);
        if (e4 != cudaSuccess) {
            if (h->graph_swaps && par == 0) swap_state(h->B);
            return cuda_fail(h, e4, "cudaGraphInstantiate");
        }
    }
    h->graph_dt = dt;
    h->graph_valid = true;
    return SD_OK;
}

sd_status resort_if_needed(sd_engine* h) {
    if (!h->need_resort) return SD_OK;
    sd::DemBuffers& B = h->B;
    if (B.n) {
        SD_CUDA(h, cudaMemcpyAsync(B.pos_n, B.pos, sizeof(float4) * B.n, cudaMemcpyDeviceToDevice, h->stream));
        SD_CUDA(h, cudaMemcpyAsync(B.vel_n, B.vel, sizeof(float4) * B.n, cudaMemcpyDeviceToDevice, h->stream));
        SD_CUDA(h, cudaMemcpyAsync(B.omg_n, B.omg, sizeof(float4) * B.n, cudaMemcpyDeviceToDevice, h->stream));
    }
    SD_CUDA(h, sd::dem_keys_from_state_async(h->P, B, h->stream));
    SD_CUDA(h, sd::dem_sort_reorder_async(h->P, B, h->stream));
    h->need_resort = false;
    h->keys_current = true;
    // the plain reorder does not carry the contact lists: build them again
    return force_list_build(h);
}

sd_status read_device_errors(sd_engine* h, uint32_t* bits) {
    uint32_t a = 0, b = 0;
    if (h->hull_mode()) {
        SD_CUDA(h, cudaMemcpyAsync(&a, h->hull.tree.status, 4, cudaMemcpyDeviceToHost, h->stream));
        SD_CUDA(h, cudaStreamSynchronize(h->stream));
        *bits = a;
        return SD_OK;
    }
    SD_CUDA(h, cudaMemcpyAsync(&a, h->B.dev_status, 4, cudaMemcpyDeviceToHost, h->stream));
    SD_CUDA(h, cudaMemcpyAsync(&b, h->B.sort_scratch, 4, cudaMemcpyDeviceToHost, h->stream));
    SD_CUDA(h, cudaStreamSynchronize(h->stream));
    *bits = a | b;
    return SD_OK;
}

sd_status errors_to_status(sd_engine* h, uint32_t bits) {
    if (bits & sd::kErrLookbackTimeout)
        return fail(h, SD_ERR_ITER_LIMIT, "device: a decoupled look-back wait hit its spin limit");
    if (bits & sd::kErrPairOverflow) return fail(h, SD_ERR_CAPACITY, "device: contact-pair buffer overflow");
    if (bits & sd::kErrWaitTimeout)
        return fail(h, SD_ERR_ITER_LIMIT, "device: a TMA tile wait hit its limit (the step used global loads)");
    if (bits & sd::kErrBadInput)
        return fail(h, SD_ERR_INVALID_ARG, h->hull_mode() ? "device: a malformed bounding-volume tree was detected"
                                                          : "device: a sphere's cell disagreed with its key");
    return SD_OK;
}


}  // namespace

uint32_t graph_kernel_nodes(cudaGraph_t g) {
    size_t count = 0;
    if (cudaGraphGetNodes(g, nullptr, &count) != cudaSuccess || count == 0) return 0;
    std::vector<cudaGraphNode_t> nodes(count);
    if (cudaGraphGetNodes(g, nodes.data(), &count) != cudaSuccess) return 0;
    uint32_t k = 0;
    for (size_t i = 0; i < count; ++i) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
    }
    return k;
}

namespace sd {
// Records the message sd_last_error(NULL, ...) returns, for entry points
// defined in other translation units.
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace sd

sd_status sd_fail(sd_engine* h, sd_status code, const std::string& msg) { return fail(h, code, msg); }
sd_status sd_cuda_fail(sd_engine* h, cudaError_t e, const char* where) { return cuda_fail(h, e, where); }
sd_status sd_alloc_bytes(sd_engine* h, void** p, size_t bytes) {
    char* q = nullptr;
    sd_status s = dev_alloc(h, &q, bytes);
    *p = q;
    return s;
}
float sd_damp_from(float kn, float e) { return damp_from(kn, e); }
uint64_t sd_tune_epoch() { return g_tune_epoch.load(); }

// =================================================================== C ABI
extern "C" {

sd_status sd_config_default(sd_config* cfg) {
    if (!cfg) return fail(nullptr, SD_ERR_INVALID_ARG, "cfg is NULL");
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->struct_size = sizeof(sd_config);
    cfg->collision_engine = SD_ENGINE_SHP;
    cfg->device = SD_DEVICE_GPU;
    cfg->cuda_device = 0;
    cfg->domain = 1.0f;
    cfg->walls = 0x3f;
    cfg->cell = 0.0f;
    cfg->kn = 1e5f;
    cfg->restitution = 0.5f;
    cfg->mu = 0.3f;
    cfg->gravity[2] = -9.81f;
    cfg->pair_capacity = 1u << 20;
    cfg->flags = 0;
    return SD_OK;
}

sd_status sd_engine_create(const sd_config* cfg, sd_engine** out) {
    if (!cfg || !out) return fail(nullptr, SD_ERR_INVALID_ARG, "NULL argument");
    if (cfg->struct_size != sizeof(sd_config))
        return fail(nullptr, SD_ERR_INVALID_ARG, "sd_config.struct_size mismatch (use sd_config_default)");
    if (cfg->device != SD_DEVICE_GPU)
        return fail(nullptr, SD_ERR_UNSUPPORTED, "only SD_DEVICE_GPU is implemented");
    if (cfg->collision_engine != SD_ENGINE_SHP && cfg->collision_engine != SD_ENGINE_SAP)
        return fail(nullptr, SD_ERR_INVALID_ARG, "unknown collision engine");
    if (cfg->cuda_device < 0) return fail(nullptr, SD_ERR_INVALID_ARG, "cuda_device < 0");
    sd_engine* h = new (std::nothrow) sd_engine();
    if (!h) return fail(nullptr, SD_ERR_NOMEM, "out of host memory");
    h->cfg = *cfg;
    h->device = cfg->cuda_device;
    *out = h;
    return SD_OK;
}

sd_status sd_engine_destroy(sd_engine* h) {
    if (!h) return SD_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    release_device(h);
    delete h;
    return SD_OK;
}

sd_status sd_last_error(const sd_engine* h, char* buf, size_t len) {
    if (!buf || len == 0) return SD_ERR_INVALID_ARG;
    const std::string& m = h ? h->err : g_last_error;
    size_t k = std::min(len - 1, m.size());
    std::memcpy(buf, m.data(), k);
    buf[k] = 0;
    return SD_OK;
}

// ---------------------------------------------------------- runtime changes
// The reference declares EntityHandler::addEntityRuntime and leaves it empty
// (entity_handler.cpp:116-119).  Here a prepared engine takes new spheres and
// clumps and loses free spheres: its state comes back to the host in sphere-
// id order (spheres with their id lanes, body states, the mesh pose), the
// change is applied there, and the engine is prepared again -- new buffers,
// the cell sort from id order, the step graph rebuilt on the next step.  The
// step count and the mesh pose carry over.  A batch of scenes and convex-hull
// scenes do not change at runtime.

// The device state back into the host arrays, in sphere-id order.
static sd_status pull_state(sd_engine* h, std::vector<float>* mesh_state) {
    sd::DemBuffers& B = h->B;
    const uint32_t n = B.n;
    SD_CUDA(h, cudaSetDevice(h->device));
    std::vector<float4>* dst[3] = {&h->h_pos, &h->h_vel, &h->h_omg};
    const float4* src[3] = {B.pos, B.vel, B.omg};
    for (int f = 0; f < 3; ++f) {
        dst[f]->resize(n);
        if (!n) continue;
        // unsorted by the id lane, which the omega copy keeps (id + clump flag)
        SD_CUDA(h, sd::dem_unsort_async(src[f], B.omg, h->d_tmp, n, h->stream));
        SD_CUDA(h, cudaMemcpyAsync(dst[f]->data(), h->d_tmp, 16 * (size_t)n, cudaMemcpyDeviceToHost, h->stream));
        SD_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    const size_t nb = h->hb_pos.size();
    std::vector<float4>* bdst[5] = {&h->hb_pos, &h->hb_vel, &h->hb_quat, &h->hb_omg, &h->hb_ang};
    float4* const bsrc[5] = {B.bpos, B.bvel, B.bquat, B.bomg, B.bang};
    for (int k = 0; k < 5 && nb; ++k)
        SD_CUDA(h, cudaMemcpyAsync(bdst[k]->data(), bsrc[k], 16 * nb, cudaMemcpyDeviceToHost, h->stream));
    mesh_state->clear();
    if (B.mesh.ntri) {
        mesh_state->resize(24);
        SD_CUDA(h, cudaMemcpyAsync(mesh_state->data(), B.mesh.state, 24 * sizeof(float), cudaMemcpyDeviceToHost,
                                   h->stream));
    }
    SD_CUDA(h, cudaStreamSynchronize(h->stream));
    return SD_OK;
}

struct Change {
    std::vector<float> mesh_state;
    uint64_t steps = 0;
    bool active = false;
};

// A prepared engine's state to the host and its device buffers released.
static sd_status begin_change(sd_engine* h, Change* c) {
    if (!h->prepared) return SD_OK;
    if (h->hull_mode()) return fail(h, SD_ERR_UNSUPPORTED, "convex-hull scenes do not change after prepare");
    if (h->scenes.size() > 1) return fail(h, SD_ERR_UNSUPPORTED, "a batch of scenes does not change after prepare");
    sd_status s = pull_state(h, &c->mesh_state);
    if (s) return s;
    c->steps = h->steps;
    c->active = true;
    release_device(h);
    return SD_OK;
}

// Prepared again on the changed host state (status: the change's own).
static sd_status finish_change(sd_engine* h, const Change& c, sd_status status) {
    if (!c.active) return status;
    sd_status s = prepare_with(h, h->h_pos.data(), h->h_vel.data(), h->h_omg.data(), (uint32_t)h->h_pos.size());
    if (s) return s;
    h->steps = c.steps;
    if (!c.mesh_state.empty() && h->B.mesh.ntri) {
        SD_CUDA(h, cudaMemcpyAsync(h->B.mesh.state, c.mesh_state.data(), 24 * sizeof(float), cudaMemcpyHostToDevice,
                                   h->stream));
        SD_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    return status;
}

sd_status sd_engine_remove_spheres(sd_engine* h, uint64_t n, const uint32_t* ids) {
    if (!h || (n && !ids)) return fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (h->hull_mode()) return fail(h, SD_ERR_UNSUPPORTED, "not available for convex-hull scenes");
    if (!h->scenes.empty()) return fail(h, SD_ERR_UNSUPPORTED, "spheres of a batch of scenes cannot be removed");
    const uint64_t total = h->prepared ? h->B.n : h->h_pos.size();
    std::vector<char> gone(total, 0);
    for (uint64_t k = 0; k < n; ++k) {
        const uint32_t id = ids[k];
        if (id >= total) return fail(h, SD_ERR_INVALID_ARG, "sphere id " + std::to_string(id) + " out of range");
        if (gone[id]) return fail(h, SD_ERR_INVALID_ARG, "sphere id " + std::to_string(id) + " listed twice");
        if (h->h_body_of[id] >= 0)
            return fail(h, SD_ERR_UNSUPPORTED, "sphere " + std::to_string(id) + " belongs to a rigid clump");
        gone[id] = 1;
    }
    if (n == 0) return SD_OK;
    Change c;
    sd_status s = begin_change(h, &c);
    if (s) return s;
    // compact in id order; the kept spheres' ids are their ranks
    std::vector<uint32_t> new_id(total);
    uint32_t k = 0;
    for (uint64_t i = 0; i < total; ++i) {
        new_id[i] = k;
        if (gone[i]) continue;
        h->h_pos[k] = h->h_pos[i];
        h->h_vel[k] = h->h_vel[i];
        h->h_omg[k] = h->h_omg[i];
        h->h_body_of[k] = h->h_body_of[i];
        h->h_r0[k] = h->h_r0[i];
        const uint32_t bits = id_bits(k) | (h->h_body_of[k] >= 0 ? 0x80000000u : 0u);
        std::memcpy(&h->h_omg[k].w, &bits, 4);
        ++k;
    }
    for (auto* v : {&h->h_pos, &h->h_vel, &h->h_omg, &h->h_r0}) v->resize(k);
    h->h_body_of.resize(k);
    for (uint32_t& f : h->hb_first) f = new_id[f];  // a clump's spheres are all kept, still consecutive
    return finish_change(h, c, SD_OK);
}

sd_status sd_engine_add_spheres(sd_engine* h, uint64_t n, const float* pos4, const float* vel4,
                                const float* omega4) {
    if (!h) return fail(nullptr, SD_ERR_INVALID_ARG, "NULL engine");
    if (h->prepared) {
        Change c;
        sd_status s = begin_change(h, &c);
        if (s) return s;
        return finish_change(h, c, sd_engine_add_spheres(h, n, pos4, vel4, omega4));
    }
    if (!h->scenes.empty() && !h->adding_scene)
        return fail(h, SD_ERR_STATE, "spheres added outside a scene of the batch (use sd_engine_add_scene)");
    if (n && (!pos4 || !vel4)) return fail(h, SD_ERR_INVALID_ARG, "pos4/vel4 NULL");
    if (h->h_pos.size() + n >= 0x7fffffffull) return fail(h, SD_ERR_CAPACITY, "more than 2^31-1 spheres");
    for (uint64_t i = 0; i < n; ++i) {
        const float* p = pos4 + 4 * i;
        const float* v = vel4 + 4 * i;
        if (!(p[3] > 0.0f) || !(v[3] > 0.0f) || !std::isfinite(p[0]) || !std::isfinite(p[1]) ||
            !std::isfinite(p[2]) || !std::isfinite(v[0]) || !std::isfinite(v[1]) || !std::isfinite(v[2]))
            return fail(h, SD_ERR_INVALID_ARG, "sphere " + std::to_string(i) + ": radius and mass must be > 0 and values finite");
    }
    h->h_pos.reserve(h->h_pos.size() + n);
    for (uint64_t i = 0; i < n; ++i) {
        uint32_t id = (uint32_t)h->h_pos.size();
        h->h_pos.push_back(f4(pos4 + 4 * i));
        h->h_vel.push_back(f4(vel4 + 4 * i));
        float4 w = omega4 ? f4(omega4 + 4 * i) : make_float4(0.f, 0.f, 0.f, 0.f);
        w.w = id_as_float(id);
        h->h_omg.push_back(w);
        h->h_body_of.push_back(-1);
        h->h_r0.push_back(make_float4(0.f, 0.f, 0.f, 0.f));
    }
    return SD_OK;
}

sd_status sd_engine_add_mesh(sd_engine* h, uint32_t n_tris, const float* tri9, const int32_t* patch,
                             const float centre[3], const float axis[3], float omega) {
    if (!h || (n_tris && !tri9) || !centre) return fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (h->prepared) return fail(h, SD_ERR_STATE, "meshes cannot be added after prepare");
    if (n_tris == 0 || n_tris >= (1u << 26)) return fail(h, SD_ERR_INVALID_ARG, "n_tris must be in 1..2^26");
    double a[3] = {axis ? axis[0] : 0.0, axis ? axis[1] : 0.0, axis ? axis[2] : 1.0};
    const double an = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    if (!(an > 0.0)) return fail(h, SD_ERR_INVALID_ARG, "mesh axis is zero");
    if (!std::isfinite(omega)) return fail(h, SD_ERR_INVALID_ARG, "omega must be finite");
    auto& M = h->mesh;
    // Static meshes combine into one (triangles appended in the first mesh's
    // frame, patches renumbered after the ones already there); a rotating
    // mesh must be the only one.
    const bool merge = !M.tri.empty();
    if (merge && (M.omega != 0.0f || omega != 0.0f))
        return fail(h, SD_ERR_UNSUPPORTED, "a rotating mesh must be the engine's only mesh (static meshes combine)");
    if (merge && M.patch.size() + n_tris >= (1u << 26))
        return fail(h, SD_ERR_INVALID_ARG, "the meshes hold 2^26 triangles or more");
    for (uint32_t t = 0; t < n_tris; ++t) {
        for (int k = 0; k < 9; ++k)
            if (!std::isfinite(tri9[9 * (size_t)t + k])) return fail(h, SD_ERR_INVALID_ARG, "mesh vertex not finite");
        if (patch && patch[t] < 0) return fail(h, SD_ERR_INVALID_ARG, "mesh patch ids must be >= 0");
    }
    const float c[3] = {merge ? M.centre[0] : centre[0], merge ? M.centre[1] : centre[1],
                        merge ? M.centre[2] : centre[2]};
    int32_t poff = 0;
    for (int32_t pid : M.patch) poff = std::max(poff, pid + 1);
    const size_t t0 = M.patch.size();
    M.tri.resize(3 * (t0 + n_tris));
    M.patch.resize(t0 + n_tris);
    for (uint32_t t = 0; t < n_tris; ++t) {
        for (int k = 0; k < 3; ++k) {
            const float* v = tri9 + 9 * (size_t)t + 3 * k;
            M.tri[3 * (t0 + t) + k] = make_float4(v[0] - c[0], v[1] - c[1], v[2] - c[2], 0.0f);
        }
        M.patch[t0 + t] = poff + (patch ? patch[t] : (int32_t)t);
    }
    if (!merge) {
        for (int k = 0; k < 3; ++k) {
            M.centre[k] = centre[k];
            M.axis[k] = (float)(a[k] / an);
        }
        M.omega = omega;
    }
    return SD_OK;
}

sd_status sd_engine_get_mesh(sd_engine* h, uint64_t cap, float* tri9, int32_t* patch, float* centre3,
                             uint64_t* n_tris) {
    if (!h || !n_tris) return fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    const auto& M = h->mesh;
    *n_tris = M.patch.size();
    if (centre3)
        for (int k = 0; k < 3; ++k) centre3[k] = M.centre[k];
    if (tri9 || patch) {
        if (cap < *n_tris) return fail(h, SD_ERR_CAPACITY, "capacity below the mesh's triangle count");
        for (uint64_t t = 0; t < *n_tris; ++t) {
            if (tri9)
                for (int k = 0; k < 3; ++k) {
                    const float4 v = M.tri[3 * t + k];
                    tri9[9 * t + 3 * k] = v.x;
                    tri9[9 * t + 3 * k + 1] = v.y;
                    tri9[9 * t + 3 * k + 2] = v.z;
                }
            if (patch) patch[t] = M.patch[t];
        }
    }
    return SD_OK;
}

sd_status sd_engine_get_mesh_state(sd_engine* h, float* state24) {
    if (!h || !state24) return fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (!h->prepared || !h->B.mesh.ntri) return fail(h, SD_ERR_STATE, "no prepared mesh");
    SD_CUDA(h, cudaMemcpyAsync(state24, h->B.mesh.state, 24 * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    SD_CUDA(h, cudaStreamSynchronize(h->stream));
    return SD_OK;
}

sd_status sd_engine_add_scene(sd_engine* h, uint64_t n, const float* pos4, const float* vel4, const float* omega4,
                              const float lo[3], const float hi[3], float cell) {
    if (!h || !lo || !hi) return fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (h->prepared) return fail(h, SD_ERR_STATE, "scenes cannot be added after prepare");
    if (!h->hb_pos.empty()) return fail(h, SD_ERR_UNSUPPORTED, "rigid clumps are not supported in a batch");
    if (h->scenes.empty() && !h->h_pos.empty())
        return fail(h, SD_ERR_STATE, "spheres added outside a scene: use sd_engine_add_scene for every sphere");
    if (h->scenes.size() >= (1u << 20)) return fail(h, SD_ERR_CAPACITY, "too many scenes");
    for (int a = 0; a < 3; ++a)
        if (!(hi[a] > lo[a]) || !std::isfinite(lo[a]) || !std::isfinite(hi[a]))
            return fail(h, SD_ERR_INVALID_ARG, "scene box: hi must exceed lo on every axis");
    if (cell < 0.0f || !std::isfinite(cell)) return fail(h, SD_ERR_INVALID_ARG, "scene cell must be >= 0");
    sd_engine::SceneHost sc{};
    for (int a = 0; a < 3; ++a) {
        sc.lo[a] = lo[a];
        sc.hi[a] = hi[a];
    }
    sc.cell = cell;
    sc.first = (uint32_t)h->h_pos.size();
    sc.count = (uint32_t)n;
    h->adding_scene = true;
    sd_status s = sd_engine_add_spheres(h, n, pos4, vel4, omega4);
    h->adding_scene = false;
    if (s) return s;
    h->scenes.push_back(sc);
    return SD_OK;
}

sd_status sd_engine_add_clump(sd_engine* h, uint32_t n, const float* rel4, float mass, const float com[3],
                              const float vel[3], const float omega[3]) {
    if (!h || !rel4 || !com || !vel) return fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (h->prepared) {
        Change c;
        sd_status s = begin_change(h, &c);
        if (s) return s;
        return finish_change(h, c, sd_engine_add_clump(h, n, rel4, mass, com, vel, omega));
    }
    if (n == 0) return fail(h, SD_ERR_INVALID_ARG, "a clump needs at least one sphere");
    if (!(mass > 0.0f) || !std::isfinite(mass)) return fail(h, SD_ERR_INVALID_ARG, "clump mass must be > 0");
    if (h->h_pos.size() + n >= 0x7fffffffull) return fail(h, SD_ERR_CAPACITY, "more than 2^31-1 spheres");
    for (uint32_t i = 0; i < n; ++i)
        if (!(rel4[4 * i + 3] > 0.0f) || !std::isfinite(rel4[4 * i]) || !std::isfinite(rel4[4 * i + 1]) ||
            !std::isfinite(rel4[4 * i + 2]))
            return fail(h, SD_ERR_INVALID_ARG, "clump sphere " + std::to_string(i) + ": bad offset or radius");
    // inertia of the spheres as solid balls of mass/n about the centre, in
    // double, and its inverse by cofactors
    const double ms = (double)mass / n;
    double I[9] = {0};
    for (uint32_t i = 0; i < n; ++i) {
        const double x = rel4[4 * i], y = rel4[4 * i + 1], z = rel4[4 * i + 2], r = rel4[4 * i + 3];
        const double self = 0.4 * ms * r * r, d2 = x * x + y * y + z * z;
        const double v[3] = {x, y, z};
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) I[3 * a + b] += ms * ((a == b ? d2 : 0.0) - v[a] * v[b]) + (a == b ? self : 0.0);
    }
    const double c00 = I[4] * I[8] - I[5] * I[7], c01 = I[5] * I[6] - I[3] * I[8], c02 = I[3] * I[7] - I[4] * I[6];
    const double det = I[0] * c00 + I[1] * c01 + I[2] * c02;
    if (!(det > 0.0)) return fail(h, SD_ERR_INVALID_ARG, "clump inertia is singular");
    double inv[9] = {c00 / det, (I[2] * I[7] - I[1] * I[8]) / det, (I[1] * I[5] - I[2] * I[4]) / det,
                     c01 / det, (I[0] * I[8] - I[2] * I[6]) / det, (I[2] * I[3] - I[0] * I[5]) / det,
                     c02 / det, (I[1] * I[6] - I[0] * I[7]) / det, (I[0] * I[4] - I[1] * I[3]) / det};
    const double w[3] = {omega ? omega[0] : 0.0, omega ? omega[1] : 0.0, omega ? omega[2] : 0.0};
    const uint32_t b = (uint32_t)h->hb_pos.size();
    h->hb_pos.push_back(make_float4(com[0], com[1], com[2], mass));
    h->hb_vel.push_back(make_float4(vel[0], vel[1], vel[2], 0.f));
    h->hb_quat.push_back(make_float4(1.f, 0.f, 0.f, 0.f));
    h->hb_omg.push_back(make_float4((float)w[0], (float)w[1], (float)w[2], 0.f));
    h->hb_ang.push_back(make_float4((float)(I[0] * w[0] + I[1] * w[1] + I[2] * w[2]),
                                    (float)(I[3] * w[0] + I[4] * w[1] + I[5] * w[2]),
                                    (float)(I[6] * w[0] + I[7] * w[1] + I[8] * w[2]), 0.f));
    for (int r = 0; r < 3; ++r)
        h->hb_inv.push_back(make_float4((float)inv[3 * r], (float)inv[3 * r + 1], (float)inv[3 * r + 2], 0.f));
    h->hb_first.push_back((uint32_t)h->h_pos.size());
    h->hb_count.push_back(n);
    for (uint32_t i = 0; i < n; ++i) {
        const float* r = rel4 + 4 * i;
        const uint32_t id = (uint32_t)h->h_pos.size();
        h->h_pos.push_back(make_float4(com[0] + r[0], com[1] + r[1], com[2] + r[2], r[3]));
        const double sv[3] = {w[1] * r[2] - w[2] * r[1], w[2] * r[0] - w[0] * r[2], w[0] * r[1] - w[1] * r[0]};
        h->h_vel.push_back(make_float4((float)(vel[0] + sv[0]), (float)(vel[1] + sv[1]), (float)(vel[2] + sv[2]), mass));
        float4 o = make_float4((float)w[0], (float)w[1], (float)w[2], 0.f);
        const uint32_t bits = id_bits(id) | 0x80000000u;
        std::memcpy(&o.w, &bits, 4);
        h->h_omg.push_back(o);
        h->h_body_of.push_back((int32_t)b);
        h->h_r0.push_back(make_float4(r[0], r[1], r[2], 0.f));
    }
    return SD_OK;
}

sd_status sd_engine_add_particle(sd_engine* h, int32_t grid_resolution, float size, float diameter, float mass,
                                 const float position[3], const float velocity[3]) {
    if (!h || !position || !velocity) return fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (grid_resolution < 1 || grid_resolution > 64) return fail(h, SD_ERR_INVALID_ARG, "grid_resolution must be 1..64");
    if (!(diameter > 0.0f) || !(size > 0.0f)) return fail(h, SD_ERR_INVALID_ARG, "size and diameter must be > 0");
    if (grid_resolution == 1) {
        float p[4] = {position[0], position[1], position[2], 0.5f * diameter};
        float v[4] = {velocity[0], velocity[1], velocity[2], mass};
        return sd_engine_add_spheres(h, 1, p, v, nullptr);
    }
    // DEMParticle::initParticles / getCenterOfMass / setParticlesInWorldSpace
    // (entity.cpp:9-59): spacing size / floor(size/diameter)^2, local sphere
    // positions (i, j, k) * dx, world = position - (local - COM), so the
    // offsets from the body centre (= position) are COM - local
    const float q = std::floor(size / diameter);
    const float num = q * q;
    if (!(num > 0.0f)) return fail(h, SD_ERR_INVALID_ARG, "size smaller than diameter");
    const float dx = size / num;
    const int R = grid_resolution;
    std::vector<float> local;
    for (int i = 1; i <= R; ++i)
        for (int j = 1; j <= R; ++j)
            for (int k = 1; k <= R; ++k) {
                local.push_back((float)i * dx);
                local.push_back((float)j * dx);
                local.push_back((float)k * dx);
            }
    double c[3] = {0, 0, 0};
    const size_t cnt = local.size() / 3;
    for (size_t s = 0; s < cnt; ++s)
        for (int a = 0; a < 3; ++a) c[a] += local[3 * s + a];
    std::vector<float> rel(4 * cnt);
    for (size_t s = 0; s < cnt; ++s) {
        for (int a = 0; a < 3; ++a) rel[4 * s + a] = (float)(c[a] / (double)cnt) - local[3 * s + a];
        rel[4 * s + 3] = 0.5f * diameter;
    }
    return sd_engine_add_clump(h, (uint32_t)cnt, rel.data(), mass, position, velocity, nullptr);
}

static bool json_vec3(const sd::JsonValue* v, float out[3]) {
    if (!v || v->kind != sd::JsonValue::Array || v->arr.size() != 3) return false;
    for (int k = 0; k < 3; ++k) {
        if (v->arr[k].kind != sd::JsonValue::Number) return false;
        out[k] = (float)v->arr[k].num;
    }
    return true;
}

static bool json_num(const sd::JsonValue* v, float* out) {
    if (!v || v->kind != sd::JsonValue::Number) return false;
    *out = (float)v->num;
    return true;
}

static bool keys_subset(const sd::JsonValue& o, std::initializer_list<const char*> allowed, std::string* bad) {
    for (auto& kv : o.obj) {
        bool ok = false;
        for (const char* a : allowed) ok = ok || kv.first == a;
        if (!ok) {
            *bad = kv.first;
            return false;
        }
    }
    return true;
}

sd_status sd_engine_load_scene_json(sd_engine* h, const char* path) {
    if (!h || !path) return fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (h->prepared) return fail(h, SD_ERR_STATE, "scene must be loaded before prepare");
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(h, SD_ERR_IO, std::string("cannot open ") + path);
    std::stringstream ss;
    ss << f.rdbuf();
    std::string text = ss.str();
    sd::JsonValue root;
    std::string perr;
    if (!sd::JsonParser(text).parse(&root, &perr)) return fail(h, SD_ERR_JSON, perr);
    std::string bad;
    if (root.kind != sd::JsonValue::Object) return fail(h, SD_ERR_JSON, "top level must be an object");
    if (!keys_subset(root, {"scene"}, &bad)) return fail(h, SD_ERR_JSON, "unknown top-level key \"" + bad + "\"");
    const sd::JsonValue* scene = root.get("scene");
    if (!scene || scene->kind != sd::JsonValue::Object) return fail(h, SD_ERR_JSON, "missing object \"scene\"");
    if (!keys_subset(*scene, {"domain", "entities", "gravity", "box", "walls", "cell", "material", "spheres"}, &bad))
        return fail(h, SD_ERR_JSON, "unknown key scene." + bad);
    sd_config c = h->cfg;
    float tmp;
    if (const sd::JsonValue* d = scene->get("domain")) {
        if (!json_num(d, &tmp) || !(tmp > 0)) return fail(h, SD_ERR_JSON, "scene.domain must be a positive number");
        c.domain = tmp;
    }
    if (const sd::JsonValue* g = scene->get("gravity")) {
        if (!json_num(g, &tmp)) return fail(h, SD_ERR_JSON, "scene.gravity must be a number (magnitude along -z)");
        c.gravity[0] = 0.f;
        c.gravity[1] = 0.f;
        c.gravity[2] = -tmp;
    }
    if (const sd::JsonValue* b = scene->get("box")) {
        if (b->kind != sd::JsonValue::Object || !keys_subset(*b, {"lo", "hi"}, &bad) || !json_vec3(b->get("lo"), c.box_lo) ||
            !json_vec3(b->get("hi"), c.box_hi))
            return fail(h, SD_ERR_JSON, "scene.box must be {lo:[3], hi:[3]}");
    }
    if (const sd::JsonValue* w = scene->get("walls")) {
        if (!json_num(w, &tmp) || tmp < 0 || tmp > 63 || tmp != std::floor(tmp))
            return fail(h, SD_ERR_JSON, "scene.walls must be an integer mask 0..63");
        c.walls = (int32_t)tmp;
    }
    if (const sd::JsonValue* ce = scene->get("cell")) {
        if (!json_num(ce, &tmp) || !(tmp > 0)) return fail(h, SD_ERR_JSON, "scene.cell must be a positive number");
        c.cell = tmp;
    }
    if (const sd::JsonValue* m = scene->get("material")) {
        if (m->kind != sd::JsonValue::Object || !keys_subset(*m, {"kn", "restitution", "mu"}, &bad))
            return fail(h, SD_ERR_JSON, "scene.material may hold kn, restitution, mu");
        if (m->get("kn") && !json_num(m->get("kn"), &c.kn)) return fail(h, SD_ERR_JSON, "material.kn");
        if (m->get("restitution") && !json_num(m->get("restitution"), &c.restitution))
            return fail(h, SD_ERR_JSON, "material.restitution");
        if (m->get("mu") && !json_num(m->get("mu"), &c.mu)) return fail(h, SD_ERR_JSON, "material.mu");
    }
    std::vector<float> pos, vel;
    // cube clumps (grid_resolution > 1) are added after the plain spheres
    // parsed before them, so ids follow the file order
    struct Cube {
        size_t after;  // number of plain spheres (x4 floats) parsed before it
        int32_t res;
        float size, diameter, mass, p3[3], v3[3];
    };
    std::vector<Cube> cubes;
    // mesh entities (DEMMesh): an STL file placed by position + quaternion,
    // static or rotating; the file name is relative to the JSON file
    struct MeshEnt {
        std::string file;
        float p3[3] = {0, 0, 0}, q4[4] = {1, 0, 0, 0}, centre[3] = {0, 0, 0}, axis[3] = {0, 0, 1};
        float omega = 0.0f, angle = 30.0f;
    };
    std::vector<MeshEnt> meshes;
    std::string dir(path);
    dir = dir.find('/') == std::string::npos ? std::string() : dir.substr(0, dir.rfind('/') + 1);
    if (const sd::JsonValue* ents = scene->get("entities")) {
        if (ents->kind != sd::JsonValue::Array) return fail(h, SD_ERR_JSON, "scene.entities must be an array");
        for (size_t i = 0; i < ents->arr.size(); ++i) {
            const sd::JsonValue& e = ents->arr[i];
            std::string where = "scene.entities[" + std::to_string(i) + "]";
            if (e.kind != sd::JsonValue::Object) return fail(h, SD_ERR_JSON, where + " must be an object");
            const sd::JsonValue* t = e.get("type");
            if (t && t->kind == sd::JsonValue::String && t->str == "mesh") {
                if (!keys_subset(e, {"type", "file", "position", "quaternion", "rotation", "patch_angle"}, &bad))
                    return fail(h, SD_ERR_JSON, "unknown key " + where + "." + bad);
                MeshEnt me;
                const sd::JsonValue* fn = e.get("file");
                if (!fn || fn->kind != sd::JsonValue::String || fn->str.empty())
                    return fail(h, SD_ERR_JSON, where + ".file must name an STL file");
                me.file = fn->str[0] == '/' ? fn->str : dir + fn->str;
                if (e.get("position") && !json_vec3(e.get("position"), me.p3))
                    return fail(h, SD_ERR_JSON, where + ".position must be [x,y,z]");
                if (const sd::JsonValue* q = e.get("quaternion")) {
                    if (q->kind != sd::JsonValue::Array || q->arr.size() != 4)
                        return fail(h, SD_ERR_JSON, where + ".quaternion must be [s,x,y,z]");
                    for (int k = 0; k < 4; ++k)
                        if (!json_num(&q->arr[k], &me.q4[k])) return fail(h, SD_ERR_JSON, where + ".quaternion must be [s,x,y,z]");
                }
                if (const sd::JsonValue* r = e.get("rotation")) {
                    if (r->kind != sd::JsonValue::Object || !keys_subset(*r, {"centre", "axis", "omega"}, &bad) ||
                        !json_vec3(r->get("centre"), me.centre) || !json_vec3(r->get("axis"), me.axis) ||
                        !json_num(r->get("omega"), &me.omega))
                        return fail(h, SD_ERR_JSON, where + ".rotation must be {centre:[3], axis:[3], omega}");
                }
                if (e.get("patch_angle") &&
                    (!json_num(e.get("patch_angle"), &me.angle) || !(me.angle >= 0.0f && me.angle <= 180.0f)))
                    return fail(h, SD_ERR_JSON, where + ".patch_angle must be in [0, 180] degrees");
                meshes.push_back(me);
                continue;
            }
            if (!keys_subset(e, {"type", "position", "size", "mass", "velocity", "grid_resolution", "diameter"}, &bad))
                return fail(h, SD_ERR_JSON, "unknown key " + where + "." + bad);
            if (!t || t->kind != sd::JsonValue::String || t->str != "generic")
                return fail(h, SD_ERR_JSON, where + ".type must be \"generic\" or \"mesh\"");
            float p3[3], v3[3] = {0, 0, 0}, size, mass;
            if (!json_vec3(e.get("position"), p3)) return fail(h, SD_ERR_JSON, where + ".position must be [x,y,z]");
            if (e.get("velocity") && !json_vec3(e.get("velocity"), v3))
                return fail(h, SD_ERR_JSON, where + ".velocity must be [vx,vy,vz]");
            if (!json_num(e.get("size"), &size) || !(size > 0)) return fail(h, SD_ERR_JSON, where + ".size must be > 0");
            if (!json_num(e.get("mass"), &mass) || !(mass > 0)) return fail(h, SD_ERR_JSON, where + ".mass must be > 0");
            float res = 1.0f, diam = size;
            if (e.get("grid_resolution") &&
                (!json_num(e.get("grid_resolution"), &res) || res != std::floor(res) || res < 1.0f || res > 64.0f))
                return fail(h, SD_ERR_JSON, where + ".grid_resolution must be an integer in 1..64");
            if (e.get("diameter") && (!json_num(e.get("diameter"), &diam) || !(diam > 0) || diam > size))
                return fail(h, SD_ERR_JSON, where + ".diameter must be in (0, size]");
            if (res > 1.0f) {
                cubes.push_back(Cube{pos.size(), (int32_t)res, size, diam, mass, {p3[0], p3[1], p3[2]},
                                     {v3[0], v3[1], v3[2]}});
                continue;
            }
            float p4[4] = {p3[0], p3[1], p3[2], 0.5f * size}, v4[4] = {v3[0], v3[1], v3[2], mass};
            pos.insert(pos.end(), p4, p4 + 4);
            vel.insert(vel.end(), v4, v4 + 4);
        }
    }
    if (const sd::JsonValue* sph = scene->get("spheres")) {
        if (sph->kind != sd::JsonValue::Array) return fail(h, SD_ERR_JSON, "scene.spheres must be an array");
        for (size_t i = 0; i < sph->arr.size(); ++i) {
            const sd::JsonValue& e = sph->arr[i];
            std::string where = "scene.spheres[" + std::to_string(i) + "]";
            if (e.kind != sd::JsonValue::Object || !keys_subset(e, {"position", "radius", "mass", "velocity"}, &bad))
                return fail(h, SD_ERR_JSON, where + ": expected {position, radius, mass, velocity}");
            float p3[3], v3[3] = {0, 0, 0}, r, m;
            if (!json_vec3(e.get("position"), p3) || !json_num(e.get("radius"), &r) || !json_num(e.get("mass"), &m) ||
                !(r > 0) || !(m > 0) || (e.get("velocity") && !json_vec3(e.get("velocity"), v3)))
                return fail(h, SD_ERR_JSON, where + ": bad position/radius/mass/velocity");
            float p4[4] = {p3[0], p3[1], p3[2], r}, v4[4] = {v3[0], v3[1], v3[2], m};
            pos.insert(pos.end(), p4, p4 + 4);
            vel.insert(vel.end(), v4, v4 + 4);
        }
    }
    for (const Cube& cb : cubes) {
        const float q = std::floor(cb.size / cb.diameter);
        if (!(q >= 1.0f)) return fail(h, SD_ERR_JSON, "a cube entity's size is smaller than its diameter");
    }
    h->cfg = c;
    for (const MeshEnt& me : meshes)
        if (sd_status s = sd_engine_add_mesh_stl(h, me.file.c_str(), me.p3, me.q4, me.centre, me.axis, me.omega,
                                                 me.angle))
            return s;
    size_t done = 0;  // floats of `pos` added so far
    for (const Cube& cb : cubes) {
        if (cb.after > done) {
            if (sd_status s = sd_engine_add_spheres(h, (cb.after - done) / 4, pos.data() + done, vel.data() + done,
                                                    nullptr))
                return s;
            done = cb.after;
        }
        if (sd_status s = sd_engine_add_particle(h, cb.res, cb.size, cb.diameter, cb.mass, cb.p3, cb.v3)) return s;
    }
    if (pos.size() == done) return SD_OK;
    return sd_engine_add_spheres(h, (pos.size() - done) / 4, pos.data() + done, vel.data() + done, nullptr);
}

sd_status sd_engine_prepare(sd_engine* h) {
    if (!h) return fail(nullptr, SD_ERR_INVALID_ARG, "NULL engine");
    if (h->prepared) return fail(h, SD_ERR_STATE, "already prepared");
    if (h->hull_mode()) {
        if (!h->h_pos.empty())
            return fail(h, SD_ERR_UNSUPPORTED, "a scene holds spheres/clumps or convex hulls, not both");
        sd_status s = hull_prepare(h);
        if (s) release_device(h);
        return s;
    }
    return prepare_with(h, h->h_pos.data(), h->h_vel.data(), h->h_omg.data(), (uint32_t)h->h_pos.size());
}

sd_status sd_engine_step(sd_engine* h, float dt, int32_t n_steps) {
    if (!h) return fail(nullptr, SD_ERR_INVALID_ARG, "NULL engine");
    if (!h->prepared) return fail(h, SD_ERR_STATE, "call sd_engine_prepare first");
    if (!(dt > 0.0f) || !std::isfinite(dt)) return fail(h, SD_ERR_INVALID_ARG, "dt must be positive and finite");
    if (n_steps < 0) return fail(h, SD_ERR_INVALID_ARG, "n_steps < 0");
    if (h->hull_mode()) return hull_step(h, dt, n_steps);
    SD_CUDA(h, cudaSetDevice(h->device));
    sd_status s = resort_if_needed(h);
    if (s) return s;
    if (!h->graph_valid || h->graph_dt != dt || h->graph_epoch != g_tune_epoch.load()) {
        h->graph_epoch = g_tune_epoch.load();
        if ((s = build_graph(h, dt))) return s;
        // steps of the previous graph may have used no lists (a knob change
        // turned them off) and moved spheres without checking their skin:
        // the first step of a list graph builds them again
        if ((s = force_list_build(h))) return s;
    }
    for (int32_t i = 0; i < n_steps; ++i) {
        SD_CUDA(h, cudaGraphLaunch(h->graph_parity ? h->graph_alt : h->graph, h->stream));
        if (h->graph_swaps) {  // the next state was sorted in place in the *_n buffers
            swap_state(h->B);
            h->graph_parity ^= 1;
        }
    }
    if (n_steps > 0 && !h->hull_mode()) h->keys_current = true;  // every step ends with a sort + reorder
    h->steps += (uint64_t)n_steps;
    return SD_OK;
}

sd_status sd_engine_update(sd_engine* h, float dt) { return sd_engine_step(h, dt, 1); }

sd_status sd_tune_set(const char* knob, int32_t value) {
    if (!knob) return fail(nullptr, SD_ERR_INVALID_ARG, "knob NULL");
    std::string k(knob);
    if (k == "contact_mode") {
        if (value != 0 && value != 1) return fail(nullptr, SD_ERR_INVALID_ARG, "contact_mode must be 0 or 1");
        sd::dem_set_contact_mode(value);
    } else if (k == "sort_items") {
        if (value != 8 && value != 16) return fail(nullptr, SD_ERR_INVALID_ARG, "sort_items must be 8 or 16");
        sd::sort_set_items(value);
    } else if (k == "z_div") {
        if (value != 0 && value != 1 && value != 2 && value != 4 && value != 8)
            return fail(nullptr, SD_ERR_INVALID_ARG, "z_div must be 0, 1, 2, 4 or 8");
        g_z_div = value;
    } else if (k == "contact_block") {
        if (value != 64 && value != 128 && value != 256)
            return fail(nullptr, SD_ERR_INVALID_ARG, "contact_block must be 64, 128 or 256");
        sd::dem_set_contact_block(value);
    } else if (k == "fix_blocks") {
        if (value != 2 && value != 4 && value != 8) return fail(nullptr, SD_ERR_INVALID_ARG, "fix_blocks must be 2, 4 or 8");
        sd::dem_set_fix_blocks(value);
    } else if (k == "listed_blocks") {
        if (value != 4 && value != 5 && value != 6 && value != 8)
            return fail(nullptr, SD_ERR_INVALID_ARG, "listed_blocks must be 4, 5, 6 or 8");
        sd::dem_set_listed_blocks(value);
    } else if (k == "lbvh_rebuild") {
        if (value < 1 || value > 4096) return fail(nullptr, SD_ERR_INVALID_ARG, "lbvh_rebuild must be in [1, 4096]");
        sd::lbvh_set_rebuild_every(value);
    } else if (k == "hull_blocks") {
        if (value != 3 && value != 4) return fail(nullptr, SD_ERR_INVALID_ARG, "hull_blocks must be 3 or 4");
        sd::hull_set_blocks(value);
    } else if (k == "skin_um") {
        if (value < 0 || value > 100000) return fail(nullptr, SD_ERR_INVALID_ARG, "skin_um must be in [0, 100000]");
        g_skin_um = value;
    } else if (k == "pair_lists") {
        if (value < 0 || value > 2) return fail(nullptr, SD_ERR_INVALID_ARG, "pair_lists must be 0, 1 or 2");
        sd::dem_set_pair_lists(value);
    } else if (k == "resort_max") {
        if (value < 0 || value > (int32_t)sd::kResortMaxCap || (value & (value - 1)) != 0)
            return fail(nullptr, SD_ERR_INVALID_ARG, "resort_max must be 0 or a power of two up to 1024");
        sd::dem_set_resort_max((uint32_t)value);
    } else {
        return fail(nullptr, SD_ERR_INVALID_ARG, "unknown knob " + k);
    }
    g_tune_epoch.fetch_add(1);
    return SD_OK;
}

sd_status sd_tune_get(const char* knob, int32_t* value) {
    if (!knob || !value) return fail(nullptr, SD_ERR_INVALID_ARG, "NULL argument");
    std::string k(knob);
    if (k == "contact_mode") *value = sd::dem_contact_mode();
    else if (k == "sort_items") *value = sd::sort_items();
    else if (k == "z_div") *value = g_z_div;
    else if (k == "resort_max") *value = (int32_t)sd::dem_resort_max();
    else if (k == "pair_lists") *value = sd::dem_pair_lists();
    else if (k == "skin_um") *value = g_skin_um;
    else if (k == "listed_blocks") *value = sd::dem_listed_blocks();
    else if (k == "contact_block") *value = sd::dem_contact_block();
    else if (k == "fix_blocks") *value = sd::dem_fix_blocks();
    else if (k == "hull_blocks") *value = sd::hull_blocks();
    else if (k == "lbvh_rebuild") *value = sd::lbvh_rebuild_every();
    else return fail(nullptr, SD_ERR_INVALID_ARG, "unknown knob " + k);
    return SD_OK;
}

sd_status sd_engine_sync(sd_engine* h) {
    if (!h) return fail(nullptr, SD_ERR_INVALID_ARG, "NULL engine");
    if (!h->prepared) return SD_OK;
    SD_CUDA(h, cudaStreamSynchronize(h->stream));
    uint32_t bits = 0;
    sd_status s = read_device_errors(h, &bits);
    if (s) return s;
    return errors_to_status(h, bits);
}

static const float4* field_ptr(sd_engine* h, int32_t field) {
    switch (field) {
        case SD_FIELD_POSITION: return h->B.pos;
        case SD_FIELD_VELOCITY: return h->B.vel;
        case SD_FIELD_OMEGA: return h->B.omg;
        case SD_FIELD_FORCE: return h->B.force;
        case SD_FIELD_TORQUE: return h->B.torque;
        default: return nullptr;
    }
}

// Device address of a host buffer that kernels can read and write in place:
// page-locked memory mapped into the device's address space (cudaHostAlloc,
// cudaHostRegister, torch's pinned tensors).  Kernels then move the data
// over the host link themselves, with no staging copy; for other memory
// this returns nullptr and the caller stages through device memory.
static void* mapped_host(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // unregistered pointers may report an error: clear it
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

sd_status sd_engine_get_state(sd_engine* h, int32_t field, void* host_dst, size_t bytes) {
    if (!h || !host_dst) return fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (!h->prepared) return fail(h, SD_ERR_STATE, "call sd_engine_prepare first");
    if (h->hull_mode()) return fail(h, SD_ERR_UNSUPPORTED, "not available for convex-hull scenes (use sd_engine_get_bodies)");
    uint32_t n = h->B.n;
    if (bytes != (size_t)n * sizeof(float4)) return fail(h, SD_ERR_INVALID_ARG, "bytes must be n_spheres * 16");
    if (field == SD_FIELD_IDS) return fail(h, SD_ERR_INVALID_ARG, "SD_FIELD_IDS is a device-pointer field");
    if ((field == SD_FIELD_FORCE || field == SD_FIELD_TORQUE) && !(h->cfg.flags & SD_FLAG_RECORD))
        return fail(h, SD_ERR_STATE, "force/torque need SD_FLAG_RECORD");
    const float4* src = field_ptr(h, field);
    if (!src) return fail(h, SD_ERR_INVALID_ARG, "unknown field");
    SD_CUDA(h, cudaSetDevice(h->device));
    sd_status s = resort_if_needed(h);
    if (s) return s;
    if (field == SD_FIELD_FORCE || field == SD_FIELD_TORQUE) {
        // recorded by sphere id already
        SD_CUDA(h, cudaMemcpyAsync(host_dst, src, bytes, cudaMemcpyDeviceToHost, h->stream));
    } else if (float4* dev_view = static_cast<float4*>(mapped_host(host_dst))) {
        SD_CUDA(h, sd::dem_host_out_async(src, h->B.omg, dev_view, reinterpret_cast<uint32_t*>(h->d_tmp), n,
                                          h->stream));
    } else {
        SD_CUDA(h, sd::dem_unsort_async(src, h->B.omg, h->d_tmp, n, h->stream));
        SD_CUDA(h, cudaMemcpyAsync(host_dst, h->d_tmp, bytes, cudaMemcpyDeviceToHost, h->stream));
    }
    SD_CUDA(h, cudaStreamSynchronize(h->stream));
    if (field == SD_FIELD_OMEGA) {
        float4* o = static_cast<float4*>(host_dst);
        for (uint32_t i = 0; i < n; ++i) o[i].w = 0.0f;
    }
    return SD_OK;
}

sd_status sd_engine_set_state(sd_engine* h, int32_t field, const void* host_src, size_t bytes) {
    if (!h || !host_src) return fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (!h->prepared) return fail(h, SD_ERR_STATE, "call sd_engine_prepare first");
    if (h->hull_mode()) return fail(h, SD_ERR_UNSUPPORTED, "not available for convex-hull scenes (use sd_engine_get_bodies)");
    uint32_t n = h->B.n;
    if (bytes != (size_t)n * sizeof(float4)) return fail(h, SD_ERR_INVALID_ARG, "bytes must be n_spheres * 16");
    if (field != SD_FIELD_POSITION && field != SD_FIELD_VELOCITY && field != SD_FIELD_OMEGA)
        return fail(h, SD_ERR_INVALID_ARG, "only POSITION, VELOCITY, OMEGA can be set");
    SD_CUDA(h, cudaSetDevice(h->device));
    sd_status s = resort_if_needed(h);
    if (s) return s;
    float4* dst = const_cast<float4*>(field_ptr(h, field));
    // the omega array's w lane holds the slot's sphere id: keep it
    const bool keep_w = field == SD_FIELD_OMEGA;
    if (const float4* in = static_cast<const float4*>(mapped_host(host_src))) {
        SD_CUDA(h, sd::dem_host_in_async(in, h->B.omg, dst, reinterpret_cast<uint32_t*>(h->d_tmp), n, keep_w,
                                         h->stream));
    } else {
        SD_CUDA(h, cudaMemcpyAsync(h->d_tmp, host_src, bytes, cudaMemcpyHostToDevice, h->stream));
        SD_CUDA(h, sd::dem_scatter_in_async(h->d_tmp, h->B.omg, dst, n, keep_w, h->stream));
    }
    // Only a position change can change cell keys.  When every sphere stays
    // in the cell it is sorted under, a stable re-sort is the identity and
    // the cell table still holds: count the slots whose key changed, and
    // re-sort before the next step only if there are any.
    const bool check = field == SD_FIELD_POSITION && h->keys_current && !h->need_resort;
    uint32_t changed = 1;
    if (check) {
        uint32_t* d_changed = h->B.dev_status + 4;
        SD_CUDA(h, sd::dem_keys_changed_async(h->P, h->B, d_changed, h->stream));
        SD_CUDA(h, cudaMemcpyAsync(&changed, d_changed, 4, cudaMemcpyDeviceToHost, h->stream));
    }
    // new positions: the contact lists are built again at the next step if
    // a sphere left its skin (lists that are off are rebuilt when they come
    // back on)
    if (field == SD_FIELD_POSITION) SD_CUDA(h, sd::dem_skin_check_async(h->B, h->stream));
    SD_CUDA(h, cudaStreamSynchronize(h->stream));
    if (field == SD_FIELD_POSITION && changed != 0) h->need_resort = true;
    return SD_OK;
}

sd_status sd_engine_launch_stage(sd_engine* h, int32_t stage, float dt) {
    if (!h) return fail(nullptr, SD_ERR_INVALID_ARG, "NULL engine");
    if (!h->prepared) return fail(h, SD_ERR_STATE, "call sd_engine_prepare first");
    if (h->hull_mode()) {
        if (stage != SD_STAGE_CONTACT) return fail(h, SD_ERR_UNSUPPORTED, "convex-hull scenes have the contact stage only");
        return hull_launch_narrow(h);
    }
    SD_CUDA(h, cudaSetDevice(h->device));
    sd_status s = resort_if_needed(h);
    if (s) return s;
    h->keys_current = false;  // a lone stage can leave keys and slots apart
    // the contact stage alone leaves the state as it is (it writes the
    // next-state buffers), so the lists stay valid; a lone sort or reorder
    // moves the state without checking the skin: the next step builds them
    if (stage != SD_STAGE_CONTACT && (s = force_list_build(h))) return s;
    switch (stage) {
        case SD_STAGE_CONTACT: {
            if (!(dt > 0.0f) || !std::isfinite(dt)) return fail(h, SD_ERR_INVALID_ARG, "dt must be positive");
            sd::DemParams p = h->P;
            p.dt = dt;
            SD_CUDA(h, sd::dem_contact_integrate_async(p, h->B, (h->cfg.flags & SD_FLAG_RECORD) != 0, h->stream));
            return SD_OK;
        }
        case SD_STAGE_SORT: SD_CUDA(h, sd::dem_sort_async(h->B, h->stream)); return SD_OK;
        case SD_STAGE_REORDER: SD_CUDA(h, sd::dem_reorder_async(h->B, h->stream)); return SD_OK;
        default: return fail(h, SD_ERR_INVALID_ARG, "unknown stage");
    }
}

sd_status sd_engine_get_bodies(sd_engine* h, int32_t field, void* host_dst, size_t bytes) {
    if (!h || !host_dst) return fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (!h->prepared) return fail(h, SD_ERR_STATE, "call sd_engine_prepare first");
    if (h->hull_mode()) return hull_get_bodies(h, field, host_dst, bytes);
    const size_t nb = h->B.nb;
    const float4* src = nullptr;
    size_t per = 16;
    switch (field) {
        case SD_BODY_POSITION: src = h->B.bpos; break;
        case SD_BODY_VELOCITY: src = h->B.bvel; break;
        case SD_BODY_QUATERNION: src = h->B.bquat; break;
        case SD_BODY_OMEGA: src = h->B.bomg; break;
        case SD_BODY_ANGMOM: src = h->B.bang; break;
        case SD_BODY_INV_INERTIA: src = h->B.binv; per = 48; break;
        default: return fail(h, SD_ERR_INVALID_ARG, "unknown body field");
    }
    if (bytes != nb * per) return fail(h, SD_ERR_INVALID_ARG, "bytes must be n_bodies * " + std::to_string(per));
    if (nb == 0) return SD_OK;
    SD_CUDA(h, cudaSetDevice(h->device));
    SD_CUDA(h, cudaMemcpyAsync(host_dst, src, bytes, cudaMemcpyDeviceToHost, h->stream));
    SD_CUDA(h, cudaStreamSynchronize(h->stream));
    if (field == SD_BODY_VELOCITY || field == SD_BODY_OMEGA || field == SD_BODY_ANGMOM) {
        float4* o = static_cast<float4*>(host_dst);
        for (size_t i = 0; i < nb; ++i) o[i].w = 0.0f;
    }
    return SD_OK;
}

sd_status sd_engine_device_ptr(sd_engine* h, int32_t field, void** out) {
    if (!h || !out) return fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (!h->prepared) return fail(h, SD_ERR_STATE, "call sd_engine_prepare first");
    if (h->hull_mode()) return fail(h, SD_ERR_UNSUPPORTED, "not available for convex-hull scenes (use sd_engine_get_bodies)");
    if (field == SD_FIELD_IDS) {
        // ids live in the w lane of the omega array
        *out = reinterpret_cast<char*>(h->B.omg) + 12;
        return SD_OK;
    }
    const float4* p = field_ptr(h, field);
    if (!p) return fail(h, SD_ERR_INVALID_ARG, "field not available");
    *out = const_cast<float4*>(p);
    return SD_OK;
}

sd_status sd_engine_stream(sd_engine* h, void** out) {
    if (!h || !out) return fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (!h->prepared) return fail(h, SD_ERR_STATE, "call sd_engine_prepare first");
    *out = h->stream;
    return SD_OK;
}

sd_status sd_engine_get_pairs(sd_engine* h, uint64_t* dst, uint64_t cap, uint64_t* n) {
    if (!h || !n) return fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (!h->prepared) return fail(h, SD_ERR_STATE, "call sd_engine_prepare first");
    if (h->hull_mode()) return fail(h, SD_ERR_UNSUPPORTED, "not available for convex-hull scenes (use sd_engine_get_bodies)");
    SD_CUDA(h, cudaSetDevice(h->device));
    sd_status s = resort_if_needed(h);
    if (s) return s;
    SD_CUDA(h, sd::dem_pairs_async(h->P, h->B, h->stream));
    unsigned long long total = 0;
    SD_CUDA(h, cudaMemcpyAsync(&total, h->B.npairs, 8, cudaMemcpyDeviceToHost, h->stream));
    SD_CUDA(h, cudaStreamSynchronize(h->stream));
    *n = total;
    if (total > h->B.pair_cap) {
        uint32_t zero = 0;
        SD_CUDA(h, cudaMemcpy(h->B.dev_status, &zero, 4, cudaMemcpyHostToDevice));
        return fail(h, SD_ERR_CAPACITY, "engine pair_capacity too small for " + std::to_string(total) + " pairs");
    }
    if (total > cap) return fail(h, SD_ERR_CAPACITY, "dst too small for " + std::to_string(total) + " pairs");
    if (total) {
        if (!dst) return fail(h, SD_ERR_INVALID_ARG, "dst NULL");
        SD_CUDA(h, cudaMemcpy(dst, h->B.pairs, total * 8, cudaMemcpyDeviceToHost));
        std::sort(dst, dst + total);
    }
    return SD_OK;
}

sd_status sd_engine_params(sd_engine* h, sd_params* out) {
    if (!h || !out) return fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    // a prepared engine reports the parameters its buffers were sized for
    // (a later "z_div" knob change applies to engines prepared after it)
    if (!h->prepared) {
        sd_status s = derive_params(h);
        if (s) return s;
    }
    static_assert(sizeof(sd_params) == sizeof(sd::DemParams), "sd_params mirrors DemParams");
    std::memcpy(out, &h->P, sizeof(sd_params));
    out->dt = h->graph_valid ? h->graph_dt : 0.0f;
    return SD_OK;
}

sd_status sd_engine_stats(sd_engine* h, sd_stats* out) {
    if (!h || !out) return fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    std::memset(out, 0, sizeof(*out));
    out->n_spheres = h->prepared ? h->B.n : h->h_pos.size();
    out->n_bodies = h->hb_pos.size();
    out->steps = h->steps;
    if (h->hull_mode()) return hull_stats(h, out);
    if (!h->prepared) return SD_OK;
    SD_CUDA(h, cudaSetDevice(h->device));
    sd_status s = resort_if_needed(h);
    if (s) return s;
    SD_CUDA(h, sd::dem_energy_async(h->B, h->d_energy, h->stream));
    double e[4];
    SD_CUDA(h, cudaMemcpyAsync(e, h->d_energy, sizeof e, cudaMemcpyDeviceToHost, h->stream));
    // contacts of the current state (count of overlapping pairs)
    SD_CUDA(h, sd::dem_pairs_async(h->P, h->B, h->stream));
    unsigned long long np = 0;
    SD_CUDA(h, cudaMemcpyAsync(&np, h->B.npairs, 8, cudaMemcpyDeviceToHost, h->stream));
    uint32_t moved = 0, vl[4] = {0u, 0u, 0u, 0u};
    if (h->graph_valid && h->B.rs_max && h->B.n)
        SD_CUDA(h, cudaMemcpyAsync(&moved, h->B.rs_scratch + 1, 4, cudaMemcpyDeviceToHost, h->stream));
    if (h->B.vl_flags) SD_CUDA(h, cudaMemcpyAsync(vl, h->B.vl_flags, sizeof vl, cudaMemcpyDeviceToHost, h->stream));
    SD_CUDA(h, cudaStreamSynchronize(h->stream));
    out->moved_keys = h->steps ? moved : 0;
    out->list_builds = vl[2];
    out->listed_steps = vl[3];
    out->step_kernels = h->graph_valid ? h->graph_kernels : 0;
    // bodies: the kernel above counted free spheres only
    const size_t nb = h->B.nb;
    if (nb) {
        std::vector<float4> bp(nb), bv(nb), bw(nb), bl(nb);
        SD_CUDA(h, cudaMemcpy(bp.data(), h->B.bpos, 16 * nb, cudaMemcpyDeviceToHost));
        SD_CUDA(h, cudaMemcpy(bv.data(), h->B.bvel, 16 * nb, cudaMemcpyDeviceToHost));
        SD_CUDA(h, cudaMemcpy(bw.data(), h->B.bomg, 16 * nb, cudaMemcpyDeviceToHost));
        SD_CUDA(h, cudaMemcpy(bl.data(), h->B.bang, 16 * nb, cudaMemcpyDeviceToHost));
        for (size_t b = 0; b < nb; ++b) {
            const double m = bp[b].w;
            e[0] += 0.5 * m * ((double)bv[b].x * bv[b].x + (double)bv[b].y * bv[b].y + (double)bv[b].z * bv[b].z) +
                    0.5 * ((double)bw[b].x * bl[b].x + (double)bw[b].y * bl[b].y + (double)bw[b].z * bl[b].z);
            e[1] += m * bv[b].x;
            e[2] += m * bv[b].y;
            e[3] += m * bv[b].z;
        }
    }
    out->kinetic_energy = e[0];
    out->momentum[0] = e[1];
    out->momentum[1] = e[2];
    out->momentum[2] = e[3];
    out->contacts = np;
    out->n_cells = h->B.ncells;
    out->n_bodies = nb;
    uint32_t bits = 0;
    if ((s = read_device_errors(h, &bits))) return s;
    // a pair overflow from this stats pass is not an error of the run
    if (np > h->B.pair_cap) {
        bits &= ~sd::kErrPairOverflow;
        uint32_t clear = bits;
        SD_CUDA(h, cudaMemcpy(h->B.dev_status, &clear, 4, cudaMemcpyHostToDevice));
    }
    out->device_errors = bits;
    return SD_OK;
}

static const char kCkptMagic[8] = {'S', 'D', 'G', 'B', 'C', 'K', 'P', '1'};

sd_status sd_engine_save_checkpoint(sd_engine* h, const char* path) {
    if (!h || !path) return fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (h->scenes.size() > 1) return fail(h, SD_ERR_UNSUPPORTED, "checkpoints of a batch of scenes are not supported");
    if (!h->mesh.tri.empty()) return fail(h, SD_ERR_UNSUPPORTED, "checkpoints of a scene with a mesh are not supported");
    if (!h->prepared) return fail(h, SD_ERR_STATE, "call sd_engine_prepare first");
    if (h->hull_mode()) return fail(h, SD_ERR_UNSUPPORTED, "not available for convex-hull scenes (use sd_engine_get_bodies)");
    SD_CUDA(h, cudaSetDevice(h->device));
    sd_status s = resort_if_needed(h);
    if (s) return s;
    uint32_t n = h->B.n;
    std::vector<float4> buf(3 * (size_t)n);
    if (n) {
        SD_CUDA(h, cudaMemcpyAsync(buf.data(), h->B.pos, 16 * (size_t)n, cudaMemcpyDeviceToHost, h->stream));
        SD_CUDA(h, cudaMemcpyAsync(buf.data() + n, h->B.vel, 16 * (size_t)n, cudaMemcpyDeviceToHost, h->stream));
        SD_CUDA(h, cudaMemcpyAsync(buf.data() + 2 * (size_t)n, h->B.omg, 16 * (size_t)n, cudaMemcpyDeviceToHost, h->stream));
    }
    // rigid bodies: the moving state from the device, the constant tables
    // (inverse inertia, sphere ranges, body of each sphere, offsets) from the host
    const uint32_t nb = h->B.nb;
    std::vector<float4> bstate(5 * (size_t)nb);
    float4* const bsrc[5] = {h->B.bpos, h->B.bvel, h->B.bquat, h->B.bomg, h->B.bang};
    for (int k = 0; k < 5 && nb; ++k)
        SD_CUDA(h, cudaMemcpyAsync(bstate.data() + k * (size_t)nb, bsrc[k], 16 * (size_t)nb, cudaMemcpyDeviceToHost,
                                   h->stream));
    SD_CUDA(h, cudaStreamSynchronize(h->stream));
    std::ofstream f(path, std::ios::binary);
    if (!f) return fail(h, SD_ERR_IO, std::string("cannot write ") + path);
    uint32_t ver = 3;  // 3: DemParams carries cell_z and z_div
    f.write(kCkptMagic, 8);
    f.write(reinterpret_cast<const char*>(&ver), 4);
    f.write(reinterpret_cast<const char*>(&n), 4);
    f.write(reinterpret_cast<const char*>(&h->steps), 8);
    f.write(reinterpret_cast<const char*>(&h->cfg), sizeof(sd_config));
    f.write(reinterpret_cast<const char*>(&h->P), sizeof(sd::DemParams));
    f.write(reinterpret_cast<const char*>(buf.data()), (std::streamsize)(buf.size() * sizeof(float4)));
    f.write(reinterpret_cast<const char*>(&nb), 4);
    if (nb) {
        f.write(reinterpret_cast<const char*>(bstate.data()), (std::streamsize)(bstate.size() * sizeof(float4)));
        f.write(reinterpret_cast<const char*>(h->hb_inv.data()), (std::streamsize)(h->hb_inv.size() * sizeof(float4)));
        f.write(reinterpret_cast<const char*>(h->hb_first.data()), 4 * (std::streamsize)nb);
        f.write(reinterpret_cast<const char*>(h->hb_count.data()), 4 * (std::streamsize)nb);
        f.write(reinterpret_cast<const char*>(h->h_body_of.data()), 4 * (std::streamsize)n);
        f.write(reinterpret_cast<const char*>(h->h_r0.data()), 16 * (std::streamsize)n);
    }
    if (!f) return fail(h, SD_ERR_IO, "write failed");
    return SD_OK;
}

sd_status sd_engine_load_checkpoint(sd_engine* h, const char* path) {
    if (!h || !path) return fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (h->scenes.size() > 1) return fail(h, SD_ERR_UNSUPPORTED, "checkpoints of a batch of scenes are not supported");
    if (h->hull_mode()) return fail(h, SD_ERR_UNSUPPORTED, "not available for convex-hull scenes");
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(h, SD_ERR_IO, std::string("cannot open ") + path);
    char magic[8];
    uint32_t ver = 0, n = 0;
    uint64_t steps = 0;
    sd_config cfg;
    sd::DemParams P;
    f.read(magic, 8);
    f.read(reinterpret_cast<char*>(&ver), 4);
    f.read(reinterpret_cast<char*>(&n), 4);
    f.read(reinterpret_cast<char*>(&steps), 8);
    f.read(reinterpret_cast<char*>(&cfg), sizeof cfg);
    if (!f || std::memcmp(magic, kCkptMagic, 8) != 0 || ver < 1 || ver > 3)
        return fail(h, SD_ERR_IO, "not a stardust-gb300 checkpoint");
    // versions 1 and 2 end the parameters at rmax and were written with z_div 1
    f.read(reinterpret_cast<char*>(&P), ver >= 3 ? sizeof P : offsetof(sd::DemParams, cell_z));
    if (ver < 3) {
        P.cell_z = P.cell;
        P.z_div = 1;
    }
    if (!f || P.z_div < 1 || P.z_div > 8) return fail(h, SD_ERR_IO, "truncated or corrupt checkpoint (grid)");
    std::vector<float4> buf(3 * (size_t)n);
    f.read(reinterpret_cast<char*>(buf.data()), (std::streamsize)(buf.size() * sizeof(float4)));
    if (!f) return fail(h, SD_ERR_IO, "truncated checkpoint");
    uint32_t nb = 0;
    if (ver >= 2) f.read(reinterpret_cast<char*>(&nb), 4);
    if (!f || nb > n) return fail(h, SD_ERR_IO, "truncated or corrupt checkpoint (bodies)");
    std::vector<float4> bstate(5 * (size_t)nb), binv(3 * (size_t)nb), r0(nb ? n : 0);
    std::vector<uint32_t> bfirst(nb), bcount(nb);
    std::vector<int32_t> body_of(nb ? n : 0);
    if (nb) {
        f.read(reinterpret_cast<char*>(bstate.data()), (std::streamsize)(bstate.size() * sizeof(float4)));
        f.read(reinterpret_cast<char*>(binv.data()), (std::streamsize)(binv.size() * sizeof(float4)));
        f.read(reinterpret_cast<char*>(bfirst.data()), 4 * (std::streamsize)nb);
        f.read(reinterpret_cast<char*>(bcount.data()), 4 * (std::streamsize)nb);
        f.read(reinterpret_cast<char*>(body_of.data()), 4 * (std::streamsize)n);
        f.read(reinterpret_cast<char*>(r0.data()), 16 * (std::streamsize)n);
        if (!f) return fail(h, SD_ERR_IO, "truncated checkpoint (bodies)");
        for (uint32_t b = 0; b < nb; ++b)
            if ((uint64_t)bfirst[b] + bcount[b] > n || bcount[b] == 0) return fail(h, SD_ERR_IO, "corrupt body table");
        for (uint32_t i = 0; i < n; ++i)
            if (body_of[i] < -1 || body_of[i] >= (int32_t)nb) return fail(h, SD_ERR_IO, "corrupt body table");
    }
    if (std::memcmp(&cfg, &h->cfg, sizeof cfg) != 0)
        return fail(h, SD_ERR_STATE, "checkpoint was written by an engine with a different config");
    release_device(h);
    const size_t nbz = nb;
    h->hb_pos.assign(bstate.begin(), bstate.begin() + nbz);
    h->hb_vel.assign(bstate.begin() + nbz, bstate.begin() + 2 * nbz);
    h->hb_quat.assign(bstate.begin() + 2 * nbz, bstate.begin() + 3 * nbz);
    h->hb_omg.assign(bstate.begin() + 3 * nbz, bstate.begin() + 4 * nbz);
    h->hb_ang.assign(bstate.begin() + 4 * nbz, bstate.begin() + 5 * nbz);
    h->hb_inv = std::move(binv);
    h->hb_first = std::move(bfirst);
    h->hb_count = std::move(bcount);
    if (nb) {
        h->h_body_of = std::move(body_of);
        h->h_r0 = std::move(r0);
    } else {
        h->h_body_of.assign(n, -1);
        h->h_r0.assign(n, make_float4(0.f, 0.f, 0.f, 0.f));
    }
    // host copy in original id order
    h->h_pos.assign(n, float4{});
    h->h_vel.assign(n, float4{});
    h->h_omg.assign(n, float4{});
    for (uint32_t s = 0; s < n; ++s) {
        uint32_t id;
        std::memcpy(&id, &buf[2 * (size_t)n + s].w, 4);
        id &= 0x7fffffffu;
        if (id >= n) return fail(h, SD_ERR_IO, "corrupt checkpoint ids");
        h->h_pos[id] = buf[s];
        h->h_vel[id] = buf[n + s];
        h->h_omg[id] = buf[2 * (size_t)n + s];
    }
    // upload in the saved (sorted) slot order, on the saved grid: a stable
    // re-sort of a sorted state is the identity, so slot order -- and with
    // it every summation order -- is exactly that of the run that wrote the
    // checkpoint
    h->z_div_fixed = P.z_div;
    sd_status s = prepare_with(h, buf.data(), buf.data() + n, buf.data() + 2 * (size_t)n, n);
    if (s) return s;
    if (std::memcmp(&P.cell, &h->P.cell, sizeof(float)) != 0 || P.nz != h->P.nz)
        return fail(h, SD_ERR_STATE, "checkpoint grid differs from the derived grid");
    h->steps = steps;
    return SD_OK;
}

// ------------------------------------------------------------- raw operators
sd_status sd_hash_construct_collision_list(uint32_t n, float cell_dim, uint32_t* d_cells, uint32_t* d_spheres,
                                           const float* d_sizes, const float* d_pos4, uint32_t* d_count,
                                           void* stream) {
    if (n && (!d_cells || !d_spheres || !d_sizes || !d_pos4)) return fail(nullptr, SD_ERR_INVALID_ARG, "NULL pointer");
    if (!d_count) return fail(nullptr, SD_ERR_INVALID_ARG, "d_count NULL");
    if (n > 0x7fffffffu / 9) return fail(nullptr, SD_ERR_CAPACITY, "n too large for 9n entries");
    if (!(cell_dim > 0.0f)) return fail(nullptr, SD_ERR_INVALID_ARG, "cell_dim must be > 0");
    if (reinterpret_cast<uintptr_t>(d_pos4) & 15u) return fail(nullptr, SD_ERR_INVALID_ARG, "d_pos4 must be 16-byte aligned");
    cudaError_t e = sd::ref_hash_build_async(n, cell_dim, d_cells, d_spheres, d_sizes,
                                             reinterpret_cast<const float4*>(d_pos4), d_count,
                                             static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "ref_hash_build");
    return SD_OK;
}

sd_status sd_sort_scratch_bytes(uint64_t n, int32_t key_bits, uint64_t* bytes) {
    if (!bytes) return fail(nullptr, SD_ERR_INVALID_ARG, "bytes NULL");
    if (key_bits < 1 || key_bits > 32) return fail(nullptr, SD_ERR_INVALID_ARG, "key_bits must be 1..32");
    if (n >= (1ull << 30)) return fail(nullptr, SD_ERR_CAPACITY, "n must be < 2^30");
    *bytes = sd::sort_scratch_words(n, key_bits) * sizeof(uint32_t);
    return SD_OK;
}

sd_status sd_sort_pairs(uint32_t* d_keys, uint32_t* d_vals, uint32_t* d_keys_tmp, uint32_t* d_vals_tmp, uint64_t n,
                        int32_t key_bits, void* d_scratch, uint64_t scratch_bytes, void* stream) {
    if (key_bits < 1 || key_bits > 32) return fail(nullptr, SD_ERR_INVALID_ARG, "key_bits must be 1..32");
    if (n >= (1ull << 30)) return fail(nullptr, SD_ERR_CAPACITY, "n must be < 2^30");
    if (n == 0) return SD_OK;
    if (!d_keys || !d_vals || !d_keys_tmp || !d_vals_tmp || !d_scratch)
        return fail(nullptr, SD_ERR_INVALID_ARG, "NULL pointer");
    if (scratch_bytes < sd::sort_scratch_words(n, key_bits) * sizeof(uint32_t))
        return fail(nullptr, SD_ERR_CAPACITY, "scratch smaller than sd_sort_scratch_bytes");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    bool in_tmp = false;
    cudaError_t e = sd::sort_pairs_async(d_keys, d_vals, d_keys_tmp, d_vals_tmp, (uint32_t)n, key_bits,
                                         static_cast<uint32_t*>(d_scratch), st, &in_tmp);
    if (e == cudaSuccess && in_tmp) {
        e = cudaMemcpyAsync(d_keys, d_keys_tmp, 4 * n, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_vals, d_vals_tmp, 4 * n, cudaMemcpyDeviceToDevice, st);
    }
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "sort_pairs");
    return SD_OK;
}

sd_status sd_hash_sort_collision_list(uint32_t* d_cells, uint32_t* d_spheres, uint32_t* d_cells_tmp,
                                      uint32_t* d_spheres_tmp, uint64_t n, void* d_scratch, uint64_t scratch_bytes,
                                      void* stream) {
    return sd_sort_pairs(d_cells, d_spheres, d_cells_tmp, d_spheres_tmp, n, 32, d_scratch, scratch_bytes, stream);
}

sd_status sd_sort_status(const void* d_scratch, void* stream, uint32_t* errors) {
    if (!d_scratch || !errors) return fail(nullptr, SD_ERR_INVALID_ARG, "NULL argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(errors, d_scratch, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "sort_status");
    return SD_OK;
}

sd_status sd_hash_pairs_scratch_bytes(uint64_t n_entries, uint64_t* bytes) {
    if (!bytes) return fail(nullptr, SD_ERR_INVALID_ARG, "bytes NULL");
    *bytes = sd::ref_pairs_scratch_words(n_entries) * sizeof(uint32_t);
    return SD_OK;
}

sd_status sd_hash_candidate_pairs(const uint32_t* d_cells, const uint32_t* d_spheres, const uint32_t* d_count,
                                  uint32_t n_entries, const int32_t* d_body_of, uint32_t* d_pair_a,
                                  uint32_t* d_pair_b, uint64_t cap, uint64_t* d_npairs, void* d_scratch,
                                  uint64_t scratch_bytes, void* stream) {
    if (!d_count || !d_npairs || !d_scratch) return fail(nullptr, SD_ERR_INVALID_ARG, "NULL pointer");
    if (n_entries && (!d_cells || !d_spheres)) return fail(nullptr, SD_ERR_INVALID_ARG, "NULL pointer");
    if (cap && (!d_pair_a || !d_pair_b)) return fail(nullptr, SD_ERR_INVALID_ARG, "pair buffers NULL");
    if (reinterpret_cast<uintptr_t>(d_npairs) & 7u) return fail(nullptr, SD_ERR_INVALID_ARG, "d_npairs must be 8-byte aligned");
    if (scratch_bytes < sd::ref_pairs_scratch_words(n_entries) * sizeof(uint32_t))
        return fail(nullptr, SD_ERR_CAPACITY, "scratch smaller than sd_hash_pairs_scratch_bytes");
    cudaError_t e = sd::ref_candidate_pairs_async(d_cells, d_spheres, d_count, n_entries, d_body_of, d_pair_a,
                                                  d_pair_b, cap, reinterpret_cast<unsigned long long*>(d_npairs),
                                                  static_cast<uint32_t*>(d_scratch), static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "candidate_pairs");
    return SD_OK;
}

}  // extern "C"
