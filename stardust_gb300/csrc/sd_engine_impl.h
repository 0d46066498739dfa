// sd_engine_impl.h -- the engine handle, shared by the translation units that
// implement the C ABI (sd_engine.cu: spheres and clumps; sd_hull_engine.cu:
// convex hulls).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/stardust.h"
#include "sd_internal.h"

// Host copy and device state of a convex-hull scene (sd_hull_engine.cu).
struct HullScene {
    // host, in insertion order
    std::vector<float4> pos, vel, quat, omg, ang, iinv, verts;
    std::vector<uint32_t> vstart, vcount;
    // device
    sd::HullParams P{};
    sd::HullBuffers H{};
    sd::Lbvh tree{};
    uint32_t* off[2] = {nullptr, nullptr};        // partner lists of even / odd steps
    uint32_t* partners[2] = {nullptr, nullptr};
    float4* dir[2] = {nullptr, nullptr};
    unsigned long long* stats = nullptr;          // 4 counters of the last step
    sd::MlpState mlp{};                           // warm-start network (device)
    uint32_t mlp_step = 0;                        // Adam steps taken
    // online training of the network (sd_engine_set_gjk_training): every
    // train_every steps the step logs max-margin targets, then train_iters
    // Adam steps of rate train_lr run on them
    int32_t train_every = 0, train_iters = 0;
    float train_lr = 0.0f;
    uint32_t* teach_flag = nullptr;               // [0] on (read by the step), [1] = 0, [2] = 1
    // a training step's samples gathered for the Adam iterations
    float* teach_feat = nullptr;
    float4* teach_tgt = nullptr;
    uint32_t *teach_flags = nullptr, *teach_pos = nullptr, *teach_scan = nullptr, *teach_total = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};        // full LBVH build
    cudaGraphExec_t graph_refit[2] = {nullptr, nullptr};  // refit of the last build's tree
    bool tree_built = false;                              // a full build ran since prepare
    int parity = 0;
    int seed_mode = 0;                            // SD_GJK_SEED_*
    float graph_dt = 0.0f;
    bool graph_valid = false;
    uint64_t graph_epoch = 0;
    uint32_t graph_kernels = 0;                   // kernel nodes of one step's graph
};

struct sd_engine {
    sd_config cfg{};
    std::string err;

    // host sphere set in insertion order; omega.w carries the id bits
    std::vector<float4> h_pos, h_vel, h_omg;
    // rigid clumps: per body (centre, mass), v, q, w, L, inverse inertia rows,
    // first sphere id and sphere count; per sphere id its body and offset
    std::vector<float4> hb_pos, hb_vel, hb_quat, hb_omg, hb_ang, hb_inv;
    std::vector<uint32_t> hb_first, hb_count;
    std::vector<int32_t> h_body_of;
    std::vector<float4> h_r0;
    // convex hulls (a scene holds spheres/clumps or hulls, not both)
    HullScene hull;
    // a batch of independent sphere scenes (sd_engine_add_scene): box, cell
    // (0: 2 x the scene's largest radius), first sphere id, sphere count
    struct SceneHost {
        float lo[3], hi[3], cell;
        uint32_t first, count;
    };
    std::vector<SceneHost> scenes;
    std::vector<sd::SceneGrid> scene_grids;  // derived at prepare
    std::vector<uint32_t> scene_first;
    bool adding_scene = false;
    // a rigid triangle mesh rotating about an axis (sd_engine_add_mesh)
    struct MeshHost {
        std::vector<float4> tri;       // 3 rows per triangle, mesh frame (world at t = 0 minus centre)
        std::vector<int32_t> patch;
        float centre[3] = {0, 0, 0}, axis[3] = {0, 0, 1}, omega = 0.0f;
        float state[24] = {0};
        float dt = 0.0f;               // dq of the graph's time step
    } mesh;

    bool prepared = false;
    int32_t z_div_fixed = 0;  // z cells per cell edge taken from a checkpoint (0: the "z_div" knob)
    int device = 0;
    cudaStream_t stream = nullptr;
    sd::DemParams P{};
    sd::DemBuffers B{};
    std::vector<void*> allocations;
    double* d_energy = nullptr;
    float4* d_tmp = nullptr;
    cudaGraphExec_t graph = nullptr;
    // when the step leaves the next state in the *_n buffers (graph_swaps),
    // a second graph captured on the swapped buffers alternates with the
    // first; graph_parity names the one whose input is the current state
    cudaGraphExec_t graph_alt = nullptr;
    bool graph_swaps = false;
    int graph_parity = 0;
    float graph_dt = 0.0f;
    bool graph_valid = false;
    uint32_t graph_kernels = 0;  // kernel nodes of the step graph
    uint64_t steps = 0;
    bool need_resort = false;
    // the sorted key arrays hold the cell key of every slot's sphere (true
    // after a full sort + reorder; a partial sd_engine_launch_stage clears it)
    bool keys_current = false;
    uint64_t graph_epoch = 0;

    bool hull_mode() const { return !hull.pos.empty(); }
};

// shared helpers (sd_engine.cu)
sd_status sd_fail(sd_engine* h, sd_status code, const std::string& msg);
sd_status sd_cuda_fail(sd_engine* h, cudaError_t e, const char* where);
// Kernel nodes in a captured graph (the kernels one launch of it runs).
uint32_t graph_kernel_nodes(cudaGraph_t g);
sd_status sd_alloc_bytes(sd_engine* h, void** p, size_t bytes);
float sd_damp_from(float kn, float e);
uint64_t sd_tune_epoch();

// hull mode (sd_hull_engine.cu)
sd_status hull_prepare(sd_engine* h);
sd_status hull_step(sd_engine* h, float dt, int32_t n_steps);
sd_status hull_launch_narrow(sd_engine* h);
sd_status hull_stats(sd_engine* h, sd_stats* out);
sd_status hull_get_bodies(sd_engine* h, int32_t field, void* host_dst, size_t bytes);
sd_status hull_get_state(sd_engine* h, int32_t field, void* host_dst, size_t bytes);
void hull_release(sd_engine* h);
