// sd_internal.h -- declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace sd {

void set_last_error(const std::string& msg);  // message for sd_last_error(NULL, ...)

// Device-side error word bits (read back by the host through sd_engine_stats
// or the raw API's status word); equal to the public SD_DEVERR_* values.
enum : uint32_t {
    kErrLookbackTimeout = 1u << 0,  // a decoupled look-back spin hit its limit
    kErrPairOverflow = 1u << 1,     // a pair buffer was too small
    kErrBadInput = 1u << 2,         // non-finite or out-of-range input seen
    kErrWaitTimeout = 1u << 3,      // a bounded wait on a TMA copy gave up
};

// ---- radix sort (sd_sort.cu)
// Digit plan of an LSD sort over key bits [0, key_bits): up to 4 passes of
// at most 9 bits, as even as possible.
struct SortPlan {
    int passes;
    int shift[4];
    int bits[4];
};
SortPlan sort_plan(int key_bits);
uint64_t sort_scratch_words(uint64_t n, int key_bits);
int sort_num_passes(int key_bits);
void sort_set_items(int items);
int sort_items();
uint32_t* sort_hist_ptr(uint32_t* scratch);  // [4][512] global digit histograms
cudaError_t sort_clear_async(uint32_t n, const SortPlan& plan, uint32_t* scratch, cudaStream_t st);
cudaError_t sort_histogram_async(const uint32_t* keys, uint32_t n, const SortPlan& plan, uint32_t* scratch,
                                 cudaStream_t st);
cudaError_t sort_passes_async(uint32_t* keys, uint32_t* vals, uint32_t* keys_tmp, uint32_t* vals_tmp,
                              uint32_t n, const SortPlan& plan, uint32_t* scratch, cudaStream_t st,
                              bool* in_tmp);
cudaError_t sort_pairs_async(uint32_t* keys, uint32_t* vals, uint32_t* keys_tmp, uint32_t* vals_tmp,
                             uint32_t n, int key_bits, uint32_t* scratch, cudaStream_t st,
                             bool* in_tmp);

// ---- reference-compatible spatial hash (sd_hash_ref.cu)
cudaError_t ref_hash_build_async(uint32_t n, float cell_dim, uint32_t* cells, uint32_t* spheres,
                                 const float* sizes, const float4* pos, uint32_t* d_count,
                                 cudaStream_t st);
uint64_t ref_pairs_scratch_words(uint64_t n_entries);
cudaError_t ref_candidate_pairs_async(const uint32_t* cells, const uint32_t* spheres,
                                      const uint32_t* d_count, uint32_t n_entries,
                                      const int32_t* body_of, uint32_t* pair_a, uint32_t* pair_b,
                                      uint64_t cap, unsigned long long* d_npairs, uint32_t* scratch,
                                      cudaStream_t st);

// ---- physics pipeline (sd_dem.cu)
struct DemParams {
    float lo[3], hi[3];
    float cell;
    int32_t nx, ny, nz;
    float kn, damp, mu;
    float g[3];
    float dt;
    int32_t walls;
    float rmax;  // largest sphere radius: bounds every contact partner's reach
};

struct DemBuffers {
    uint32_t n;
    uint32_t ncells;
    float4 *pos, *vel, *omg;        // current state, cell-sorted
    float4 *pos_n, *vel_n, *omg_n;  // next state, slot order of the current
    uint32_t *keys, *vals;          // sort keys / slot indices
    uint32_t *keys_tmp, *vals_tmp;  // sort ping-pong
    uint32_t* cell_start;           // ncells + 1
    uint32_t* sort_scratch;
    uint32_t* dev_status;           // [0] error bits, [1] contacts lo, [2] contacts hi
    float4 *force, *torque;         // optional per-slot outputs (may be null)
    unsigned long long* pairs;      // optional contact pairs (may be null)
    unsigned long long* npairs;
    uint64_t pair_cap;
    bool sorted_in_tmp;             // set by dem_sort_async: result in the *_tmp buffers
    // rigid clumps (all null / 0 when the scene has none).  A clump sphere's
    // id (omg.w bits) has bit 31 set.
    uint32_t nb;                    // bodies
    int32_t* body_of;               // per sphere id: its body, -1 for free spheres
    float4* r0;                     // per sphere id: body-frame offset from the body's centre
    uint32_t* slot_of;              // per sphere id: current slot (kept by the reorder)
    float4 *sf, *st;                // per slot: contact force / torque of clump spheres
    float4 *bpos, *bvel, *bquat, *bomg, *bang;  // per body: (x,y,z,m), v, q=(s,x,y,z), w, L
    float4* binv;                   // per body: 3 rows of the body-frame inverse inertia
    uint32_t *bfirst, *bcount;      // per body: first sphere id, number of spheres
};

constexpr uint32_t kClumpFlag = 0x80000000u;

int dem_key_bits(uint32_t ncells);
cudaError_t dem_init_kernels();  // once per device, outside stream capture
cudaError_t dem_keys_from_state_async(const DemParams& p, DemBuffers& b, cudaStream_t st);
cudaError_t dem_sort_async(DemBuffers& b, cudaStream_t st);
cudaError_t dem_reorder_async(DemBuffers& b, cudaStream_t st);
cudaError_t dem_sort_reorder_async(const DemParams& p, DemBuffers& b, cudaStream_t st);
cudaError_t dem_contact_integrate_async(const DemParams& p, DemBuffers& b, bool record,
                                        cudaStream_t st);
cudaError_t dem_step_async(const DemParams& p, DemBuffers& b, bool record, cudaStream_t st);
void dem_set_contact_mode(int mode);
int dem_contact_mode();
cudaError_t dem_pairs_async(const DemParams& p, DemBuffers& b, cudaStream_t st);
cudaError_t dem_unsort_async(const float4* src, const float4* omg, float4* dst, uint32_t n,
                             cudaStream_t st);
cudaError_t dem_scatter_in_async(const float4* src_by_id, const float4* omg, float4* dst, uint32_t n, bool keep_w,
                                 cudaStream_t st);
cudaError_t dem_energy_async(const DemBuffers& b, double* d_out, cudaStream_t st);

}  // namespace sd
