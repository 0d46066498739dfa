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
    int stride;  // words per pass of the digit histograms and per tile of the look-back status: 512, or 1024
                 // when a digit is 10 bits wide (19- and 20-bit keys, sorted in two passes)
};
SortPlan sort_plan(int key_bits);
uint64_t sort_scratch_words(uint64_t n, int key_bits);
int sort_num_passes(int key_bits);
void sort_set_items(int items);
int sort_items();
uint32_t* sort_hist_ptr(uint32_t* scratch);  // global digit histograms, pass q at q * plan.stride (2048 words)
cudaError_t sort_clear_async(uint32_t n, const SortPlan& plan, uint32_t* scratch, cudaStream_t st);
cudaError_t sort_histogram_async(const uint32_t* keys, uint32_t n, const SortPlan& plan, uint32_t* scratch,
                                 cudaStream_t st);
// skip (may be null): the passes return at once when skip[1] <= skip_max
// (the incremental re-sort has written the result)
// The radix fallback of the incremental re-sort: when skip[1] > skip_max,
// clears the tile status, sets vals[i] = i, builds the histograms (tile counters and
// histograms -- the first sort_fallback_clear_words() words after word 4 of
// the scratch -- must be zero) and runs the passes; otherwise its kernels
// return at once.
uint64_t sort_fallback_clear_words();
cudaError_t sort_fallback_async(uint32_t* keys, uint32_t* vals, uint32_t* keys_tmp, uint32_t* vals_tmp, uint32_t n,
                                const SortPlan& plan, uint32_t* scratch, cudaStream_t st, bool* in_tmp,
                                const uint32_t* skip, uint32_t skip_max);
cudaError_t sort_passes_async(uint32_t* keys, uint32_t* vals, uint32_t* keys_tmp, uint32_t* vals_tmp,
                              uint32_t n, const SortPlan& plan, uint32_t* scratch, cudaStream_t st,
                              bool* in_tmp, const uint32_t* skip = nullptr, uint32_t skip_max = 0);
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

// ---- scans and the LBVH broad phase (sd_lbvh.cu)
uint64_t scan_scratch_words(uint32_t n);
// out[0..n) = exclusive prefix sums of in, out[n] = total
cudaError_t scan_exclusive_async(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* scratch, cudaStream_t st);

struct Lbvh {
    uint32_t n;                          // leaves (boxes)
    uint32_t *keys, *vals, *keys_tmp, *vals_tmp;
    const uint32_t *skeys, *svals;       // sorted Morton codes / box ids (after the build)
    uint32_t* sort_scratch;
    float *bounds, *bound_part;          // global box (lo xyz, hi xyz) and per-block partials
    int2* children;                      // n-1 internal nodes; bit 31 marks a leaf child
    int32_t* parent;                     // internal nodes [0, n-1), leaves [n-1, 2n-1); root -1
    uint32_t* visit;                     // refit arrival counters
    float4 *node_lo, *node_hi, *leaf_lo, *leaf_hi;
    uint32_t* counts;                    // per box id
    uint32_t* first;                     // per leaf: its first kLbvhFirst partners found (counting pass)
    float4* rec;                         // per internal node: both children's boxes (lo.w = child ref)
    uint32_t* scan_scratch;
    uint32_t* status;                    // device error bits
};
constexpr int kLbvhFirst = 16;
uint64_t lbvh_scratch_bytes(uint32_t n);
void lbvh_carve(void* scratch, uint32_t n, Lbvh* t);
cudaError_t lbvh_morton_async(Lbvh& t, const float4* lo, const float4* hi, cudaStream_t st);
cudaError_t lbvh_build_async(Lbvh& t, const float4* lo, const float4* hi, cudaStream_t st);
// new boxes in the tree the last build made (its leaf order and topology):
// bounds stay exact, so the pair sets do too; only the tree's quality ages
cudaError_t lbvh_refit_async(Lbvh& t, const float4* lo, const float4* hi, cudaStream_t st);
// steps between full LBVH builds of a moving scene (knob "lbvh_rebuild")
void lbvh_set_rebuild_every(int k);
int lbvh_rebuild_every();
// per box id: partners at [off[id], off[id+1]) ascending, self[] = id; off has n+1
cudaError_t lbvh_partners_async(Lbvh& t, uint32_t* off, uint32_t* partners, uint32_t* self, uint64_t cap,
                                cudaStream_t st);
// ascending unique pairs (i < j) of any per-box partner lists (CSR, partners
// ascending per box); counts n, pos n+1 (pos[n] = count), scan scratch
cudaError_t csr_unique_pairs_async(uint32_t n, const uint32_t* off, const uint32_t* partners, uint64_t partners_cap,
                                   uint32_t* counts, uint32_t* scan_scratch, uint32_t* pos, unsigned long long* out,
                                   uint64_t cap, cudaStream_t st);
// ascending unique pairs (i < j) from the partner lists; pos has n+1 (pos[n] = count)
cudaError_t lbvh_unique_pairs_async(Lbvh& t, const uint32_t* off, const uint32_t* partners, uint64_t partners_cap,
                                    uint32_t* pos, unsigned long long* out, uint64_t cap, cudaStream_t st);

// ---- sweep and prune (sd_sap.cu)
uint64_t sap_scratch_bytes(uint64_t n, uint64_t pair_cap);
cudaError_t sap_aabb_async(uint32_t n, const float4* pos, const float* radius, float4* lo, float4* hi,
                           cudaStream_t st);
cudaError_t sap_sort_lower_x_async(uint32_t n, const float4* lo, bool ordered, uint32_t* keys, uint32_t* vals,
                                   uint32_t* keys_tmp, uint32_t* vals_tmp, uint32_t* sort_scratch, bool* in_tmp,
                                   cudaStream_t st);
cudaError_t sap_sweep_ref_async(uint32_t n, const float* upperx, const float* lowerx_sorted, const float* uppery,
                                const float* lowery, const uint32_t* idx_sorted, int32_t* rows, cudaStream_t st);
// exact pair set; d_count2[0] = pairs, d_count2[1] = device error bits
cudaError_t sap_pairs_async(uint32_t n, const float4* lo, const float4* hi, void* scratch, uint64_t pair_cap,
                            unsigned long long* out, uint32_t* d_count2, cudaStream_t st);

// ---- convex hulls (sd_hull.cu)
struct HullParams {
    float lo[3], hi[3];
    float kn, damp, mu;
    float g[3];
    float dt;
    int32_t walls;
};

struct HullBuffers {
    uint32_t nb;
    float4 *pos, *vel, *quat, *omg, *ang;  // (x,y,z,m), v, q=(s,x,y,z), w, world L
    float4* iinv;                          // body-frame principal inverse inertia, w = bounding radius
    uint32_t *vstart, *vcount;
    float4* verts;                         // body-frame vertices
    float4 *lo, *hi;                       // world AABBs
    uint32_t* ext;                         // 2 per body: vertex index of min x|y<<8|z<<16, of max
    uint32_t *off, *partners, *self;       // candidate entries (CSR, off has nb+1)
    uint64_t cap;                          // entry capacity
    float4 *ef, *et;                       // per entry: force / torque on self
    uint32_t* info;                        // per entry: status | gjk iters << 8 | epa iters << 16
    float4* dir;                           // per entry: final search direction in A's frame, w = 1 if separated
    float4* seeds;                         // per entry: seed in A's frame, w = 1 to use (may be null)
    float* feat;                           // per entry: 16 MLP inputs (may be null)
    // training targets of the warm-start network (may be null): when
    // *teach_on, per unique entry the converged closest-point direction of
    // a separated pair in A's frame (w = 1), else w = 0
    float4* teach;
    const uint32_t* teach_on;
    // learned seeds: a pair whose seeded run certified separation keeps its
    // previous direction (inputs 8..10, the anchor) as the next step's, so
    // the network is never fed its own outputs
    bool keep_anchor;
    // the pairs GJK found intersecting, for the EPA kernel: count, and per
    // hit the unique-pair index and the GJK support evaluations spent, and
    // the support keys of the enclosing tetrahedron
    uint32_t* hit_count;
    uint2* hits;
    uint4* hit_keys;
    const uint32_t *prev_off, *prev_partners;  // the previous step's lists
    const float4* prev_dir;
    float4 *force, *torque;                // optional per body totals
    uint32_t *ucount, *upos, *ulist, *uscan;  // unique pairs: per body count, offsets (nb+1), entry list, scan scratch
};
cudaError_t hull_aabb_async(HullBuffers& H, cudaStream_t st);
cudaError_t hull_seed_async(HullBuffers& H, uint32_t mode, cudaStream_t st);
cudaError_t hull_narrow_async(const HullParams& p, HullBuffers& H, cudaStream_t st);
void hull_set_blocks(int b);
int hull_blocks();
// The training samples of a step (teach[e].w == 1 among the d_count[0]
// entries), gathered in entry order into feat_c (16 floats per row) and
// teach_c (cap / 2 + 1 rows each); *d_total = their number.  flags and pos
// hold cap words, scan the scan scratch of cap words.
cudaError_t hull_teach_compact_async(const HullBuffers& H, const uint32_t* d_count, float* feat_c, float4* teach_c,
                                     uint32_t* flags, uint32_t* pos, uint32_t* scan, uint32_t* d_total,
                                     cudaStream_t st);
cudaError_t hull_integrate_async(const HullParams& p, HullBuffers& H, cudaStream_t st);
cudaError_t hull_stats_async(HullBuffers& H, unsigned long long* out, cudaStream_t st);

// ---- GJK warm-start network (sd_mlp.cu)
struct MlpState {
    float *params, *m1, *m2, *grad;  // FP32 master parameters, Adam moments, last gradient
    uint8_t* img;                    // packed BF16 operand images
    float* part;                     // per-CTA gradient partials
    uint32_t* status;                // device error bits
};
uint64_t mlp_state_bytes();
uint32_t mlp_param_count();
MlpState mlp_carve(void* base);
cudaError_t mlp_init_kernels();
cudaError_t mlp_set_params_async(MlpState& s, const float* host_params, cudaStream_t st);
// seeds == true: out[e] = (y, 1) for rows with feat[7] == 1 (else 0), e < *d_count;
// seeds == false: out[e] = (y, 0), e < n
cudaError_t mlp_forward_async(const MlpState& s, const float* feat, float4* out, const uint32_t* d_count, uint64_t n,
                              bool seeds, cudaStream_t st);
// one full-batch gradient of the cosine loss (grad[] = its value) and, when
// update, an Adam step (adam_step counts from 1); d_count (may be null): a
// device word capping the rows below n
cudaError_t mlp_train_async(MlpState& s, const float* feat, const float4* tgt, uint32_t n, uint32_t n_valid, float lr,
                            uint32_t adam_step, bool update, cudaStream_t st, const uint32_t* d_count = nullptr);

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
    // z cells are `cell / z_div` high (nz counts them): a finer z split
    // shortens each neighbour column's candidate range without adding
    // columns; cell keys stay (ix*ny + iy)*nz + iz
    float cell_z;
    int32_t z_div;
};

// One scene of a batch: its box and grid, the first global cell key of its
// grid (scenes occupy consecutive key ranges) and its first sphere slot
// (scenes occupy consecutive slot ranges, in every step, because the sort
// keeps each scene's keys together and no sphere leaves its scene).
struct SceneGrid {
    float lo[3], hi[3];
    float cell;
    int32_t nx, ny, nz;
    uint32_t base;
};

// A rigid triangle mesh (walls of a rotating drum): triangles in the mesh's
// own frame, a static uniform grid over that frame listing, per cell, every
// triangle within the largest sphere radius (ascending triangle ids), and
// the pose.  state (device, 24 floats): R[9] (mesh to world), c[3] (centre
// of rotation), axis[3] (unit), omega, q[4] (s,x,y,z), dq[4] (the rotation of
// one step); mesh_advance_async applies q <- normalize(dq q), R <- R(q).
struct MeshView {
    uint32_t ntri;
    const float4* tri;        // 3 rows per triangle (x, y, z, 0), mesh frame
    const int32_t* patch;     // per triangle: the face it belongs to
    const uint32_t* cell_off; // ncells + 1
    const uint32_t* cell_tri;
    float lo[3];
    float h;
    int32_t nx, ny, nz;
    float* state;
    // sweep and prune of the triangles (collision engine SD_ENGINE_SAP): the
    // triangles' boxes (mesh frame) sorted by their lower bound along axis
    // sap_axis -- sap_box[2k] = (lo, lower bound), sap_box[2k+1] = (hi,
    // triangle id as float bits) -- and the largest box extent along it;
    // sap_n == 0: the static grid above gives the candidates
    uint32_t sap_n;
    const float4* sap_box;
    const float* sap_lo;      // sorted lower bounds (the binary search's array)
    int32_t sap_axis;
    float sap_len;
};
constexpr int kMeshPatches = 4;  // deepest contact kept per patch, up to this many patches per sphere
constexpr int kSapHits = 32;     // triangles in contact with one sphere the sweep can order (more: error bit)

struct DemBuffers {
    uint32_t n;
    uint32_t ncells;
    MeshView mesh;                  // mesh.ntri == 0: no mesh
    uint32_t nscenes;               // 0 or 1: one scene (DemParams' grid); > 1: a batch
    const SceneGrid* scenes;        // [nscenes]
    const uint32_t* scene_first;    // [nscenes + 1] first slot of each scene, then n
    float4 *pos, *vel, *omg;        // current state, cell-sorted
    float4 *pos_n, *vel_n, *omg_n;  // next state, slot order of the current
    uint32_t *keys, *vals;          // sort keys / slot indices
    uint32_t *keys_tmp, *vals_tmp;  // sort ping-pong
    uint32_t* cell_start;           // ncells + 1
    uint32_t* sort_scratch;
    uint32_t* dev_status;           // [0] error bits, [2..3] contact count (u64), [4] changed keys
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
    // incremental re-sort (sd_resort.cu): rs_max 0 = the step always radix-sorts
    uint32_t* keys_prev;            // per slot: the sorted key it sits under (written by the reorder)
    unsigned long long* rs_list;    // the moved entries, (key << 32 | slot), up to kResortMaxCap
    uint32_t* rs_pos;               // per moved entry (in (key, slot) order): its sorted position
    uint32_t* rs_q;                 // per moved slot (ascending): slot - rank
    uint32_t* rs_iv_lo;             // per moved entry: first position its move shifts
    uint32_t* rs_iv_pre;            // exclusive prefix sums of those intervals' lengths (M + 1 entries)
    uint32_t* rs_scratch;           // [0] moved count, [1] M of the step, [3] total interval length
    uint32_t rs_max;                // most moved entries re-sorted incrementally (power of two, or 0)
    // contact partner lists (scenes without clumps): per slot a count, zero
    // between steps, and kNbrCap partner slots; null when not allocated
    uint32_t *nbr_cnt, *nbr;
    // skin lists (single scenes of free spheres, vl_skin > 0): per sphere id
    // its neighbours within r_i + r_j + skin at the last build and the
    // position then; vl_flags[0] = build this step, [1] = build next step,
    // [2] = steps that built the lists, [3] = steps that used them
    uint32_t *vl_cnt, *vl_nbr, *vl_flags;
    float4* vl_ref;
    // the reorder's buffers for the list entries it moves (same sizes)
    uint32_t *vl_cnt_t, *vl_nbr_t;
    float4* vl_ref_t;
    float vl_skin;
};

constexpr uint32_t kClumpFlag = 0x80000000u;
constexpr uint32_t kNbrCap = 16;  // contact partners listed per sphere by the pair kernel
constexpr uint32_t kVlCap = 24;   // skin-list neighbours per sphere (more: the sphere scans)

int dem_key_bits(uint32_t ncells);
// incremental re-sort (sd_resort.cu): the step's key writers append the
// slots whose key changed to rs_list (count in rs_scratch[0]); when at most
// b.rs_max did (the count is published in rs_scratch[1]; b.cell_start must
// still be the previous sort's table), the plan kernel orders the moved
// entries by (key, slot) with their sorted positions and the intervals of
// positions they shift, which the reorder turns into the sorted order
// (ResortView); otherwise it clears the radix fallback's counters
constexpr uint32_t kResortMaxCap = 1024;  // largest rs_max (two sorted lists in 16 KB of shared memory)
uint64_t resort_scratch_words(uint32_t n);
// vl_flags (may be null): the skin lists' flags, [0] <- [1], [1] <- 0
cudaError_t resort_plan_async(const DemBuffers& b, cudaStream_t st, uint32_t* vl_flags = nullptr);
void dem_set_resort_max(uint32_t m);
uint32_t dem_resort_max();
void dem_set_pair_lists(int on);
void dem_set_listed_blocks(int b);
void dem_set_contact_block(int t);
int dem_contact_block();
void dem_set_fix_blocks(int b);
int dem_fix_blocks();
int dem_listed_blocks();
int dem_pair_lists();
cudaError_t dem_init_kernels();  // once per device, outside stream capture
// Counts, into *count (device), the slots whose key from the current position
// differs from the sorted key they sit under.
cudaError_t dem_keys_changed_async(const DemParams& p, const DemBuffers& b, uint32_t* count, cudaStream_t st);
cudaError_t dem_keys_from_state_async(const DemParams& p, DemBuffers& b, cudaStream_t st);
cudaError_t dem_sort_async(DemBuffers& b, cudaStream_t st);
cudaError_t dem_reorder_async(DemBuffers& b, cudaStream_t st);
// True when dem_step_async leaves the next state in the *_n buffers (sorted
// in place there): the caller then swaps pos/pos_n, vel/vel_n, omg/omg_n.
bool dem_step_swaps(const DemBuffers& b);
// True when the step uses the skin lists (single scene of free spheres, knob
// skin_um > 0, re-sort on).
bool dem_step_skin(const DemBuffers& b);
cudaError_t dem_sort_reorder_async(const DemParams& p, DemBuffers& b, cudaStream_t st);
cudaError_t dem_contact_integrate_async(const DemParams& p, DemBuffers& b, bool record,
                                        cudaStream_t st);
cudaError_t dem_step_async(const DemParams& p, DemBuffers& b, bool record, cudaStream_t st);
void dem_set_contact_mode(int mode);
int dem_contact_mode();
cudaError_t dem_pairs_async(const DemParams& p, DemBuffers& b, cudaStream_t st);
cudaError_t dem_unsort_async(const float4* src, const float4* omg, float4* dst, uint32_t n,
                             cudaStream_t st);
// State fields between a host buffer in sphere-id order that the device can
// address (mapped page-locked memory) and the slot-ordered device arrays;
// slot_of_id (n words) receives the id -> slot table.
// After the host wrote positions: sets the lists' build flag when a sphere
// left 0.45 skin of its position at the last build (no-op without lists).
cudaError_t dem_skin_check_async(const DemBuffers& b, cudaStream_t st);
// slot_of[id] = slot of every sphere of the current state (ids in omg.w).
cudaError_t dem_slot_of_all_async(const float4* omg, uint32_t* slot_of, uint32_t n, cudaStream_t st);
cudaError_t dem_host_in_async(const float4* host_src, const float4* omg, float4* dst, uint32_t* slot_of_id,
                              uint32_t n, bool keep_w, cudaStream_t st);
cudaError_t dem_host_out_async(const float4* src, const float4* omg, float4* host_dst, uint32_t* slot_of_id,
                               uint32_t n, cudaStream_t st);
cudaError_t dem_scatter_in_async(const float4* src_by_id, const float4* omg, float4* dst, uint32_t n, bool keep_w,
                                 cudaStream_t st);
cudaError_t dem_energy_async(const DemBuffers& b, double* d_out, cudaStream_t st);
// advance != 0: q <- normalize(dq q); then R <- R(q)
cudaError_t mesh_advance_async(const MeshView& m, int advance, cudaStream_t st);

}  // namespace sd
