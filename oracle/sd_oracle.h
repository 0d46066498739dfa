/*
 * sd_oracle.h -- CPU oracle for the stardust-gb300 DEM step.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code.  Only tests/, __graft_entry__.smoke() and bench.py (its
 * cpu_baseline leg and its `--impl reference` arm) may use it, and only as
 * the checker or as the timed CPU restatement of the reference.
 *
 * Two families of functions live here:
 *
 *  1. ref_compat: a plain-C restatement of the reference's spatial-hash broad
 *     phase, bit-for-bit, including its quirks:
 *       - cell keys / phantom entries  : src/engine/cuda/sh_collision_detection.cu:27-127
 *       - LSD radix sort (stable, 8-bit digits; the intended semantics of
 *         sh_collision_detection.cu:129-360 with the chunk-offset defect at
 *         :241-242 corrected)
 *       - run traversal / candidate pairs: src/engine/cuda/collision_resolution.cu:30-199
 *       - the reference contact law, evaluated sequentially
 *         (collision_resolution.cu:30-98, cuda_helpers.cuh:43-63)
 *       - rigid-body update kernels
 *         (src/engine/cuda/physics_update.cu:26-310, cuda_helpers.cuh:65-171)
 *     These are pinned against the reference's own kernels: oracle/ref_build.py
 *     compiles the reference sources unchanged into sm_103a cubins,
 *     oracle/ref_harness.cpp runs them on a GPU, tests/golden/make_ref_golden.py
 *     stores their outputs in tests/golden/, and tests/test_oracle_ref.py
 *     checks this restatement against them (keys bit-exact; traversal forces
 *     and rigid-body kernels to 1e-6 relative).
 *
 *  2. physics: the per-step pipeline of the GPU engine (linear spring-dashpot
 *     with restitution damping, Coulomb friction, box walls, symplectic Euler)
 *     restated in FP32 with the same operation order as the CUDA kernels, and
 *     in FP64 for the error statement.  The reference has no correct contact
 *     law (collision_resolution.cu:90-95 multiplies by velocity signs and
 *     races), so this half is pinned only against its own FP64 twin and the
 *     physics tests (energy, momentum, restitution).
 *
 * All arithmetic is compiled with -ffp-contract=off so that every float
 * operation rounds exactly once, as the CUDA kernels do (-fmad=false plus the
 * explicit __fmaf_rn where the reference's compiled code fuses).
 */
#ifndef SD_ORACLE_H
#define SD_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- ref_compat */

/* constructCollisionListCUDA (sh_collision_detection.cu:27-127).
 * Writes 9 (cell, sphere) slots per sphere at [9i, 9i+9): the home entry,
 * then one phantom entry per valid neighbour offset in ascending offset order,
 * then padding (cell 0xffffffff, sphere i<<2).  Returns the number of
 * non-padding entries (the value the kernel accumulates into d_temp[0]). */
uint32_t sdo_ref_hash_build(uint32_t n, float cell_dim, const float* pos4,
                            const float* sizes, uint32_t* cells, uint32_t* spheres);

/* Stable LSD radix sort of (key, value) pairs over key bits [0, nbits),
 * 8 bits per pass, in place.  tmp_k/tmp_v are n-element scratch. */
void sdo_radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t n, int nbits,
                          uint32_t* tmp_k, uint32_t* tmp_v);

/* Run traversal of tranverseCollisionListCUDA (collision_resolution.cu:100-199)
 * over the first `count` sorted entries: for every maximal run of equal
 * cell (key >> 1), every home entry j pairs with every later entry k of the
 * run.  Pairs whose spheres share a rigid body (body_of, may be NULL) are
 * skipped, as collision_resolution.cu:69 does.  Writes (home, other) sphere
 * ids in traversal order; returns the number of pairs (may exceed cap, in
 * which case only cap are written). */
uint64_t sdo_ref_candidate_pairs(const uint32_t* cells, const uint32_t* spheres,
                                 uint32_t count, const int32_t* body_of,
                                 uint32_t* pair_a, uint32_t* pair_b, uint64_t cap);

/* The reference contact law applied sequentially over the candidate runs
 * (resolveCollisionsCUDA, collision_resolution.cu:30-98), forces accumulated
 * into force4 (which the caller zeroes), with the reference's hard-coded
 * stiffness 2e6, tangential 200, damping 200 and contact distance 0.2.
 * Used only to pin the traversal against the reference source run on the
 * host; it is NOT the engine's contact law. */
void sdo_ref_resolve_forces(const uint32_t* cells, const uint32_t* spheres,
                            uint32_t count, const int32_t* body_of,
                            const float* pos4, const float* vel4, float* force4);

/* Rigid-body kernels of physics_update.cu restated per body. */
void sdo_ref_update_spheres(int n_spheres, const float* init_rel4, const int32_t* body_of,
                            const float* body_pos4, const float* body_vel4,
                            const float* body_quat4, const float* body_omega4,
                            float* pos4, float* rel4, float* vel4);
void sdo_ref_body_forces(int n_bodies, const int32_t* start, const int32_t* length,
                         const float* body_mass, const float* rel4, const float* sphere_force4,
                         float* body_force4, float* body_torque4);
void sdo_ref_advect(int n_bodies, float dt, const float* body_mass, const float* inertia9,
                    const float* body_force4, const float* body_torque4,
                    float* body_pos4, float* body_vel4, float* body_omega4,
                    float* body_quat4, float* lin_mom4, float* ang_mom4);

/* ------------------------------------------------------------------ physics */

typedef struct sdo_params {
    float lo[3], hi[3];     /* box; walls on the six faces when walls != 0 */
    float cell;             /* grid cell edge */
    int32_t nx, ny, nz;     /* grid dims (nz counts z cells of cell_z); key = (ix*ny + iy)*nz + iz */
    float kn;               /* normal stiffness, N/m */
    float damp;             /* 2*beta*sqrt(kn); gamma_n = damp*sqrt(m_eff) */
    float mu;               /* Coulomb coefficient */
    float g[3];             /* gravity */
    float dt;
    int32_t walls;          /* bit a*2+s: wall on axis a, side s (0 low, 1 high) */
    float cell_z;           /* z cell edge (cell / z_div of the engine); 0 = cell.
                               iz = clamp(trunc((z - lo[2]) / cell_z), 0, nz-1) */
} sdo_params;

/* Cell key of a position (clamped into the grid). */
uint32_t sdo_cell_key(const sdo_params* p, float x, float y, float z);
/* Cell keys of n positions (pos4 rows). */
void sdo_cell_keys(const sdo_params* p, uint32_t n, const float* pos4, uint32_t* keys);

/* Sort a freshly integrated state into cell order:
 *   keys[i] = cell key of slot i of (pos_n, vel_n, omg_n)
 *   stable sort of (keys, slot) -> gather into (pos, vel, omg)
 *   cell_start[c] = first sorted slot with key >= c, c in [0, ncells]
 * keys_out (n) receives the sorted keys. */
void sdo_sort_reorder(const sdo_params* p, uint32_t n,
                      const float* pos_n, const float* vel_n, const float* omg_n,
                      const uint32_t* keys, uint32_t* keys_out,
                      float* pos, float* vel, float* omg, uint32_t* cell_start);

/* Contact gather + integration over a cell-sorted state (FP32).
 * Writes the next state into *_n and its cell keys into keys_n.
 * force4/torque4 (may be NULL) receive the total contact+wall force and
 * torque on each slot.  Returns the number of particle-particle contacts
 * seen (each pair counted from both sides). */
uint64_t sdo_contact_integrate(const sdo_params* p, uint32_t n,
                               const float* pos, const float* vel, const float* omg,
                               const uint32_t* cell_start,
                               float* pos_n, float* vel_n, float* omg_n, uint32_t* keys_n,
                               float* force4, float* torque4);

/* FP64 twin of sdo_contact_integrate (same algorithm, double arithmetic). */
uint64_t sdo_contact_integrate_f64(const sdo_params* p, uint32_t n,
                                   const double* pos, const double* vel, const double* omg,
                                   const uint32_t* cell_start,
                                   double* pos_n, double* vel_n, double* omg_n, uint32_t* keys_n,
                                   double* force4, double* torque4);

/* Contact pair set of a cell-sorted state: u64 (min_id << 32 | max_id) of
 * every overlapping particle pair, ids from omg.w.  Returns the count. */
uint64_t sdo_contact_pairs(const sdo_params* p, uint32_t n, const float* pos,
                           const float* omg, const uint32_t* cell_start,
                           uint64_t* out, uint64_t cap);

/* Full engine run: prepare (key + sort) then `steps` steps of
 * contact_integrate + sort_reorder.  State arrays are in slot order and are
 * updated in place.  Scratch is allocated internally. */
int sdo_run(const sdo_params* p, uint32_t n, float* pos, float* vel, float* omg,
            int steps, int prepare);
/* FP64 twin of sdo_run (error statement of long runs): n x 4 doubles, ids
 * permuted with the cell sort; contacts[s] (s < steps, may be NULL) = the
 * contact pairs of state s. */
int sdo_run_f64(const sdo_params* p, uint32_t n, double* pos, double* vel, double* omg, uint32_t* ids, int steps,
                uint64_t* contacts);

/* A rigid triangle mesh: tri holds 12 floats per triangle (3 rows x, y, z,
 * unused) in the mesh frame, patch a face id per triangle, state 24 floats
 * R[9] (mesh to world), c[3], axis[3], omega, q[4], dq[4] (as the engine's
 * device state).  Every triangle is tested, in ascending order; the deepest
 * contact per patch is kept. */
typedef struct sdo_mesh {
    uint32_t ntri;
    const float* tri;
    const int32_t* patch;
    float state[24];
} sdo_mesh;
void sdo_mesh_advance(float* state24, int advance);

/* ---- rigid clumps (spheres whose id has bit 31 set belong to body
 * body_of[id]; pairs within one body are skipped, collision_resolution.cu:69) */

/* sdo_contact_integrate with clumps: a clump sphere's contact force and
 * torque go to sf4/st4 (slot order) instead of being integrated. */
uint64_t sdo_contact_integrate_bodies(const sdo_params* p, uint32_t n, const float* pos, const float* vel,
                                      const float* omg, const uint32_t* cell_start, const int32_t* body_of,
                                      float* pos_n, float* vel_n, float* omg_n, uint32_t* keys_n,
                                      float* force4, float* torque4, float* sf4, float* st4);
/* slot_of[id] = slot of every sphere of a cell-sorted state. */
void sdo_slot_of(uint32_t n, const float* omg, uint32_t* slot_of);
/* One step of every body and the next state of its spheres. */
void sdo_body_step(const sdo_params* p, uint32_t nb, float* bpos4, float* bvel4, float* bquat4, float* bomg4,
                   float* bang4, const float* binv12, const uint32_t* first, const uint32_t* count,
                   const float* r0_4, const uint32_t* slot_of, const float* pos, const float* omg,
                   const float* sf4, const float* st4, float* pos_n, float* vel_n, float* omg_n,
                   uint32_t* keys_n);
/* sdo_run with rigid bodies (state arrays and body arrays updated in place). */
int sdo_run_bodies(const sdo_params* p, uint32_t n, float* pos, float* vel, float* omg, int steps,
                   uint32_t nb, float* bpos4, float* bvel4, float* bquat4, float* bomg4, float* bang4,
                   const float* binv12, const uint32_t* first, const uint32_t* count, const float* r0_4,
                   const int32_t* body_of);

/* ------------------------------------------------------ convex hulls
 * (sd_oracle_hull.c).  Bodies: pos4 (x, y, z, mass), vel4, quat4 (s, x, y, z),
 * omg4, ang4 (world angular momentum), iinv4 (body-frame principal inverse
 * inertia xyz, bounding radius w); vertices verts4 (body frame) at
 * [vstart[b], vstart[b] + vcount[b]). */

typedef struct sdo_hull_params {
    float lo[3], hi[3];
    float kn, damp, mu;
    float g[3];
    float dt;
    int32_t walls;
} sdo_hull_params;

/* Reference Morton code of each box centroid (testLBVH.cu:113-151). */
void sdo_morton_ref(uint32_t n, const float* lo4, const float* hi4, const float* glo, const float* ghi,
                    uint32_t* codes);
/* Exact closed-box overlap pair set, ascending u64 (i << 32 | j), i < j. */
uint64_t sdo_aabb_pairs(uint32_t n, const float* lo4, const float* hi4, uint64_t* out, uint64_t cap);
/* World AABBs of rotated hulls; ext6 (may be NULL): per body the vertex
 * index of the min x, y, z and max x, y, z. */
void sdo_hull_aabbs(uint32_t nb, const float* pos4, const float* quat4, const uint32_t* vstart,
                    const uint32_t* vcount, const float* verts4, float* lo4, float* hi4, uint32_t* ext6);
/* GJK + EPA of one pair A < B (seed NULL: x_A - x_B). */
void sdo_gjk_epa(const float* pos4, const float* quat4, const float* iinv4, const uint32_t* vstart,
                 const uint32_t* vcount, const float* verts4, uint32_t A, uint32_t B, const float* seed,
                 int32_t* status_iters3, float* res10);
/* Per-body candidate partner lists (CSR, ascending) from the AABB pairs. */
int64_t sdo_hull_partners(uint32_t nb, const float* lo4, const float* hi4, uint32_t* off, uint32_t* partners,
                          uint64_t cap);
/* One hull step over given partner lists (state updated in place). */
void sdo_hull_step(const sdo_hull_params* p, uint32_t nb, float* pos4, float* vel4, float* quat4, float* omg4,
                   float* ang4, const float* iinv4, const uint32_t* vstart, const uint32_t* vcount,
                   const float* verts4, const uint32_t* off, const uint32_t* partners, const float* seeds4,
                   int32_t* status, int32_t* iters, float* dir4, float* force4, float* torque4);

/* The reference's windowed sweep (sap_detection.cu:385-440) and its whole
 * processCollisions pipeline; rows are 16 int32 per sorted position. */
void sdo_sap_sweep_ref(uint32_t n, const float* upperx, const float* lowerx_sorted, const float* uppery,
                       const float* lowery, const uint32_t* idx_sorted, int32_t* rows);
void sdo_sap_process(uint32_t n, const float* pos4, const float* radius, int32_t* rows);

/* sdo_run_bodies with an optional mesh (mesh may be NULL, nb may be 0); the
 * mesh state advances after every step. */
int sdo_run_full(const sdo_params* p, uint32_t n, float* pos, float* vel, float* omg, int steps,
                 uint32_t nb, float* bpos4, float* bvel4, float* bquat4, float* bomg4, float* bang4,
                 const float* binv12, const uint32_t* first, const uint32_t* count, const float* r0_4,
                 const int32_t* body_of, sdo_mesh* mesh);

/* Number of OpenMP threads the oracle uses (1 when built without OpenMP). */
int sdo_num_threads(void);
void sdo_set_num_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
