/*
 * stardust.h -- C ABI of stardust-gb300, a GB300-native (sm_103a) DEM step.
 *
 * The reference engine (spacesuit825/stardust) exposes its per-step DEM path
 * as C++ classes: STARDUST::DEMEngine (src/engine/engine.hpp:37-447) and the
 * static operator class STARDUST::SpatialPartition
 * (src/engine/cuda/collision_detection.cuh:30-66).  This header is the drop-in
 * boundary for that path: plain C, opaque handles, pointers and sizes, int
 * status codes instead of exit() (src/engine/cuda/cuda_utils.hpp:8-14).
 *
 * Conventions
 *   - Every function returns an sd_status; 0 is success.  sd_last_error()
 *     gives a message for the last failure on a handle (or globally for
 *     handle-less calls when h is NULL).
 *   - Ownership: an engine owns all device memory it allocates; raw operator
 *     calls (sd_hash_*, sd_sort_*) use caller-owned device memory only.
 *   - Threading: calls on one engine handle must be serialised.  Different
 *     handles may be used from different host threads.  `stream` arguments
 *     are cudaStream_t values passed as void* (NULL = legacy default stream).
 *   - Layouts: float4 arrays are 16-byte aligned, 4 floats per element.
 *     Sphere position = (x, y, z, radius); velocity = (vx, vy, vz, mass);
 *     angular velocity = (wx, wy, wz, 0).
 */
#ifndef STARDUST_GB300_H
#define STARDUST_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SD_ABI_VERSION 1

typedef enum sd_status {
    SD_OK = 0,
    SD_ERR_INVALID_ARG = 1, /* bad pointer, size or option */
    SD_ERR_CUDA = 2,        /* a CUDA runtime call failed */
    SD_ERR_JSON = 3,        /* scene file unreadable or not the expected schema */
    SD_ERR_CAPACITY = 4,    /* an output or pair buffer was too small */
    SD_ERR_ITER_LIMIT = 5,  /* a bounded device wait or iteration gave up */
    SD_ERR_STATE = 6,       /* call not valid in the engine's current state */
    SD_ERR_IO = 7,          /* file read/write failed */
    SD_ERR_NOMEM = 8,       /* host or device allocation failed */
    SD_ERR_UNSUPPORTED = 9  /* feature not available in this build/config */
} sd_status;

/* Collision engine selector; mirrors STARDUST::CollisionEngine
 * (src/engine/engine.hpp:21-24).  SD_ENGINE_SAP: sphere-triangle candidates
 * of a mesh come from sweep and prune along one axis (the rotation axis of
 * a rotating mesh, else the mesh's longest extent: triangle boxes sorted by
 * their lower bound, each sphere sweeps the window its box can meet);
 * SD_ENGINE_SHP: from a static grid in the mesh frame.  Sphere-sphere
 * candidates come from the spatial hash under both (the reference's SAP
 * step keeps at most 9 partners per sorted box in a window of 64 and is not
 * a correct broad phase; sd_sap_pairs is the exact SAP operator).  Both
 * engines give the same contacts in the same order, so the same bits. */
typedef enum sd_collision_engine {
    SD_ENGINE_SAP = 0,
    SD_ENGINE_SHP = 1 /* spatial hash */
} sd_collision_engine;

/* Mirrors STARDUST::Device (engine.hpp:26-29).  Only SD_DEVICE_GPU runs;
 * the reference never implemented its CPU device either. */
typedef enum sd_device { SD_DEVICE_CPU = 0, SD_DEVICE_GPU = 1 } sd_device;

typedef struct sd_config {
    uint32_t struct_size;     /* sizeof(sd_config), set by sd_config_default */
    int32_t collision_engine; /* sd_collision_engine */
    int32_t device;           /* sd_device */
    int32_t cuda_device;      /* CUDA ordinal */
    float domain;             /* reference m_domain (engine.hpp:43); used as the box edge
                                 when box_hi is left at 0 */
    float box_lo[3], box_hi[3];
    int32_t walls;            /* bit 2*axis+side: wall on that face (0x3f = closed box) */
    float cell;               /* hash cell edge; 0 = 2 * largest radius */
    float kn;                 /* normal stiffness N/m */
    float restitution;        /* normal restitution coefficient (0, 1] */
    float mu;                 /* Coulomb friction coefficient */
    float gravity[3];
    uint64_t pair_capacity;   /* capacity of the contact-pair validation buffer */
    uint32_t flags;           /* SD_FLAG_* */
    uint32_t reserved;        /* must be 0 (keeps the struct free of padding) */
} sd_config;

/* Record per-sphere force/torque and the contact count at every step
 * (needed for SD_FIELD_FORCE/TORQUE; costs 32 B per sphere-step). */
#define SD_FLAG_RECORD 0x1u

typedef struct sd_stats {
    uint64_t n_spheres;
    uint64_t steps;           /* steps taken since prepare */
    uint64_t contacts;        /* particle-particle contacts at the last step (pairs) */
    double kinetic_energy;    /* translational + rotational, J */
    double momentum[3];
    uint32_t device_errors;   /* OR of device error bits (see SD_DEVERR_*) */
    uint32_t n_cells;
    uint64_t n_bodies;        /* rigid clumps, or convex hulls */
    /* convex-hull scenes, last step: candidate pairs (AABB overlaps), GJK
     * support evaluations and EPA iterations summed over them */
    uint64_t gjk_pairs;
    uint64_t gjk_iters;
    uint64_t epa_iters;
    /* sphere scenes, last step: slots whose cell key changed (the step
     * re-sorts incrementally when at most knob "resort_max" changed, else it
     * runs the radix passes); 0 when the knob is 0 */
    uint64_t moved_keys;
    /* kernels one step launches (the kernel nodes of the captured step
     * graph; 0 before the first step) */
    uint64_t step_kernels;
    /* sphere scenes with contact lists (knob "skin_um"), since prepare:
     * steps that built the lists (a scan over the window widened by the
     * skin) and steps that tested only the listed neighbours */
    uint64_t list_builds;
    uint64_t listed_steps;
} sd_stats;

#define SD_DEVERR_LOOKBACK_TIMEOUT 0x1u
#define SD_DEVERR_PAIR_OVERFLOW 0x2u
#define SD_DEVERR_BAD_INPUT 0x4u
#define SD_DEVERR_WAIT_TIMEOUT 0x8u /* a bounded wait on a TMA copy gave up (results still exact) */

typedef enum sd_field {
    SD_FIELD_POSITION = 0, /* float4 (x, y, z, r) */
    SD_FIELD_VELOCITY = 1, /* float4 (vx, vy, vz, m) */
    SD_FIELD_OMEGA = 2,    /* float4 (wx, wy, wz, 0) */
    SD_FIELD_FORCE = 3,    /* float4 contact + wall force of the last step (fx, fy, fz, 0);
                              with SD_FLAG_RECORD; the device array is indexed by sphere id */
    SD_FIELD_TORQUE = 4,   /* float4 contact torque of the last step (indexed by sphere id) */
    SD_FIELD_IDS = 5       /* uint32 original sphere id of each sorted slot (device ptr only) */
} sd_field;

/* Derived step parameters (box, grid, contact-law constants).  Cell key of
 * a position: ix = clamp(trunc((x - lo[0]) / cell), 0, nx-1) (same for y),
 * iz = clamp(trunc((z - lo[2]) / cell_z), 0, nz-1), key = (ix*ny + iy)*nz + iz.
 * cell_z = cell / z_div: the z axis is split z_div times finer than x and y
 * (knob "z_div"), which shortens the candidate range of each neighbour
 * column.  Normal damping gamma_n = damp * sqrt(m_eff). */
typedef struct sd_params {
    float lo[3], hi[3];
    float cell;
    int32_t nx, ny, nz;
    float kn, damp, mu;
    float gravity[3];
    float dt;        /* dt of the captured step graph (0 before the first step) */
    int32_t walls;
    float rmax;      /* largest sphere radius */
    float cell_z;    /* z edge of a cell: cell / z_div */
    int32_t z_div;   /* z cells per cell edge (1 for a batch of scenes) */
} sd_params;

typedef struct sd_engine sd_engine;

/* ------------------------------------------------------------ engine API */

/* Fills the defaults: GPU, spatial hash, unit box with all walls, kn 1e5,
 * restitution 0.5, mu 0.3, gravity (0, 0, -9.81). */
sd_status sd_config_default(sd_config* cfg);

/* DEMEngine(engineConfig, Scalar domain): engine.hpp:43-166. */
sd_status sd_engine_create(const sd_config* cfg, sd_engine** out);
/* ~DEMEngine: engine.hpp:192-296 (frees every device buffer). */
sd_status sd_engine_destroy(sd_engine* h);
/* Removes free spheres (not spheres of rigid clumps) by id, before or after
 * prepare; the remaining spheres keep their order and take ids 0..n-1 in
 * it (clump tables follow).  Ids must be distinct and in range. */
sd_status sd_engine_remove_spheres(sd_engine* h, uint64_t n, const uint32_t* ids);
/* Copies the last error message of h (or of handle-less calls when h is
 * NULL) into buf; always NUL-terminates when len > 0. */
sd_status sd_last_error(const sd_engine* h, char* buf, size_t len);

/* Adds n free spheres.  pos4 = (x, y, z, r), vel4 = (vx, vy, vz, m) host
 * arrays; omega4 may be NULL (zero spin).  Replaces the bulk of
 * DEMEngine::add(DEMParticle) for one-sphere entities
 * (engine.cpp:601-603, entity_handler.cpp:101-107).
 *
 * Runtime changes (the reference's EntityHandler::addEntityRuntime,
 * entity_handler.cpp:116, is a stub): on a prepared engine,
 * sd_engine_add_spheres, sd_engine_add_clump and sd_engine_remove_spheres
 * bring the state back to the host in sphere-id order, apply the change
 * and prepare again (new buffers, cell sort, step graph on the next step);
 * the step count and the mesh pose carry over.  New spheres take the next
 * ids.  Not for a batch of scenes or convex-hull scenes. */
sd_status sd_engine_add_spheres(sd_engine* h, uint64_t n, const float* pos4,
                                const float* vel4, const float* omega4);

/* DEMEngine::add(DEMParticle(id, grid_resolution, size, diameter, mass,
 * position, velocity)) (entity.cpp:9-59, entity.hpp:24-32).  grid_resolution
 * 1 adds a free sphere of radius diameter/2; larger values add the
 * reference's cube clump as one rigid body: grid_resolution^3 spheres of
 * radius diameter/2 at (i, j, k) * size / floor(size/diameter)^2,
 * i, j, k = 1..grid_resolution, placed about `position` as
 * setParticlesInWorldSpace does (world = position - (local - COM)), total
 * mass `mass`. */
sd_status sd_engine_add_particle(sd_engine* h, int32_t grid_resolution, float size,
                                 float diameter, float mass, const float position[3],
                                 const float velocity[3]);

/* Adds one rigid body made of n spheres (the reference's DEMParticle, a
 * clump of spheres integrated as one body, physics_update.cu).  rel4[i] =
 * (x, y, z, r): sphere offsets from the body's centre of mass in the body
 * frame (equal to the world frame at t = 0); com, vel: the body's centre and
 * velocity; omega (may be NULL): angular velocity.  The body's inertia is
 * that of its spheres as solid balls of mass/n each.  Spheres of one body
 * do not collide with each other (collision_resolution.cu:69). */
sd_status sd_engine_add_clump(sd_engine* h, uint32_t n, const float* rel4, float mass,
                              const float com[3], const float vel[3], const float omega[3]);

/* A rigid triangle mesh -- the walls of a rotating drum -- that rotates at
 * omega rad/s about the line through centre along axis (omega = 0: a static
 * mesh).  tri9: n_tris triangles, 9 floats each (three vertices, world frame
 * at time 0); patch (may be NULL: each triangle its own): the face a
 * triangle belongs to -- per sphere, only the deepest contact of each face
 * acts, so a sphere touching several triangles of one flat or gently curved
 * face feels one contact.  Sphere-triangle contacts use the sphere contact
 * law against the moving wall.  Candidate triangles come from a static grid
 * in the mesh's own frame (the mesh moves rigidly, so the grid is built
 * once).  Static meshes combine: a later static mesh is appended, its
 * patch ids renumbered after the earlier ones (ids must be >= 0); a rotating
 * mesh must be the engine's only mesh.  Not in a batch.  Replaces
 * DEMEngine::addMesh (engine.cpp:117-121) with DEMMesh (entity.hpp:64-120),
 * whose triangles the reference never used in a step. */
sd_status sd_engine_add_mesh(sd_engine* h, uint32_t n_tris, const float* tri9, const int32_t* patch,
                             const float centre[3], const float axis[3], float omega);
/* Triangles of an STL file (ASCII or binary), 9 floats each, as stored.
 * Call with tri9 = NULL for the count (*n_tris), then with cap >= *n_tris.
 * Replaces loadAndConvertMesh (src/IO/mesh_loader.cpp:9-45), which reads
 * through the third-party stl_reader header (external/stl_reader). */
sd_status sd_stl_read(const char* path, uint64_t cap, float* tri9, uint64_t* n_tris);
/* Smooth faces of a triangle soup: triangles sharing an edge (bit-identical
 * endpoints) whose normals, as unoriented lines, differ by less than
 * angle_deg share a patch id; ids count up from 0 in order of each patch's
 * first triangle. */
sd_status sd_mesh_patches(uint64_t n_tris, const float* tri9, float angle_deg, int32_t* patch);
/* DEMMesh(filename, position, quaternion) (entity.hpp:68-73) as a wall of
 * the step: the STL's triangles placed at R(quat) v + position (quat = (s,
 * x, y, z), normalised; NULL = identity; position NULL = 0), grouped into
 * patches with patch_angle_deg (30 is a good default), then added with
 * sd_engine_add_mesh (centre NULL = origin; omega 0: static). */
sd_status sd_engine_add_mesh_stl(sd_engine* h, const char* path, const float position[3], const float quat[4],
                                 const float centre[3], const float axis[3], float omega, float patch_angle_deg);
/* The engine's mesh as it steps it (host copy; before or after prepare):
 * n_tris triangles in the mesh frame -- world at time 0 minus centre --,
 * 9 floats each, their patch ids, and the centre.  tri9 / patch / centre3
 * may be NULL; with either array, cap must be >= the triangle count. */
sd_status sd_engine_get_mesh(sd_engine* h, uint64_t cap, float* tri9, int32_t* patch, float* centre3,
                             uint64_t* n_tris);
/* Headless snapshots in place of the reference's OpenGL renderer
 * (src/graphics/renderer.cpp:15-22, 146-147), which writes nothing to disk.
 * SD_SNAPSHOT_CSV: one row per sphere in id order, id,x,y,z,r,vx,vy,vz,m,
 * wx,wy,wz, each the shortest decimal that reads back as the same float32; with
 * SD_SNAPSHOT_CONTACTS also <path>.contacts.csv (i,j per contact pair).
 * SD_SNAPSHOT_VTK: legacy VTK, BINARY POLYDATA -- spheres as points (point
 * i = sphere i, VERTICES cells), contact pairs as LINES, the mesh at its
 * current pose as POLYGONS over extra points (SD_SNAPSHOT_MESH); point data
 * radius, mass, id (-1 on mesh points), velocity, spin. */
typedef enum sd_snapshot_format { SD_SNAPSHOT_CSV = 0, SD_SNAPSHOT_VTK = 1 } sd_snapshot_format;
#define SD_SNAPSHOT_CONTACTS 0x1u
#define SD_SNAPSHOT_MESH 0x2u
sd_status sd_engine_write_snapshot(sd_engine* h, const char* path, int32_t format, uint32_t flags);
/* The mesh pose on the device: R[9] (mesh to world, row-major), centre[3],
 * axis[3], omega, q[4] (s, x, y, z), dq[4] (the rotation of one step). */
sd_status sd_engine_get_mesh_state(sd_engine* h, float* state24);

/* A batch of independent sphere scenes stepped together (one launch per
 * stage for all of them): each call adds one scene -- n spheres (pos4, vel4,
 * omega4 as sd_engine_add_spheres) in its own walled box [lo, hi] with its
 * own hash cell (0: 2 x the scene's largest radius).  Scenes share the
 * material, gravity and time step of the config.  Once a scene is added,
 * every sphere must come through this call; clumps are not batched.  Each
 * scene's grid occupies its own range of cell keys, so one sort orders all
 * scenes and no pair ever spans two scenes.  No counterpart in the
 * reference (its engine holds one scene). */
sd_status sd_engine_add_scene(sd_engine* h, uint64_t n, const float* pos4, const float* vel4, const float* omega4,
                              const float lo[3], const float hi[3], float cell);

/* DEMEngine::loadJSONSetup (engine.cpp:65-108, schema of
 * setup/star_test.json): scene.domain, scene.gravity (magnitude, along -z),
 * scene.entities[] of {type: "generic", position[3], size, mass,
 * velocity[3]}; a generic entity becomes one sphere of diameter `size`.  Extension keys (all optional): scene.box {lo[3], hi[3]},
 * scene.walls (int mask), scene.cell, scene.material {kn, restitution, mu},
 * scene.spheres[] of {position[3], radius, mass, velocity[3]}.  Unknown keys
 * are rejected with SD_ERR_JSON. */
sd_status sd_engine_load_scene_json(sd_engine* h, const char* path);

/* prep() + transfer(): engine.cpp:605-614.  Allocates device state, uploads
 * it and sorts it into cell order. */
sd_status sd_engine_prepare(sd_engine* h);

/* Runs n_steps steps of length dt on the engine's stream (captured once as a
 * CUDA graph).  Returns after enqueueing; use sd_engine_sync to wait. */
sd_status sd_engine_step(sd_engine* h, float dt, int32_t n_steps);
/* DEMEngine::update(float dt): simulation_kernel.cu:52-153 -- one step. */
sd_status sd_engine_update(sd_engine* h, float dt);

/* Stages of one step, for profiling: launching CONTACT, SORT, REORDER in
 * that order is one step.  CONTACT alone is idempotent (it reads the
 * current state and writes the next-state buffers).  In a convex-hull scene
 * CONTACT is the narrow phase (GJK, EPA, contact forces) of the last step's
 * candidate lists at the current bodies, and the only stage: it changes no
 * body, and the entry results it rewrites are rewritten by the next step. */
#define SD_STAGE_CONTACT 0
#define SD_STAGE_SORT 1
#define SD_STAGE_REORDER 2
sd_status sd_engine_launch_stage(sd_engine* h, int32_t stage, float dt);
/* Waits for queued work and reports device error bits as SD_ERR_ITER_LIMIT /
 * SD_ERR_CAPACITY. */
sd_status sd_engine_sync(sd_engine* h);

/* Copies a field in ORIGINAL sphere order (the order spheres were added)
 * into host memory; bytes must be n_spheres * 16. */
sd_status sd_engine_get_state(sd_engine* h, int32_t field, void* host_dst, size_t bytes);
typedef enum sd_body_field {
    SD_BODY_POSITION = 0,   /* float4 (x, y, z, mass) of the centre of mass */
    SD_BODY_VELOCITY = 1,   /* float4 (vx, vy, vz, 0) */
    SD_BODY_QUATERNION = 2, /* float4 (s, x, y, z), body to world */
    SD_BODY_OMEGA = 3,      /* float4 (wx, wy, wz, 0) */
    SD_BODY_ANGMOM = 4,     /* float4 (Lx, Ly, Lz, 0), world frame */
    SD_BODY_INV_INERTIA = 5, /* clumps: 3 float4 rows of the body-frame inverse inertia (12 floats) */
    SD_BODY_HULL_INV_INERTIA = 6, /* hulls: (1/Ix, 1/Iy, 1/Iz, bounding radius), principal frame */
    SD_BODY_FORCE = 7,      /* hulls, SD_FLAG_RECORD: total force of the last step */
    SD_BODY_TORQUE = 8      /* hulls, SD_FLAG_RECORD: total torque of the last step */
} sd_body_field;

/* Copies a rigid-body field into host memory (bodies in the order they
 * were added); bytes must be n_bodies * 16 (48 for SD_BODY_INV_INERTIA). */
sd_status sd_engine_get_bodies(sd_engine* h, int32_t field, void* host_dst, size_t bytes);

/* ------------------------------------------------------ convex hulls
 * A scene holds either spheres and clumps or convex hulls.  Hull scenes
 * step through: world AABBs, an LBVH broad phase (sandbox/testLBVH.cu),
 * GJK + EPA per candidate pair (sandbox/testGJK.cu:52-315 plus a
 * penetration depth), the spring-dashpot law at the EPA contact point, and
 * quaternion integration with a diagonal body-frame inertia. */

/* One hull: the convex hull of n_points points (pts4 rows x, y, z, unused,
 * in the body's local frame placed at pos with orientation quat (s, x, y, z),
 * NULL = identity).  The centre of mass is the mean of the points and the
 * inertia that of the points as equal masses; both are reduced to a
 * principal frame.  No counterpart in the reference (its Hull struct,
 * sandbox/primitives.hpp:37-57, is filled by hand in testGJK.cu:328-352). */
sd_status sd_engine_add_hull(sd_engine* h, uint32_t n_points, const float* pts4, float mass,
                             const float pos[3], const float quat[4], const float vel[3],
                             const float omega[3]);

/* The stored shapes: per hull its first vertex and vertex count, and the
 * principal-frame vertices (float4 rows); *n_verts = total vertex count. */
sd_status sd_engine_get_hull_shapes(sd_engine* h, uint32_t* vstart, uint32_t* vcount, float* verts4,
                                    uint64_t verts_cap, uint64_t* n_verts);

/* GJK seed of a candidate pair.  PLAIN: x_A - x_B, the reference seed
 * (testGJK.cu:266).  PREVIOUS: the pair's final search direction of the
 * previous step (in A's body frame) when it was separated then.  LEARNED:
 * the warm-start network's direction for pairs seen in the previous step.
 * A seeded run has two support evaluations to certify separation; any other
 * outcome is decided by GJK rerun from the plain seed to its own
 * termination test, so the seed changes only the iteration count. */
#define SD_GJK_SEED_PLAIN 0
#define SD_GJK_SEED_LEARNED 1
#define SD_GJK_SEED_PREVIOUS 2
sd_status sd_engine_set_gjk_seed(sd_engine* h, int32_t mode);

/* Online training of the warm-start network while the scene steps (seed mode
 * LEARNED): every `every` steps (0 = off) the step also logs, per separated
 * pair that the network seeds, the separating direction of largest margin
 * (the closest-point direction, GJK run to convergence) in A's frame, and
 * then `iters` Adam steps of rate `lr` on that step's inputs and targets run
 * on the GPU before the next step.  Trains on the simulation's own pairs;
 * contact results are unchanged (seeds only move the iteration count).  No
 * counterpart in the reference. */
sd_status sd_engine_set_gjk_training(sd_engine* h, int32_t every, int32_t iters, float lr);

/* The candidate entries of the last step: off[n_bodies+1] (CSR), partner
 * ids (ascending per body), info (status | GJK iterations << 8 | EPA
 * iterations << 16; status 0 separated, 1 intersecting, 2 touching,
 * 3 not converged), final GJK direction in A's frame (w = 1 when separated),
 * the seeds used (w = 1 when seeded) and the 16 network inputs.  Any output
 * may be NULL; *n_entries receives the count. */
sd_status sd_engine_hull_entries(sd_engine* h, uint32_t* off, uint32_t* partners, uint32_t* info, float* dir4,
                                 float* seed4, float* feat16, uint64_t cap, uint64_t* n_entries);

/* ------------------------------------------------- GJK warm-start network
 * 16 inputs (per candidate pair, in the body frame of its first hull A:
 * relative quaternion conj(qA) qB (4), centre offset / (rhoA + rhoB) (3),
 * previous-contact flag (1), the pair's previous separating direction (3),
 * |offset| / (rhoA + rhoB) (1), zeros (4)) -> 64 -> ReLU -> 64 -> ReLU -> 3,
 * added to inputs 8..10 (a residual network over the previous direction; its
 * last layer starts at zero): a search direction in A's frame.  BF16 weights, FP32 accumulation on the
 * tensor cores, trained on the GPU with Adam on the cosine loss
 * 1 - y.t/|y| against separating directions plain GJK logged
 * (sd_engine_hull_entries).  Parameters: 6288 floats, W1[64][16], b1[64],
 * W2[64][64], b2[64], W3[16][64] (rows 3.. zero), b3[16].  No counterpart in
 * the reference. */
sd_status sd_engine_mlp_params(sd_engine* h, float* host, uint64_t n, int32_t set);
/* Device rows of 16 inputs -> device rows (y0, y1, y2, 0). */
sd_status sd_engine_mlp_forward(sd_engine* h, const float* d_feat16, float* d_out4, uint64_t n);
/* Full-batch training on n device rows (inputs, target (tx, ty, tz, valid)):
 * iters Adam steps of rate lr (iters = 0: the gradient only).  host_grad
 * (may be NULL) receives the last gradient (6288 floats, mean over rows). */
sd_status sd_engine_mlp_train(sd_engine* h, const float* d_feat16, const float* d_tgt4, uint64_t n, int32_t iters,
                              float lr, float* host_grad);

/* ------------------------------------------------------ sweep and prune
 * (SAPCollision, src/engine/cuda/collisions/SAP/sap_detection.cu:135-706). */

/* Device scratch for sd_sap_pairs (pair_cap pairs) and
 * sd_sap_process_collisions (pair_cap 0). */
sd_status sd_sap_scratch_bytes(uint64_t n, uint64_t pair_cap, uint64_t* bytes);
/* Exact broad phase: every pair (i < j) of overlapping closed boxes,
 * ascending u64 (i << 32 | j), by sorting the lower x extents (order-
 * preserving keys, negative coordinates allowed) and sweeping.  d_count[0] =
 * pairs, d_count[1] = device error bits. */
sd_status sd_sap_pairs(uint64_t n, const float* d_lo4, const float* d_hi4, uint64_t* d_pairs, uint64_t cap,
                       uint32_t* d_count, void* d_scratch, uint64_t scratch_bytes, void* stream);
/* sweepAndPruneCUDA (sap_detection.cu:385-440) on given sorted inputs: per
 * sorted position tid a row of 16 int32 at d_rows[16 * tid] -- partner ids
 * found in the next 64 sorted positions whose lower x <= the home upper x
 * (which the kernel replaces by the home upper y once a y test has run) and
 * lower y <= the home upper y; at most 9, unique, ids equal to tid skipped;
 * unused entries -1 (every row is cleared first). */
sd_status sd_sap_sweep(uint64_t n, const float* d_upperx, const float* d_lowerx_sorted, const float* d_uppery,
                       const float* d_lowery, const uint32_t* d_idx_sorted, int32_t* d_rows, void* stream);
/* SAPCollision::processCollisions (sap_detection.cu:668-706): AABBs of
 * spheres (radius from d_radius, or pos.w when NULL), a stable radix sort of
 * the lower x extents as uint32 float bits, then the sweep above. */
sd_status sd_sap_process_collisions(uint64_t n, const float* d_pos4, const float* d_radius, int32_t* d_rows,
                                    void* d_scratch, uint64_t scratch_bytes, void* stream);

/* ------------------------------------------------------ LBVH operators
 * (sandbox/testLBVH.cu:42-907 as raw device operators).  Boxes are float4
 * rows lo (x, y, z, -) and hi, 16-byte aligned, n < 2^30. */

/* Device scratch for sd_lbvh_pairs / sd_lbvh_morton. */
sd_status sd_lbvh_scratch_bytes(uint64_t n, uint64_t pair_cap, uint64_t* bytes);
/* Every pair (i < j) of overlapping closed boxes, ascending u64
 * (i << 32 | j).  d_count[0] = number of pairs (written up to cap),
 * d_count[1] = device error bits (SD_DEVERR_PAIR_OVERFLOW when the partner
 * lists exceeded 2 * cap entries). */
sd_status sd_lbvh_pairs(uint64_t n, const float* d_lo4, const float* d_hi4, uint64_t* d_pairs, uint64_t cap,
                        uint32_t* d_count, void* d_scratch, uint64_t scratch_bytes, void* stream);
/* The reference's 30-bit Morton code of each box centroid relative to the
 * boxes' global bounds (computeSpaceFillingCurveCUDA, testLBVH.cu:113-151). */
sd_status sd_lbvh_morton(uint64_t n, const float* d_lo4, const float* d_hi4, uint32_t* d_codes, void* d_scratch,
                         uint64_t scratch_bytes, void* stream);

/* Overwrites a field (POSITION, VELOCITY, OMEGA) from host memory in
 * original sphere order.  The engine re-sorts before the next step. */
sd_status sd_engine_set_state(sd_engine* h, int32_t field, const void* host_src, size_t bytes);
/* Device pointer of a field in current SORTED slot order (headless
 * replacement of the GL VBO interop, engine.hpp:165-168).  Valid until the
 * next step: the step alternates between two state buffers, so ask again
 * after stepping, as the reference maps its VBO each frame. */
sd_status sd_engine_device_ptr(sd_engine* h, int32_t field, void** out);
/* The engine's CUDA stream (cudaStream_t as void*). */
sd_status sd_engine_stream(sd_engine* h, void** out);

/* Contact pairs of the current state: u64 (min_id << 32 | max_id), sorted
 * ascending, original ids.  *n receives the total; SD_ERR_CAPACITY if it
 * exceeds cap (the first cap are not guaranteed to be the smallest). */
sd_status sd_engine_get_pairs(sd_engine* h, uint64_t* dst, uint64_t cap, uint64_t* n);

sd_status sd_engine_stats(sd_engine* h, sd_stats* out);

/* The step parameters derived from the config and the sphere set (valid
 * before prepare once spheres are added). */
sd_status sd_engine_params(sd_engine* h, sd_params* out);

/* Binary snapshot of the engine state (config, step count, all sphere
 * fields in sorted order).  Loading it into an engine created with the
 * same config resumes bit-exactly. */
sd_status sd_engine_save_checkpoint(sd_engine* h, const char* path);
sd_status sd_engine_load_checkpoint(sd_engine* h, const char* path);

/* ------------------------------------------------------------ launch knobs
 * Process-wide kernel variants and tile sizes, set by the autotuner
 * (stardust_gb300.autotune) in place of the reference's hand block sweeps
 * (profiling/blocksweep*.txt).  Engines re-capture their step graph on the
 * next step after a change.  Knobs:
 *   "contact_mode"  0 = one thread per sphere, candidates read through L1 (default);
 *                   1 = one CTA per grid column, neighbour columns staged in shared
 *                       memory by TMA bulk copies
 *   "sort_items"    keys per thread of the sort's digit pass: 8 or 16 (default)
 *   "z_div"         z cells per cell edge for engines prepared afterwards: 1, 2, 4 or 8,
 *                   or 0 (default) = 2 when that keeps keys within 20 bits and the
 *                   sort's pass count, else 1; a batch of scenes always uses 1
 *   "resort_max"    most changed cell keys the step re-sorts incrementally (a merge of
 *                   the changed entries into the previous order) instead of running the
 *                   radix passes: 0 (always the passes) or a power of two up to 1024;
 *                   default 1024.  Same result either way (a stable sort by key)
 *   "pair_lists"    scenes without clumps or meshes: 1 = a pair kernel tests each candidate
 *                   pair once and lists up to 16 contacts per sphere, which the contact
 *                   kernel applies in slot order (a full scan for an overflowed list);
 *                   0 = one scan kernel; 2 (default) = lists for batches of scenes only.
 *                   Steps with contact lists (knob skin_um) use those instead.
 *                   Same bits either way
 *   "skin_um"       scenes of free spheres (one, or a batch), from the next step: contact lists with a
 *                   skin of this many micrometres (0 = none; default 50).  A step that
 *                   follows a sphere moving 0.45 skin from its position at the last build
 *                   scans the window widened by the skin and lists each sphere's neighbours
 *                   within r_i + r_j + skin; other steps test only the listed neighbours.
 *                   Same contact set and order as the scan, so the same bits
 *   "listed_blocks" resident 256-thread blocks per SM the contact-list kernel is compiled
 *                   for: 4 (64 registers) or 5 (48 registers, the default); single scenes
 *                   without clumps or meshes also 6 (40) or 8 (32 registers, more spills)
 *   "contact_block" threads per block of the per-sphere contact kernels: 64, 128 or 256
 *                   (default)
 *   "fix_blocks"    blocks per SM of the in-place reorder's fixed grid: 2, 4 or 8 (default)
 *   "hull_blocks"   convex-hull scenes: resident 128-thread blocks per SM the GJK kernel is
 *                   compiled for: 3 (168 registers) or 4 (128, the default)
 *   "lbvh_rebuild"  convex-hull scenes: steps between full LBVH builds (1..4096, default 16);
 *                   the steps between refit the last build's tree (exact bounds, so the
 *                   same candidate pairs) */
sd_status sd_tune_set(const char* knob, int32_t value);
sd_status sd_tune_get(const char* knob, int32_t* value);

/* --------------------------------------------------- raw operator API ---
 * Device pointers, caller-owned memory, asynchronous on `stream`. */

/* SpatialPartition::constructCollisionList (sh_collision_detection.cu:285-306,
 * kernel :27-127): writes 9*n (cell, sphere) entries -- home entry, phantom
 * entries, padding -- and the number of non-padding entries into *d_count
 * (device u32, overwritten).  Bit-exact with the reference's rule,
 * including its phantom-offset behaviour. */
sd_status sd_hash_construct_collision_list(uint32_t n, float cell_dim, uint32_t* d_cells,
                                           uint32_t* d_spheres, const float* d_sizes,
                                           const float* d_pos4, uint32_t* d_count,
                                           void* stream);

/* Bytes of device scratch sd_sort_pairs / sd_hash_sort_collision_list need
 * for n keys of key_bits bits. */
sd_status sd_sort_scratch_bytes(uint64_t n, int32_t key_bits, uint64_t* bytes);

/* Stable LSD radix sort of (key, value) u32 pairs by key bits
 * [0, key_bits), onesweep style (one histogram pass + one pass per digit
 * with decoupled look-back).  The sorted result is left in d_keys/d_vals;
 * d_keys_tmp/d_vals_tmp are n-element ping-pong buffers.  The first 16
 * bytes of scratch hold a status word (see sd_sort_status); the caller
 * zeroes it once. */
sd_status sd_sort_pairs(uint32_t* d_keys, uint32_t* d_vals, uint32_t* d_keys_tmp,
                        uint32_t* d_vals_tmp, uint64_t n, int32_t key_bits, void* d_scratch,
                        uint64_t scratch_bytes, void* stream);

/* SpatialPartition::sortCollisionList (sh_collision_detection.cu:310-360):
 * sorts the first n (cell, sphere) entries by the full 32-bit cell word,
 * result back in d_cells/d_spheres, like the reference's four-pass
 * ping-pong. */
sd_status sd_hash_sort_collision_list(uint32_t* d_cells, uint32_t* d_spheres,
                                      uint32_t* d_cells_tmp, uint32_t* d_spheres_tmp,
                                      uint64_t n, void* d_scratch, uint64_t scratch_bytes,
                                      void* stream);

/* Reads the sort status word (synchronises the stream): *errors receives
 * the device error bits accumulated since the caller last zeroed it. */
sd_status sd_sort_status(const void* d_scratch, void* stream, uint32_t* errors);

/* sd_sort_pairs without a caller scratch buffer, for callers that cannot
 * allocate device memory (a stepping loop that must never block on the
 * device allocator, or a host that only hands over the key/value buffers it
 * owns).  No counterpart in the reference, whose sort takes its radix
 * buffers from the engine's allocations.  Allocates nothing: the scratch is
 * a fixed 8 MiB array in the library's device memory, held on every GPU
 * that loads the library until exit.  Sorts whose scratch need
 * (sd_sort_scratch_bytes) exceeds 8 MiB return SD_ERR_CAPACITY -- up to
 * 2,093,056 keys of 32 bits, 4,188,160 keys of at most 18 bits.  Every call
 * looks up the array's device address on the current device; the first call
 * on a device also loads the library's device code there (make that first
 * call before any stream capture).  All calls share the array, so calls
 * that overlap on the GPU race; each call re-clears what must start at zero.
 * Same result layout as sd_sort_pairs (sorted pairs in d_keys/d_vals);
 * d_status, when not NULL, receives the device error bits (one u32). */
sd_status sd_sort_pairs_noalloc(uint32_t* d_keys, uint32_t* d_vals, uint32_t* d_keys_tmp,
                                uint32_t* d_vals_tmp, uint64_t n, int32_t key_bits,
                                uint32_t* d_status, void* stream);

/* Candidate pairs of SpatialPartition::tranverseAndResolveCollisionList
 * (collision_resolution.cu:100-199): over the first *d_count sorted
 * entries, every home entry pairs with every later entry of its cell run;
 * pairs within one rigid body (d_body_of, may be NULL) are skipped
 * (collision_resolution.cu:69).  Writes (home, other) sphere ids in the
 * reference's traversal order to d_pair_a/d_pair_b and the total into
 * *d_npairs (device u64).  Pairs beyond cap are counted, not written. */
sd_status sd_hash_candidate_pairs(const uint32_t* d_cells, const uint32_t* d_spheres,
                                  const uint32_t* d_count, uint32_t n_entries,
                                  const int32_t* d_body_of, uint32_t* d_pair_a,
                                  uint32_t* d_pair_b, uint64_t cap, uint64_t* d_npairs,
                                  void* d_scratch, uint64_t scratch_bytes, void* stream);

/* Bytes of device scratch sd_hash_candidate_pairs needs for n_entries. */
sd_status sd_hash_pairs_scratch_bytes(uint64_t n_entries, uint64_t* bytes);

/* ------------------------------------------------------ scene generators
 * Seeded, deterministic host-side scene builders (the reference builds its
 * scenes in sandbox/testDEM.cpp:60-98 with unseeded rand()). */

/* nx*ny*nz spheres on a cubic lattice of the given spacing starting at
 * origin (first centre = origin), each coordinate jittered by
 * U[-jitter, jitter]; velocities U[-vmax, vmax] per axis.  Writes pos4/vel4
 * (n*4 floats each), sphere i = (ix*ny + iy)*nz + iz. */
sd_status sd_scene_lattice(int32_t nx, int32_t ny, int32_t nz, float spacing, float jitter,
                           const float origin[3], float radius, float mass, float vmax,
                           uint64_t seed, float* pos4, float* vel4);

/* Random sequential addition of n non-overlapping spheres in the box
 * [lo, hi], radii lognormal(r_median, r_sigma) clipped to [r_min, r_max],
 * inserted largest first; mass = density * 4/3 pi r^3; velocities
 * U[-vmax, vmax].  Gives up with SD_ERR_CAPACITY after max_attempts
 * placements attempts for one sphere.  *volume_fraction (may be NULL)
 * receives the packed fraction. */
sd_status sd_scene_rsa(uint64_t n, const float lo[3], const float hi[3], float r_median,
                       float r_sigma, float r_min, float r_max, float density, float vmax,
                       uint64_t seed, uint64_t max_attempts, float* pos4, float* vel4,
                       double* volume_fraction);

#ifdef __cplusplus
}
#endif
#endif /* STARDUST_GB300_H */
