// ref_harness.cpp -- runs the reference's own kernels (test infrastructure).
//
// oracle/ref_build.py compiles the reference's kernel sources
// (src/engine/cuda/sh_collision_detection.cu, collision_resolution.cu,
// physics_update.cu) unchanged, where they lie, into sm_103a cubins in
// oracle/_ref/.  This harness loads those cubins with the CUDA driver API and
// launches the reference kernels with the reference's launch shapes, so the
// CPU restatement in sd_oracle.c can be pinned against the reference's own
// code (tests/golden/make_ref_golden.py writes the golden vectors).
//
// Only kernels that are deterministic and stay in bounds on the inputs the
// golden script builds are exposed: the key/phantom construction, the run
// traversal on inputs where every sphere sits in exactly one run (so the
// reference's non-atomic force writes do not race), and the three
// rigid-body kernels (one thread per body or sphere).
#include <cuda.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct Kern {
    const char* part;  // substring of the mangled name
    const char* module;
    bool optional = false;  // the LBVH/GJK prototypes, loaded when their cubins exist
    CUfunction fn = nullptr;
};

Kern g_k[] = {
    {"constructCollisionListCUDA", "sh_collision_detection"},
    {"tranverseCollisionListCUDA", "collision_resolution"},
    {"updateSphereDataCUDA", "physics_update"},
    {"computeForcesAndTorquesCUDA", "physics_update"},
    {"advectParticlesCUDA", "physics_update"},
    {"RadixTabulateCUDA", "sh_collision_detection"},
    {"RadixSumCUDA", "sh_collision_detection"},
    {"RadixReorderCUDA", "sh_collision_detection"},
    {"sweepAndPruneCUDA", "sap_detection"},
    {"computeSpaceFillingCurveCUDA", "testLBVH", true},
    {"gjkCUDA", "testGJK", true},
};
constexpr int kConstruct = 0, kTraverse = 1, kUpdate = 2, kForces = 3, kAdvect = 4, kTab = 5, kSum = 6,
              kReorder = 7, kSweep = 8, kMorton = 9, kGjk = 10;

std::string g_err;

int fail(const char* what, CUresult r) {
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    g_err = std::string(what) + ": " + (s ? s : "?");
    return 1;
}

int launch_async(int k, unsigned grid, unsigned block, unsigned smem, CUstream st, void** args) {
    if (!g_k[k].fn) {
        g_err = std::string("kernel not loaded: ") + g_k[k].part;
        return 1;
    }
    CUresult r = cuLaunchKernel(g_k[k].fn, grid, 1, 1, block, 1, 1, smem, st, args, nullptr);
    if (r != CUDA_SUCCESS) return fail("cuLaunchKernel", r);
    return 0;
}

int launch(int k, unsigned grid, unsigned block, unsigned smem, CUstream st, void** args) {
    if (launch_async(k, grid, block, smem, st, args)) return 1;
    CUresult r = cuStreamSynchronize(st);
    if (r != CUDA_SUCCESS) return fail("cuStreamSynchronize", r);
    return 0;
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

// Loads the three cubins from `dir` into the current context and finds the
// kernels by name.
int ref_init(const char* dir) {
    const char* mods[] = {"sh_collision_detection", "collision_resolution", "physics_update", "sap_detection",
                          "testLBVH", "testGJK"};
    for (const char* m : mods) {
        const bool optional = std::strncmp(m, "test", 4) == 0;
        std::string path = std::string(dir) + "/" + m + ".cubin";
        if (optional) {
            FILE* f = std::fopen(path.c_str(), "rb");
            if (!f) continue;
            std::fclose(f);
        }
        CUmodule mod;
        CUresult r = cuModuleLoad(&mod, path.c_str());
        if (r != CUDA_SUCCESS) return fail(path.c_str(), r);
        unsigned count = 0;
        if ((r = cuModuleGetFunctionCount(&count, mod)) != CUDA_SUCCESS) return fail("cuModuleGetFunctionCount", r);
        std::vector<CUfunction> fns(count);
        if ((r = cuModuleEnumerateFunctions(fns.data(), count, mod)) != CUDA_SUCCESS)
            return fail("cuModuleEnumerateFunctions", r);
        for (CUfunction f : fns) {
            const char* name = nullptr;
            if (cuFuncGetName(&name, f) != CUDA_SUCCESS || !name) continue;
            for (Kern& k : g_k)
                if (std::strcmp(k.module, m) == 0 && std::strstr(name, k.part)) k.fn = f;
        }
    }
    for (Kern& k : g_k)
        if (!k.fn && !k.optional) {
            g_err = std::string("kernel not found: ") + k.part;
            return 1;
        }
    return 0;
}

// computeSpaceFillingCurveCUDA<<<ceil(n/256), 256>>> (sandbox/testLBVH.cu:
// 113-151, launched as at :153-171): boxes as the sandbox's AABB rows
// (upper extent, then lower extent, float4 each), the domain passed by value.
int ref_morton(int n, const float* dom_upper4, const float* dom_lower4, CUdeviceptr aabbs, CUdeviceptr codes,
               CUdeviceptr idx, CUstream st) {
    struct {
        float u[4], l[4];
    } __attribute__((aligned(16))) dom;
    std::memcpy(dom.u, dom_upper4, sizeof dom.u);
    std::memcpy(dom.l, dom_lower4, sizeof dom.l);
    void* args[] = {&n, &dom, &aabbs, &codes, &idx};
    return launch(kMorton, (unsigned)((n + 255) / 256), 256, 0, st, args);
}

// STARDUST::gjkCUDA (sandbox/testGJK.cu:237-315) on ONE candidate pair
// (n_collisions = 1, one block of one thread).  The kernel keeps its verdict
// in a local and only prints "Yo, you just collided!" for a hit, so one pair
// per launch (synchronised) ties each printed line to its pair; the caller
// captures the process's standard output.
int ref_gjk_one(unsigned n_primitives, CUdeviceptr pair, CUdeviceptr hulls, CUdeviceptr verts, CUstream st) {
    unsigned n_collisions = 1;
    void* args[] = {&n_collisions, &n_primitives, &pair, &hulls, &verts};
    return launch(kGjk, 1, 1, 0, st, args);
}

// sweepAndPruneCUDA<<<ceil(n/256), 256>>> (sap_detection.cu:613-629) on given
// sorted inputs; rows (16 per sorted position) must be set to -1 first.
int ref_sap_sweep(int n, CUdeviceptr upperx, CUdeviceptr lowerx_sorted, CUdeviceptr uppery, CUdeviceptr lowery,
                  CUdeviceptr idx_sorted, CUdeviceptr idx, CUdeviceptr rows, CUstream st) {
    int padding = 16;
    void* args[] = {&n, &upperx, &lowerx_sorted, &uppery, &lowery, &idx_sorted, &idx, &rows, &padding};
    return launch(kSweep, (unsigned)((n + 255) / 256), 256, 0, st, args);
}

// constructCollisionListCUDA<<<16, tpb, tpb*4>>> (sh_collision_detection.cu:298);
// d_temp[0] must be zero on entry (the reference memsets it, :296).
int ref_construct(unsigned n, float cell_dim, CUdeviceptr cells, CUdeviceptr spheres, CUdeviceptr sizes,
                  CUdeviceptr pos, CUdeviceptr d_temp, unsigned tpb, CUstream st) {
    void* args[] = {&n, &cell_dim, &cells, &spheres, &sizes, &pos, &d_temp};
    return launch(kConstruct, 16, tpb, tpb * 4, st, args);
}

// tranverseCollisionListCUDA, run by ONE thread.  Every thread of that
// kernel reads the entry count from collision_count[0] and then zeroes it
// (collision_resolution.cu:117-120), so a multi-thread launch races.  With
// one block of one thread and threads_per_block = 1, the thread's chunk is
// (count - 1) / 16 + 1 entries (the kernel divides by its 16 blocks), so the
// caller stores 16 * count in d_temp[0]: the single thread then walks every
// run in order.  It reads up to entry 16 * count, so cells/spheres must hold
// at least 16 * count + 1 entries, padded with the sentinel key 0xffffffff.
int ref_traverse_serial(CUdeviceptr cells, CUdeviceptr spheres, CUdeviceptr pos, CUdeviceptr vel,
                        CUdeviceptr force, CUdeviceptr mass, CUdeviceptr size, CUdeviceptr rigid, unsigned n,
                        CUdeviceptr d_temp, CUstream st) {
    CUdeviceptr test_count = d_temp + 4;
    int tpb = 1;
    void* args[] = {&cells, &spheres, &pos, &vel, &force, &mass, &size, &rigid, &n, &d_temp, &test_count, &tpb};
    return launch(kTraverse, 1, 1, 4, st, args);
}

// updateSphereDataCUDA<<<ceil(n/64), 64>>> (physics_update.cu:124-139).
int ref_update_spheres(int n_spheres, int n_bodies, CUdeviceptr pos, CUdeviceptr vel, CUdeviceptr init_rel,
                       CUdeviceptr rel, CUdeviceptr body_of, CUdeviceptr bpos, CUdeviceptr bvel, CUdeviceptr bquat,
                       CUdeviceptr bomega, CUstream st) {
    void* args[] = {&n_spheres, &n_bodies, &pos, &vel, &init_rel, &rel, &body_of, &bpos, &bvel, &bquat, &bomega};
    return launch(kUpdate, (unsigned)(n_spheres + 63) / 64, 64, 0, st, args);
}

// computeForcesAndTorquesCUDA<<<ceil(nb/64), 64>>> (physics_update.cu:210-227).
int ref_body_forces(int n_spheres, int n_bodies, CUdeviceptr bforce, CUdeviceptr btorque, CUdeviceptr bmass,
                    CUdeviceptr start, CUdeviceptr length, CUdeviceptr rel, CUdeviceptr sforce, CUdeviceptr body_of,
                    CUstream st) {
    void* args[] = {&n_spheres, &n_bodies, &bforce, &btorque, &bmass, &start, &length, &rel, &sforce, &body_of};
    return launch(kForces, (unsigned)(n_bodies + 63) / 64, 64, 0, st, args);
}

// advectParticlesCUDA<<<ceil(nb/64), 64>>> (physics_update.cu:329-347).
int ref_advect(int n_spheres, int n_bodies, float dt, CUdeviceptr bpos, CUdeviceptr bvel, CUdeviceptr bomega,
               CUdeviceptr bforce, CUdeviceptr btorque, CUdeviceptr bquat, CUdeviceptr bmass, CUdeviceptr lin,
               CUdeviceptr ang, CUdeviceptr inertia, CUstream st) {
    void* args[] = {&n_spheres, &n_bodies, &dt, &bpos, &bvel, &bomega, &bforce, &btorque, &bquat, &bmass,
                    &lin, &ang, &inertia};
    return launch(kAdvect, (unsigned)(n_bodies + 63) / 64, 64, 0, st, args);
}

// Buffers of one step of the reference's spatial-hash path.
struct RefStep {
    unsigned n;            // spheres (one-sphere bodies)
    float cell_dim;
    CUdeviceptr cells, spheres, cells_tmp, spheres_tmp;  // 9n u32 each
    CUdeviceptr radices, radix_sums;                     // 16*256*12 and 256 u32
    CUdeviceptr d_temp;                                  // 2 u32
    CUdeviceptr pos, vel, force, size, mass, rigid;      // spheres
    CUdeviceptr init_rel, rel;                           // spheres
    CUdeviceptr bpos, bvel, bomega, bforce, btorque, bquat, bmass, lin, ang, inertia, start, length;  // bodies
    float dt;
};

// Enqueues one step of the reference's spatial-hash path on `st`, with the
// reference's launch shapes: constructCollisionList
// (sh_collision_detection.cu:285-306), sortCollisionList over the 9n
// entries -- 4 passes of Tabulate/Sum/Reorder, 16 blocks of 192 threads
// (:310-360), run as written -- tranverseAndResolveCollisionList
// (collision_resolution.cu:201-231), then computeForcesAndTorques, advect and
// updateSphereData (physics_update.cu).  Nothing is synchronised; the caller
// times it with events on `st`.
// Stage masks for ref_step_async: construct, sort, traverse, rigid-body.
enum { kStageConstruct = 1, kStageSort = 2, kStageTraverse = 4, kStageRigid = 8 };

int ref_stages_async(const RefStep* b, int stages, CUstream st);

int ref_step_async(const RefStep* b, CUstream st) { return ref_stages_async(b, 15, st); }

int ref_stages_async(const RefStep* b, int stages, CUstream st) {
    unsigned n = b->n, entries = 9 * b->n;
    int tpb = 128;
    if (stages & kStageConstruct) {
        if (cuMemsetD32Async(b->d_temp, 0, 2, st) != CUDA_SUCCESS) return fail("memset", CUDA_ERROR_UNKNOWN);
        float cd = b->cell_dim;
        CUdeviceptr c = b->cells, s = b->spheres, sz = b->size, p = b->pos, t = b->d_temp;
        void* a[] = {&n, &cd, &c, &s, &sz, &p, &t};
        if (launch_async(kConstruct, 16, tpb, tpb * 4, st, a)) return 1;
    }
    if (stages & kStageSort) {
        unsigned cells_per_group = (entries - 1) / 16 / 12 + 1;
        CUdeviceptr k = b->cells, v = b->spheres, kt = b->cells_tmp, vt = b->spheres_tmp;
        CUdeviceptr rad = b->radices, sums = b->radix_sums;
        for (int shift = 0; shift < 32; shift += 8) {
            void* a1[] = {&k, &rad, &entries, &cells_per_group, &shift};
            if (launch_async(kTab, 16, 12 * 16, 12 * 256 * 4, st, a1)) return 1;
            void* a2[] = {&rad, &sums};
            if (launch_async(kSum, 16, 12 * 16, 256 * 4, st, a2)) return 1;
            void* a3[] = {&k, &v, &kt, &vt, &rad, &sums, &entries, &cells_per_group, &shift};
            if (launch_async(kReorder, 16, 12 * 16, (256 + 12 * 256) * 4, st, a3)) return 1;
            CUdeviceptr x = k; k = kt; kt = x;
            x = v; v = vt; vt = x;
        }
    }
    if (stages & kStageTraverse) {
        CUdeviceptr c = b->cells, s = b->spheres, p = b->pos, v = b->vel, f = b->force, m = b->mass, sz = b->size,
                    rg = b->rigid, t = b->d_temp, tc = b->d_temp + 4;
        void* a[] = {&c, &s, &p, &v, &f, &m, &sz, &rg, &n, &t, &tc, &tpb};
        if (launch_async(kTraverse, 16, tpb, tpb * 4, st, a)) return 1;
    }
    if (stages & kStageRigid) {
        int ns = (int)n, nb = (int)n;
        CUdeviceptr bf = b->bforce, bt = b->btorque, bm = b->bmass, s0 = b->start, ln = b->length, rl = b->rel,
                    f = b->force, rg = b->rigid;
        void* a[] = {&ns, &nb, &bf, &bt, &bm, &s0, &ln, &rl, &f, &rg};
        if (launch_async(kForces, (n + 63) / 64, 64, 0, st, a)) return 1;
        float dt = b->dt;
        CUdeviceptr bp = b->bpos, bv = b->bvel, bw = b->bomega, bq = b->bquat, li = b->lin, an = b->ang,
                    in = b->inertia;
        void* a2[] = {&ns, &nb, &dt, &bp, &bv, &bw, &bf, &bt, &bq, &bm, &li, &an, &in};
        if (launch_async(kAdvect, (n + 63) / 64, 64, 0, st, a2)) return 1;
        CUdeviceptr p = b->pos, v = b->vel, ir = b->init_rel;
        void* a3[] = {&ns, &nb, &p, &v, &ir, &rl, &rg, &bp, &bv, &bq, &bw};
        if (launch_async(kUpdate, (n + 63) / 64, 64, 0, st, a3)) return 1;
    }
    return 0;
}

}  // extern "C"
