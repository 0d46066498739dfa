/*
 * stardust_demengine.hpp -- a header-only C++ stand-in for the reference's
 * STARDUST::DEMEngine (src/engine/engine.hpp:37-447) over the C ABI of
 * stardust.h, so that drivers written against the reference class
 * (sandbox/testDEM.cpp:60-137: construct, add, prep, transfer, update in a
 * loop) build against libstardust_gb300.so with their calls unchanged.
 *
 * Differences from the reference class: failures throw std::runtime_error
 * with the library's message (the reference calls exit()); update() is
 * asynchronous (sync() or any state read waits); the collision engine and
 * device selectors map onto sd_config (engine.hpp:21-29).
 */
#ifndef STARDUST_DEMENGINE_HPP
#define STARDUST_DEMENGINE_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "stardust.h"

namespace STARDUST {

enum class CollisionEngine { SAP = SD_ENGINE_SAP, SHP = SD_ENGINE_SHP };
enum class Device { CPU = SD_DEVICE_CPU, GPU = SD_DEVICE_GPU };

struct engineConfig {
    CollisionEngine collision_engine = CollisionEngine::SHP;
    Device device = Device::GPU;
};

class DEMEngine {
  public:
    // DEMEngine(engineConfig, Scalar domain) (engine.hpp:43): a closed cubic
    // box of edge `domain`
    DEMEngine(engineConfig cfg, float domain) {
        sd_config c;
        check(sd_config_default(&c));
        c.collision_engine = static_cast<int32_t>(cfg.collision_engine);
        c.device = static_cast<int32_t>(cfg.device);
        c.domain = domain;
        check(sd_engine_create(&c, &h_));
    }
    explicit DEMEngine(const sd_config& c) { check(sd_engine_create(&c, &h_)); }
    ~DEMEngine() {
        if (h_) sd_engine_destroy(h_);
    }
    DEMEngine(const DEMEngine&) = delete;
    DEMEngine& operator=(const DEMEngine&) = delete;

    // add(DEMParticle(id, grid_resolution, size, diameter, mass, position,
    // velocity)) (entity.hpp:24-32): grid_resolution 1 is one sphere of
    // radius diameter / 2, larger values the reference's cube clump
    void add(int32_t grid_resolution, float size, float diameter, float mass, const float position[3],
             const float velocity[3]) {
        check(sd_engine_add_particle(h_, grid_resolution, size, diameter, mass, position, velocity));
    }
    // bulk form: n spheres, (x, y, z, r) and (vx, vy, vz, m) rows
    void addSpheres(const std::vector<float>& pos4, const std::vector<float>& vel4) {
        if (pos4.size() != vel4.size() || pos4.size() % 4) throw std::invalid_argument("addSpheres: bad sizes");
        check(sd_engine_add_spheres(h_, pos4.size() / 4, pos4.data(), vel4.data(), nullptr));
    }
    // addMesh(DEMMesh) (engine.cpp:117-121): triangles in world coordinates,
    // optionally turning about an axis (a rotating drum)
    void addMesh(const std::vector<float>& tri9, const float centre[3], const float axis[3], float omega) {
        check(sd_engine_add_mesh(h_, static_cast<uint32_t>(tri9.size() / 9), tri9.data(), nullptr, centre, axis,
                                 omega));
    }
    void loadJSONSetup(const std::string& path) { check(sd_engine_load_scene_json(h_, path.c_str())); }
    void prep() {}                                  // folded into transfer()
    void transfer() { check(sd_engine_prepare(h_)); }  // engine.cpp:605-614
    void update(float dt) { check(sd_engine_update(h_, dt)); }  // simulation_kernel.cu:52-153
    void sync() { check(sd_engine_sync(h_)); }

    // the state in the order spheres were added
    std::vector<float> positions() { return field(SD_FIELD_POSITION); }
    std::vector<float> velocities() { return field(SD_FIELD_VELOCITY); }
    sd_stats stats() {
        sd_stats s;
        check(sd_engine_stats(h_, &s));
        return s;
    }
    sd_engine* handle() { return h_; }

  private:
    std::vector<float> field(int32_t f) {
        const sd_stats s = stats();
        std::vector<float> out(4 * s.n_spheres);
        check(sd_engine_get_state(h_, f, out.data(), out.size() * sizeof(float)));
        return out;
    }
    void check(sd_status s) {
        if (s != SD_OK) {
            char m[512];
            sd_last_error(h_, m, sizeof m);
            throw std::runtime_error(std::string(m));
        }
    }
    sd_engine* h_ = nullptr;
};

}  // namespace STARDUST

#endif
