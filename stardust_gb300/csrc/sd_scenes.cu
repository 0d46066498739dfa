// sd_scenes.cu -- seeded host-side scene builders (include/stardust.h:
// sd_scene_lattice, sd_scene_rsa).  The reference builds its scenes with
// unseeded rand() in sandbox/testDEM.cpp:60-98; these are deterministic for a
// given seed on every host (SplitMix64 stream, double arithmetic, one float
// rounding per stored value).
//
// Host code only.  The library compiles it with the rest of csrc/; the CPU
// oracle's build compiles the same file with SD_SCENES_STANDALONE (names
// prefixed sdo_, no CUDA), so both sides of a comparison draw identical
// inputs without the oracle loading this library.
#ifdef SD_SCENES_STANDALONE
#define sd_scene_lattice sdo_scene_lattice
#define sd_scene_rsa sdo_scene_rsa
#endif
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/stardust.h"
#ifndef SD_SCENES_STANDALONE
#include "sd_internal.h"
#endif

namespace {

constexpr double kPi = 3.14159265358979323846;

// SplitMix64 (Steele, Lea, Flood 2014): one 64-bit state, one output per call.
struct SplitMix {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    double u01() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

sd_status scene_fail(sd_status code, const std::string& msg) {
#ifdef SD_SCENES_STANDALONE
    (void)msg;
#else
    sd::set_last_error(msg);
#endif
    return code;
}

}  // namespace

extern "C" {

sd_status sd_scene_lattice(int32_t nx, int32_t ny, int32_t nz, float spacing, float jitter, const float origin[3],
                           float radius, float mass, float vmax, uint64_t seed, float* pos4, float* vel4) {
    if (nx < 0 || ny < 0 || nz < 0 || !origin || !pos4 || !vel4)
        return scene_fail(SD_ERR_INVALID_ARG, "bad lattice arguments");
    SplitMix rng{seed};
    size_t i = 0;
    for (int32_t x = 0; x < nx; ++x)
        for (int32_t y = 0; y < ny; ++y)
            for (int32_t z = 0; z < nz; ++z, ++i) {
                int32_t idx[3] = {x, y, z};
                for (int a = 0; a < 3; ++a) {
                    double j = (2.0 * rng.u01() - 1.0) * jitter;
                    pos4[4 * i + a] = (float)((double)origin[a] + (double)idx[a] * spacing + j);
                }
                pos4[4 * i + 3] = radius;
                for (int a = 0; a < 3; ++a) vel4[4 * i + a] = (float)((2.0 * rng.u01() - 1.0) * vmax);
                vel4[4 * i + 3] = mass;
            }
    return SD_OK;
}

sd_status sd_scene_rsa(uint64_t n, const float lo[3], const float hi[3], float r_median, float r_sigma, float r_min,
                       float r_max, float density, float vmax, uint64_t seed, uint64_t max_attempts, float* pos4,
                       float* vel4, double* volume_fraction) {
    if (!lo || !hi || (n && (!pos4 || !vel4)) || !(r_min > 0) || !(r_max >= r_min) || !(density > 0))
        return scene_fail(SD_ERR_INVALID_ARG, "bad RSA arguments");
    for (int a = 0; a < 3; ++a)
        if (!(hi[a] - lo[a] > 2 * r_max)) return scene_fail(SD_ERR_INVALID_ARG, "box smaller than a sphere");
    SplitMix rng{seed};
    std::vector<double> r(n);
    for (uint64_t i = 0; i < n; ++i) {
        double u1 = rng.u01(), u2 = rng.u01();
        double g = std::sqrt(-2.0 * std::log(u1 + 1e-300)) * std::cos(2.0 * kPi * u2);
        double x = (double)r_median * std::exp((double)r_sigma * g);
        r[i] = std::min<double>(std::max<double>(x, r_min), r_max);
    }
    std::sort(r.begin(), r.end(), [](double a, double b) { return a > b; });
    const double c = 2.0 * r_max;
    int dims[3];
    for (int a = 0; a < 3; ++a) dims[a] = std::max(1, (int)std::ceil((hi[a] - lo[a]) / c));
    size_t ncell = (size_t)dims[0] * dims[1] * dims[2];
    // cell-binned occupancy; a cell of edge 2*r_max holds few spheres
    std::vector<std::vector<uint32_t>> bins(ncell);
    std::vector<double> P(3 * n);
    double vol = 0;
    for (uint64_t i = 0; i < n; ++i) {
        double ri = r[i];
        bool placed = false;
        for (uint64_t att = 0; att < max_attempts && !placed; ++att) {
            double x[3];
            for (int a = 0; a < 3; ++a) x[a] = lo[a] + ri + rng.u01() * ((double)hi[a] - lo[a] - 2 * ri);
            int ci[3];
            for (int a = 0; a < 3; ++a) ci[a] = std::min(dims[a] - 1, (int)((x[a] - lo[a]) / c));
            bool clash = false;
            for (int dx = -1; dx <= 1 && !clash; ++dx)
                for (int dy = -1; dy <= 1 && !clash; ++dy)
                    for (int dz = -1; dz <= 1 && !clash; ++dz) {
                        int X = ci[0] + dx, Y = ci[1] + dy, Z = ci[2] + dz;
                        if (X < 0 || Y < 0 || Z < 0 || X >= dims[0] || Y >= dims[1] || Z >= dims[2]) continue;
                        for (uint32_t j : bins[((size_t)X * dims[1] + Y) * dims[2] + Z]) {
                            double ex = x[0] - P[3 * j], ey = x[1] - P[3 * j + 1], ez = x[2] - P[3 * j + 2];
                            double rr = ri + r[j];
                            if (ex * ex + ey * ey + ez * ez < rr * rr) {
                                clash = true;
                                break;
                            }
                        }
                    }
            if (clash) continue;
            for (int a = 0; a < 3; ++a) P[3 * i + a] = x[a];
            bins[((size_t)ci[0] * dims[1] + ci[1]) * dims[2] + ci[2]].push_back((uint32_t)i);
            placed = true;
        }
        if (!placed)
            return scene_fail(SD_ERR_CAPACITY, "RSA could not place sphere " + std::to_string(i) + " within max_attempts");
        double vi = 4.0 / 3.0 * kPi * ri * ri * ri;
        vol += vi;
        for (int a = 0; a < 3; ++a) {
            pos4[4 * i + a] = (float)P[3 * i + a];
            vel4[4 * i + a] = (float)((2.0 * rng.u01() - 1.0) * vmax);
        }
        pos4[4 * i + 3] = (float)ri;
        vel4[4 * i + 3] = (float)(density * vi);
    }
    if (volume_fraction)
        *volume_fraction = vol / (((double)hi[0] - lo[0]) * ((double)hi[1] - lo[1]) * ((double)hi[2] - lo[2]));
    return SD_OK;
}

}  // extern "C"
