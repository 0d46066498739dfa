// sd_snapshot.cu -- headless snapshots of the engine state (host code).
//
// The reference shows its spheres through an OpenGL renderer
// (src/graphics/renderer.cpp:15-22, 146-147, fed by the VBO interop of
// engine.hpp:165-168) and writes nothing to disk.  This file writes the
// state instead, through the public C ABI only (sd_engine_get_state,
// sd_engine_get_pairs, sd_engine_get_mesh, sd_engine_get_mesh_state):
//
//   * CSV: one row per sphere in id order --
//     id,x,y,z,r,vx,vy,vz,m,wx,wy,wz -- each value the shortest decimal that
//     reads back as the same float32; with SD_SNAPSHOT_CONTACTS a second file,
//     <path>.contacts.csv, lists the contact pairs (i,j with i < j).
//   * VTK (legacy format, BINARY, POLYDATA): the spheres as points (point i
//     = sphere i) with VERTICES cells, the contact pairs as LINES
//     (SD_SNAPSHOT_CONTACTS), the mesh at its current pose as POLYGONS over
//     extra points (SD_SNAPSHOT_MESH), and point data: radius, mass, id,
//     velocity, spin (zero on mesh points).  Big-endian float32 / int32 as
//     the format requires.
#include <charconv>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/stardust.h"
#include "sd_engine_impl.h"

namespace {

struct File {
    FILE* f = nullptr;
    explicit File(const std::string& path) : f(std::fopen(path.c_str(), "wb")) {}
    ~File() {
        if (f) std::fclose(f);
    }
    bool ok() const { return f != nullptr; }
    bool put(const std::string& s) { return std::fwrite(s.data(), 1, s.size(), f) == s.size(); }
    bool put(const void* p, size_t n) { return std::fwrite(p, 1, n, f) == n; }
    bool close() {
        const bool good = f && std::fflush(f) == 0 && !std::ferror(f);
        if (f) std::fclose(f);
        f = nullptr;
        return good;
    }
};

uint32_t be32(uint32_t v) {
    return (v >> 24) | ((v >> 8) & 0xff00u) | ((v << 8) & 0xff0000u) | (v << 24);
}

// big-endian copies of n 32-bit words
template <typename T>
std::vector<uint32_t> big_endian(const T* src, size_t n) {
    static_assert(sizeof(T) == 4, "32-bit words");
    std::vector<uint32_t> out(n);
    std::memcpy(out.data(), src, 4 * n);
    for (uint32_t& w : out) w = be32(w);
    return out;
}

// The shortest decimal text that reads back as exactly v (std::to_chars).
void put_float(std::string& out, float v) {
    char b[32];
    const auto r = std::to_chars(b, b + sizeof b, v);
    out.append(b, r.ptr);
}

}  // namespace

extern "C" sd_status sd_engine_write_snapshot(sd_engine* h, const char* path, int32_t format, uint32_t flags) {
    if (!h || !path) return sd_fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (format != SD_SNAPSHOT_CSV && format != SD_SNAPSHOT_VTK)
        return sd_fail(h, SD_ERR_INVALID_ARG, "format must be SD_SNAPSHOT_CSV or SD_SNAPSHOT_VTK");
    if (flags & ~(uint32_t)(SD_SNAPSHOT_CONTACTS | SD_SNAPSHOT_MESH)) return sd_fail(h, SD_ERR_INVALID_ARG, "unknown flags");
    sd_stats st{};
    if (sd_status s = sd_engine_stats(h, &st)) return s;
    const uint64_t n = st.n_spheres;
    std::vector<float> pos(4 * n), vel(4 * n), omg(4 * n);
    if (n) {
        if (sd_status s = sd_engine_get_state(h, SD_FIELD_POSITION, pos.data(), 16 * n)) return s;
        if (sd_status s = sd_engine_get_state(h, SD_FIELD_VELOCITY, vel.data(), 16 * n)) return s;
        if (sd_status s = sd_engine_get_state(h, SD_FIELD_OMEGA, omg.data(), 16 * n)) return s;
    }
    std::vector<uint64_t> pairs;
    if (flags & SD_SNAPSHOT_CONTACTS) {
        uint64_t np = 0;
        if (sd_status s = sd_engine_get_pairs(h, nullptr, 0, &np); s && s != SD_ERR_CAPACITY) return s;
        pairs.resize(np);
        if (np)
            if (sd_status s = sd_engine_get_pairs(h, pairs.data(), np, &np)) return s;
        pairs.resize(np);
    }
    std::vector<float> tri;  // world triangles at the current pose
    if (flags & SD_SNAPSHOT_MESH) {
        uint64_t nt = 0;
        float c[3];
        if (sd_status s = sd_engine_get_mesh(h, 0, nullptr, nullptr, c, &nt)) return s;
        if (nt) {
            std::vector<float> frame(9 * nt);
            if (sd_status s = sd_engine_get_mesh(h, nt, frame.data(), nullptr, c, &nt)) return s;
            float state[24];
            if (sd_status s = sd_engine_get_mesh_state(h, state)) return s;
            const float* R = state;  // mesh to world, row-major; centre at state[9..11]
            tri.resize(9 * nt);
            for (uint64_t v = 0; v < 3 * nt; ++v)
                for (int k = 0; k < 3; ++k)
                    tri[3 * v + k] = (R[3 * k] * frame[3 * v] + R[3 * k + 1] * frame[3 * v + 1]) +
                                     R[3 * k + 2] * frame[3 * v + 2] + state[9 + k];
        }
    }
    const std::string p(path);
    if (format == SD_SNAPSHOT_CSV) {
        File f(p);
        if (!f.ok()) return sd_fail(h, SD_ERR_IO, "cannot write " + p);
        std::string buf = "id,x,y,z,r,vx,vy,vz,m,wx,wy,wz\n";
        for (uint64_t i = 0; i < n; ++i) {
            buf += std::to_string(i);
            const float* row[3] = {&pos[4 * i], &vel[4 * i], &omg[4 * i]};
            for (int fld = 0; fld < 3; ++fld)
                for (int k = 0; k < (fld == 2 ? 3 : 4); ++k) {  // spin: no w lane
                    buf += ',';
                    put_float(buf, row[fld][k]);
                }
            buf += '\n';
            if (buf.size() > (1u << 20)) {
                if (!f.put(buf)) return sd_fail(h, SD_ERR_IO, "write failed: " + p);
                buf.clear();
            }
        }
        if (!f.put(buf) || !f.close()) return sd_fail(h, SD_ERR_IO, "write failed: " + p);
        if (flags & SD_SNAPSHOT_CONTACTS) {
            File g(p + ".contacts.csv");
            if (!g.ok()) return sd_fail(h, SD_ERR_IO, "cannot write " + p + ".contacts.csv");
            std::string b = "i,j\n";
            for (uint64_t q : pairs) b += std::to_string(q >> 32) + "," + std::to_string(q & 0xffffffffu) + "\n";
            if (!g.put(b) || !g.close()) return sd_fail(h, SD_ERR_IO, "write failed: " + p + ".contacts.csv");
        }
        return SD_OK;
    }
    // VTK legacy, binary polydata
    const uint64_t nt = tri.size() / 9, npts = n + 3 * nt;
    if (npts >= (1ull << 31) || pairs.size() >= (1ull << 30))
        return sd_fail(h, SD_ERR_CAPACITY, "snapshot too large for the VTK legacy format");
    File f(p);
    if (!f.ok()) return sd_fail(h, SD_ERR_IO, "cannot write " + p);
    bool good = f.put("# vtk DataFile Version 3.0\nstardust-gb300 snapshot, step " + std::to_string(st.steps) +
                      "\nBINARY\nDATASET POLYDATA\nPOINTS " + std::to_string(npts) + " float\n");
    {
        std::vector<float> xyz(3 * npts);
        for (uint64_t i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) xyz[3 * i + k] = pos[4 * i + k];
        std::memcpy(xyz.data() + 3 * n, tri.data(), 4 * tri.size());
        const auto w = big_endian(xyz.data(), xyz.size());
        good = good && f.put(w.data(), 4 * w.size());
    }
    auto cells = [&](const char* kind, uint64_t ncell, uint64_t per, auto&& fill) {
        std::vector<int32_t> c(ncell * (per + 1));
        for (uint64_t i = 0; i < ncell; ++i) {
            c[i * (per + 1)] = (int32_t)per;
            fill(i, &c[i * (per + 1) + 1]);
        }
        const auto w = big_endian(c.data(), c.size());
        return f.put(std::string("\n") + kind + " " + std::to_string(ncell) + " " + std::to_string(c.size()) + "\n") &&
               f.put(w.data(), 4 * w.size());
    };
    good = good && cells("VERTICES", n, 1, [](uint64_t i, int32_t* o) { o[0] = (int32_t)i; });
    if (flags & SD_SNAPSHOT_CONTACTS)
        good = good && cells("LINES", pairs.size(), 2, [&](uint64_t i, int32_t* o) {
                   o[0] = (int32_t)(pairs[i] >> 32);
                   o[1] = (int32_t)(pairs[i] & 0xffffffffu);
               });
    if (nt)
        good = good && cells("POLYGONS", nt, 3, [&](uint64_t i, int32_t* o) {
                   for (int k = 0; k < 3; ++k) o[k] = (int32_t)(n + 3 * i + k);
               });
    auto scalars = [&](const char* name, const char* type, const std::vector<uint32_t>& words) {
        const auto w = big_endian(words.data(), words.size());
        return f.put(std::string("\nSCALARS ") + name + " " + type + " 1\nLOOKUP_TABLE default\n") &&
               f.put(w.data(), 4 * w.size());
    };
    auto vectors = [&](const char* name, const std::vector<float>& src4) {
        std::vector<float> v(3 * npts, 0.0f);
        for (uint64_t i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) v[3 * i + k] = src4[4 * i + k];
        const auto w = big_endian(v.data(), v.size());
        return f.put(std::string("\nVECTORS ") + name + " float\n") && f.put(w.data(), 4 * w.size());
    };
    std::vector<uint32_t> rad(npts, 0), mass(npts, 0), ids(npts);
    for (uint64_t i = 0; i < n; ++i) {
        std::memcpy(&rad[i], &pos[4 * i + 3], 4);
        std::memcpy(&mass[i], &vel[4 * i + 3], 4);
    }
    for (uint64_t i = 0; i < npts; ++i) ids[i] = i < n ? (uint32_t)i : 0xffffffffu;  // -1 on mesh points
    good = good && f.put("\nPOINT_DATA " + std::to_string(npts)) && scalars("radius", "float", rad) &&
           scalars("mass", "float", mass) && scalars("id", "int", ids) && vectors("velocity", vel) &&
           vectors("spin", omg) && f.put("\n");
    if (!good || !f.close()) return sd_fail(h, SD_ERR_IO, "write failed: " + p);
    return SD_OK;
}
