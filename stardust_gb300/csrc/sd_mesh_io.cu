// sd_mesh_io.cu -- mesh entities from STL files (host code).
//
// The reference's DEMMesh (src/engine/entities/entity.hpp:64-93) reads an
// STL file through the third-party stl_reader header
// (src/IO/mesh_loader.cpp:9-45), keeps a position and a quaternion, and
// computes a circumscribed sphere per triangle (entity.cpp:75-120); its
// engine counts the triangles (entity_handler.cpp:110-115) but no kernel ever
// reads them, and the JSON "mesh" branch is commented out
// (engine.cpp:64-108).  Here an STL mesh becomes a wall of the step:
//
//   * sd_stl_read: ASCII or binary STL -> a triangle soup (9 floats per
//     triangle).  Binary when the file is exactly 84 + 50 * count bytes
//     (count = the u32 at byte 80), which also covers binary files whose
//     80-byte header starts with "solid"; otherwise ASCII (facets of exactly
//     three "vertex x y z" lines, any number of solids).  The stored facet
//     normals are not used: orientation comes from the vertices.
//   * sd_mesh_patches: groups triangles into smooth faces ("patches": per
//     sphere, only the deepest contact of each patch acts).  Two triangles
//     that share an edge (both endpoints bit-identical) belong to one patch
//     when their normals, taken as unoriented lines (STL winding is often
//     inconsistent), differ by less than angle_deg; patches are numbered
//     by their first triangle.  A tessellated cylinder wall is one patch, its
//     flat caps two more, and a box has six.
//   * sd_engine_add_mesh_stl: read, place with a position and a unit
//     quaternion (v' = R(q) v + position, in double, rounded once), group,
//     and add with sd_engine_add_mesh (static or rotating about an axis).
//
// No bounding spheres per triangle: candidate triangles come from the
// mesh's static grid (sd_engine_add_mesh).
#include <algorithm>
#include <array>
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <map>
#include <numeric>
#include <string>
#include <string_view>
#include <utility>
#include <vector>

#include "sd_engine_impl.h"

namespace sd {
namespace {

bool read_file(const std::string& path, std::string* out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    f.seekg(0, std::ios::end);
    const std::streamoff size = f.tellg();
    if (size < 0) return false;
    out->resize((size_t)size);
    f.seekg(0, std::ios::beg);
    if (size) f.read(&(*out)[0], size);
    return (bool)f;
}

bool parse_binary(const std::string& d, std::vector<float>* tri9) {
    uint32_t count = 0;
    std::memcpy(&count, d.data() + 80, 4);  // little-endian on every supported host
    if (d.size() != 84 + 50 * (uint64_t)count) return false;
    tri9->resize(9 * (size_t)count);
    for (uint32_t t = 0; t < count; ++t)
        std::memcpy(tri9->data() + 9 * (size_t)t, d.data() + 84 + 50 * (size_t)t + 12, 36);
    return true;
}

// Whitespace-separated tokens of an ASCII STL.
struct Tokens {
    const char* p;
    const char* end;
    bool next(std::string_view* tok) {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n')) ++p;
        if (p >= end) return false;
        const char* s = p;
        while (p < end && !(*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n')) ++p;
        *tok = std::string_view(s, (size_t)(p - s));
        return true;
    }
    void skip_line() {
        while (p < end && *p != '\n') ++p;
    }
};

bool parse_float(std::string_view s, float* v) {
    const auto r = std::from_chars(s.data(), s.data() + s.size(), *v);
    return r.ec == std::errc() && r.ptr == s.data() + s.size() && std::isfinite(*v);
}

bool parse_ascii(const std::string& d, std::vector<float>* tri9, std::string* err) {
    Tokens tk{d.data(), d.data() + d.size()};
    std::string_view tok;
    size_t facets = 0;
    bool any_solid = false;
    {
        Tokens first = tk;
        if (!first.next(&tok) || tok != "solid") {
            *err = "not an STL file (neither a binary STL of matching size nor ASCII starting with \"solid\")";
            return false;
        }
    }
    while (tk.next(&tok)) {
        if (tok == "solid") {  // the rest of the line is the solid's name
            any_solid = true;
            tk.skip_line();
        } else if (tok == "endsolid") {
            tk.skip_line();
        } else if (tok == "facet") {
            int nv = 0;
            float v[9];
            while (true) {
                if (!tk.next(&tok)) {
                    *err = "ASCII STL ends inside facet " + std::to_string(facets);
                    return false;
                }
                if (tok == "endfacet") break;
                if (tok == "vertex") {
                    if (nv == 3) {
                        *err = "ASCII STL facet " + std::to_string(facets) + " has more than three vertices";
                        return false;
                    }
                    for (int k = 0; k < 3; ++k) {
                        if (!tk.next(&tok) || !parse_float(tok, &v[3 * nv + k])) {
                            *err = "ASCII STL facet " + std::to_string(facets) + ": bad vertex coordinate";
                            return false;
                        }
                    }
                    ++nv;
                }
                // "normal nx ny nz", "outer loop", "endloop": not needed
            }
            if (nv != 3) {
                *err = "ASCII STL facet " + std::to_string(facets) + " has " + std::to_string(nv) + " vertices";
                return false;
            }
            tri9->insert(tri9->end(), v, v + 9);
            ++facets;
        } else {
            *err = "ASCII STL: unexpected token \"" + std::string(tok.substr(0, 32)) + "\"";
            return false;
        }
    }
    if (!any_solid) {
        *err = "not an STL file (neither a binary STL of matching size nor ASCII \"solid\")";
        return false;
    }
    return true;
}

}  // namespace

bool read_stl(const std::string& path, std::vector<float>* tri9, std::string* err) {
    tri9->clear();
    std::string d;
    if (!read_file(path, &d)) {
        *err = "cannot read " + path;
        return false;
    }
    if (d.size() >= 84 && parse_binary(d, tri9)) return true;
    tri9->clear();
    if (!parse_ascii(d, tri9, err)) {
        tri9->clear();
        return false;
    }
    for (float v : *tri9)
        if (!std::isfinite(v)) {
            *err = "STL vertex not finite";
            tri9->clear();
            return false;
        }
    return true;
}

void smooth_patches(uint64_t n, const float* tri9, float angle_deg, int32_t* patch) {
    // unit normals from the vertices, in double (zero for a degenerate triangle)
    std::vector<double> nrm(3 * n);
    for (uint64_t t = 0; t < n; ++t) {
        const float* v = tri9 + 9 * t;
        const double e1[3] = {(double)v[3] - v[0], (double)v[4] - v[1], (double)v[5] - v[2]};
        const double e2[3] = {(double)v[6] - v[0], (double)v[7] - v[1], (double)v[8] - v[2]};
        double c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        const double l = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        for (int k = 0; k < 3; ++k) nrm[3 * t + k] = l > 0.0 ? c[k] / l : 0.0;
    }
    constexpr double kPi = 3.14159265358979323846;
    const double cos_max = std::cos((double)angle_deg * kPi / 180.0);
    // union-find over triangles, joined across shared edges
    std::vector<uint64_t> parent(n);
    std::iota(parent.begin(), parent.end(), 0);
    auto find = [&](uint64_t x) {
        while (parent[x] != x) x = parent[x] = parent[parent[x]];
        return x;
    };
    // an edge: its two endpoints' bit patterns, ordered
    using Vtx = std::array<uint32_t, 3>;
    std::map<std::pair<Vtx, Vtx>, std::vector<uint64_t>> edges;
    for (uint64_t t = 0; t < n; ++t) {
        Vtx p[3];
        for (int k = 0; k < 3; ++k) std::memcpy(p[k].data(), tri9 + 9 * t + 3 * k, 12);
        for (int k = 0; k < 3; ++k) {
            Vtx a = p[k], b = p[(k + 1) % 3];
            if (b < a) std::swap(a, b);
            if (a == b) continue;
            edges[{a, b}].push_back(t);
        }
    }
    for (auto& kv : edges) {
        const auto& ts = kv.second;
        for (size_t i = 0; i < ts.size(); ++i)
            for (size_t j = i + 1; j < ts.size(); ++j) {
                const double* a = &nrm[3 * ts[i]];
                const double* b = &nrm[3 * ts[j]];
                const double c = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
                // the crease-angle rule on unsigned normals: STL files are often
                // wound inconsistently, and a patch only merges contacts
                if (std::fabs(c) > cos_max && (a[0] != 0.0 || a[1] != 0.0 || a[2] != 0.0) &&
                    (b[0] != 0.0 || b[1] != 0.0 || b[2] != 0.0)) {
                    const uint64_t ra = find(ts[i]), rb = find(ts[j]);
                    if (ra != rb) parent[std::max(ra, rb)] = std::min(ra, rb);
                }
            }
    }
    // number the patches by their first triangle
    std::vector<int64_t> id(n, -1);
    int32_t next = 0;
    for (uint64_t t = 0; t < n; ++t) {
        const uint64_t r = find(t);
        if (id[r] < 0) id[r] = next++;
        patch[t] = (int32_t)id[r];
    }
}

}  // namespace sd

extern "C" sd_status sd_stl_read(const char* path, uint64_t cap, float* tri9, uint64_t* n_tris) {
    if (!path || !n_tris) return sd_fail(nullptr, SD_ERR_INVALID_ARG, "NULL argument");
    std::vector<float> t;
    std::string err;
    if (!sd::read_stl(path, &t, &err)) return sd_fail(nullptr, SD_ERR_IO, err);
    *n_tris = t.size() / 9;
    if (tri9) {
        if (cap < *n_tris)
            return sd_fail(nullptr, SD_ERR_CAPACITY,
                           "STL has " + std::to_string(*n_tris) + " triangles, capacity " + std::to_string(cap));
        std::copy(t.begin(), t.end(), tri9);
    }
    return SD_OK;
}

extern "C" sd_status sd_mesh_patches(uint64_t n_tris, const float* tri9, float angle_deg, int32_t* patch) {
    if ((n_tris && (!tri9 || !patch))) return sd_fail(nullptr, SD_ERR_INVALID_ARG, "NULL argument");
    if (!(angle_deg >= 0.0f && angle_deg <= 180.0f)) return sd_fail(nullptr, SD_ERR_INVALID_ARG, "angle_deg must be in [0, 180]");
    sd::smooth_patches(n_tris, tri9, angle_deg, patch);
    return SD_OK;
}

extern "C" sd_status sd_engine_add_mesh_stl(sd_engine* h, const char* path, const float position[3],
                                            const float quat[4], const float centre[3], const float axis[3],
                                            float omega, float patch_angle_deg) {
    if (!h || !path) return sd_fail(h, SD_ERR_INVALID_ARG, "NULL argument");
    if (!(patch_angle_deg >= 0.0f && patch_angle_deg <= 180.0f))
        return sd_fail(h, SD_ERR_INVALID_ARG, "patch_angle_deg must be in [0, 180]");
    std::vector<float> t;
    std::string err;
    if (!sd::read_stl(path, &t, &err)) return sd_fail(h, SD_ERR_IO, err);
    const uint64_t n = t.size() / 9;
    if (n == 0) return sd_fail(h, SD_ERR_INVALID_ARG, std::string(path) + " holds no triangles");
    double q[4] = {1.0, 0.0, 0.0, 0.0}, p[3] = {0.0, 0.0, 0.0};
    if (quat)
        for (int k = 0; k < 4; ++k) q[k] = quat[k];
    if (position)
        for (int k = 0; k < 3; ++k) p[k] = position[k];
    const double qn = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    if (!(qn > 0.0) || !std::isfinite(qn)) return sd_fail(h, SD_ERR_INVALID_ARG, "quaternion must be non-zero");
    for (double& x : q) x /= qn;
    const bool identity = q[0] == 1.0 && p[0] == 0.0 && p[1] == 0.0 && p[2] == 0.0;
    if (!identity) {
        const double s = q[0], x = q[1], y = q[2], z = q[3];
        const double R[9] = {1 - 2 * (y * y + z * z), 2 * (x * y - s * z),     2 * (x * z + s * y),
                             2 * (x * y + s * z),     1 - 2 * (x * x + z * z), 2 * (y * z - s * x),
                             2 * (x * z - s * y),     2 * (y * z + s * x),     1 - 2 * (x * x + y * y)};
        for (uint64_t v = 0; v < 3 * n; ++v) {
            const double a = t[3 * v], b = t[3 * v + 1], c = t[3 * v + 2];
            for (int k = 0; k < 3; ++k) t[3 * v + k] = (float)(R[3 * k] * a + R[3 * k + 1] * b + R[3 * k + 2] * c + p[k]);
        }
    }
    std::vector<int32_t> patch(n);
    sd::smooth_patches(n, t.data(), patch_angle_deg, patch.data());
    const float zero[3] = {0.0f, 0.0f, 0.0f};
    if (n >= (1u << 26)) return sd_fail(h, SD_ERR_CAPACITY, "mesh has more than 2^26 triangles");
    return sd_engine_add_mesh(h, (uint32_t)n, t.data(), patch.data(), centre ? centre : zero, axis, omega);
}
