// rt_obj.cpp -- Wavefront OBJ meshes as build input (include/rtcore_scene.h).
//
// The reference sample hard-codes its vertex and index arrays
// (vulkan-raytraced-triangle/main.cpp:676-682) and leaves loading a mesh from
// an OBJ file as an exercise (vulkan-raytraced-triangle/README.md:217-218).
// This loader produces exactly the arrays rt_build_blas takes: FP32 xyz
// vertices and uint32 triangle indices, plus a material index per triangle
// from the `usemtl` statements.
//
// Accepted: `v x y z [w ...]` (the first three numbers), `f` with three or more
// vertex references of the forms a, a/t, a//n, a/t/n (1-based, or negative =
// relative to the vertices read so far), split into a triangle fan
// (a0, ai, ai+1); `usemtl name`.  Other statements (vt, vn, o, g, s, mtllib,
// l, p, ...) are skipped.  Numbers are parsed with std::from_chars, which
// rounds correctly and does not depend on the C locale.
#include <charconv>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <system_error>
#include <vector>

#include "../../include/rtcore_scene.h"

namespace {

struct ObjMesh {
    std::vector<float> v;
    std::vector<uint32_t> idx;
    std::vector<uint32_t> mat;
    uint32_t n_materials = 0;
};

bool read_file(const char *path, std::string &out) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) out.append(buf, n);
    const bool ok = !std::ferror(f);
    std::fclose(f);
    return ok;
}

inline bool blank(char c) { return c == ' ' || c == '\t' || c == '\r'; }

// Splits [p, e) at blanks into views.
void split(const char *p, const char *e, std::vector<std::pair<const char *, const char *>> &out) {
    out.clear();
    while (p < e) {
        while (p < e && blank(*p)) ++p;
        const char *s = p;
        while (p < e && !blank(*p)) ++p;
        if (p > s) out.emplace_back(s, p);
    }
}

bool parse_float(const char *s, const char *e, float &x) {
    if (s < e && *s == '+') ++s;
    auto r = std::from_chars(s, e, x);
    return r.ec == std::errc() && r.ptr == e;
}

// The vertex index of one face reference ("a", "a/t", "a//n", "a/t/n"):
// 0-based, possibly not yet checked against the final vertex count.
bool parse_ref(const char *s, const char *e, uint64_t n_vertices_so_far, int64_t &out) {
    const char *slash = static_cast<const char *>(std::memchr(s, '/', (size_t)(e - s)));
    const char *end = slash ? slash : e;
    if (s < end && *s == '+') ++s;
    long long a = 0;
    auto r = std::from_chars(s, end, a);
    if (r.ec != std::errc() || r.ptr != end || a == 0) return false;
    out = a > 0 ? (int64_t)a - 1 : (int64_t)n_vertices_so_far + (int64_t)a;
    return out >= 0;
}

rt_status parse(const char *path, ObjMesh &m) {
    if (!path) return RT_ERR_INVALID_ARG;
    std::string text;
    if (!read_file(path, text)) return RT_ERR_INVALID_ARG;
    std::map<std::string, uint32_t> names;
    std::string current;  // faces before any usemtl use the unnamed material
    std::vector<std::pair<const char *, const char *>> tok;
    std::vector<int64_t> face;
    const char *p = text.data(), *end = text.data() + text.size();
    while (p < end) {
        const char *nl = static_cast<const char *>(std::memchr(p, '\n', (size_t)(end - p)));
        const char *le = nl ? nl : end;
        const char *hash = static_cast<const char *>(std::memchr(p, '#', (size_t)(le - p)));
        split(p, hash ? hash : le, tok);
        p = nl ? nl + 1 : end;
        if (tok.empty()) continue;
        const std::string kw(tok[0].first, tok[0].second);
        if (kw == "v") {
            if (tok.size() < 4) return RT_ERR_INVALID_ARG;
            for (int k = 1; k <= 3; ++k) {
                float x;
                if (!parse_float(tok[k].first, tok[k].second, x)) return RT_ERR_INVALID_ARG;
                m.v.push_back(x);
            }
            if (m.v.size() / 3 > 0xffffffffull) return RT_ERR_UNSUPPORTED;
        } else if (kw == "f") {
            if (tok.size() < 4) return RT_ERR_INVALID_ARG;
            face.clear();
            for (size_t k = 1; k < tok.size(); ++k) {
                int64_t a;
                if (!parse_ref(tok[k].first, tok[k].second, m.v.size() / 3, a)) return RT_ERR_INVALID_ARG;
                face.push_back(a);
            }
            auto it = names.find(current);
            if (it == names.end()) it = names.emplace(current, (uint32_t)names.size()).first;
            for (size_t k = 1; k + 1 < face.size(); ++k) {
                if (face[0] > 0xfffffffell || face[k] > 0xfffffffell || face[k + 1] > 0xfffffffell)
                    return RT_ERR_INVALID_ARG;
                m.idx.push_back((uint32_t)face[0]);
                m.idx.push_back((uint32_t)face[k]);
                m.idx.push_back((uint32_t)face[k + 1]);
                m.mat.push_back(it->second);
            }
            if (m.mat.size() > 0xffffffffull) return RT_ERR_UNSUPPORTED;
        } else if (kw == "usemtl") {
            current = tok.size() > 1 ? std::string(tok[1].first, tok.back().second) : std::string();
        }
    }
    const uint64_t nv = m.v.size() / 3;
    for (uint32_t i : m.idx)
        if (i >= nv) return RT_ERR_INVALID_ARG;  // a positive reference beyond the last vertex
    m.n_materials = (uint32_t)names.size();
    return RT_OK;
}

}  // namespace

extern "C" rt_status rt_obj_counts(const char *path, uint32_t *n_vertices, uint32_t *n_tris, uint32_t *n_materials) {
    if (!n_vertices || !n_tris) return RT_ERR_INVALID_ARG;
    ObjMesh m;
    const rt_status rc = parse(path, m);
    if (rc != RT_OK) return rc;
    *n_vertices = (uint32_t)(m.v.size() / 3);
    *n_tris = (uint32_t)m.mat.size();
    if (n_materials) *n_materials = m.n_materials;
    return RT_OK;
}

extern "C" rt_status rt_obj_load(const char *path, float *vertices, uint32_t *indices, uint32_t *tri_material) {
    if (!vertices || !indices) return RT_ERR_INVALID_ARG;
    ObjMesh m;
    const rt_status rc = parse(path, m);
    if (rc != RT_OK) return rc;
    if (!m.v.empty()) std::memcpy(vertices, m.v.data(), m.v.size() * sizeof(float));
    if (!m.idx.empty()) std::memcpy(indices, m.idx.data(), m.idx.size() * sizeof(uint32_t));
    if (tri_material && !m.mat.empty()) std::memcpy(tri_material, m.mat.data(), m.mat.size() * sizeof(uint32_t));
    return RT_OK;
}
