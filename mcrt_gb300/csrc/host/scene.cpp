// scene.cpp — the reference's Scene/Material/Camera/YAML API on the host:
// load_scene_from_str / load_scene_from_yaml (src/scene.rs:640-999), the OBJ
// loader (src/mesh.rs:474-642), compute_camera (src/camera.rs:76-127) and the
// environment map (src/texture.rs:124-220).  The reference runs all of these on
// the CPU; so does this file.  Compiled with -ffp-contract=off: the float
// sequences are the ones written (and the reference's), identical on x86-64
// and aarch64.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "../fmath.h"
#include "mcrt_cuda.h"
#include "scene_internal.h"
#include "yaml.h"

using mcrt::fm_sincos;

struct mcrt_loaded_scene {
    mcrt_host::LoadedScene s;
};

namespace mcrt_host {

namespace {

constexpr uint32_t kBackfaceCull = 1u << 31;    // scene.rs:709-718
constexpr float kPiF = 3.14159265358979323846f;

struct SceneErr {
    mcrt_status code;
    std::string msg;
};

bool read_file(const std::string &path, std::string *out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    *out = ss.str();
    return true;
}

// ---- typed access to YAML nodes (serde semantics: unknown keys are ignored)
bool as_f32(const YNode *n, float *out) {
    if (!n || n->kind != YNode::Scalar || n->quoted) return false;
    const std::string &s = n->scalar;
    if (s == ".inf" || s == "+.inf") { *out = INFINITY; return true; }
    if (s == "-.inf") { *out = -INFINITY; return true; }
    if (s == ".nan") { *out = NAN; return true; }
    char *end = nullptr;
    double v = strtod(s.c_str(), &end);
    if (end == s.c_str() || *end != '\0') return false;
    if (s.find('x') != std::string::npos || s.find('X') != std::string::npos) return false;
    *out = (float)v;
    return true;
}
bool as_u32(const YNode *n, uint32_t *out) {
    if (!n || n->kind != YNode::Scalar || n->quoted) return false;
    const std::string &s = n->scalar;
    if (s.empty() || s[0] == '-') return false;
    char *end = nullptr;
    unsigned long long v = strtoull(s.c_str(), &end, 10);
    if (*end != '\0' || v > 0xffffffffull) return false;
    *out = (uint32_t)v;
    return true;
}
bool as_bool(const YNode *n, bool *out) {
    if (!n || n->kind != YNode::Scalar || n->quoted) return false;
    if (n->scalar == "true" || n->scalar == "True" || n->scalar == "TRUE") { *out = true; return true; }
    if (n->scalar == "false" || n->scalar == "False" || n->scalar == "FALSE") { *out = false; return true; }
    return false;
}
bool as_str(const YNode *n, std::string *out) {
    if (!n || n->kind != YNode::Scalar) return false;
    *out = n->scalar;
    return true;
}
template <int N> bool as_vec(const YNode *n, float (&out)[N]) {
    if (!n || n->kind != YNode::Seq || (int)n->seq.size() != N) return false;
    for (int i = 0; i < N; ++i)
        if (!as_f32(&n->seq[i], &out[i])) return false;
    return true;
}

SceneErr perr(const std::string &src, const YNode *n, const std::string &m) {
    std::string where = n ? (" at line " + std::to_string(n->line)) : "";
    return {MCRT_ERR_PARSE, "parse error: failed to parse '" + src + "': " + m + where};
}

// MaterialDesc (scene.rs:103-125) -> GpuMaterial (material_desc_to_gpu, scene.rs:354-381)
bool material_from_yaml(const YNode *n, const std::string &src, mcrt_gpu_material *out, SceneErr *e) {
    if (!n || n->kind != YNode::Map) { *e = perr(src, n, "material must be a mapping"); return false; }
    std::string kind;
    if (!as_str(n->get("type"), &kind)) { *e = perr(src, n, "material: missing field `type`"); return false; }
    float albedo[3] = {1.0f, 1.0f, 1.0f};
    if (const YNode *a = n->get("albedo"))
        if (a->kind != YNode::Null && !as_vec<3>(a, albedo)) { *e = perr(src, a, "albedo: expected [f32; 3]"); return false; }
    auto opt_f = [&](const char *key, float def, float *v) {
        *v = def;
        const YNode *x = n->get(key);
        if (!x || x->kind == YNode::Null) return true;
        if (!as_f32(x, v)) { *e = perr(src, x, std::string(key) + ": expected f32"); return false; }
        return true;
    };
    uint32_t layer = 0;
    if (const YNode *t = n->get("texture_layer"))
        if (!as_u32(t, &layer)) { *e = perr(src, t, "texture_layer: expected u32"); return false; }
    std::memset(out, 0, sizeof(*out));
    float f = 0.0f;
    if (kind == "lambertian") {
        out->type_pad[0] = MCRT_MAT_LAMBERTIAN; out->type_pad[1] = layer;
        out->albedo_fuzz[0] = albedo[0]; out->albedo_fuzz[1] = albedo[1]; out->albedo_fuzz[2] = albedo[2];
        out->ior_pad[0] = 1.0f;
    } else if (kind == "metal") {
        if (!opt_f("fuzz", 0.0f, &f)) return false;
        out->type_pad[0] = MCRT_MAT_METAL; out->type_pad[1] = layer;
        out->albedo_fuzz[0] = albedo[0]; out->albedo_fuzz[1] = albedo[1]; out->albedo_fuzz[2] = albedo[2];
        out->albedo_fuzz[3] = f;
        out->ior_pad[0] = 1.0f;
    } else if (kind == "dielectric") {
        if (!opt_f("ior", 1.5f, &f)) return false;
        out->type_pad[0] = MCRT_MAT_DIELECTRIC;
        out->albedo_fuzz[0] = 1.0f; out->albedo_fuzz[1] = 1.0f; out->albedo_fuzz[2] = 1.0f;
        out->ior_pad[0] = f;
    } else if (kind == "emissive") {
        if (!opt_f("emission_strength", 1.0f, &f)) return false;
        out->type_pad[0] = MCRT_MAT_EMISSIVE;
        out->albedo_fuzz[0] = albedo[0]; out->albedo_fuzz[1] = albedo[1]; out->albedo_fuzz[2] = albedo[2];
        out->ior_pad[0] = f;
    } else if (kind == "ggx") {   // extension: GGX conductor, roughness in albedo_fuzz.w
        if (!opt_f("roughness", 0.5f, &f)) return false;
        out->type_pad[0] = MCRT_MAT_GGX; out->type_pad[1] = layer;
        out->albedo_fuzz[0] = albedo[0]; out->albedo_fuzz[1] = albedo[1]; out->albedo_fuzz[2] = albedo[2];
        out->albedo_fuzz[3] = f;
        out->ior_pad[0] = 1.0f;
    } else {
        *e = perr(src, n->get("type"), "unknown variant `" + kind + "`");
        return false;
    }
    return true;
}

// ---- rotation helpers (scene.rs:386-408)
inline float to_rad(float deg) { return deg * kPiF / 180.0f; }
struct M3 { float m[3][3]; };
M3 euler_to_mat3(float rx, float ry, float rz) {
    float sx, cx, sy, cy, sz, cz;
    fm_sincos(to_rad(rx), &sx, &cx);
    fm_sincos(to_rad(ry), &sy, &cy);
    fm_sincos(to_rad(rz), &sz, &cz);
    M3 r;
    r.m[0][0] = cy * cz; r.m[0][1] = sx * sy * cz - cx * sz; r.m[0][2] = cx * sy * cz + sx * sz;
    r.m[1][0] = cy * sz; r.m[1][1] = sx * sy * sz + cx * cz; r.m[1][2] = cx * sy * sz - sx * cz;
    r.m[2][0] = -sy;     r.m[2][1] = sx * cy;                r.m[2][2] = cx * cy;
    return r;
}
inline void rot3(const M3 &m, const float v[3], float out[3]) {
    float r[3];
    for (int i = 0; i < 3; ++i) r[i] = m.m[i][0] * v[0] + m.m[i][1] * v[1] + m.m[i][2] * v[2];
    for (int i = 0; i < 3; ++i) out[i] = r[i];
}

// TransformDesc (scene.rs:438-495)
struct Transform {
    bool has_t = false, has_r = false, has_s = false;
    float t[3] = {0, 0, 0}, r[3] = {0, 0, 0}, s = 1.0f;
    bool identity() const { return !has_t && !has_r && !has_s; }
    void apply_point(const float p[3], float out[3]) const {
        float q[3] = {p[0] * s, p[1] * s, p[2] * s};
        if (has_r) rot3(euler_to_mat3(r[0], r[1], r[2]), q, q);
        out[0] = q[0] + t[0]; out[1] = q[1] + t[1]; out[2] = q[2] + t[2];
    }
    void apply_normal(const float n[3], float out[3]) const {
        if (has_r) rot3(euler_to_mat3(r[0], r[1], r[2]), n, out);
        else { out[0] = n[0]; out[1] = n[1]; out[2] = n[2]; }
    }
};
bool transform_from_yaml(const YNode *n, const std::string &src, Transform *t, SceneErr *e) {
    if (!n || n->kind == YNode::Null) return true;
    if (n->kind != YNode::Map) { *e = perr(src, n, "transform must be a mapping"); return false; }
    if (const YNode *x = n->get("translate"); x && x->kind != YNode::Null) {
        if (!as_vec<3>(x, t->t)) { *e = perr(src, x, "translate: expected [f32; 3]"); return false; }
        t->has_t = true;
    }
    if (const YNode *x = n->get("rotate"); x && x->kind != YNode::Null) {
        if (!as_vec<3>(x, t->r)) { *e = perr(src, x, "rotate: expected [f32; 3]"); return false; }
        t->has_r = true;
    }
    if (const YNode *x = n->get("scale"); x && x->kind != YNode::Null) {
        if (!as_f32(x, &t->s)) { *e = perr(src, x, "scale: expected f32"); return false; }
        t->has_s = true;
    }
    return true;
}

// ---- plane tessellation (scene.rs:497-590)
inline void pcross(const float a[3], const float b[3], float o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}
inline void pnormalize(const float v[3], float o[3]) {
    float len = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (len > 1e-9f) { o[0] = v[0] / len; o[1] = v[1] / len; o[2] = v[2] / len; }
    else { o[0] = 0.0f; o[1] = 1.0f; o[2] = 0.0f; }
}
void push_quad_face(const float c[3], const float n[3], float hw, float hh, uint32_t mat,
                    std::vector<mcrt_gpu_vertex> &verts, std::vector<mcrt_gpu_triangle> &tris) {
    float a0 = fabsf(n[0]), a1 = fabsf(n[1]), a2 = fabsf(n[2]);
    float helper[3] = {0, 0, 0};
    if (a0 <= a1 && a0 <= a2) helper[0] = 1.0f;
    else if (a1 <= a2) helper[1] = 1.0f;
    else helper[2] = 1.0f;
    float tmp[3], t1[3], t2[3];
    pcross(helper, n, tmp);
    pnormalize(tmp, t1);
    pcross(n, t1, t2);
    auto corner = [&](float s1, float s2, float out[4]) {
        for (int i = 0; i < 3; ++i) out[i] = c[i] + t1[i] * s1 * hw + t2[i] * s2 * hh;
        out[3] = 1.0f;
    };
    const float sgn[4][2] = {{-1.0f, -1.0f}, {1.0f, -1.0f}, {1.0f, 1.0f}, {-1.0f, 1.0f}};
    const float uvs[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
    uint32_t base = (uint32_t)verts.size();
    for (int k = 0; k < 4; ++k) {
        mcrt_gpu_vertex v{};
        corner(sgn[k][0], sgn[k][1], v.position);
        v.normal[0] = n[0]; v.normal[1] = n[1]; v.normal[2] = n[2]; v.normal[3] = 0.0f;
        v.uv[0] = uvs[k][0]; v.uv[1] = uvs[k][1];
        verts.push_back(v);
    }
    tris.push_back({{base, base + 1, base + 2}, mat});
    tris.push_back({{base, base + 2, base + 3}, mat});
}

}  // namespace

// ---- OBJ loader (mesh.rs:474-642), with the Rust string rules it relies on
namespace {
inline void normalize3_obj(const float v[3], float o[3]) {     // mesh.rs:663-670
    float len = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (len < 1e-8f) { o[0] = 0.0f; o[1] = 1.0f; o[2] = 0.0f; return; }
    o[0] = v[0] / len; o[1] = v[1] / len; o[2] = v[2] / len;
}
// String::from_utf8: the first invalid sequence and its length (0: the text
// ends inside it), as core::str::run_utf8_validation reports them.
bool utf8_valid(const std::string &t, size_t *at, int *error_len) {
    const size_t n = t.size();
    auto byte = [&](size_t i) { return (unsigned char)t[i]; };
    auto cont = [](unsigned char b) { return (b & 0xC0) == 0x80; };
    for (size_t i = 0; i < n;) {
        const unsigned char b = byte(i);
        if (b < 0x80) { ++i; continue; }
        *at = i;
        const int w = (b >= 0xC2 && b <= 0xDF) ? 2 : (b >= 0xE0 && b <= 0xEF) ? 3 : (b >= 0xF0 && b <= 0xF4) ? 4 : 0;
        if (w == 0) { *error_len = 1; return false; }
        if (i + 1 >= n) { *error_len = 0; return false; }
        const unsigned char b1 = byte(i + 1);
        const bool ok = w == 2   ? cont(b1)
                        : w == 3 ? (b == 0xE0 && b1 >= 0xA0 && b1 <= 0xBF) || (b >= 0xE1 && b <= 0xEC && cont(b1)) ||
                                       (b == 0xED && b1 >= 0x80 && b1 <= 0x9F) || (b >= 0xEE && cont(b1))
                                 : (b == 0xF0 && b1 >= 0x90 && b1 <= 0xBF) || (b >= 0xF1 && b <= 0xF3 && cont(b1)) ||
                                       (b == 0xF4 && b1 >= 0x80 && b1 <= 0x8F);
        if (!ok) { *error_len = 1; return false; }
        for (int k = 2; k < w; ++k) {
            if (i + k >= n) { *error_len = 0; return false; }
            if (!cont(byte(i + k))) { *error_len = k; return false; }
        }
        i += w;
    }
    return true;
}
// char::is_whitespace of the character that starts at s[i] (bytes), or 0.
int ws_len_at(const std::string &s, size_t i, size_t end) {
    const unsigned char c = s[i];
    auto at = [&](size_t k) { return i + k < end ? (unsigned char)s[i + k] : 0u; };
    if (c == ' ' || (c >= 0x09 && c <= 0x0D)) return 1;
    if (c == 0xC2 && (at(1) == 0x85 || at(1) == 0xA0)) return 2;
    if (c == 0xE1 && at(1) == 0x9A && at(2) == 0x80) return 3;
    if (c == 0xE2 && at(1) == 0x80 && i + 2 < end && (at(2) <= 0x8A || at(2) == 0xA8 || at(2) == 0xA9 || at(2) == 0xAF))
        return 3;
    if (c == 0xE2 && at(1) == 0x81 && at(2) == 0x9F) return 3;
    if (c == 0xE3 && at(1) == 0x80 && at(2) == 0x80) return 3;
    return 0;
}
// str::trim of s[b, e) (valid UTF-8).
void trim_range(const std::string &s, size_t *b, size_t *e) {
    int n;
    while (*b < *e && (n = ws_len_at(s, *b, *e)) > 0) *b += n;
    for (;;) {
        if (*e > *b && ws_len_at(s, *e - 1, *e) == 1) { *e -= 1; continue; }
        if (*e >= *b + 2 && ws_len_at(s, *e - 2, *e) == 2) { *e -= 2; continue; }
        if (*e >= *b + 3 && ws_len_at(s, *e - 3, *e) == 3) { *e -= 3; continue; }
        break;
    }
}
inline bool ascii_ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\x0C' || c == '\r'; }
std::vector<std::string> split_ascii_ws(const std::string &s, size_t b, size_t e) {   // str::split_ascii_whitespace
    std::vector<std::string> out;
    while (b < e) {
        while (b < e && ascii_ws(s[b])) ++b;
        size_t t = b;
        while (b < e && !ascii_ws(s[b])) ++b;
        if (b > t) out.push_back(s.substr(t, b - t));
    }
    return out;
}
// str::parse::<f32> (core::num::dec2flt grammar; strtof rounds correctly).
bool parse_f32_strict(const std::string &s, float *out) {
    size_t i = 0;
    bool neg = false;
    if (i < s.size() && (s[i] == '+' || s[i] == '-')) { neg = s[i] == '-'; ++i; }
    std::string body = s.substr(i);
    for (char &c : body) c = (char)((c >= 'A' && c <= 'Z') ? c - 'A' + 'a' : c);
    if (body == "inf" || body == "infinity") { *out = neg ? -INFINITY : INFINITY; return true; }
    if (body == "nan") {
        const uint32_t bits = neg ? 0xFFC00000u : 0x7FC00000u;
        std::memcpy(out, &bits, 4);
        return true;
    }
    size_t digits = 0;
    while (i < s.size() && s[i] >= '0' && s[i] <= '9') { ++i; ++digits; }
    if (i < s.size() && s[i] == '.')
        for (++i; i < s.size() && s[i] >= '0' && s[i] <= '9'; ++i) ++digits;
    if (digits == 0) return false;
    if (i < s.size() && (s[i] == 'e' || s[i] == 'E')) {
        ++i;
        if (i < s.size() && (s[i] == '+' || s[i] == '-')) ++i;
        size_t ed = 0;
        for (; i < s.size() && s[i] >= '0' && s[i] <= '9'; ++i) ++ed;
        if (ed == 0) return false;
    }
    if (i != s.size()) return false;
    *out = strtof(s.c_str(), nullptr);
    return true;
}
// str::parse::<i64>: optional sign, digits, no overflow.
bool parse_i64_strict(const std::string &s, long long *out) {
    size_t i = 0;
    bool neg = false;
    if (i < s.size() && (s[i] == '+' || s[i] == '-')) { neg = s[i] == '-'; ++i; }
    if (i == s.size()) return false;
    const unsigned long long lim = neg ? 9223372036854775808ull : 9223372036854775807ull;
    unsigned long long v = 0;
    for (; i < s.size(); ++i) {
        if (s[i] < '0' || s[i] > '9') return false;
        const unsigned d = (unsigned)(s[i] - '0');
        if (v > (lim - d) / 10) return false;
        v = v * 10 + d;
    }
    *out = neg ? (long long)(0ull - v) : (long long)v;
    return true;
}
std::vector<std::string> split_char(const std::string &s, char c) {
    std::vector<std::string> out;
    size_t b = 0;
    for (;;) {
        size_t e = s.find(c, b);
        out.push_back(s.substr(b, e == std::string::npos ? std::string::npos : e - b));
        if (e == std::string::npos) break;
        b = e + 1;
    }
    return out;
}
}  // namespace

bool load_obj_text(const std::string &content, uint32_t mat_idx, std::vector<mcrt_gpu_vertex> *verts_out,
                   std::vector<mcrt_gpu_triangle> *tris_out, std::string *err) {
    size_t bad_at = 0;
    int bad_len = 0;
    if (!utf8_valid(content, &bad_at, &bad_len)) {                              // mesh.rs:477-478
        *err = std::string(" is not valid UTF-8: ") +
               (bad_len ? "invalid utf-8 sequence of " + std::to_string(bad_len) + " bytes from index "
                        : std::string("incomplete utf-8 byte sequence from index ")) +
               std::to_string(bad_at);
        return false;
    }
    std::vector<float> pos, nrm, uvs;   // flattened 3 / 3 / 2
    std::vector<mcrt_gpu_vertex> vertices;
    std::vector<mcrt_gpu_triangle> triangles;
    std::unordered_map<uint64_t, uint32_t> cache_pt;               // (pos, uv) -> dense id
    std::unordered_map<uint64_t, uint32_t> cache;                  // (dense id, normal) -> vertex
    auto resolve = [](const std::string &raw, size_t len, uint32_t *out) {
        long long i;
        if (!parse_i64_strict(raw, &i)) return false;
        long long idx = i < 0 ? (long long)len + i : i - 1;
        if (idx >= 0 && (size_t)idx < len) { *out = (uint32_t)idx; return true; }
        return false;
    };
    for (size_t lb = 0; lb < content.size();) {                                // str::lines + str::trim
        size_t nl = content.find('\n', lb);
        size_t b = lb, e = nl == std::string::npos ? content.size() : nl;
        lb = nl == std::string::npos ? content.size() : nl + 1;
        trim_range(content, &b, &e);
        if (b == e || content[b] == '#') continue;
        std::vector<std::string> parts = split_ascii_ws(content, b, e);
        const std::string &tag = parts[0];
        std::vector<std::string> rest(parts.begin() + 1, parts.end());
        auto f = [&](size_t k) { float v = 0.0f; if (!parse_f32_strict(rest[k], &v)) v = 0.0f; return v; };
        if (tag == "v" && rest.size() >= 3) {
            pos.push_back(f(0)); pos.push_back(f(1)); pos.push_back(f(2));
        } else if (tag == "vn" && rest.size() >= 3) {
            float v[3] = {f(0), f(1), f(2)}, o[3];
            normalize3_obj(v, o);
            nrm.insert(nrm.end(), o, o + 3);
        } else if (tag == "vt" && rest.size() >= 2) {
            uvs.push_back(f(0)); uvs.push_back(f(1));
        } else if (tag == "f" && rest.size() >= 3) {
            std::vector<uint32_t> face;
            for (const std::string &tok : rest) {
                std::vector<std::string> p = split_char(tok, '/');
                uint32_t pi = 0, ti = 0xffffffffu, ni = 0xffffffffu;
                if (!resolve(p[0], pos.size() / 3, &pi)) pi = 0;
                if (p.size() > 1 && !p[1].empty() && !resolve(p[1], uvs.size() / 2, &ti)) ti = 0xffffffffu;
                if (p.size() > 2 && !resolve(p[2], nrm.size() / 3, &ni)) ni = 0xffffffffu;
                auto make_vertex = [&](bool with_normal) {
                    mcrt_gpu_vertex v{};
                    if ((size_t)pi * 3 + 2 < pos.size()) { v.position[0] = pos[3 * pi]; v.position[1] = pos[3 * pi + 1]; v.position[2] = pos[3 * pi + 2]; }
                    v.position[3] = 1.0f;
                    if (with_normal && (size_t)ni * 3 + 2 < nrm.size()) {
                        v.normal[0] = nrm[3 * ni]; v.normal[1] = nrm[3 * ni + 1]; v.normal[2] = nrm[3 * ni + 2];
                    } else {
                        v.normal[1] = 1.0f;
                    }
                    if (ti != 0xffffffffu && (size_t)ti * 2 + 1 < uvs.size()) { v.uv[0] = uvs[2 * ti]; v.uv[1] = uvs[2 * ti + 1]; }
                    return v;
                };
                uint32_t vi;
                if (ni != 0xffffffffu) {                                       // vert_cache, mesh.rs:556-575
                    auto ins = cache_pt.emplace((uint64_t)pi | ((uint64_t)ti << 32), (uint32_t)cache_pt.size());
                    const uint64_t key = (uint64_t)ins.first->second | ((uint64_t)ni << 32);
                    auto it = cache.find(key);
                    if (it == cache.end()) {
                        vi = (uint32_t)vertices.size();
                        vertices.push_back(make_vertex(true));
                        cache.emplace(key, vi);
                    } else {
                        vi = it->second;
                    }
                } else {
                    vi = (uint32_t)vertices.size();
                    vertices.push_back(make_vertex(false));
                }
                face.push_back(vi);
            }
            for (size_t i = 1; i + 1 < face.size(); ++i) {              // fan, mesh.rs:593-630
                uint32_t v0 = face[0], v1 = face[i], v2 = face[i + 1];
                const std::string keys[3] = {rest[0], rest[i], i + 1 < rest.size() ? rest[i + 1] : std::string()};
                const uint32_t vis[3] = {v0, v1, v2};
                for (int k = 0; k < 3; ++k) {
                    std::vector<std::string> p = split_char(keys[k], '/');
                    long long dummy;
                    bool has_norm = p.size() > 2 && !p[2].empty() && parse_i64_strict(p[2], &dummy);
                    if (!has_norm) {
                        const float *p0 = vertices[v0].position, *p1 = vertices[v1].position, *p2 = vertices[v2].position;
                        float e1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
                        float e2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
                        float cr[3], gn[3];
                        pcross(e1, e2, cr);
                        normalize3_obj(cr, gn);
                        vertices[vis[k]].normal[0] = gn[0]; vertices[vis[k]].normal[1] = gn[1];
                        vertices[vis[k]].normal[2] = gn[2]; vertices[vis[k]].normal[3] = 0.0f;
                    }
                }
                triangles.push_back({{v0, v1, v2}, mat_idx});
            }
        }
    }
    if (vertices.empty() || triangles.empty()) { *err = ": no geometry found after parsing"; return false; }
    *verts_out = std::move(vertices);
    *tris_out = std::move(triangles);
    return true;
}

void rotation_matrix(const float deg[3], float m[9]) {
    M3 r = euler_to_mat3(deg[0], deg[1], deg[2]);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) m[3 * i + j] = r.m[i][j];
}

// ---- load_scene_from_str (scene.rs:640-978)
mcrt_status load_scene(const std::string &text, const std::string &src, LoadedScene *out, std::string *errmsg,
                       bool defer_meshes) {
    YNode root;
    std::string yerr;
    if (!yaml_parse(text, &root, &yerr)) {
        *errmsg = "parse error: failed to parse '" + src + "': " + yerr;
        return MCRT_ERR_PARSE;
    }
    if (root.kind == YNode::Null) root.kind = YNode::Map;
    if (root.kind != YNode::Map) { *errmsg = "parse error: failed to parse '" + src + "': expected a mapping"; return MCRT_ERR_PARSE; }
    SceneErr e{MCRT_OK, ""};
    LoadedScene S;
    std::vector<mcrt_gpu_material> mats;
    std::unordered_map<std::string, uint32_t> name_to_idx;
    std::vector<std::string> palette_names;
    for (const char *section : {"world_materials", "materials"}) {            // scene.rs:656-667
        const YNode *m = root.get(section);
        if (!m || m->kind == YNode::Null) continue;
        if (m->kind != YNode::Map) { e = perr(src, m, std::string(section) + ": expected a mapping"); *errmsg = e.msg; return e.code; }
        for (const auto &kv : m->map) {
            if (name_to_idx.count(kv.first)) continue;
            mcrt_gpu_material gm;
            if (!material_from_yaml(&kv.second, src, &gm, &e)) { *errmsg = e.msg; return e.code; }
            name_to_idx[kv.first] = (uint32_t)mats.size();
            palette_names.push_back(kv.first);
            mats.push_back(gm);
        }
    }
    auto resolve_mat = [&](const YNode *ref, uint32_t *idx) -> bool {
        if (!ref) { e = perr(src, nullptr, "object: missing field `material`"); return false; }
        if (ref->kind == YNode::Scalar) {
            auto it = name_to_idx.find(ref->scalar);
            if (it == name_to_idx.end()) { e = {MCRT_ERR_UNKNOWN_MATERIAL, "unknown material '" + ref->scalar + "'"}; return false; }
            *idx = it->second;
            return true;
        }
        mcrt_gpu_material gm;
        if (!material_from_yaml(ref, src, &gm, &e)) return false;
        *idx = (uint32_t)mats.size();
        mats.push_back(gm);
        return true;
    };
    if (const YNode *objs = root.get("objects"); objs && objs->kind != YNode::Null) {
        if (objs->kind != YNode::Seq) { e = perr(src, objs, "objects: expected a sequence"); *errmsg = e.msg; return e.code; }
        for (const YNode &o : objs->seq) {
            if (o.kind != YNode::Map) { e = perr(src, &o, "object: expected a mapping"); *errmsg = e.msg; return e.code; }
            std::string type;
            if (!as_str(o.get("type"), &type)) { e = perr(src, &o, "object: missing field `type`"); *errmsg = e.msg; return e.code; }
            if (type == "sphere") {
                float c[3], r;
                if (!as_vec<3>(o.get("center"), c)) { e = perr(src, &o, "sphere: missing or invalid `center`"); *errmsg = e.msg; return e.code; }
                if (!as_f32(o.get("radius"), &r)) { e = perr(src, &o, "sphere: missing or invalid `radius`"); *errmsg = e.msg; return e.code; }
                uint32_t mi;
                if (!resolve_mat(o.get("material"), &mi)) { *errmsg = e.msg; return e.code; }
                mcrt_gpu_sphere s{};
                s.center_r[0] = c[0]; s.center_r[1] = c[1]; s.center_r[2] = c[2]; s.center_r[3] = r;
                s.mat_and_pad[0] = mi;
                S.spheres.push_back(s);
            } else if (type == "plane") {                                         // scene.rs:701-734
                float n[3], he[2];
                if (!as_vec<3>(o.get("normal"), n)) { e = perr(src, &o, "plane: missing or invalid `normal`"); *errmsg = e.msg; return e.code; }
                if (!as_vec<2>(o.get("half_extents"), he)) { e = perr(src, &o, "plane: missing or invalid `half_extents`"); *errmsg = e.msg; return e.code; }
                Transform t;
                if (!transform_from_yaml(o.get("transform"), src, &t, &e)) { *errmsg = e.msg; return e.code; }
                bool cull = false;
                if (const YNode *b = o.get("backface_culling"); b && b->kind != YNode::Null && !as_bool(b, &cull)) {
                    e = perr(src, b, "backface_culling: expected bool"); *errmsg = e.msg; return e.code;
                }
                uint32_t mi;
                if (!resolve_mat(o.get("material"), &mi)) { *errmsg = e.msg; return e.code; }
                if (cull) mi |= kBackfaceCull;
                float en[3];
                t.apply_normal(n, en);
                push_quad_face(t.t, en, he[0], he[1], mi, S.vertices, S.triangles);
            } else if (type == "box") {                                           // scene.rs:736-827
                float he[3];
                if (!as_vec<3>(o.get("half_extents"), he)) { e = perr(src, &o, "box: missing or invalid `half_extents`"); *errmsg = e.msg; return e.code; }
                Transform t;
                if (!transform_from_yaml(o.get("transform"), src, &t, &e)) { *errmsg = e.msg; return e.code; }
                uint32_t mi;
                if (!resolve_mat(o.get("material"), &mi)) { *errmsg = e.msg; return e.code; }
                M3 rot = t.has_r ? euler_to_mat3(t.r[0], t.r[1], t.r[2]) : M3{{{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}};
                const float hx = he[0], hy = he[1], hz = he[2];
                const float faces[6][5][3] = {
                    {{1, 0, 0}, {hx, -hy, -hz}, {hx, -hy, hz}, {hx, hy, hz}, {hx, hy, -hz}},
                    {{-1, 0, 0}, {-hx, -hy, hz}, {-hx, -hy, -hz}, {-hx, hy, -hz}, {-hx, hy, hz}},
                    {{0, 1, 0}, {-hx, hy, -hz}, {hx, hy, -hz}, {hx, hy, hz}, {-hx, hy, hz}},
                    {{0, -1, 0}, {hx, -hy, -hz}, {-hx, -hy, -hz}, {-hx, -hy, hz}, {hx, -hy, hz}},
                    {{0, 0, 1}, {hx, -hy, hz}, {-hx, -hy, hz}, {-hx, hy, hz}, {hx, hy, hz}},
                    {{0, 0, -1}, {-hx, -hy, -hz}, {hx, -hy, -hz}, {hx, hy, -hz}, {-hx, hy, -hz}},
                };
                const float uvs[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
                for (int f = 0; f < 6; ++f) {
                    float rn[3];
                    rot3(rot, faces[f][0], rn);
                    uint32_t base = (uint32_t)S.vertices.size();
                    for (int k = 0; k < 4; ++k) {
                        float rc[3];
                        rot3(rot, faces[f][1 + k], rc);
                        mcrt_gpu_vertex v{};
                        v.position[0] = t.t[0] + rc[0]; v.position[1] = t.t[1] + rc[1];
                        v.position[2] = t.t[2] + rc[2]; v.position[3] = 1.0f;
                        v.normal[0] = rn[0]; v.normal[1] = rn[1]; v.normal[2] = rn[2];
                        v.uv[0] = uvs[k][0]; v.uv[1] = uvs[k][1];
                        S.vertices.push_back(v);
                    }
                    S.triangles.push_back({{base, base + 1, base + 2}, mi});
                    S.triangles.push_back({{base, base + 2, base + 3}, mi});
                }
            } else if (type == "mesh") {                                          // scene.rs:829-879
                std::string path;
                if (!as_str(o.get("path"), &path)) { e = perr(src, &o, "mesh: missing field `path`"); *errmsg = e.msg; return e.code; }
                Transform t;
                if (!transform_from_yaml(o.get("transform"), src, &t, &e)) { *errmsg = e.msg; return e.code; }
                uint32_t mi;
                if (!resolve_mat(o.get("material"), &mi)) { *errmsg = e.msg; return e.code; }
                std::string content;
                if (!read_file(path, &content)) {
                    *errmsg = "mesh load error: failed to load mesh '" + path + "': cannot read '" + path + "'";
                    return MCRT_ERR_MESH_LOAD;
                }
                if (defer_meshes) {                       // parsed on the device by mcrt_mesh_append_scene
                    LoadedScene::MeshRef m;
                    m.path = path;
                    m.text = std::move(content);
                    m.mat_idx = mi;
                    m.xf.has_translate = t.has_t; m.xf.has_rotate = t.has_r; m.xf.has_scale = t.has_s;
                    for (int k = 0; k < 3; ++k) { m.xf.translate[k] = t.t[k]; m.xf.rotate_deg[k] = t.r[k]; }
                    m.xf.scale = t.s;
                    m.at_vertex = S.vertices.size();
                    m.at_triangle = S.triangles.size();
                    S.meshes.push_back(std::move(m));
                    continue;
                }
                std::vector<mcrt_gpu_vertex> mv;
                std::vector<mcrt_gpu_triangle> mt;
                std::string oerr;
                if (!load_obj_text(content, mi, &mv, &mt, &oerr)) {
                    *errmsg = "mesh load error: failed to load mesh '" + path + "': '" + path + "'" + oerr;
                    return MCRT_ERR_MESH_LOAD;
                }
                if (!(t.s > 0.0f)) {
                    *errmsg = "mesh '" + path + "' transform.scale must be positive";
                    return MCRT_ERR_INVALID_ARG;
                }
                if (!t.identity())
                    for (auto &v : mv) {
                        float p[3] = {v.position[0], v.position[1], v.position[2]}, q[3];
                        t.apply_point(p, q);
                        v.position[0] = q[0]; v.position[1] = q[1]; v.position[2] = q[2];
                        float n[3] = {v.normal[0], v.normal[1], v.normal[2]}, m2[3];
                        t.apply_normal(n, m2);
                        v.normal[0] = m2[0]; v.normal[1] = m2[1]; v.normal[2] = m2[2];
                    }
                uint32_t off = (uint32_t)S.vertices.size();
                S.vertices.insert(S.vertices.end(), mv.begin(), mv.end());
                for (auto tr : mt) {
                    tr.v[0] += off; tr.v[1] += off; tr.v[2] += off;
                    S.triangles.push_back(tr);
                }
            } else {
                e = perr(src, o.get("type"), "unknown variant `" + type + "`");
                *errmsg = e.msg;
                return e.code;
            }
        }
    }
    S.deferred = defer_meshes;
    if (S.vertices.empty() && S.meshes.empty()) {                                 // scene.rs:887-899
        mcrt_gpu_vertex v{};
        v.position[0] = 1.0e9f; v.position[1] = 1.0e9f; v.position[2] = 1.0e9f; v.position[3] = 1.0f;
        v.normal[1] = 1.0f;
        S.vertices.push_back(v);
        S.triangles.push_back({{0, 0, 0}, 0});
    }
    if (mats.size() > MCRT_MAX_MATERIALS) {                                       // scene.rs:902-907
        *errmsg = "scene uses " + std::to_string(mats.size()) + " materials but limit is " +
                  std::to_string(MCRT_MAX_MATERIALS);
        return MCRT_ERR_TOO_MANY_MATERIALS;
    }
    std::memset(&S.materials, 0, sizeof(S.materials));
    S.materials.mat_count = (uint32_t)mats.size();
    for (size_t i = 0; i < mats.size(); ++i) S.materials.materials[i] = mats[i];
    for (const auto &s : S.spheres) {                                             // scene.rs:915-923
        uint32_t idx = s.mat_and_pad[0];
        if (idx < mats.size() && mats[idx].type_pad[0] == MCRT_MAT_EMISSIVE) S.emissive_spheres.push_back(s);
    }
    S.materials.n_emissive = (uint32_t)S.emissive_spheres.size();
    if (const YNode *c = root.get("camera"); c && c->kind != YNode::Null) {      // scene.rs:926-944
        if (c->kind != YNode::Map) { e = perr(src, c, "camera: expected a mapping"); *errmsg = e.msg; return e.code; }
        if (!as_vec<3>(c->get("look_from"), S.look_from)) { e = perr(src, c, "camera: missing or invalid `look_from`"); *errmsg = e.msg; return e.code; }
        if (!as_vec<3>(c->get("look_at"), S.look_at)) { e = perr(src, c, "camera: missing or invalid `look_at`"); *errmsg = e.msg; return e.code; }
        S.has_camera = true;
        float d[3] = {S.look_from[0] - S.look_at[0], S.look_from[1] - S.look_at[1], S.look_from[2] - S.look_at[2]};
        float dist = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        S.vfov = 60.0f;
        S.aperture = 0.0f;
        S.focus_dist = dist;
        auto opt = [&](const char *k, float *v) {
            const YNode *x = c->get(k);
            if (!x || x->kind == YNode::Null) return true;
            if (!as_f32(x, v)) { e = perr(src, x, std::string(k) + ": expected f32"); return false; }
            return true;
        };
        if (!opt("vfov", &S.vfov) || !opt("aperture", &S.aperture) || !opt("focus_dist", &S.focus_dist)) {
            *errmsg = e.msg;
            return e.code;
        }
    }
    if (const YNode *env = root.get("env_map"); env && env->kind != YNode::Null) {
        if (!as_str(env, &S.env_map_path)) { e = perr(src, env, "env_map: expected a string"); *errmsg = e.msg; return e.code; }
        S.has_env_map = true;
    }
    S.material_names.resize(mats.size());                                        // scene.rs:962-975
    for (size_t i = 0; i < mats.size(); ++i) S.material_names[i] = "inline-" + std::to_string(i);
    for (const auto &kv : name_to_idx) S.material_names[kv.second] = kv.first;
    *out = std::move(S);
    return MCRT_OK;
}

// ---- compute_camera (camera.rs:76-127), glam Vec3 arithmetic
namespace {
struct V { float x, y, z; };
inline V vsub(V a, V b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V vscale(V a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline float vdot(V a, V b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline V vcross(V a, V b) { return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
inline V vnormalize(V a) { float r = 1.0f / sqrtf(vdot(a, a)); return vscale(a, r); }
}  // namespace

void compute_camera(uint32_t width, uint32_t height, const float lf[3], const float la[3], float vfov_deg,
                    float aperture, float focus_dist, mcrt_camera_uniform *out) {
    const float rads_per_deg = kPiF / 180.0f;
    float aspect = (float)width / (float)height;
    V vup = {0.0f, 1.0f, 0.0f};
    float vfov_rad = vfov_deg * rads_per_deg;
    float h = mcrt::fm_tan(vfov_rad * 0.5f);
    float vh = 2.0f * h;
    float vw = aspect * vh;
    V from = {lf[0], lf[1], lf[2]}, at = {la[0], la[1], la[2]};
    V w = vnormalize(vsub(from, at));
    V c = vcross(vup, w);
    V vup_safe = vdot(c, c) > 1e-10f ? vup : V{0.0f, 0.0f, 1.0f};
    V u = vnormalize(vcross(vup_safe, w));
    V v = vcross(w, u);
    V horizontal = vscale(u, focus_dist * vw);
    V vertical = vscale(v, focus_dist * vh);
    V ll = vsub(vsub(vsub(from, vscale(horizontal, 0.5f)), vscale(vertical, 0.5f)), vscale(w, focus_dist));
    float lens = aperture * 0.5f;
    V du = vscale(u, lens), dv = vscale(v, lens);
    std::memset(out, 0, sizeof(*out));
    auto put = [](float *d, V a) { d[0] = a.x; d[1] = a.y; d[2] = a.z; d[3] = 0.0f; };
    put(out->origin, from);
    put(out->lower_left, ll);
    put(out->horizontal, horizontal);
    put(out->vertical, vertical);
    put(out->defocus_u, du);
    put(out->defocus_v, dv);
    out->frame_count = 0;
}

// ---- environment map (texture.rs)
void gradient_env_map(float *data) {                                              // texture.rs:158-199
    for (uint32_t y = 0; y < MCRT_ENV_MAP_HEIGHT; ++y) {
        float v = ((float)y + 0.5f) / (float)MCRT_ENV_MAP_HEIGHT;
        float el = 1.0f - 2.0f * v;
        float r, g, b;
        if (el >= 0.0f) {
            float t = el;
            r = 1.0f - 0.5f * t; g = 1.0f - 0.3f * t; b = 1.0f;
        } else {
            float t = std::min(-el, 1.0f);
            r = (1.0f - t) * 0.8f; g = (1.0f - t) * 0.4f; b = (1.0f - t) * 0.1f;
        }
        for (uint32_t x = 0; x < MCRT_ENV_MAP_WIDTH; ++x) {
            float *p = data + 4 * ((size_t)y * MCRT_ENV_MAP_WIDTH + x);
            p[0] = r; p[1] = g; p[2] = b; p[3] = 1.0f;
        }
    }
}

// Radiance RGBE decode (flat and run-length scanlines), as the image crate 0.25
// decodes it: component * 2^(e - 136), e == 0 -> black.
bool read_hdr(const std::string &path, std::vector<float> *rgb, uint32_t *w_out, uint32_t *h_out) {
    std::string d;
    if (!read_file(path, &d)) return false;
    size_t pos = 0;
    auto getline = [&](std::string *l) {
        if (pos >= d.size()) return false;
        size_t e = d.find('\n', pos);
        if (e == std::string::npos) return false;
        *l = d.substr(pos, e - pos);
        pos = e + 1;
        return true;
    };
    std::string l;
    if (!getline(&l) || (l.rfind("#?", 0) != 0)) return false;
    for (;;) {
        if (!getline(&l)) return false;
        if (l.empty()) break;
        if (l.rfind("FORMAT=", 0) == 0 && l != "FORMAT=32-bit_rle_rgbe") return false;
    }
    if (!getline(&l)) return false;
    int H = 0, W = 0;
    if (sscanf(l.c_str(), "-Y %d +X %d", &H, &W) != 2 || H <= 0 || W <= 0 || (uint64_t)W * H > (1ull << 28)) return false;
    std::vector<uint8_t> px((size_t)W * H * 4);
    for (int y = 0; y < H; ++y) {
        uint8_t *row = px.data() + (size_t)y * W * 4;
        if (pos + 4 <= d.size() && W >= 8 && W < 32768 && (uint8_t)d[pos] == 2 && (uint8_t)d[pos + 1] == 2 &&
            !((uint8_t)d[pos + 2] & 0x80)) {
            int sw = ((uint8_t)d[pos + 2] << 8) | (uint8_t)d[pos + 3];
            if (sw != W) return false;
            pos += 4;
            for (int c = 0; c < 4; ++c) {
                int x = 0;
                while (x < W) {
                    if (pos >= d.size()) return false;
                    int n = (uint8_t)d[pos++];
                    if (n > 128) {
                        n -= 128;
                        if (pos >= d.size() || x + n > W) return false;
                        uint8_t v = (uint8_t)d[pos++];
                        for (int k = 0; k < n; ++k) row[4 * (x++) + c] = v;
                    } else {
                        if (n == 0 || pos + n > d.size() || x + n > W) return false;
                        for (int k = 0; k < n; ++k) row[4 * (x++) + c] = (uint8_t)d[pos++];
                    }
                }
            }
        } else {
            if (pos + (size_t)W * 4 > d.size()) return false;
            std::memcpy(row, d.data() + pos, (size_t)W * 4);
            pos += (size_t)W * 4;
        }
    }
    rgb->resize((size_t)W * H * 3);
    for (size_t i = 0; i < (size_t)W * H; ++i) {
        uint8_t e = px[4 * i + 3];
        for (int c = 0; c < 3; ++c) {
            float v = 0.0f;
            if (e != 0) v = mcrt::fm_ldexp(1.0f, (int)e - 136) * (float)px[4 * i + c];
            (*rgb)[3 * i + c] = v;
        }
    }
    *w_out = (uint32_t)W;
    *h_out = (uint32_t)H;
    return true;
}

// try_load_hdr (texture.rs:124-148): nearest resize to 1024x512, clamp to [0, 1e10], alpha 1.
bool try_load_hdr(const std::string &path, float *out) {
    std::vector<float> rgb;
    uint32_t W, H;
    if (!read_hdr(path, &rgb, &W, &H)) return false;
    const uint32_t OW = MCRT_ENV_MAP_WIDTH, OH = MCRT_ENV_MAP_HEIGHT;
    const float rx = (float)W / (float)OW, ry = (float)H / (float)OH;
    for (uint32_t y = 0; y < OH; ++y) {
        uint32_t sy = (W == OW && H == OH) ? y : std::min(mcrt::fm_f2u_sat(((float)y + 0.5f) * ry), H - 1);
        for (uint32_t x = 0; x < OW; ++x) {
            uint32_t sx = (W == OW && H == OH) ? x : std::min(mcrt::fm_f2u_sat(((float)x + 0.5f) * rx), W - 1);
            const float *s = rgb.data() + 3 * ((size_t)sy * W + sx);
            float *o = out + 4 * ((size_t)y * OW + x);
            for (int c = 0; c < 3; ++c) o[c] = std::min(std::max(s[c], 0.0f), 1e10f);
            o[3] = 1.0f;
        }
    }
    return true;
}

// load_env_map_data (texture.rs:209-220)
void load_env_map_data(const char *scene_path, float *out) {
    if (scene_path && try_load_hdr(scene_path, out)) return;
    if (try_load_hdr("textures/env.hdr", out)) return;
    gradient_env_map(out);
}

}  // namespace mcrt_host

// ====================================================================== ABI
extern "C" {

mcrt_status mcrt_scene_load_yaml_str_ex(const char *text, const char *source, uint32_t flags,
                                        mcrt_loaded_scene **out) {
    if (!text || !out) { mcrt::set_global_error("NULL argument"); return MCRT_ERR_INVALID_ARG; }
    if (flags & ~(uint32_t)MCRT_LOAD_DEFER_MESHES) { mcrt::set_global_error("unknown flags"); return MCRT_ERR_INVALID_ARG; }
    *out = nullptr;
    auto *ls = new mcrt_loaded_scene();
    std::string err;
    mcrt_status s = mcrt_host::load_scene(text, source ? source : "<inline>", &ls->s, &err,
                                          (flags & MCRT_LOAD_DEFER_MESHES) != 0);
    if (s != MCRT_OK) {
        delete ls;
        mcrt::set_global_error(err);
        return s;
    }
    *out = ls;
    return MCRT_OK;
}

mcrt_status mcrt_scene_load_yaml_str(const char *text, const char *source, mcrt_loaded_scene **out) {
    return mcrt_scene_load_yaml_str_ex(text, source, 0, out);
}

mcrt_status mcrt_scene_load_yaml_ex(const char *path, uint32_t flags, mcrt_loaded_scene **out) {
    if (!path || !out) { mcrt::set_global_error("NULL argument"); return MCRT_ERR_INVALID_ARG; }
    std::string text;
    if (!mcrt_host::read_file(path, &text)) {
        mcrt::set_global_error(std::string("I/O error: cannot read '") + path + "'");
        return MCRT_ERR_IO;
    }
    return mcrt_scene_load_yaml_str_ex(text.c_str(), path, flags, out);
}

mcrt_status mcrt_scene_load_yaml(const char *path, mcrt_loaded_scene **out) {
    return mcrt_scene_load_yaml_ex(path, 0, out);
}

// The scene's objects in order (scene.rs:687-899): runs of host records
// between the deferred mesh objects, each mesh parsed on the device.
mcrt_status mcrt_mesh_append_scene(mcrt_ctx *ctx, const mcrt_loaded_scene *scene) {
    if (!ctx || !scene) { mcrt::set_global_error("NULL argument"); return MCRT_ERR_INVALID_ARG; }
    const mcrt_host::LoadedScene &S = scene->s;
    size_t v_done = 0, t_done = 0;
    auto host_run = [&](size_t v_end, size_t t_end) -> mcrt_status {
        std::vector<mcrt_gpu_triangle> tris(S.triangles.begin() + t_done, S.triangles.begin() + t_end);
        for (auto &t : tris)
            for (int k = 0; k < 3; ++k) t.v[k] -= (uint32_t)v_done;
        mcrt_status st = mcrt_mesh_append(ctx, S.vertices.data() + v_done, (uint32_t)(v_end - v_done), tris.data(),
                                          (uint32_t)tris.size());
        v_done = v_end;
        t_done = t_end;
        return st;
    };
    for (const auto &m : S.meshes) {
        mcrt_status st = host_run(m.at_vertex, m.at_triangle);
        if (st != MCRT_OK) return st;
        st = mcrt_mesh_append_obj(ctx, m.text.data(), m.text.size(), m.mat_idx, &m.xf, m.path.c_str(), nullptr,
                                  nullptr);
        if (st != MCRT_OK) return st;
    }
    return host_run(S.vertices.size(), S.triangles.size());
}

void mcrt_scene_free(mcrt_loaded_scene *scene) { delete scene; }

mcrt_status mcrt_scene_view_get(const mcrt_loaded_scene *scene, mcrt_scene_view *v) {
    if (!scene || !v) { mcrt::set_global_error("NULL argument"); return MCRT_ERR_INVALID_ARG; }
    const mcrt_host::LoadedScene &s = scene->s;
    std::memset(v, 0, sizeof(*v));
    v->spheres = s.spheres.data(); v->n_spheres = (uint32_t)s.spheres.size();
    v->vertices = s.vertices.data(); v->n_vertices = (uint32_t)s.vertices.size();
    v->triangles = s.triangles.data(); v->n_triangles = (uint32_t)s.triangles.size();
    v->emissive_spheres = s.emissive_spheres.data(); v->n_emissive_spheres = (uint32_t)s.emissive_spheres.size();
    v->materials = &s.materials;
    v->has_camera = s.has_camera ? 1 : 0;
    for (int i = 0; i < 3; ++i) { v->look_from[i] = s.look_from[i]; v->look_at[i] = s.look_at[i]; }
    v->vfov = s.vfov; v->aperture = s.aperture; v->focus_dist = s.focus_dist;
    v->env_map_path = s.has_env_map ? s.env_map_path.c_str() : nullptr;
    v->n_material_names = (uint32_t)s.material_names.size();
    return MCRT_OK;
}

const char *mcrt_scene_material_name(const mcrt_loaded_scene *scene, uint32_t index) {
    if (!scene || index >= scene->s.material_names.size()) return nullptr;
    return scene->s.material_names[index].c_str();
}

mcrt_status mcrt_compute_camera(uint32_t width, uint32_t height, const float look_from[3], const float look_at[3],
                                float vfov_deg, float aperture, float focus_dist, mcrt_camera_uniform *out) {
    if (!look_from || !look_at || !out || width == 0 || height == 0) {
        mcrt::set_global_error("invalid camera arguments");
        return MCRT_ERR_INVALID_ARG;
    }
    mcrt_host::compute_camera(width, height, look_from, look_at, vfov_deg, aperture, focus_dist, out);
    return MCRT_OK;
}

mcrt_status mcrt_load_env_map(const char *path, float *out) {
    if (!out) { mcrt::set_global_error("NULL argument"); return MCRT_ERR_INVALID_ARG; }
    mcrt_host::load_env_map_data(path, out);
    return MCRT_OK;
}

mcrt_status mcrt_albedo_layers(uint8_t *out) {
    if (!out) { mcrt::set_global_error("NULL argument"); return MCRT_ERR_INVALID_ARG; }
    // build_checker_texture (texture.rs:46-61): tiles of size/8 pixels
    auto checker = [](uint8_t *dst, const uint8_t a[4], const uint8_t b[4]) {
        const uint32_t n = MCRT_TEXTURE_SIZE, tile = n / 8 ? n / 8 : 1;
        for (uint32_t y = 0; y < n; ++y)
            for (uint32_t x = 0; x < n; ++x) memcpy(dst + 4 * ((size_t)y * n + x), ((x / tile + y / tile) % 2 == 0) ? a : b, 4);
    };
    const size_t layer = (size_t)MCRT_TEXTURE_SIZE * MCRT_TEXTURE_SIZE * 4;
    memset(out, 255, layer);                                                        // layer 0: white
    const uint8_t grey_a[4] = {220, 220, 220, 255}, grey_b[4] = {50, 50, 50, 255};  // texture.rs:245-252
    const uint8_t mag_a[4] = {200, 0, 200, 255}, mag_b[4] = {30, 30, 30, 255};      // texture.rs:105-107
    checker(out + layer, grey_a, grey_b);
    checker(out + 2 * layer, mag_a, mag_b);
    checker(out + 3 * layer, mag_a, mag_b);
    return MCRT_OK;
}

mcrt_status mcrt_gradient_env_map(float *out) {
    if (!out) { mcrt::set_global_error("NULL argument"); return MCRT_ERR_INVALID_ARG; }
    mcrt_host::gradient_env_map(out);
    return MCRT_OK;
}

}  // extern "C"
