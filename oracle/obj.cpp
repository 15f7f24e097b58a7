// obj.cpp — CPU restatement of the reference's Wavefront OBJ loader, load_obj
// (src/mesh.rs:474-642), together with the Rust standard-library rules that
// loader relies on: String::from_utf8 (the UTF-8 check and its error text),
// str::lines, str::trim, str::split_ascii_whitespace, str::split('/'),
// str::parse::<f32> and str::parse::<i64>.  Written as a literal sequential
// loop with a hash map keyed by (position, uv, normal) indices, as the
// reference is.  Test infrastructure only: it is the checker of the device OBJ
// parser and is never linked into the library.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "oracle.h"

namespace {

// String::from_utf8 -> core::str::run_utf8_validation: the first invalid
// sequence's start (valid_up_to) and its error_len (0 = incomplete at the end).
bool utf8_validate(const unsigned char *v, size_t len, size_t *valid_up_to, int *error_len) {
    size_t i = 0;
    auto cont = [](unsigned char b) { return (b & 0xC0) == 0x80; };
    while (i < len) {
        const unsigned char first = v[i];
        if (first < 0x80) { ++i; continue; }
        const size_t start = i;
        auto fail = [&](int el) { *valid_up_to = start; *error_len = el; return false; };
        int w = 0;
        if (first >= 0xC2 && first <= 0xDF) w = 2;
        else if (first >= 0xE0 && first <= 0xEF) w = 3;
        else if (first >= 0xF0 && first <= 0xF4) w = 4;
        if (w == 0) return fail(1);
        if (i + 1 >= len) return fail(0);
        const unsigned char b1 = v[i + 1];
        if (w == 2) {
            if (!cont(b1)) return fail(1);
        } else if (w == 3) {
            bool ok = (first == 0xE0 && b1 >= 0xA0 && b1 <= 0xBF) ||
                      (first >= 0xE1 && first <= 0xEC && cont(b1)) ||
                      (first == 0xED && b1 >= 0x80 && b1 <= 0x9F) ||
                      (first >= 0xEE && first <= 0xEF && cont(b1));
            if (!ok) return fail(1);
            if (i + 2 >= len) return fail(0);
            if (!cont(v[i + 2])) return fail(2);
        } else {
            bool ok = (first == 0xF0 && b1 >= 0x90 && b1 <= 0xBF) ||
                      (first >= 0xF1 && first <= 0xF3 && cont(b1)) ||
                      (first == 0xF4 && b1 >= 0x80 && b1 <= 0x8F);
            if (!ok) return fail(1);
            if (i + 2 >= len) return fail(0);
            if (!cont(v[i + 2])) return fail(2);
            if (i + 3 >= len) return fail(0);
            if (!cont(v[i + 3])) return fail(3);
        }
        i += w;
    }
    return true;
}

// Decode the scalar value of the (valid) UTF-8 character starting at s[i].
uint32_t decode_at(const std::string &s, size_t i, size_t *n) {
    const unsigned char c = s[i];
    if (c < 0x80) { *n = 1; return c; }
    if (c < 0xE0) { *n = 2; return ((c & 0x1Fu) << 6) | (s[i + 1] & 0x3Fu); }
    if (c < 0xF0) { *n = 3; return ((c & 0x0Fu) << 12) | ((s[i + 1] & 0x3Fu) << 6) | (s[i + 2] & 0x3Fu); }
    *n = 4;
    return ((c & 0x07u) << 18) | ((s[i + 1] & 0x3Fu) << 12) | ((s[i + 2] & 0x3Fu) << 6) | (s[i + 3] & 0x3Fu);
}

// char::is_whitespace (the Unicode White_Space property).
bool is_white_space(uint32_t c) {
    return (c >= 0x09 && c <= 0x0D) || c == 0x20 || c == 0x85 || c == 0xA0 || c == 0x1680 ||
           (c >= 0x2000 && c <= 0x200A) || c == 0x2028 || c == 0x2029 || c == 0x202F || c == 0x205F ||
           c == 0x3000;
}

// str::trim: strip White_Space characters from both ends.
std::string trim(const std::string &s) {
    std::vector<std::pair<size_t, uint32_t>> chars;   // (byte offset, scalar)
    for (size_t i = 0; i < s.size();) {
        size_t n;
        uint32_t c = decode_at(s, i, &n);
        chars.push_back({i, c});
        i += n;
    }
    size_t b = 0, e = chars.size();
    while (b < e && is_white_space(chars[b].second)) ++b;
    while (e > b && is_white_space(chars[e - 1].second)) --e;
    if (b == e) return std::string();
    size_t off_b = chars[b].first, off_e = e < chars.size() ? chars[e].first : s.size();
    return s.substr(off_b, off_e - off_b);
}

// str::lines: split at '\n', drop one '\r' before it, no empty last line.
std::vector<std::string> lines(const std::string &s) {
    std::vector<std::string> out;
    size_t b = 0;
    while (b < s.size()) {
        size_t e = s.find('\n', b);
        size_t end = e == std::string::npos ? s.size() : e;
        std::string l = s.substr(b, end - b);
        if (e != std::string::npos && !l.empty() && l.back() == '\r') l.pop_back();
        out.push_back(l);
        if (e == std::string::npos) break;
        b = e + 1;
    }
    return out;
}

// str::split_ascii_whitespace (u8::is_ascii_whitespace: space, \t, \n, \x0C, \r).
std::vector<std::string> split_ascii_ws(const std::string &s) {
    std::vector<std::string> out;
    auto ws = [](char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\x0C' || c == '\r'; };
    size_t i = 0;
    while (i < s.size()) {
        while (i < s.size() && ws(s[i])) ++i;
        size_t b = i;
        while (i < s.size() && !ws(s[i])) ++i;
        if (i > b) out.push_back(s.substr(b, i - b));
    }
    return out;
}

std::vector<std::string> split_slash(const std::string &s) {
    std::vector<std::string> out;
    size_t b = 0;
    for (;;) {
        size_t e = s.find('/', b);
        out.push_back(s.substr(b, e == std::string::npos ? std::string::npos : e - b));
        if (e == std::string::npos) return out;
        b = e + 1;
    }
}

bool ieq(const std::string &a, const char *lit) {
    if (a.size() != strlen(lit)) return false;
    for (size_t i = 0; i < a.size(); ++i) {
        char c = a[i];
        if (c >= 'A' && c <= 'Z') c = (char)(c - 'A' + 'a');
        if (c != lit[i]) return false;
    }
    return true;
}

// str::parse::<f32> (core::num::dec2flt): optional sign, then "inf",
// "infinity" or "nan" in any case, or digits with an optional fraction and an
// optional exponent; at least one mantissa digit; nothing else.  The value is
// the correctly rounded binary32 (strtof in the C locale rounds correctly).
bool parse_f32(const std::string &s, float *out) {
    size_t i = 0;
    bool neg = false;
    if (i < s.size() && (s[i] == '+' || s[i] == '-')) { neg = s[i] == '-'; ++i; }
    std::string body = s.substr(i);
    if (ieq(body, "inf") || ieq(body, "infinity")) { *out = neg ? -INFINITY : INFINITY; return true; }
    if (ieq(body, "nan")) {
        uint32_t bits = neg ? 0xFFC00000u : 0x7FC00000u;
        std::memcpy(out, &bits, 4);
        return true;
    }
    size_t digits = 0;
    while (i < s.size() && s[i] >= '0' && s[i] <= '9') { ++i; ++digits; }
    if (i < s.size() && s[i] == '.') {
        ++i;
        while (i < s.size() && s[i] >= '0' && s[i] <= '9') { ++i; ++digits; }
    }
    if (digits == 0) return false;
    if (i < s.size() && (s[i] == 'e' || s[i] == 'E')) {
        ++i;
        if (i < s.size() && (s[i] == '+' || s[i] == '-')) ++i;
        size_t ed = 0;
        while (i < s.size() && s[i] >= '0' && s[i] <= '9') { ++i; ++ed; }
        if (ed == 0) return false;
    }
    if (i != s.size()) return false;
    *out = strtof(s.c_str(), nullptr);
    return true;
}

// str::parse::<i64>: optional sign, one or more digits, no overflow.
bool parse_i64(const std::string &s, long long *out) {
    size_t i = 0;
    bool neg = false;
    if (i < s.size() && (s[i] == '+' || s[i] == '-')) { neg = s[i] == '-'; ++i; }
    if (i == s.size()) return false;
    unsigned long long v = 0;
    const unsigned long long lim = neg ? 9223372036854775808ull : 9223372036854775807ull;
    for (; i < s.size(); ++i) {
        if (s[i] < '0' || s[i] > '9') return false;
        unsigned d = (unsigned)(s[i] - '0');
        if (v > (lim - d) / 10) return false;
        v = v * 10 + d;
    }
    *out = neg ? (long long)(0ull - v) : (long long)v;
    return true;
}

// mesh.rs:663-670 / :650-661
void normalize3(const float v[3], float o[3]) {
    float len = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (len < 1e-8f) { o[0] = 0.0f; o[1] = 1.0f; o[2] = 0.0f; return; }
    o[0] = v[0] / len; o[1] = v[1] / len; o[2] = v[2] / len;
}

struct KeyHash {
    size_t operator()(const std::tuple<uint32_t, uint32_t, uint32_t> &k) const {
        uint64_t h = std::get<0>(k) * 0x9E3779B97F4A7C15ull;
        h ^= (std::get<1>(k) + 0x632BE59BD9B4E019ull) * 0xBF58476D1CE4E5B9ull;
        h ^= (std::get<2>(k) + 0x94D049BB133111EBull) * 0x94D049BB133111EBull;
        return (size_t)(h ^ (h >> 31));
    }
};

struct ObjResult {
    std::vector<orc_vertex> vertices;
    std::vector<orc_triangle> triangles;
};

}  // namespace

extern "C" {

// load_obj on the text of one file.  Returns a handle (NULL on error, with the
// reference's message after "'<path>': " / "'<path>' " in err).
void *orc_obj_load(const char *text, uint64_t len, uint32_t mat_idx, uint32_t *n_vertices, uint32_t *n_triangles,
                   char *err, uint32_t err_cap) {
    auto set_err = [&](const std::string &m) {
        if (err && err_cap) {
            size_t n = std::min<size_t>(m.size(), err_cap - 1);
            std::memcpy(err, m.data(), n);
            err[n] = '\0';
        }
    };
    size_t vu = 0;
    int el = 0;
    if (!utf8_validate(reinterpret_cast<const unsigned char *>(text), (size_t)len, &vu, &el)) {   // mesh.rs:477-478
        set_err(el ? "is not valid UTF-8: invalid utf-8 sequence of " + std::to_string(el) + " bytes from index " +
                         std::to_string(vu)
                   : "is not valid UTF-8: incomplete utf-8 byte sequence from index " + std::to_string(vu));
        return nullptr;
    }
    const std::string content(text, (size_t)len);
    std::vector<std::array<float, 3>> positions, normals;
    std::vector<std::array<float, 2>> uvs;
    auto *R = new ObjResult();
    std::vector<orc_vertex> &vertices = R->vertices;
    std::vector<orc_triangle> &triangles = R->triangles;
    std::unordered_map<std::tuple<uint32_t, uint32_t, uint32_t>, uint32_t, KeyHash> vert_cache;
    auto resolve = [](const std::string &raw, size_t n, uint32_t *out) {             // mesh.rs:491-500
        long long i;
        if (!parse_i64(raw, &i)) return false;
        long long idx = i < 0 ? (long long)n + i : i - 1;
        if (idx >= 0 && (size_t)idx < n) { *out = (uint32_t)idx; return true; }
        return false;
    };
    auto f32_or_zero = [](const std::string &s) { float v; return parse_f32(s, &v) ? v : 0.0f; };
    for (const std::string &raw_line : lines(content)) {                              // mesh.rs:502-617
        const std::string line = trim(raw_line);
        if (line.empty() || line[0] == '#') continue;
        std::vector<std::string> parts = split_ascii_ws(line);
        if (parts.empty()) continue;
        const std::string tag = parts[0];
        std::vector<std::string> rest(parts.begin() + 1, parts.end());
        if (tag == "v" && rest.size() >= 3) {
            positions.push_back({f32_or_zero(rest[0]), f32_or_zero(rest[1]), f32_or_zero(rest[2])});
        } else if (tag == "vn" && rest.size() >= 3) {
            float v[3] = {f32_or_zero(rest[0]), f32_or_zero(rest[1]), f32_or_zero(rest[2])}, o[3];
            normalize3(v, o);
            normals.push_back({o[0], o[1], o[2]});
        } else if (tag == "vt" && rest.size() >= 2) {
            uvs.push_back({f32_or_zero(rest[0]), f32_or_zero(rest[1])});
        } else if (tag == "f" && rest.size() >= 3) {
            std::vector<uint32_t> face_verts;
            for (const std::string &token : rest) {
                std::vector<std::string> p = split_slash(token);
                uint32_t pi = 0, ti = 0xFFFFFFFFu, ni = 0xFFFFFFFFu, r;
                if (resolve(p[0], positions.size(), &r)) pi = r;
                if (p.size() > 1 && !p[1].empty() && resolve(p[1], uvs.size(), &r)) ti = r;
                if (p.size() > 2 && resolve(p[2], normals.size(), &r)) ni = r;
                auto make = [&](bool with_normal) {
                    orc_vertex v{};
                    if (pi < positions.size()) {
                        v.position[0] = positions[pi][0]; v.position[1] = positions[pi][1]; v.position[2] = positions[pi][2];
                    }
                    v.position[3] = 1.0f;
                    if (with_normal && ni < normals.size()) {
                        v.normal[0] = normals[ni][0]; v.normal[1] = normals[ni][1]; v.normal[2] = normals[ni][2];
                    } else {
                        v.normal[0] = 0.0f; v.normal[1] = 1.0f; v.normal[2] = 0.0f;
                    }
                    if (ti != 0xFFFFFFFFu && ti < uvs.size()) { v.uv[0] = uvs[ti][0]; v.uv[1] = uvs[ti][1]; }
                    return v;
                };
                uint32_t vert_idx;
                if (ni != 0xFFFFFFFFu) {
                    auto key = std::make_tuple(pi, ti, ni);
                    auto it = vert_cache.find(key);
                    if (it != vert_cache.end()) {
                        vert_idx = it->second;
                    } else {
                        vert_idx = (uint32_t)vertices.size();
                        vertices.push_back(make(true));
                        vert_cache.emplace(key, vert_idx);
                    }
                } else {
                    vert_idx = (uint32_t)vertices.size();
                    vertices.push_back(make(false));
                }
                face_verts.push_back(vert_idx);
            }
            for (size_t i = 1; i + 1 < face_verts.size(); ++i) {                     // mesh.rs:580-613
                const uint32_t v0 = face_verts[0], v1 = face_verts[i], v2 = face_verts[i + 1];
                const std::string keys[3] = {rest[0], rest[i], i + 1 < rest.size() ? rest[i + 1] : std::string()};
                const uint32_t vis[3] = {v0, v1, v2};
                for (int k = 0; k < 3; ++k) {
                    std::vector<std::string> p = split_slash(keys[k]);
                    long long dummy;
                    const bool has_norm = p.size() > 2 && !p[2].empty() && parse_i64(p[2], &dummy);
                    if (!has_norm) {
                        const float *p0 = vertices[v0].position, *p1 = vertices[v1].position,
                                    *p2 = vertices[v2].position;
                        const float e1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
                        const float e2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
                        const float cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                             e1[0] * e2[1] - e1[1] * e2[0]};
                        float gn[3];
                        normalize3(cr, gn);
                        float *n = vertices[vis[k]].normal;
                        n[0] = gn[0]; n[1] = gn[1]; n[2] = gn[2]; n[3] = 0.0f;
                    }
                }
                triangles.push_back({{v0, v1, v2}, mat_idx});
            }
        }
    }
    if (vertices.empty() || triangles.empty()) {                                      // mesh.rs:636-638
        delete R;
        set_err("no geometry found after parsing");
        return nullptr;
    }
    *n_vertices = (uint32_t)vertices.size();
    *n_triangles = (uint32_t)triangles.size();
    return R;
}

void orc_obj_copy(void *h, orc_vertex *vertices, orc_triangle *triangles) {
    auto *R = static_cast<ObjResult *>(h);
    std::memcpy(vertices, R->vertices.data(), R->vertices.size() * sizeof(orc_vertex));
    std::memcpy(triangles, R->triangles.data(), R->triangles.size() * sizeof(orc_triangle));
}

void orc_obj_free(void *h) { delete static_cast<ObjResult *>(h); }

// str::parse::<f32> alone (NaN payloads as the reference's: 0x7FC00000, sign
// from the text); returns 0 on a syntax error.
int orc_parse_f32(const char *s, uint32_t len, float *out) {
    return parse_f32(std::string(s, len), out) ? 1 : 0;
}

}  // extern "C"
