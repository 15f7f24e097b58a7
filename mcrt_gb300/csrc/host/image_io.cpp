// image_io.cpp — tone mapping (src/headless.rs:93-98, :350-368) and an RGBA8
// PNG writer standing in for the image crate's save (src/headless.rs:380-382).
// The PNG stream uses stored (uncompressed) deflate blocks, so no compression
// library is needed; any PNG reader decodes it.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../fmath.h"
#include "scene_internal.h"

namespace mcrt_host {

// tonemap_to_u8 per channel after the non-finite -> 0 sanitising.
void tonemap_rgba8(const float *rgba, uint32_t n, uint8_t *out) {
    const float inv_gamma = 1.0f / 2.2f;
    for (uint32_t i = 0; i < n; ++i) {
        for (int c = 0; c < 3; ++c) {
            float v = rgba[4 * (size_t)i + c];
            if (!std::isfinite(v)) v = 0.0f;
            v = std::max(v, 0.0f);
            float mapped = v / (v + 1.0f);                                   // Reinhard
            float g = mcrt::fm_pow(mapped, inv_gamma);                       // gamma 2.2
            g = std::min(std::max(g, 0.0f), 1.0f);
            out[4 * (size_t)i + c] = (uint8_t)std::min(mcrt::fm_f2u_sat(g * 255.0f + 0.5f), 255u);
        }
        out[4 * (size_t)i + 3] = 255;
    }
}

// Rust f32::clamp: NaN passes through.
static inline float rclamp(float x, float lo, float hi) { return x < lo ? lo : (x > hi ? hi : x); }

// screenshot_to_u8 (gpu.rs:1904-1939): ACES filmic (Narkowicz 2016) + sRGB.
void tonemap_aces_rgba8(const float *rgba, uint32_t n, uint8_t *out) {
    for (uint32_t i = 0; i < n; ++i) {
        for (int c = 0; c < 3; ++c) {
            float x = rgba[4 * (size_t)i + c];
            x = std::isnan(x) ? 0.0f : std::max(x, 0.0f);                          // f32::max(0.0)
            float a = rclamp((x * (2.51f * x + 0.03f)) / (x * (2.43f * x + 0.59f) + 0.14f), 0.0f, 1.0f);
            float s;
            if (a <= 0.0f) s = 0.0f;
            else if (a <= 0.0031308f) s = std::min(a * 12.92f, 1.0f);
            else if (a < 1.0f) s = rclamp(1.055f * mcrt::fm_pow(a, 1.0f / 2.4f) - 0.055f, 0.0f, 1.0f);
            else s = 1.0f;
            out[4 * (size_t)i + c] = (uint8_t)std::min(mcrt::fm_f2u_sat(s * 255.0f + 0.5f), 255u);
        }
        out[4 * (size_t)i + 3] = 255;
    }
}

// RGBE encoding as tests/assets/gen_test_skymap.py:44-94 (flat scanlines).
bool write_hdr(const std::string &path, const float *rgba, uint32_t w, uint32_t h, std::string *err) {
    std::vector<uint8_t> px((size_t)w * h * 4, 0);
    for (size_t i = 0; i < (size_t)w * h; ++i) {
        float r = rgba[4 * i], g = rgba[4 * i + 1], b = rgba[4 * i + 2];
        float mx = std::max(r, std::max(g, b));
        if (!(mx > 1e-32f)) continue;
        int e = 0;
        float m = std::frexp(mx, &e);                  // m in [0.5, 1)
        float scale = m * 256.0f / mx;
        const float ch[3] = {r, g, b};
        for (int c = 0; c < 3; ++c) px[4 * i + c] = (uint8_t)std::min(std::max(ch[c] * scale, 0.0f), 255.0f);
        px[4 * i + 3] = (uint8_t)std::min(std::max(e + 128, 0), 255);
    }
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) { *err = "cannot open '" + path + "' for writing"; return false; }
    std::string hdr = "#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y " + std::to_string(h) + " +X " + std::to_string(w) + "\n";
    bool ok = fwrite(hdr.data(), 1, hdr.size(), f) == hdr.size();
    ok = ok && fwrite(px.data(), 1, px.size(), f) == px.size();
    ok = (fclose(f) == 0) && ok;
    if (!ok) *err = "write to '" + path + "' failed";
    return ok;
}

namespace {
uint32_t crc_table[256];
bool crc_init = false;
uint32_t crc32(const uint8_t *p, size_t n, uint32_t c = 0xffffffffu) {
    if (!crc_init) {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t v = i;
            for (int k = 0; k < 8; ++k) v = (v & 1) ? 0xedb88320u ^ (v >> 1) : v >> 1;
            crc_table[i] = v;
        }
        crc_init = true;
    }
    for (size_t i = 0; i < n; ++i) c = crc_table[(c ^ p[i]) & 0xff] ^ (c >> 8);
    return c;
}
void put32(std::vector<uint8_t> &v, uint32_t x) {
    v.push_back((uint8_t)(x >> 24)); v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8)); v.push_back((uint8_t)x);
}
void chunk(std::vector<uint8_t> &out, const char *type, const std::vector<uint8_t> &data) {
    put32(out, (uint32_t)data.size());
    size_t start = out.size();
    out.insert(out.end(), type, type + 4);
    out.insert(out.end(), data.begin(), data.end());
    put32(out, crc32(out.data() + start, out.size() - start) ^ 0xffffffffu);
}
}  // namespace

bool write_png(const std::string &path, const uint8_t *rgba, uint32_t w, uint32_t h, std::string *err) {
    std::vector<uint8_t> raw;
    raw.reserve((size_t)h * (4 * (size_t)w + 1));
    for (uint32_t y = 0; y < h; ++y) {
        raw.push_back(0);   // filter: none
        raw.insert(raw.end(), rgba + (size_t)y * w * 4, rgba + (size_t)(y + 1) * w * 4);
    }
    std::vector<uint8_t> z = {0x78, 0x01};
    size_t pos = 0;
    uint32_t a = 1, b = 0;
    for (uint8_t c : raw) { a = (a + c) % 65521u; b = (b + a) % 65521u; }
    do {
        size_t len = std::min<size_t>(65535, raw.size() - pos);
        bool last = pos + len == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)len); z.push_back((uint8_t)(len >> 8));
        z.push_back((uint8_t)~len); z.push_back((uint8_t)(~len >> 8));
        z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + len);
        pos += len;
    } while (pos < raw.size());
    put32(z, (b << 16) | a);
    std::vector<uint8_t> png = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
    std::vector<uint8_t> ihdr;
    put32(ihdr, w); put32(ihdr, h);
    ihdr.push_back(8); ihdr.push_back(6); ihdr.push_back(0); ihdr.push_back(0); ihdr.push_back(0);
    chunk(png, "IHDR", ihdr);
    chunk(png, "IDAT", z);
    chunk(png, "IEND", {});
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) { *err = "cannot open '" + path + "' for writing"; return false; }
    bool ok = fwrite(png.data(), 1, png.size(), f) == png.size();
    ok = (fclose(f) == 0) && ok;
    if (!ok) *err = "write to '" + path + "' failed";
    return ok;
}

}  // namespace mcrt_host

extern "C" {

mcrt_status mcrt_tonemap_rgba8(const float *rgba, uint32_t n_pixels, uint8_t *out) {
    if ((!rgba || !out) && n_pixels) { mcrt::set_global_error("NULL argument"); return MCRT_ERR_INVALID_ARG; }
    mcrt_host::tonemap_rgba8(rgba, n_pixels, out);
    return MCRT_OK;
}

mcrt_status mcrt_tonemap_aces_rgba8(const float *rgba, uint32_t n_pixels, uint8_t *out) {
    if ((!rgba || !out) && n_pixels) { mcrt::set_global_error("NULL argument"); return MCRT_ERR_INVALID_ARG; }
    mcrt_host::tonemap_aces_rgba8(rgba, n_pixels, out);
    return MCRT_OK;
}

mcrt_status mcrt_write_hdr(const char *path, const float *rgba, uint32_t w, uint32_t h) {
    if (!path || !rgba || w == 0 || h == 0) { mcrt::set_global_error("invalid HDR arguments"); return MCRT_ERR_INVALID_ARG; }
    std::string err;
    if (!mcrt_host::write_hdr(path, rgba, w, h, &err)) { mcrt::set_global_error("I/O error: " + err); return MCRT_ERR_IO; }
    return MCRT_OK;
}

mcrt_status mcrt_write_png(const char *path, const uint8_t *rgba, uint32_t w, uint32_t h) {
    if (!path || !rgba || w == 0 || h == 0) { mcrt::set_global_error("invalid PNG arguments"); return MCRT_ERR_INVALID_ARG; }
    std::string err;
    if (!mcrt_host::write_png(path, rgba, w, h, &err)) { mcrt::set_global_error("I/O error: " + err); return MCRT_ERR_IO; }
    return MCRT_OK;
}

}  // extern "C"
