// headless.cpp — headless::run (src/headless.rs:112-386) on the CUDA library:
// parameters (CLI > sidecar [render] > 512/512/64, headless.rs:36-40, :46-77,
// :120-127), scene load, environment map, GPU upload with the BVH built on the
// GPU, camera (default INIT_LOOK_FROM/AT, camera.rs:18-21), spp frames
// 0..spp-1, tone map, PNG.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "mcrt_cuda.h"
#include "scene_internal.h"

namespace {

struct Sidecar {
    uint32_t width = 0, height = 0, spp = 0;
};

// `diffuse_sphere.yaml` -> `diffuse_sphere.test.toml` (headless.rs:69-77); the
// [render] table's integer keys.  Missing or unparsable sidecars are ignored.
Sidecar load_sidecar(const std::string &scene_path) {
    Sidecar s;
    std::string base = scene_path;
    size_t slash = base.find_last_of('/');
    size_t dot = base.find_last_of('.');
    if (dot != std::string::npos && (slash == std::string::npos || dot > slash)) base = base.substr(0, dot);
    std::ifstream f(base + ".test.toml");
    if (!f) return s;
    std::string line, section;
    while (std::getline(f, line)) {
        size_t h = line.find('#');
        if (h != std::string::npos) line = line.substr(0, h);
        auto trim = [](std::string x) {
            size_t b = x.find_first_not_of(" \t\r"), e = x.find_last_not_of(" \t\r");
            return b == std::string::npos ? std::string() : x.substr(b, e - b + 1);
        };
        line = trim(line);
        if (line.empty()) continue;
        if (line[0] == '[') { section = trim(line.substr(1, line.find(']') - 1)); continue; }
        size_t eq = line.find('=');
        if (eq == std::string::npos || section != "render") continue;
        std::string k = trim(line.substr(0, eq)), v = trim(line.substr(eq + 1));
        char *end = nullptr;
        long long x = strtoll(v.c_str(), &end, 10);
        if (*end != '\0' || x < 0 || x > 0xffffffffll) continue;
        if (k == "width") s.width = (uint32_t)x;
        else if (k == "height") s.height = (uint32_t)x;
        else if (k == "spp") s.spp = (uint32_t)x;
    }
    return s;
}

void make_parent_dirs(const std::string &path) {
    for (size_t i = 1; i < path.size(); ++i)
        if (path[i] == '/') mkdir(path.substr(0, i).c_str(), 0755);
}

}  // namespace

extern "C" mcrt_status mcrt_headless_run(const char *scene_path, const char *output_path, uint32_t width,
                                         uint32_t height, uint32_t spp, const mcrt_render_opts *opts) {
    if (!scene_path || !output_path) {
        mcrt::set_global_error("scene and output paths are required");
        return MCRT_ERR_INVALID_ARG;
    }
    Sidecar sc = load_sidecar(scene_path);
    uint32_t W = width ? width : (sc.width ? sc.width : 512);
    uint32_t H = height ? height : (sc.height ? sc.height : 512);
    uint32_t N = spp ? spp : (sc.spp ? sc.spp : 64);
    W = W ? W : 1; H = H ? H : 1; N = N ? N : 1;
    mcrt_loaded_scene *ls = nullptr;
    mcrt_status st = mcrt_scene_load_yaml_ex(scene_path, MCRT_LOAD_DEFER_MESHES, &ls);   // OBJ meshes parse on the device
    if (st != MCRT_OK) return st;
    mcrt_scene_view v;
    mcrt_scene_view_get(ls, &v);
    std::vector<float> env((size_t)MCRT_ENV_MAP_WIDTH * MCRT_ENV_MAP_HEIGHT * 4);
    mcrt_load_env_map(v.env_map_path, env.data());
    mcrt_ctx *ctx = nullptr;
    st = mcrt_create(0, nullptr, &ctx);
    if (st != MCRT_OK) { mcrt_scene_free(ls); return st; }
    mcrt_scene_desc d{};
    d.spheres = v.spheres; d.n_spheres = v.n_spheres;
    d.materials = v.materials;
    d.env_rgba = env.data(); d.env_w = MCRT_ENV_MAP_WIDTH; d.env_h = MCRT_ENV_MAP_HEIGHT;
    d.flags = MCRT_SCENE_DEVICE_MESH;
    st = mcrt_mesh_append_scene(ctx, ls);
    if (st == MCRT_OK) st = mcrt_upload_scene(ctx, &d);
    std::vector<float> img((size_t)W * H * 4);
    if (st == MCRT_OK) {
        float lf[3] = {0.0f, 1.0f, 3.5f}, la[3] = {0.0f, 0.0f, 0.0f};
        float vfov = 60.0f, ap = 0.0f;
        float focus = sqrtf(0.0f * 0.0f + 1.0f * 1.0f + 3.5f * 3.5f);
        if (v.has_camera) {
            for (int i = 0; i < 3; ++i) { lf[i] = v.look_from[i]; la[i] = v.look_at[i]; }
            vfov = v.vfov; ap = v.aperture; focus = v.focus_dist;
        }
        mcrt_camera_uniform cam;
        mcrt_compute_camera(W, H, lf, la, vfov, ap, focus, &cam);
        st = mcrt_render(ctx, &cam, W, H, N, 0, opts, img.data(), nullptr, nullptr);
    }
    if (st != MCRT_OK) mcrt::set_global_error(mcrt_last_error(ctx));
    mcrt_destroy(ctx);
    mcrt_scene_free(ls);
    if (st != MCRT_OK) return st;
    std::vector<uint8_t> px((size_t)W * H * 4);
    mcrt_host::tonemap_rgba8(img.data(), W * H, px.data());
    make_parent_dirs(output_path);
    std::string err;
    if (!mcrt_host::write_png(output_path, px.data(), W, H, &err)) {
        mcrt::set_global_error("I/O error: " + err);
        return MCRT_ERR_IO;
    }
    return MCRT_OK;
}
