// scene_internal.h — host-side scene types shared by the host translation units.
#pragma once

#include <string>
#include <vector>

#include "mcrt_cuda.h"

namespace mcrt {
// Message returned by mcrt_last_error(NULL) (defined in api.cu).
void set_global_error(const std::string &msg);
}  // namespace mcrt

namespace mcrt_host {

// LoadedScene, src/scene.rs:311-351.
struct LoadedScene {
    std::vector<mcrt_gpu_sphere> spheres;
    mcrt_gpu_material_data materials{};
    std::vector<mcrt_gpu_vertex> vertices;
    std::vector<mcrt_gpu_triangle> triangles;
    std::vector<mcrt_gpu_sphere> emissive_spheres;
    bool has_camera = false;
    float look_from[3] = {0, 0, 0}, look_at[3] = {0, 0, 0};
    float vfov = 60.0f, aperture = 0.0f, focus_dist = 1.0f;
    bool has_env_map = false;
    std::string env_map_path;
    std::vector<std::string> material_names;
    // Mesh objects of a deferred load (MCRT_LOAD_DEFER_MESHES), in object
    // order: the OBJ text, and where its records go between the host records.
    struct MeshRef {
        std::string path, text;
        uint32_t mat_idx = 0;
        mcrt_mesh_transform xf{};
        size_t at_vertex = 0, at_triangle = 0;
    };
    std::vector<MeshRef> meshes;
    bool deferred = false;
};

mcrt_status load_scene(const std::string &text, const std::string &src, LoadedScene *out, std::string *errmsg,
                       bool defer_meshes = false);
// euler_to_mat3 (scene.rs:396-405) of angles in degrees, row-major.
void rotation_matrix(const float deg[3], float m[9]);
// load_obj (mesh.rs:474-642) of OBJ text; on failure err is the reference's
// message after "'<path>'" (" is not valid UTF-8: ..." or ": no geometry ...").
bool load_obj_text(const std::string &content, uint32_t mat_idx, std::vector<mcrt_gpu_vertex> *verts,
                   std::vector<mcrt_gpu_triangle> *tris, std::string *err);
void compute_camera(uint32_t width, uint32_t height, const float lf[3], const float la[3], float vfov_deg,
                    float aperture, float focus_dist, mcrt_camera_uniform *out);
void gradient_env_map(float *data);
void load_env_map_data(const char *scene_path, float *out);
void tonemap_rgba8(const float *rgba, uint32_t n, uint8_t *out);
void tonemap_aces_rgba8(const float *rgba, uint32_t n, uint8_t *out);
bool write_png(const std::string &path, const uint8_t *rgba, uint32_t w, uint32_t h, std::string *err);
bool write_hdr(const std::string &path, const float *rgba, uint32_t w, uint32_t h, std::string *err);

}  // namespace mcrt_host
