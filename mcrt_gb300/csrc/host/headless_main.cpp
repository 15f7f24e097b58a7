// headless_main.cpp — `mcrt_headless --headless <scene.yaml> --output <out.png>
// [--width W] [--height H] [--spp N] [--max-depth D] [--nee]`, the headless
// mode of the reference's command line (src/main.rs:62-80): same flags, same
// exit behaviour (message on stderr, exit code 1 on failure).
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "mcrt_cuda.h"

static const char *next_after(const std::vector<std::string> &a, const char *flag) {
    for (size_t i = 0; i + 1 < a.size(); ++i)
        if (a[i] == flag) return a[i + 1].c_str();
    return nullptr;
}
static bool has(const std::vector<std::string> &a, const char *flag) {
    for (const auto &s : a)
        if (s == flag) return true;
    return false;
}
static uint32_t parse_u32(const char *s) {
    if (!s) return 0;
    char *end = nullptr;
    unsigned long v = strtoul(s, &end, 10);
    return (*end == '\0' && v <= 0xffffffffu) ? (uint32_t)v : 0;
}

int main(int argc, char **argv) {
    std::vector<std::string> args(argv + 1, argv + argc);
    if (!has(args, "--headless")) {
        fprintf(stderr, "error: only --headless mode is available in this build\n");
        return 1;
    }
    const char *scene = next_after(args, "--headless");
    if (!scene) { fprintf(stderr, "error: --headless requires a scene YAML path\n"); return 1; }
    const char *out = next_after(args, "--output");
    if (!out) { fprintf(stderr, "error: --headless mode requires --output <path>\n"); return 1; }
    mcrt_render_opts o{};
    o.max_depth = parse_u32(next_after(args, "--max-depth"));
    if (has(args, "--nee")) o.flags |= MCRT_RENDER_NEE;
    mcrt_status st = mcrt_headless_run(scene, out, parse_u32(next_after(args, "--width")),
                                       parse_u32(next_after(args, "--height")), parse_u32(next_after(args, "--spp")), &o);
    if (st != MCRT_OK) {
        fprintf(stderr, "headless render failed: %s\n", mcrt_last_error(nullptr));
        return 1;
    }
    return 0;
}
