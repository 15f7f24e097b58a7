"""Generate the golden fixtures under tests/golden/ (run in the build container,
where the reference checkout is available; the fixtures travel, the reference
does not).

* scene_<name>.npz — the reference's six regression scenes
  (tests/assets/scenes/*.yaml with their *.test.toml sidecars) loaded through
  this library's YAML loader and frozen as GpuSphere/GpuVertex/GpuTriangle/
  GpuMaterialData arrays, the camera (compute_camera at the sidecar size), the
  sidecar [render] parameters and [regression] thresholds.
* test_sky_128x64.hdr / test_sky_128x64.npy — the reference's synthetic HDR sky
  generator (tests/assets/gen_test_skymap.py, imported and run with the
  Makefile's gen-test-assets arguments, Makefile:67-74) at 128x64: its RGBE
  file and the float image it encodes.
* oracle_<name>.npz — the CPU oracle's 32x32, 4-spp renders (running mean,
  f64 sums, G-buffer) and closest hits of 4096 seeded rays for each scene.

Usage: python tests/golden/make_golden.py /path/to/reference-checkout
       (or MCRT_REFERENCE=/path/to/reference-checkout python tests/golden/make_golden.py)
"""
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import mcrt_gb300 as M  # noqa: E402
import pyoracle as O  # noqa: E402

SCENES = ["diffuse_sphere", "mirror_sphere", "glass_sphere", "emissive_box", "cornell_box_mini", "skymap_sphere"]


def read_sidecar(path):
    render, reg, sec = {}, {}, None
    for line in open(path):
        line = line.split("#")[0].strip()
        if not line:
            continue
        if line.startswith("["):
            sec = line.strip("[]").strip()
            continue
        k, v = [x.strip() for x in line.split("=")]
        (render if sec == "render" else reg)[k] = float(v)
    return render, reg


def seeded_rays(camera, n, seed):
    rng = np.random.default_rng(seed)
    o = np.asarray(camera["origin"][:3], np.float32)
    org = (o + rng.normal(scale=0.05, size=(n, 3))).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    # half of the rays aimed through the screen, half uniformly random
    tgt = (camera["lower_left"][:3] + rng.uniform(0, 1, (n, 1)) * camera["horizontal"][:3]
           + rng.uniform(0, 1, (n, 1)) * camera["vertical"][:3]).astype(np.float32)
    d[: n // 2] = tgt[: n // 2] - org[: n // 2]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return M.make_rays(org, d)


def main(ref):
    # ---- synthetic sky through the reference's own generator
    spec = importlib.util.spec_from_file_location("gen_test_skymap", os.path.join(ref, "tests/assets/gen_test_skymap.py"))
    sky = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(sky)
    img = sky.generate_skymap(128, 64, sky_horizon_nit=0.4, sky_zenith_nit=0.8)
    np.save(os.path.join(HERE, "test_sky_128x64.npy"), img)
    sky.save_hdr(img, os.path.join(HERE, "test_sky_128x64.hdr"))
    env_sky = M.load_env_map(os.path.join(HERE, "test_sky_128x64.hdr"))
    env_grad = M.gradient_env_map()
    for name in SCENES:
        yaml = os.path.join(ref, "tests/assets/scenes", name + ".yaml")
        s = M.load_scene_yaml(yaml)
        render, reg = read_sidecar(os.path.join(ref, "tests/assets/scenes", name + ".test.toml"))
        w, h, spp = int(render.get("width", 512)), int(render.get("height", 512)), int(render.get("spp", 64))
        c = s.camera
        cam = M.compute_camera(w, h, c["look_from"], c["look_at"], c["vfov"], c["aperture"], c["focus_dist"])
        np.savez_compressed(os.path.join(HERE, f"scene_{name}.npz"), spheres=s.spheres.view(np.uint8),
                            vertices=s.vertices.view(np.uint8), triangles=s.triangles.view(np.uint8),
                            materials=s.materials.reshape(1).view(np.uint8), camera=cam.reshape(1).view(np.uint8),
                            render=np.array([w, h, spp], np.int64),
                            thresholds=np.array([reg.get("threshold_mse", 0.002), reg.get("threshold_psnr", 38.0)]),
                            uses_sky=np.array([s.env_map_path is not None]))
        env = env_sky if s.env_map_path else env_grad
        osc = O.OracleScene(materials=s.materials, spheres=s.spheres, vertices=s.vertices, triangles=s.triangles,
                            env=env)
        cam32 = M.compute_camera(32, 32, c["look_from"], c["look_at"], c["vfov"], c["aperture"], c["focus_dist"])
        r = osc.render(cam32, 32, 32, 4, 0, 8)
        rays = seeded_rays(cam, 4096, seed=hash(name) % 1000 + 11)
        hits = osc.trace(rays)
        np.savez_compressed(os.path.join(HERE, f"oracle_{name}.npz"), rgba=r["rgba"], sum=r["sum"], gbuf=r["gbuf"],
                            rays=rays.view(np.uint8), hits=hits.view(np.uint8), camera32=cam32.reshape(1).view(np.uint8))
        print(name, len(s.spheres), len(s.triangles), (w, h, spp), "hits:", int((hits["prim"] != 0xFFFFFFFF).sum()))


if __name__ == "__main__":
    ref_dir = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MCRT_REFERENCE")
    if not ref_dir:
        sys.exit("usage: make_golden.py /path/to/reference-checkout (or set MCRT_REFERENCE)")
    main(ref_dir)
