"""Benchmark: plain path tracing of the procedural displaced-icosphere scene.

Workload (one "step"): the 1,310,720-triangle icosphere (level 8) displaced by
5-octave value noise on a ground plane, 50 % Lambertian / 30 % GGX / 20 %
dielectric material groups, seeded 512x256 HDR smooth-noise environment;
the SAH BVH rebuilt on the GPU, then 1920x1080 at 16 spp, max depth 12.
Metric: Msamples/s = 1920*1080*16 / step time.

  value : device-resident inputs (mcrt_rebuild_bvh + mcrt_render, results kept on the GPU)
  e2e   : through the C ABI with host buffers: mcrt_update_vertices (vertex upload +
          rebuild) and mcrt_render returning the image to the host, copies inside the timer

roofline : the closest-hit kernels (12 launches per frame) against the measured HBM copy
           bandwidth, with the bytes per ray of their own traversal:
           B_ray = 64 N_node + 48 N_tri + 32 + 48 bytes (compact node record, triangle record,
           root box, ray in and hit out), N_node / N_tri = record fetches per ray counted by the
           counting kernels on one frame of this run (outside the timed region; the bounce-0
           warp packets fetch a record once per warp); traffic = the DRAM bytes of a dated ncu
           capture of the same launches; roofline.l2 = L2 traffic (ncu, 960x540 case) against
           this run's L2-resident copy bandwidth; roofline.reference_traversal = the bytes the
           reference traversal would fetch on the reference BVH (oracle statistics), a
           reference figure, not a bound of these kernels.
time_to_relmse : seeded Cornell box 512x512, depth 8: wall time of the render calls until
           the running estimate reaches relMSE 1e-3 against a 4096-spp NEE reference, for
           the reference estimator ("plain"), next-event estimation and NEE + the radiance
           cache (online training inside the time), with the bound of a perfect, free cache
           (ideal_cache_bound); icosphere_cache_time_to_relmse: the same on the displaced
           icosphere (long paths, environment light only).
adjoint  : path-replay adjoint of the GGX Cornell box, 256x256, 32 spp: paths/s
           through mcrt_adjoint with host buffers.
voxel_world : the 256x128x256 voxel world generated, meshed (4.94 M triangles),
           uploaded with a GPU BVH build, rendered 1280x720 8 spp depth 6 with the
           sun and sky, denoised 5x5: device time per stage.
batched_views : 16 uneven views of the voxel world traced together (CUDA graph)
           against one call per view; batched_views_cache_time_to_relmse: the
           same views' time to relMSE 1e-3 with and without the radiance cache.
radiance_cache_mlp : inference and one training step of the cache MLP on 2^20
           queries / samples against the measured bf16 tensor peak.
cpu_baseline : the CPU oracle (a restatement of the reference's path: its single-threaded
           SAH build and the path_trace.wgsl estimator on all host cores) on 128 rows of the
           frame, scaled to one frame; cpu_baselines_other: the same oracle on the Cornell box,
           the voxel world and the adjoint (see cpu_baselines).
parity   : the GPU's images of the same frames equal the oracle's bit for bit (the 128 rows of
           the benchmark frame, the whole Cornell and voxel-world frames).
--impl reference : the oracle over whole frames, per step the single-threaded SAH build and
           the full 1920 x 1080 x 16-spp frame on all host cores (no library of this
           repository loaded).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Profiling cases (--leg bvh_build | cache_mlp | frame | adjoint | nee, and --small)
print their own timings, not a bench line.
Under torchrun each rank renders an independent replica (the path does not
shard: "replicas only"); value = all ranks' samples / max step time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W, H, SPP, DEPTH, LEVEL, SEED = 1920, 1080, 16, 12, 8, 1234
WORKLOAD = "displaced_icosphere_l8_1.31Mtri_1920x1080_16spp_depth12_gpu_rebuild"
# DRAM bytes (read + write) per traced ray of the closest-hit kernels on this
# workload: one ncu capture (dram__bytes_read.sum + dram__bytes_write.sum) of the
# 12 launches of a frame, 10.47 GB / 71.54 M rays
EXTEND_DRAM_CAPTURE = {"bytes_per_ray": 146.3, "captured": "2026-12-04",
                       "profile": "profiles/k_extend_displaced_icosphere_1080p16.md"}
# L2 traffic of the closest-hit launches of bounces 1 and 2 on the 960x540x16 case
# (ncu lts__t_bytes.sum / gpu__time_duration.sum), with the L2 and L1 sector hit rates
EXTEND_L2_CAPTURE = {"gbs": [3389.2, 4355.2], "l2_hit_pct": [72.0, 73.9], "l1_hit_pct": [66.0, 60.8],
                     "captured": "2026-12-04", "case": "960x540, 16 spp, bounces 1 and 2",
                     "profile": "profiles/k_extend_displaced_icosphere_1080p16.md"}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="mcrt", choices=["mcrt", "reference"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--small", action="store_true",
                   help="same scene at 480x270, 4 spp: the profiling case (not a bench line)")
    p.add_argument("--mid", action="store_true",
                   help="same scene at 960x540, 16 spp (2 GB of path state): the profiling case for counter "
                        "sets that need several passes (not a bench line)")
    p.add_argument("--leg", choices=["bvh_build", "cache_mlp", "frame", "adjoint", "nee", "roofline_inputs",
                                     "cache_race", "ingest"],
                   help="profiling case: only the GPU BVH builds of the workload's mesh, only the "
                        "radiance-cache MLP (2^18 queries), only frames of the workload (autotune: 8 "
                        "frames, then rebuild + render with the chosen closest-hit variant, 12 extend "
                        "launches per frame), only the adjoint calls of the adjoint leg, or only renders "
                        "of the time-to-relMSE scene (Cornell 512x512, 128 spp, depth 8) without and with "
                        "NEE; prints its timings, not a bench line")
    a = p.parse_args()
    global W, H, SPP, WORKLOAD
    if a.small:
        W, H, SPP = 480, 270, 4
        WORKLOAD = WORKLOAD.replace("1920x1080_16spp", "480x270_4spp")
    elif a.mid:
        W, H = 960, 540
        WORKLOAD = WORKLOAD.replace("1920x1080", "960x540")
    a.small = a.small or a.mid
    return a


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init(n):
    from mcrt_gb300 import replicas
    return replicas.init("nccl")


def max_over_ranks(x, world):
    from mcrt_gb300 import replicas
    return replicas.max_over_ranks(x, device="cuda") if world > 1 else x


def barrier(world):
    from mcrt_gb300 import replicas
    replicas.barrier()


def make_scene():
    from mcrt_gb300 import scenes
    return scenes.displaced_icosphere(seed=SEED, level=LEVEL, width=W, height=H)


def camera(sc):
    import mcrt_gb300 as M
    c = sc["camera"]
    return M.compute_camera(W, H, c["look_from"], c["look_at"], c["vfov"], c["aperture"])


# ------------------------------------------------------------------ CPU oracle (baseline / reference arm)
def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    return O


def oracle_camera(O, c, w, h):
    return O.compute_camera(w, h, c["look_from"], c["look_at"], c["vfov"], c.get("aperture", 0.0))


def oracle_strips(h, n_rects, rows):
    return [int((k + 0.5) * h / n_rects) - rows // 2 for k in range(n_rects)]


def cpu_frame_sample(sc, cam, rows_total=128, threads=0, stats=False):
    """Reference SAH build (single thread, as the reference runs it) + the path_trace.wgsl
    estimator on `rows_total` image rows in 8 strips spread over the frame (all host cores).
    Returns (build s, render s, rows, strips [(y0, mean rgba)], traversal stats, oracle scene)."""
    O = _oracle()
    t0 = time.perf_counter()
    osc = O.OracleScene(materials=sc["materials"], vertices=sc["vertices"], triangles=sc["triangles"], env=sc["env"])
    t_build = time.perf_counter() - t0
    rows = max(1, rows_total // 8)
    t_render, st, strips = 0.0, dict(rays=0, nodes=0, prims=0), []
    for y0 in oracle_strips(H, 8, rows):
        t1 = time.perf_counter()
        r = osc.render(cam, W, H, SPP, 0, DEPTH, threads=threads, rect=(0, y0, W, rows), stats=stats)
        t_render += time.perf_counter() - t1
        strips.append((y0, r["rgba"]))
        if stats:
            for key in st:
                st[key] += r["stats"][key]
    return t_build, t_render, rows * 8, strips, st, osc


def run_reference(args):
    """The reference's path on the host cores: its single-threaded SAH build and the
    path_trace.wgsl estimator (the oracle, a C++ restatement: the reference itself is Rust +
    WGSL and has no CPU renderer) over the whole 1920 x 1080 x 16-spp frame on every core,
    per step.  Camera and scene come from the oracle and numpy; no library of this
    repository is loaded."""
    rank = int(os.environ.get("RANK", 0))
    if rank != 0:
        return
    O = _oracle()
    sc = make_scene()
    c = sc["camera"]
    cam = oracle_camera(O, c, W, H)
    cores = os.cpu_count() or 1
    times, builds = [], []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        osc = O.OracleScene(materials=sc["materials"], vertices=sc["vertices"], triangles=sc["triangles"],
                            env=sc["env"])
        t1 = time.perf_counter()
        osc.render(cam, W, H, SPP, i * SPP, DEPTH, threads=cores)
        t2 = time.perf_counter()
        if i >= args.warmup:
            times.append(t2 - t0)
            builds.append(t1 - t0)
        del osc
    t = sum(times) / len(times)
    value = W * H * SPP / t / 1e6
    sample = (f"whole frames: reference SAH build of all {len(sc['triangles'])} triangles (1 thread, "
              f"{sum(builds) / len(builds):.2f} s) + all {H} rows x {W} px x {SPP} spp, depth {DEPTH} "
              f"({t - sum(builds) / len(builds):.2f} s on {cores} threads), per step")
    print(json.dumps({
        "impl": "reference", "metric": "Msamples/s", "value": round(value, 4), "unit": "Msamples/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1000, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "width": W, "height": H, "spp": SPP, "max_depth": DEPTH,
                   "triangles": int(len(sc["triangles"])), "seed": SEED},
        "cpu_baseline": {"value": round(value, 4), "unit": "Msamples/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def cpu_baselines(M, ctx, quality, cores):
    """The oracle on the host cores for the other workloads, each image compared bit for
    bit with the GPU's render of the same frames:
      cornell : the seeded Cornell box 512 x 512, depth 8, reference estimator, 8 of its 64
                frames of the whole image (Msamples/s and Mrays/s are rates of that sample);
      cornell time to relMSE 1e-3 : the estimators are bit-identical on both sides, so the CPU
                needs the spp the GPU leg needed; its time is that spp x the measured CPU
                seconds per spp (8 frames of the whole image, each estimator), i.e. projected;
      voxel_world : 1280 x 720, 8 spp, depth 6, sun + sky, NEE: the reference SAH build of the
                4.94 M triangles (1 thread) and the whole frame (all cores);
      adjoint : the oracle's brute-force (forward-mode) gradient of the GGX Cornell box,
                256 x 256, 32 spp, NEE, 256 parameters: paths/s of the whole call."""
    from mcrt_gb300 import scenes
    O = _oracle()
    env = M.gradient_env_map()
    out = {"cores": cores}
    parity = {}
    # ---- Cornell box
    sc = scenes.cornell_box(SEED)
    c = sc["camera"]
    cam = oracle_camera(O, c, 512, 512)
    osc = O.OracleScene(materials=sc["materials"], vertices=sc["vertices"], triangles=sc["triangles"], env=env)
    per_spp = {}
    for name, nee in (("plain", False), ("nee", True)):
        t0 = time.perf_counter()
        r = osc.render(cam, 512, 512, 8, 0, 8, threads=cores, stats=True, nee=nee)
        dt = time.perf_counter() - t0
        per_spp[name] = dt / 8
        if name == "plain":
            out["cornell"] = {"msamples_per_s": round(512 * 512 * 8 / dt / 1e6, 3),
                              "mrays_per_s": round(r["stats"]["rays"] / dt / 1e6, 3),
                              "sample": f"512x512 x 8 of 64 spp, depth 8, reference estimator, {cores} threads"}
        ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"], env=env)
        g = ctx.render(cam, 512, 512, 8, max_depth=8, nee=nee, outputs=("rgba",))["rgba"]
        parity[f"cornell_{name}"] = {"pixels": 512 * 512, "spp": 8,
                                     "bit_exact": bool(np.array_equal(g.view(np.uint32), r["rgba"].view(np.uint32)))}
    if quality:
        proj = {}
        for name in ("plain", "nee"):
            spp_needed = quality[name]["spp"]
            proj[name] = {"spp": spp_needed, "s": round(spp_needed * per_spp[name], 2),
                          "cpu_s_per_spp": round(per_spp[name], 4)}
        out["cornell_time_to_relmse"] = dict(proj, kind="projected: measured CPU s per spp x the spp the "
                                                     "bit-identical estimator needed on the GPU")
    # ---- voxel world
    w = scenes.voxel_world(SEED)
    p = w["params"]
    cw = oracle_camera(O, w["camera"], w["width"], w["height"])
    v, t = O.world_mesh(O.world_generate(p), w["block_material"], greedy=False, chunk_x0=p["chunk_x0"],
                        chunk_z0=p["chunk_z0"])
    t0 = time.perf_counter()
    osc = O.OracleScene(materials=w["materials"], vertices=v, triangles=t, env=env, sun_dir=w["sun_dir"],
                        sun_irradiance=w["sun_irradiance"])
    t_build = time.perf_counter() - t0
    t0 = time.perf_counter()
    r = osc.render(cw, w["width"], w["height"], w["spp"], 0, w["max_depth"], threads=cores, stats=True, nee=True)
    t_render = time.perf_counter() - t0
    del osc
    n = w["width"] * w["height"] * w["spp"]
    out["voxel_world"] = {"msamples_per_s": round(n / t_render / 1e6, 3),
                          "mrays_per_s": round(r["stats"]["rays"] / t_render / 1e6, 3),
                          "render_s": round(t_render, 2), "bvh_build_s": round(t_build, 2),
                          "triangles": int(len(t)),
                          "sample": f"whole frame 1280x720 x 8 spp, depth 6, NEE, {cores} threads; "
                                    "reference SAH build on 1 thread"}
    ctx.world_generate(p)
    ctx.world_mesh(w["block_material"], greedy=False)
    ctx.upload_scene(materials=w["materials"], env=env, sun_dir=w["sun_dir"], sun_irradiance=w["sun_irradiance"],
                     world_mesh=True)
    g = ctx.render(cw, w["width"], w["height"], w["spp"], max_depth=w["max_depth"], nee=True, outputs=("rgba",))["rgba"]
    parity["voxel_world"] = {"pixels": w["width"] * w["height"], "spp": w["spp"],
                             "bit_exact": bool(np.array_equal(g.view(np.uint32), r["rgba"].view(np.uint32)))}
    # ---- adjoint
    sc = scenes.cornell_box_ggx(SEED)
    c = sc["camera"]
    cam = oracle_camera(O, c, 256, 256)
    osc = O.OracleScene(materials=sc["materials"], vertices=sc["vertices"], triangles=sc["triangles"], env=env)
    d_img = np.random.default_rng(0).standard_normal((256, 256, 4)).astype(np.float32)
    t0 = time.perf_counter()
    osc.adjoint(cam, 256, 256, 32, d_img, max_depth=8, nee=True, threads=cores)
    dt = time.perf_counter() - t0
    out["adjoint"] = {"paths_per_s": round(256 * 256 * 32 / dt, 1), "s": round(dt, 3),
                      "sample": f"whole call 256x256 x 32 spp, depth 8, NEE, 256 parameters, {cores} threads"}
    return out, parity


# ------------------------------------------------------------------ GPU arm
def nee_rate(M, ctx, n_warm=1, n_calls=2, w=512, h=512, spp=128, depth=8):
    """Renders of the time-to-relMSE scene (seeded Cornell box, 512 x 512, 128
    spp, depth 8) with the reference estimator and with NEE + MIS: per-kernel
    device times of each call (the NEE shadow rays go through the persistent
    any-hit traversal)."""
    from mcrt_gb300 import scenes
    sc = scenes.cornell_box(SEED)
    c = sc["camera"]
    cam = M.compute_camera(w, h, c["look_from"], c["look_at"], c["vfov"], 0.0)
    ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"],
                     env=M.gradient_env_map())
    out = {"leg": "nee", "workload": f"cornell_box_seed{SEED}_{w}x{h}_{spp}spp_depth{depth}"}
    for name, nee in (("plain", False), ("nee", True)):
        calls = []
        for i in range(n_warm + n_calls):
            ctx.render(cam, w, h, spp, first_frame=i * spp, max_depth=depth, nee=nee, outputs=())
            t = ctx.timings()
            calls.append({k: round(t[k], 3) for k in ("extend_ms", "shade_ms", "shadow_ms", "total_ms")} |
                         {"rays": t["rays"], "shadow_rays": t["shadow_rays"],
                          "msamples_per_s": round(w * h * spp / t["total_ms"] / 1e3, 1)})
        out[name] = calls[n_warm:]
    return out


def race(read_sum, render, ref, target, max_spp, warm=None, growth=1.1, min_chunk=1, denom_ref=None):
    """Wall time for an estimator's running estimate to reach relMSE <= target
    (mean over pixels and channels of (x - r)^2 / (r^2 + 1e-2)) against ref.
    render(spp, first_frame, keep) adds spp frames to the device accumulation and
    returns when they are done (the library's calls are synchronous); its wall
    time is summed, with warm() (the cache's warm-up training) inside it.  The
    estimate grows in chunks of about 10 % (growth); read_sum() reads the f64
    sums between chunks, outside the time.  relMSE of an unbiased estimate falls
    as 1/spp, so the crossing is interpolated linearly in 1/relMSE between the
    last two checkpoints (spp_at_target, s_at_target), free of the chunk size.
    denom_ref: the image whose squares normalise the error (default ref)."""
    total, sec, hist = 0, 0.0, []
    den = (ref if denom_ref is None else denom_ref) ** 2 + 1e-2
    if warm:
        t0 = time.perf_counter()
        warm()
        sec += time.perf_counter() - t0
    rel = None
    while total < max_spp:
        chunk = min(max(min_chunk, int(total * (growth - 1.0))), max_spp - total)
        t0 = time.perf_counter()
        render(chunk, total, total > 0)
        sec += time.perf_counter() - t0
        total += chunk
        x = read_sum() / total
        rel = float(np.mean((x - ref) ** 2 / den))
        hist.append((total, sec, rel))
        if rel <= target:
            break
    out = {"spp": total, "s": round(sec, 4), "relmse": round(rel, 7), "reached": rel <= target,
           "checkpoints": len(hist)}
    if rel <= target:
        n1, s1, r1 = hist[-1]
        n0, s0, r0 = hist[-2] if len(hist) > 1 else (0, 0.0, float("inf"))
        a0 = 0.0 if r0 == float("inf") else 1.0 / r0
        f = (1.0 / target - a0) / max(1.0 / r1 - a0, 1e-30)
        f = min(max(f, 0.0), 1.0)
        out["spp_at_target"] = round(n0 + f * (n1 - n0), 1)
        out["s_at_target"] = round(s0 + f * (s1 - s0), 4)
    return out


def _speedups(out, base, names):
    for name in names:
        if out[base]["reached"] and out[name]["reached"]:
            out[f"speedup_{name}_vs_{base}"] = round(out[base]["s_at_target"] / out[name]["s_at_target"], 3)


def ideal_cache_bound(render, read, full_ref, full, target, max_spp, vertices=(1, 2), ref_spp=4096, min_chunk=2):
    """The speedup a perfect and free radiance cache could reach.  A path
    stopped at vertex k (after its next-event sample) and given the exact
    expected radiance of its remainder has at least the variance of the path
    truncated there, and the cost of the truncated path.  render(spp, first,
    keep, depth) renders with max_depth; for each k the tracer truncated to
    depth k + 1 races (wall time) against its own ref_spp reference, its error
    normalised by the full image (full_ref: the remainder a perfect cache adds
    back is the difference of the two references), and full["s_at_target"] /
    its time bounds the speedup of any cache that stops paths at vertex k.
    The bound factors into the cost per sample and the samples needed."""
    out = {}
    for k in vertices:
        render(ref_spp, 1 << 20, False, k + 1)
        ref = read() / ref_spp
        r = race(read, lambda spp, first, keep: render(spp, first, keep, k + 1), ref, target, max_spp,
                 min_chunk=min_chunk, denom_ref=full_ref)
        if r["reached"]:
            r["ideal_speedup"] = round(full["s_at_target"] / r["s_at_target"], 3)
            r["cost_per_spp_ratio"] = round((full["s"] / full["spp"]) / (r["s"] / r["spp"]), 3)
            r["spp_ratio"] = round(full["spp_at_target"] / r["spp_at_target"], 3)
        out[f"stop_at_vertex_{k}"] = r
    return out


def time_to_relmse(M, ctx, target=1e-3, w=512, h=512, depth=8, ref_spp=4096, max_spp=16384, bound=True,
                   cache_cfgs=None, plain=True):
    """Seeded Cornell box at 512 x 512, depth 8: wall time for the running
    estimate to reach relMSE <= target against a 4096-spp NEE reference (race),
    for the reference estimator ("plain"), NEE + MIS ("nee") and NEE + the
    online-trained radiance cache ("cache", warm-up and training in the time)."""
    from mcrt_gb300 import scenes
    sc = scenes.cornell_box(SEED)
    c = sc["camera"]
    cam = M.compute_camera(w, h, c["look_from"], c["look_at"], c["vfov"], 0.0)
    ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"],
                     env=M.gradient_env_map())
    ref = ctx.render(cam, w, h, ref_spp, first_frame=1 << 20, max_depth=depth, nee=True, outputs=("sum",))["sum"]
    ref /= ref_spp
    out = {"workload": f"cornell_box_seed{SEED}_{w}x{h}_depth{depth}", "target_relmse": target,
           "reference": f"NEE {ref_spp} spp, independent frames", "time": "wall clock of the render calls"}
    cache_cfgs = cache_cfgs or [dict(query_vertex=2, train_stride=64, train_steps=8, train_batch=1 << 14, lr=1e-3)]
    read = lambda: ctx.read_accum()[1]
    runs = ([("plain", False, None)] if plain else []) + [("nee", True, None)] + \
        [("cache" if k == 0 else f"cache_{k}", True, cfg) for k, cfg in enumerate(cache_cfgs)]
    for name, nee, cache_cfg in runs:
        warm = None
        cache = cache_cfg is not None
        if cache:
            ctx.cache_config(**cache_cfg)
            ctx.cache_init(0)

            def warm():
                for i in range(5):
                    ctx.render(cam, w, h, 8, first_frame=(1 << 21) + 8 * i, max_depth=depth, nee=True, cache=True,
                               outputs=())
        out[name] = race(read, lambda spp, first, keep: ctx.render(
            cam, w, h, spp, first_frame=first, max_depth=depth, nee=nee, keep=keep, outputs=(), cache=cache),
            ref, target, max_spp, warm=warm, min_chunk=4)
        if cache:
            out[name]["judged_bias"] = [round(b, 4) for b in ctx.cache_stats()["bias"]]
            out[name]["config"] = dict(cache_cfg, warmup="5 passes x 8 spp, in the time")
    caches = [r[0] for r in runs if r[2] is not None]
    if plain:
        _speedups(out, "plain", ["nee"] + caches)
    _speedups(out, "nee", caches)
    if bound and out["nee"]["reached"]:
        out["ideal_cache_bound_vs_nee"] = ideal_cache_bound(
            lambda spp, first, keep, d: ctx.render(cam, w, h, spp, first_frame=first, max_depth=d, nee=True,
                                                   keep=keep, outputs=()),
            read, ref, out["nee"], target, max_spp)
    return out


def icosphere_cache_relmse(M, ctx, target=1e-3, ref_spp=4096, max_spp=4096, configs=None, bound=True):
    """The displaced icosphere (1.31 M triangles, 1920 x 1080, depth 12; lit by
    its environment map alone, so next-event estimation has no light to sample
    and the plain tracer is the tracer without the cache): wall time to relMSE
    <= target against a 4096-spp reference for the tracer without and with the
    online-trained radiance cache (race).  Long paths through dielectric and
    GGX surfaces: what the cache stops is up to 10 more bounces per path."""
    sc = make_scene()
    c = sc["camera"]
    cam = M.compute_camera(W, H, c["look_from"], c["look_at"], c["vfov"], c["aperture"])
    ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"], env=sc["env"])
    ref = ctx.render(cam, W, H, ref_spp, first_frame=1 << 20, max_depth=DEPTH, outputs=("sum",))["sum"] / ref_spp
    out = {"workload": f"displaced_icosphere_l8_1.31Mtri_{W}x{H}_depth{DEPTH}", "target_relmse": target,
           "reference": f"{ref_spp} spp, independent frames", "time": "wall clock of the render calls"}
    read = lambda: ctx.read_accum()[1]
    out["plain"] = race(read, lambda spp, first, keep: ctx.render(
        cam, W, H, spp, first_frame=first, max_depth=DEPTH, keep=keep, outputs=(), graph=True),
        ref, target, max_spp, min_chunk=2)
    for k, cfg in enumerate(configs or [dict(query_vertex=1, train_stride=64, train_steps=16, train_batch=1 << 14,
                                             lr=3e-3)]):
        ctx.cache_config(**cfg)
        ctx.cache_init(0)

        def warm():
            for i in range(4):
                ctx.render(cam, W, H, 2, first_frame=(1 << 21) + 2 * i, max_depth=DEPTH, cache=True, graph=True,
                           outputs=())
        name = "cache" if k == 0 else f"cache_{k}"
        out[name] = race(read, lambda spp, first, keep: ctx.render(
            cam, W, H, spp, first_frame=first, max_depth=DEPTH, keep=keep, outputs=(), cache=True, graph=True),
            ref, target, max_spp, warm=warm, min_chunk=2)
        out[name]["judged_bias"] = [round(b, 4) for b in ctx.cache_stats()["bias"]]
        out[name]["config"] = dict(cfg, warmup="4 passes x 2 spp, in the time")
        _speedups(out, "plain", (name,))
    if bound and out["plain"]["reached"]:
        out["ideal_cache_bound_vs_plain"] = ideal_cache_bound(
            lambda spp, first, keep, d: ctx.render(cam, W, H, spp, first_frame=first, max_depth=d, keep=keep,
                                                   outputs=(), graph=True),
            read, ref, out["plain"], target, max_spp)
    return out


def adjoint_rate(M, ctx, stream, n_warm=3, n_calls=10, w=256, h=256, spp=32, depth=8):
    """Path-replay adjoint of the GGX Cornell box at 256 x 256, 32 spp (primal +
    replay), NEE: paths per second through mcrt_adjoint with host buffers
    (d_image in, gradient out), CUDA events on the library's stream."""
    import torch
    from mcrt_gb300 import scenes
    sc = scenes.cornell_box_ggx(SEED)
    c = sc["camera"]
    cam = M.compute_camera(w, h, c["look_from"], c["look_at"], c["vfov"], 0.0)
    ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"],
                     env=M.gradient_env_map())
    d_img = np.random.default_rng(0).standard_normal((h, w, 4)).astype(np.float32)
    for i in range(n_warm):
        ctx.adjoint(cam, w, h, spp, d_img, first_frame=i * spp, max_depth=depth, nee=True)
    ms, dev = [], []
    for i in range(n_calls):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.adjoint(cam, w, h, spp, d_img, first_frame=(n_warm + i) * spp, max_depth=depth, nee=True)
        b.record(stream)
        b.synchronize()
        ms.append(a.elapsed_time(b))
        dev.append(ctx.timings()["total_ms"])
    t = sum(ms) / len(ms)
    return {"value": round(w * h * spp / (t / 1000.0), 1), "unit": "paths/s", "ms_per_call": round(t, 3),
            "device_ms_per_call": round(sum(dev) / len(dev), 3), "calls": n_calls,
            "workload": f"cornell_box_ggx_seed{SEED}_{w}x{h}_{spp}spp_depth{depth}_nee",
            "params": "64 material slots x (albedo rgb, roughness)"}


def voxel_world_rate(M, ctx, stream, n_warm=2, n_steps=3):
    """The voxel world 256 x 128 x 256: generate on the GPU, mesh the exposed
    faces (4-6 M triangles), upload + GPU BVH build, render 1280 x 720, 8 spp,
    depth 6 with the sun (NEE) and the sky, then the 5 x 5 denoiser
    (sigma_color 0.1, sigma_normal 0.2).  Device times per stage (CUDA events)."""
    import torch
    from mcrt_gb300 import scenes
    w = scenes.voxel_world(SEED)
    c = w["camera"]
    W2, H2, S2, D2 = w["width"], w["height"], w["spp"], w["max_depth"]
    cam = M.compute_camera(W2, H2, c["look_from"], c["look_at"], c["vfov"], 0.0)
    env = M.gradient_env_map()

    def stage(fn):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        out = fn()
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b), out

    rows = []
    for i in range(n_warm + n_steps):
        t_gen, _ = stage(lambda: ctx.world_generate(w["params"]))
        t_mesh, (nv, nt) = stage(lambda: ctx.world_mesh(w["block_material"], greedy=False))
        t_up, _ = stage(lambda: ctx.upload_scene(materials=w["materials"], env=env, sun_dir=w["sun_dir"],
                                                 sun_irradiance=w["sun_irradiance"], world_mesh=True))
        t_r, _ = stage(lambda: ctx.render(cam, W2, H2, S2, first_frame=i * S2, max_depth=D2, nee=True, outputs=()))
        t_dn, _ = stage(lambda: ctx.denoise_accum(read_back=False, **w["denoise"]))
        if i >= n_warm:
            rows.append((t_gen, t_mesh, t_up, t_r, t_dn))
    m = [sum(r[k] for r in rows) / len(rows) for k in range(5)]
    total = sum(m)
    return {"workload": f"voxel_world_256x128x256_seed{SEED}_{W2}x{H2}_{S2}spp_depth{D2}_sun_nee_denoise5x5",
            "triangles": int(nt), "ms": {"generate": round(m[0], 3), "mesh": round(m[1], 3),
                                         "upload_and_bvh": round(m[2], 3), "render": round(m[3], 3),
                                         "denoise": round(m[4], 3), "total": round(total, 3)},
            "render_msamples_per_s": round(W2 * H2 * S2 / (m[3] / 1000.0) / 1e6, 1),
            "frame_msamples_per_s": round(W2 * H2 * S2 / (total / 1000.0) / 1e6, 1)}


def batched_views_rate(M, ctx, stream, spp=4, n_warm=1, n_steps=3):
    """16 seeded views of uneven sizes (256^2 .. 1920 x 1080) over the voxel
    world (the scene of voxel_world_rate, left uploaded), depth 6, sun NEE:
    all views in one batched render per frame (each bounce one launch over every
    view, the passes replayed as a CUDA graph) against the same views rendered
    one call each."""
    import torch
    from mcrt_gb300 import scenes
    w = scenes.voxel_world(SEED)
    vs = scenes.world_views(w, seed=SEED)
    views = [(M.compute_camera(v["width"], v["height"], v["look_from"], v["look_at"], v["vfov"], 0.0),
              v["width"], v["height"]) for v in vs]
    depth = w["max_depth"]
    px = sum(v[1] * v[2] for v in views)

    def timed(fn):
        ms = []
        for i in range(n_warm + n_steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn(i)
            b.record(stream)
            b.synchronize()
            if i >= n_warm:
                ms.append(a.elapsed_time(b))
        return sum(ms) / len(ms)

    t_batch = timed(lambda i: ctx.render_views(views, spp, first_frame=i * spp, max_depth=depth, nee=True, graph=True,
                                               read_back=False))
    t_seq = timed(lambda i: [ctx.render(cam, vw, vh, spp, first_frame=i * spp, max_depth=depth, nee=True, outputs=())
                             for cam, vw, vh in views])
    return {"workload": f"voxel_world_16_views_seed{SEED}_{px / 1e6:.2f}Mpix_{spp}spp_depth{depth}_sun_nee",
            "batched_graph_ms": round(t_batch, 3), "per_view_calls_ms": round(t_seq, 3),
            "batched_msamples_per_s": round(px * spp / (t_batch / 1000.0) / 1e6, 1),
            "per_view_msamples_per_s": round(px * spp / (t_seq / 1000.0) / 1e6, 1),
            "speedup": round(t_seq / t_batch, 3)}


def scenes_voxel_upload(M, ctx):
    """Generate, mesh and upload the voxel world (the scene of voxel_world_rate)."""
    from mcrt_gb300 import scenes
    w = scenes.voxel_world(SEED)
    ctx.world_generate(w["params"])
    ctx.world_mesh(w["block_material"], greedy=False)
    ctx.upload_scene(materials=w["materials"], env=M.gradient_env_map(), sun_dir=w["sun_dir"],
                     sun_irradiance=w["sun_irradiance"], world_mesh=True)
    return w


def views_cache_relmse(M, ctx, target=1e-3, ref_spp=4096, max_spp=1024, bound=True):
    """The batched workload with the radiance cache: the 16 uneven views of the
    voxel world (left uploaded by voxel_world_rate), depth 6, sun NEE + sky.
    Wall time for the views' estimates to reach relMSE <= target (over every
    pixel of every view) against a 4096-spp NEE reference (race), without the
    cache and with the online-trained cache (warm-up and training inside the
    time), both replaying their passes as CUDA graphs (the cached passes with
    their training)."""
    from mcrt_gb300 import scenes
    w = scenes.voxel_world(SEED)
    vs = scenes.world_views(w, seed=SEED)
    views = [(M.compute_camera(v["width"], v["height"], v["look_from"], v["look_at"], v["vfov"], 0.0),
              v["width"], v["height"]) for v in vs]
    depth = w["max_depth"]
    px = sum(v[1] * v[2] for v in views)
    ctx.render_views(views, ref_spp, first_frame=1 << 20, max_depth=depth, nee=True, graph=True, read_back=False)
    ref = ctx.read_accum()[1].reshape(-1, 3) / ref_spp
    out = {"workload": f"voxel_world_16_views_seed{SEED}_{px / 1e6:.2f}Mpix_depth{depth}_sun_nee",
           "target_relmse": target, "reference": f"NEE {ref_spp} spp, independent frames",
           "time": "wall clock of the render calls"}
    cache_cfg = dict(query_vertex=2, train_stride=256, train_steps=16, train_batch=1 << 14, lr=3e-3)
    read = lambda: ctx.read_accum()[1].reshape(-1, 3)
    for name, cache in (("nee", False), ("nee_cache", True)):
        warm = None
        if cache:
            ctx.cache_config(**cache_cfg)
            ctx.cache_init(0)

            def warm():
                for i in range(10):
                    ctx.render_views(views, 2, first_frame=(1 << 21) + 2 * i, max_depth=depth, nee=True, cache=True,
                                     graph=True, read_back=False)
        out[name] = race(read, lambda spp, first, keep: ctx.render_views(
            views, spp, first_frame=first, max_depth=depth, nee=True, keep=keep, cache=cache, graph=True,
            read_back=False), ref, target, max_spp, warm=warm, min_chunk=2)
        if cache:
            out[name]["judged_bias"] = [round(b, 4) for b in ctx.cache_stats()["bias"]]
    out["nee_cache"]["config"] = dict(cache_cfg, warmup="10 passes x 2 spp over all views, in the time")
    _speedups(out, "nee", ("nee_cache",))
    if bound and out["nee"]["reached"]:
        out["ideal_cache_bound_vs_nee"] = ideal_cache_bound(
            lambda spp, first, keep, d: ctx.render_views(views, spp, first_frame=first, max_depth=d, nee=True,
                                                         keep=keep, graph=True, read_back=False),
            read, ref, out["nee"], target, max_spp)
    return out


MLP_FLOP_INFER = 2 * (96 * 64 + 4 * 64 * 64 + 64 * 16)                    # per query
MLP_FLOP_TRAIN = MLP_FLOP_INFER + 2 * (16 * 64 + 4 * 64 * 64) + MLP_FLOP_INFER   # + backward data + weight grads


def ingest_rate(M, ctx, n_warm=1, n_steps=3, cpu=True):
    """Scene ingestion on the device: the benchmark meshes as Wavefront OBJ text
    (host bytes) parsed into the device mesh by mcrt_mesh_append_obj (load_obj,
    mesh.rs:474-642; the call's wall time, text copy included), then the GPU
    BVH build of the parsed mesh (mcrt_upload_scene with the device mesh).
    Parity: the icosphere's records equal the oracle's load_obj bit for bit;
    the voxel world's parsed triangles equal the device mesher's own.  CPU
    baselines: the oracle's load_obj (a restatement of the reference's
    single-threaded loader) and the library's host loader, 1 thread each."""
    from mcrt_gb300 import scenes
    out = {}
    sc = scenes.displaced_icosphere(SEED, LEVEL)
    texts = {"displaced_icosphere_l8": scenes.displaced_icosphere_obj(SEED, LEVEL)}
    wd = scenes.voxel_world(SEED)
    ctx.world_generate(wd["params"])
    ctx.world_mesh(wd["block_material"], greedy=False)
    wv, wt = ctx.world_read_mesh()
    texts["voxel_world_faces"] = scenes.world_mesh_obj(wv, wt)
    for name, text in texts.items():
        rows = []
        for i in range(n_warm + n_steps):
            ctx.mesh_reset()
            t0 = time.perf_counter()
            nv, nt = ctx.mesh_append_obj(text)
            wall = (time.perf_counter() - t0) * 1e3
            st = ctx.mesh_obj_stats()
            ctx.upload_scene(materials=sc["materials"], device_mesh=True)
            if i >= n_warm:
                rows.append((wall, st["h2d_ms"], st["kernel_ms"], ctx.timings()["bvh_build_ms"]))
        m = [statistics.median(r[k] for r in rows) for k in range(4)]
        mb = len(text) / 1e6
        r = {"text_mb": round(mb, 1), "lines": int(st["lines"]), "face_tokens": int(st["tokens"]),
             "vertices": int(nv), "triangles": int(nt), "kernel_launches": int(st["launches"]),
             "wall_ms": round(m[0], 3), "h2d_ms": round(m[1], 3), "kernel_ms": round(m[2], 3),
             "text_gbs_wall": round(mb / m[0], 2), "text_gbs_kernels": round(mb / m[2], 2),
             "h2d_gbs": round(mb / m[1], 2), "mtriangles_per_s_wall": round(nt / m[0] / 1e3, 1),
             "bvh_build_ms": round(m[3], 3), "ingest_and_build_ms": round(m[0] + m[3], 3)}
        v_d, t_d = ctx.mesh_read()
        if name == "displaced_icosphere_l8":
            O = _oracle()
            t0 = time.perf_counter()
            v_o, t_o = O.obj_load(text, 0)
            t_oracle = time.perf_counter() - t0
            canon = lambda v: np.where(np.isnan(v.view(np.float32)), np.float32(np.nan), v.view(np.float32)).view(np.uint32)
            r["parity"] = {"against": "oracle load_obj", "bit_exact": bool(
                np.array_equal(canon(v_d), canon(v_o)) and np.array_equal(t_d.view(np.uint32), t_o.view(np.uint32)))}
            if cpu:
                import tempfile
                with tempfile.NamedTemporaryFile(suffix=".obj", delete=False) as f:
                    f.write(text)
                    path = f.name
                t0 = time.perf_counter()
                M.load_scene_yaml_str(f"objects:\n  - type: mesh\n    path: {path}\n    material: {{ type: lambertian }}\n")
                t_host = time.perf_counter() - t0
                os.remove(path)
                r["cpu_baseline"] = {"oracle_load_obj_s": round(t_oracle, 3), "host_loader_s": round(t_host, 3),
                                     "cores": 1, "kind": "port",
                                     "sample": "the whole OBJ text (file read included for the host loader)"}
                r["speedup_wall_vs_oracle"] = round(t_oracle * 1e3 / m[0], 1)
        else:
            ok = (np.array_equal(v_d["position"][t_d["v"]], wv["position"][wt["v"]]) and
                  np.array_equal(v_d["normal"][t_d["v"]][..., :3], wv["normal"][wt["v"]][..., :3]))
            r["parity"] = {"against": "the device mesher's triangles (corner positions and normals)",
                           "bit_exact": bool(ok)}
        out[name] = r
    return out


def mlp_rate(M, ctx, n=1 << 20, reps=10):
    """Radiance-cache MLP on the tensor cores: inference over 2^20 synthetic
    queries and one training step on 2^20 samples (device time), against the
    measured bf16 peak (algorithmic FLOPs of the 96-64x5-3 network, output layer
    counted 16 wide)."""
    t_inf, t_train = ctx.cache_bench(n, reps)
    peak = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak = json.load(f)["bf16_tflops"]
    except (OSError, KeyError, ValueError):
        peak = 1900.0
    tf_inf = n * MLP_FLOP_INFER / (t_inf / 1000.0) / 1e12
    tf_train = n * MLP_FLOP_TRAIN / (t_train / 1000.0) / 1e12
    return {"queries": n, "infer_ms": round(t_inf, 4), "train_step_ms": round(t_train, 4),
            "infer_queries_per_s": round(n / (t_inf / 1000.0), 1),
            "train_samples_per_s": round(n / (t_train / 1000.0), 1),
            "roofline": {"bound": "tensor", "unit": "TFLOP/s", "peak": peak,
                         "infer_achieved": round(tf_inf, 2), "infer_frac": round(tf_inf / peak, 4),
                         "train_achieved": round(tf_train, 2), "train_frac": round(tf_train / peak, 4),
                         "flop_per_query": MLP_FLOP_INFER, "flop_per_train_sample": MLP_FLOP_TRAIN}}


def run_mcrt(args):
    import torch
    import mcrt_gb300 as M
    rank, world, local = dist_init(args.gpus)
    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()          # a dedicated stream shared by torch events and the library
    torch.cuda.set_stream(stream)
    sc = make_scene()
    cam = camera(sc)
    ctx = M.Context(local, stream=stream.cuda_stream)
    if args.leg == "cache_mlp":
        ctx.cache_init(0)
        print(json.dumps(mlp_rate(M, ctx, n=1 << 18, reps=args.steps)))
        return
    if args.leg == "adjoint":
        print(json.dumps(adjoint_rate(M, ctx, stream, n_warm=args.warmup, n_calls=args.steps)))
        return
    if args.leg == "nee":
        print(json.dumps(nee_rate(M, ctx, n_warm=args.warmup, n_calls=args.steps)))
        return
    if args.leg == "ingest":
        print(json.dumps({"leg": "ingest"} | ingest_rate(M, ctx, n_warm=args.warmup, n_steps=args.steps,
                                                         cpu=not args.no_cpu_baseline)))
        return
    ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"], env=sc["env"])
    if args.leg == "bvh_build":
        builds = []
        for _ in range(args.warmup + args.steps):
            ctx.rebuild_bvh()
            t = ctx.timings()
            builds.append((t["bvh_build_ms"], t["build_launches"]))
        ms = [b[0] for b in builds[args.warmup:]]
        print(json.dumps({"leg": "bvh_build", "triangles": int(len(sc["triangles"])), "ms": ms,
                          "launches_per_build": builds[-1][1]}))
        return
    if args.leg == "cache_race":          # the radiance cache against the tracer without it (wall time)
        cfgs = json.loads(os.environ["MCRT_CACHE_CONFIGS"]) if os.environ.get("MCRT_CACHE_CONFIGS") else None
        out = {"leg": "cache_race", "icosphere": icosphere_cache_relmse(M, ctx, configs=cfgs)}
        if not os.environ.get("MCRT_CACHE_ICOSPHERE_ONLY"):
            out["cornell"] = time_to_relmse(M, ctx)
            cfgs_c = [dict(query_vertex=v, train_stride=64, train_steps=8, train_batch=1 << 14, lr=1e-3) for v in (1, 2)]
            for tgt in (1e-2, 3e-3):
                out[f"cornell_target_{tgt:g}"] = time_to_relmse(M, ctx, target=tgt, cache_cfgs=cfgs_c, plain=False,
                                                                bound=False)
        if os.environ.get("MCRT_CACHE_VIEWS"):
            w = scenes_voxel_upload(M, ctx)
            out["views"] = views_cache_relmse(M, ctx)
        print(json.dumps(out))
        return
    if args.leg == "roofline_inputs":
        variant, _ = ctx.autotune(cam, W, H, SPP, max_depth=DEPTH)
        out = {"leg": "roofline_inputs", "workload": WORKLOAD, "variant": variant,
               "copy_gbs": {f"{mb}MB": round(ctx.copy_bandwidth(mb << 20, 50), 1) for mb in (8, 16, 32, 48, 64, 96)}}
        out["copy_gbs"]["2048MB"] = round(ctx.copy_bandwidth(2048 << 20, 10), 1)
        ctx.rebuild_bvh()
        ctx.render(cam, W, H, SPP, first_frame=0, max_depth=DEPTH, outputs=(), count=True)
        t = ctx.timings()
        out["counted"] = {k: int(t[k]) for k in ("rays", "node_fetches", "triangle_fetches", "extend_launches")}
        out["counted_per_variant"] = {}
        for v in range(8):                      # each variant's own fetches and extend time on the same frame
            ctx.render(cam, W, H, SPP, first_frame=0, max_depth=DEPTH, outputs=(), count=True, variant=v)
            tv = ctx.timings()
            ctx.render(cam, W, H, SPP, first_frame=0, max_depth=DEPTH, outputs=(), variant=v)
            out["counted_per_variant"][v] = {"node_fetches_per_ray": round(tv["node_fetches"] / tv["rays"], 3),
                                             "triangle_fetches_per_ray": round(tv["triangle_fetches"] / tv["rays"], 3),
                                             "extend_ms": round(ctx.timings()["extend_ms"], 3)}
        ctx.rebuild_bvh()
        ctx.render(cam, W, H, SPP, first_frame=0, max_depth=DEPTH, outputs=())
        out["extend_ms"] = round(ctx.timings()["extend_ms"], 3)
        print(json.dumps(out))
        return
    if args.leg == "frame":
        variant, tune_ms = ctx.autotune(cam, W, H, SPP, max_depth=DEPTH)  # 8 frames, 12 extend launches each
        frames = []
        for i in range(args.warmup + args.steps):
            ctx.rebuild_bvh()
            ctx.render(cam, W, H, SPP, first_frame=i * SPP, max_depth=DEPTH, outputs=())
            t = ctx.timings()
            frames.append({k: round(t[k], 3) for k in ("extend_ms", "shade_ms", "total_ms")} |
                          {"rays": t["rays"], "extend_launches": t["extend_launches"]})
        print(json.dumps({"leg": "frame", "workload": WORKLOAD, "variant": variant,
                          "autotune_extend_ms": [round(x, 3) for x in tune_ms], "frames": frames[args.warmup:]}))
        return
    # set-up, outside the timed region: one frame of the workload per variant
    variant, tune_ms = ctx.autotune(cam, W, H, SPP, max_depth=DEPTH)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")   # > 129 MB L2

    def step_device(i):
        ctx.rebuild_bvh()
        ctx.render(cam, W, H, SPP, first_frame=i * SPP, max_depth=DEPTH, outputs=())

    # the end-to-end step's host buffers: the vertices in and the image out, in pinned memory
    pin_vertices = torch.empty(sc["vertices"].nbytes, dtype=torch.uint8, pin_memory=True).numpy().view(M.VERTEX)
    np.copyto(pin_vertices, sc["vertices"])
    pin_image = torch.empty(H * W * 4, dtype=torch.float32, pin_memory=True).numpy().reshape(H, W, 4)

    def step_e2e(i):
        ctx.update_vertices(pin_vertices)
        ctx.render(cam, W, H, SPP, first_frame=i * SPP, max_depth=DEPTH, outputs=(), out_rgba=pin_image)

    breakdown = {}

    def timed(fn, n_warm, n_steps, sampler=None):
        for i in range(n_warm):
            fn(i)
        torch.cuda.synchronize()
        ms, extend = [], []
        launches = 0
        breakdown.clear()
        for i in range(n_steps):
            flush.fill_(float(i))                         # evict the scene and path state from L2
            barrier(world)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn(n_warm + i)
            b.record(stream)
            b.synchronize()
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
            t = ctx.timings()
            extend.append((t["extend_ms"], t["extend_launches"], t["rays"]))
            launches += t["render_launches"] + t["build_launches"]
            for k in ("bvh_build_ms", "extend_ms", "shade_ms", "shadow_ms", "resolve_ms", "total_ms"):
                breakdown[k] = breakdown.get(k, 0.0) + t[k] / n_steps
        return ms, extend, launches

    with ClockSampler(local) as clk:
        ms, ext, launches = timed(step_device, args.warmup, args.steps)
    device_breakdown = {k: round(v, 3) for k, v in breakdown.items()}
    e2e_ms, _, _ = timed(step_e2e, args.warmup, args.steps)
    step_ms = max_over_ranks(sum(ms) / len(ms), world)
    e2e_step_ms = max_over_ranks(sum(e2e_ms) / len(e2e_ms), world)
    samples = W * H * SPP * world
    value = samples / (step_ms / 1000.0) / 1e6
    e2e_value = samples / (e2e_step_ms / 1000.0) / 1e6
    if rank != 0:
        barrier(world)
        return
    # ---- roofline of the extend kernel (bytes per ray from oracle statistics of this workload)
    peak, peak_kind = peaks()
    cpu = None
    st = None
    parity = {}
    cores = os.cpu_count() or 1
    if not args.no_cpu_baseline:
        t_build, t_render, n_rows, strips, st, _ = cpu_frame_sample(sc, cam, rows_total=128, threads=cores, stats=True)
        t_frame = t_build + t_render * (H / n_rows)
        cpu = {"value": round(W * H * SPP / t_frame / 1e6, 4), "unit": "Msamples/s", "cores": cores, "kind": "port",
               "sample": (f"reference SAH build of all {len(sc['triangles'])} triangles (1 thread, {t_build:.2f} s) + "
                          f"{n_rows} of {H} rows x {W} px x {SPP} spp (depth {DEPTH}, {t_render:.2f} s on {cores} "
                          f"threads), render time scaled by {H / n_rows:.1f} to one frame")}
        # the same frames on the GPU (outside the timed region): the oracle's rows, bit for bit
        ctx.rebuild_bvh()
        g = ctx.render(cam, W, H, SPP, first_frame=0, max_depth=DEPTH, outputs=("rgba",))["rgba"]
        ok = all(np.array_equal(g[y0:y0 + m.shape[0]].view(np.uint32), m.view(np.uint32)) for y0, m in strips)
        parity["displaced_icosphere"] = {"rows": n_rows, "pixels": n_rows * W, "spp": SPP, "bit_exact": bool(ok)}
    ext_ms = sum(e[0] for e in ext)
    ext_launches = sum(e[1] for e in ext)
    rays = sum(e[2] for e in ext)
    roof = None
    if not args.small:
        # outside the timed region: this run's copy bandwidths and the traversal's own record fetches
        l2_copy = ctx.copy_bandwidth(16 << 20, 50)
        hbm_copy = ctx.copy_bandwidth(2048 << 20, 10)
        ctx.rebuild_bvh()
        ctx.render(cam, W, H, SPP, first_frame=0, max_depth=DEPTH, outputs=(), count=True)
        tc = ctx.timings()
        n_node = tc["node_fetches"] / max(tc["rays"], 1)
        n_tri = tc["triangle_fetches"] / max(tc["rays"], 1)
        b_ray = 64 * n_node + 48 * n_tri + 32 + 48
        sec = ext_ms / 1000.0
        achieved = rays * b_ray / sec / 1e9
        rays_per_launch = rays / max(ext_launches, 1)
        dram_b = EXTEND_DRAM_CAPTURE["bytes_per_ray"]
        l2_gbs = sum(EXTEND_L2_CAPTURE["gbs"]) / len(EXTEND_L2_CAPTURE["gbs"])
        roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                "traffic": round(dram_b * rays_per_launch), "traffic_unit": "B per launch",
                "traffic_source": dict(EXTEND_DRAM_CAPTURE, note="DRAM bytes per ray of the capture x this run's "
                                                                 "rays per launch"),
                "kernel": "k_extend_packet (bounce 0) + k_extend (bounces 1-11)",
                "bytes_per_ray": round(b_ray, 1), "node_fetches_per_ray": round(n_node, 3),
                "triangle_fetches_per_ray": round(n_tri, 3),
                "fetch_source": "counting kernels, one frame of this run",
                "mrays_per_s": round(rays / sec / 1e6, 1), "avg_launch_ms": round(ext_ms / max(ext_launches, 1), 4),
                "hbm_copy_gbs_this_run": round(hbm_copy, 1),
                "dram": {"achieved": round(dram_b * rays / sec / 1e9, 1), "frac": round(dram_b * rays / sec / 1e9 / peak, 4),
                         "bytes_per_ray": dram_b},
                "l2": {"achieved": round(l2_gbs, 1), "peak": round(l2_copy, 1), "frac": round(l2_gbs / l2_copy, 4),
                       "unit": "GB/s", "peak_kind": "this run's float4 copy over 2 x 16 MB (L2-resident)",
                       "source": EXTEND_L2_CAPTURE}}
        if st and st["rays"]:
            rn, rt = st["nodes"] / st["rays"], st["prims"] / st["rays"]
            rb = 48 * rn + 64 * rt + 32 + 16
            roof["reference_traversal"] = {
                "bytes_per_ray": round(rb, 1), "node_visits_per_ray": round(rn, 2), "triangle_tests_per_ray": round(rt, 2),
                "equivalent_gbs": round(rays * rb / sec / 1e9, 1),
                "note": "the reference traversal's visits on the reference BVH (48 B node, 16 B triangle + 3 x 16 B "
                        "positions), oracle statistics of this run's sample: more than HBM could deliver in the "
                        "kernels' time, since these kernels fetch fewer records, most from L2 and L1"}
    clocks = clk.summary()
    quality = adjoint = voxel = views = views_cache = icosphere_cache = mlp = cpu_more = ingest = None
    if not args.small:
        mlp = mlp_rate(M, ctx)
        quality = time_to_relmse(M, ctx)
        adjoint = adjoint_rate(M, ctx, stream)
        voxel = voxel_world_rate(M, ctx, stream)
        views = batched_views_rate(M, ctx, stream)
        views_cache = views_cache_relmse(M, ctx, bound=False)
        icosphere_cache = icosphere_cache_relmse(M, ctx)
        if not args.no_cpu_baseline:
            cpu_more, more_parity = cpu_baselines(M, ctx, quality, cores)
            parity.update(more_parity)
        ingest = ingest_rate(M, ctx, cpu=not args.no_cpu_baseline)
        parity.update({f"obj_{k}": v["parity"] for k, v in ingest.items()})
    out = {
        "metric": "Msamples/s", "value": round(value, 3), "unit": "Msamples/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_ms, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "width": W, "height": H, "spp": SPP, "max_depth": DEPTH,
                   "triangles": int(len(sc["triangles"])), "seed": SEED, "estimator": "reference (no NEE)",
                   "parallelism": f"replicas{world}", "l2": "256 MB buffer written between timed steps",
                   "e2e_host_buffers": "pinned (vertices in, f32 RGBA image out)",
                   "extend_variant": variant, "extend_variant_info": M.variant_info(variant),
                   "autotune_extend_ms_per_frame": [round(x, 3) for x in tune_ms]},
        "e2e": {"value": round(e2e_value, 3), "unit": "Msamples/s",
                "h2d_bytes_per_step": int(sc["vertices"].nbytes), "d2h_bytes_per_step": W * H * 16},
        "gpu_launches": int(launches),
        "roofline": roof,
        "cpu_baseline": cpu,
        "cpu_baselines_other": cpu_more,
        "parity": parity or None,
        "clocks": clocks,
        "extend_ms_per_step": round(ext_ms / len(ext), 3),
        "breakdown_ms_per_step": device_breakdown,
        "time_to_relmse": quality,
        "adjoint": adjoint,
        "voxel_world": voxel,
        "batched_views": views,
        "batched_views_cache_time_to_relmse": views_cache,
        "icosphere_cache_time_to_relmse": icosphere_cache,
        "radiance_cache_mlp": mlp,
        "scene_ingestion": ingest,
    }
    print(json.dumps(out))
    barrier(world)


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_mcrt(a)
