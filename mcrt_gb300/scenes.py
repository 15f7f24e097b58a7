"""Seeded synthetic scenes for the benchmark workloads (numpy).

* ``cornell_box(seed)`` — 512x512, 64 spp, depth 8: five walls of the unit cube
  (10 triangles), two boxes 0.3 and 0.6 tall with yaw drawn from U[-20, 20]
  degrees (24 triangles), a 0.25 x 0.25 ceiling quad light of radiance
  (17, 12, 4); Lambertian red (0.63, 0.065, 0.05), green (0.14, 0.45, 0.09),
  white 0.73; pinhole camera, 40 degree field of view.
* ``displaced_icosphere(seed, level=8)`` — 1920x1080, 16 spp, depth 12: an
  icosphere subdivided ``level`` times (20 * 4**level triangles; 1,310,720 at
  level 8) displaced along its normals by 5-octave seeded value noise
  (amplitude 0.08) on a ground plane; per-triangle-group materials 50 %
  Lambertian (albedo U[0.2, 0.8]), 30 % GGX conductor (roughness U[0.05, 0.5]),
  20 % dielectric (IOR 1.5); a seeded 512x256 smooth-noise HDR environment,
  resized nearest to 1024x512 as the reference's loader does
  (src/texture.rs:124-148).

The reference ships no such scenes; these are the synthetic stand-ins with the
stated shapes, sizes and value distributions.
"""
from __future__ import annotations

import numpy as np

from ._native import MATERIAL_DATA, SPHERE, TRIANGLE, VERTEX, MAT_DIELECTRIC, MAT_EMISSIVE, MAT_GGX, MAT_LAMBERTIAN

__all__ = ["cornell_box", "cornell_box_ggx", "ggx_materials", "displaced_icosphere", "icosphere", "value_noise3", "smooth_noise_env"]


def _mat(md, i, t, alb, w=0.0, x=1.0):
    md["materials"][i]["type_pad"][0] = t
    md["materials"][i]["albedo_fuzz"][:3] = alb
    md["materials"][i]["albedo_fuzz"][3] = w
    md["materials"][i]["ior_pad"][0] = x


def _quads_to_mesh(quads, normals, mats, verts, tris):
    """Append quads (4 corners CCW seen from the normal side) as 2 triangles each."""
    for q, n, m in zip(quads, normals, mats):
        base = len(verts)
        for k, c in enumerate(q):
            v = np.zeros((), VERTEX)
            v["position"] = (*c, 1.0)
            v["normal"] = (*n, 0.0)
            v["uv"][:2] = [(0, 0), (1, 0), (1, 1), (0, 1)][k]
            verts.append(v)
        tris.append(((base, base + 1, base + 2), m))
        tris.append(((base, base + 2, base + 3), m))


def _box_quads(cx, cz, sx, h, sz, yaw_deg):
    c, s = np.cos(np.radians(yaw_deg)), np.sin(np.radians(yaw_deg))

    def P(x, y, z):
        return (cx + c * x + s * z, y, cz - s * x + c * z)

    def R(nx, ny, nz):
        return (c * nx + s * nz, ny, -s * nx + c * nz)

    hx, hz = sx / 2, sz / 2
    faces = [
        ([P(hx, 0, -hz), P(hx, 0, hz), P(hx, h, hz), P(hx, h, -hz)], R(1, 0, 0)),
        ([P(-hx, 0, hz), P(-hx, 0, -hz), P(-hx, h, -hz), P(-hx, h, hz)], R(-1, 0, 0)),
        ([P(-hx, h, -hz), P(hx, h, -hz), P(hx, h, hz), P(-hx, h, hz)], R(0, 1, 0)),
        ([P(hx, 0, -hz), P(-hx, 0, -hz), P(-hx, 0, hz), P(hx, 0, hz)], R(0, -1, 0)),
        ([P(hx, 0, hz), P(-hx, 0, hz), P(-hx, h, hz), P(hx, h, hz)], R(0, 0, 1)),
        ([P(-hx, 0, -hz), P(hx, 0, -hz), P(hx, h, -hz), P(-hx, h, -hz)], R(0, 0, -1)),
    ]
    return faces


def cornell_box(seed: int = 1234, box_mats=(0, 0)):
    rng = np.random.default_rng(seed)
    md = np.zeros((), MATERIAL_DATA)
    _mat(md, 0, MAT_LAMBERTIAN, (0.73, 0.73, 0.73))
    _mat(md, 1, MAT_LAMBERTIAN, (0.63, 0.065, 0.05))
    _mat(md, 2, MAT_LAMBERTIAN, (0.14, 0.45, 0.09))
    _mat(md, 3, MAT_EMISSIVE, (17.0, 12.0, 4.0), 0.0, 1.0)
    md["mat_count"] = 4
    verts, tris = [], []
    walls = [  # floor, ceiling, back, left (red), right (green); inward normals
        ([(0, 0, 1), (1, 0, 1), (1, 0, 0), (0, 0, 0)], (0, 1, 0), 0),
        ([(0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1)], (0, -1, 0), 0),
        ([(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0)], (0, 0, 1), 0),
        ([(0, 0, 1), (0, 0, 0), (0, 1, 0), (0, 1, 1)], (1, 0, 0), 1),
        ([(1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0)], (-1, 0, 0), 2),
    ]
    _quads_to_mesh([w[0] for w in walls], [w[1] for w in walls], [w[2] for w in walls], verts, tris)
    yaws = rng.uniform(-20.0, 20.0, size=2)
    for (cx, cz, h), yaw, bm in zip([(0.68, 0.62, 0.3), (0.32, 0.35, 0.6)], yaws, box_mats):
        faces = _box_quads(cx, cz, 0.28, h, 0.28, yaw)
        _quads_to_mesh([f[0] for f in faces], [f[1] for f in faces], [bm] * 6, verts, tris)
    L = 0.125
    _quads_to_mesh([[(0.5 - L, 0.999, 0.5 - L), (0.5 + L, 0.999, 0.5 - L), (0.5 + L, 0.999, 0.5 + L),
                     (0.5 - L, 0.999, 0.5 + L)]], [(0, -1, 0)], [3], verts, tris)
    V = np.array(verts, VERTEX)
    T = np.zeros(len(tris), TRIANGLE)
    T["v"] = [t[0] for t in tris]
    T["mat_idx"] = [t[1] for t in tris]
    camera = dict(look_from=[0.5, 0.5, 2.4], look_at=[0.5, 0.5, 0.0], vfov=40.0, aperture=0.0)
    return dict(vertices=V, triangles=T, materials=md, spheres=np.zeros(0, SPHERE), camera=camera,
                width=512, height=512, spp=64, max_depth=8)


GGX_SLOTS = (0, 1, 2, 4, 5)      # white walls, red wall, green wall, short box, tall box
LIGHT_SLOT = 3


def ggx_materials(albedo, roughness, radiance):
    """Material table of the differentiable Cornell box: GGX conductors in the
    slots GGX_SLOTS with per-material albedo (5 x 3) and roughness (5), and the
    quad light in LIGHT_SLOT with radiance = 1 * albedo (3)."""
    md = np.zeros((), MATERIAL_DATA)
    albedo = np.asarray(albedo, np.float32).reshape(5, 3)
    roughness = np.asarray(roughness, np.float32).reshape(5)
    for k, slot in enumerate(GGX_SLOTS):
        _mat(md, slot, MAT_GGX, albedo[k], float(roughness[k]))
    _mat(md, LIGHT_SLOT, MAT_EMISSIVE, np.asarray(radiance, np.float32).reshape(3), 0.0, 1.0)
    md["mat_count"] = 6
    return md


def cornell_box_ggx(seed: int = 1234):
    """The inverse-rendering scene: the seeded Cornell box geometry (boxes in
    their own material slots) with GGX materials whose target parameters are
    drawn from the seed -- albedo U[0.1, 0.9]^3 and roughness U[0.1, 0.8] per
    material, light radiance (17, 12, 4) scaled by U[0.5, 1.5] -- and the
    optimisation's starting point (albedo 0.5, roughness 0.5, radiance
    (17, 12, 4)).  Rendered at 256 x 256."""
    base = cornell_box(seed, box_mats=(4, 5))
    rng = np.random.default_rng(seed + 1)
    target = dict(albedo=rng.uniform(0.1, 0.9, (5, 3)).astype(np.float32),
                  roughness=rng.uniform(0.1, 0.8, 5).astype(np.float32),
                  radiance=(np.array([17.0, 12.0, 4.0]) * rng.uniform(0.5, 1.5)).astype(np.float32))
    start = dict(albedo=np.full((5, 3), 0.5, np.float32), roughness=np.full(5, 0.5, np.float32),
                 radiance=np.array([17.0, 12.0, 4.0], np.float32))
    base["materials"] = ggx_materials(**target)
    base.update(target=target, start=start, width=256, height=256, spp=32)
    return base


# Block ids of the reference's registry (world/block.rs:14-24) that the world
# generator places, their material slots and Lambertian albedos (the registry's
# tints, block.rs:64-125, where it has them).
WORLD_BLOCKS = [  # (block id, name, albedo)
    (1, "limestone", (0.82, 0.78, 0.70)),
    (2, "red_soil", (0.55, 0.25, 0.15)),
    (3, "grass", (0.35, 0.42, 0.18)),
    (4, "sand", (0.86, 0.78, 0.56)),
    (5, "water", (0.10, 0.25, 0.40)),
    (8, "shrub", (0.22, 0.36, 0.12)),
    (9, "gravel", (0.50, 0.48, 0.45)),
    (10, "cave_glow", (0.40, 0.80, 0.60)),
]


def world_params(seed: int = 1234, nx: int = 256, ny: int = 128, nz: int = 256):
    """mcrt_world_params of the voxel-world workload: a seeded 2D fBm heightmap
    (4 octaves, lacunarity 2, gain 0.5) and 3D-noise caves carved where the
    value exceeds 0.6; the grid is centred on the origin."""
    return dict(nx=nx, ny=ny, nz=nz, seed=seed, chunk_x0=-(nx // 32), chunk_z0=-(nz // 32),
                height_base=0.6 * ny, height_amp=0.3 * ny, height_freq=1.0 / 80.0, height_octaves=4,
                lacunarity=2.0, gain=0.5, cave_freq=0.25, cave_octaves=2, cave_threshold=0.6, cave_contrast=1.5,
                cave_min_y=2, sea_level=0.42 * ny, sand_line=0.45 * ny)


def voxel_world(seed: int = 1234, nx: int = 256, ny: int = 128, nz: int = 256):
    """The voxel-world scene: world parameters, the block -> material map and
    the 8 Lambertian block materials, a sun (directional light) over the
    gradient sky, a camera over the terrain; rendered at 1280 x 720, 8 spp,
    depth 6, then denoised (5 x 5, sigma_color 0.1, sigma_normal 0.2)."""
    md = np.zeros((), MATERIAL_DATA)
    block_material = np.zeros(256, np.uint32)
    for slot, (bid, _, alb) in enumerate(WORLD_BLOCKS):
        _mat(md, slot, MAT_LAMBERTIAN, alb)
        block_material[bid] = slot
    md["mat_count"] = len(WORLD_BLOCKS)
    s = 0.125                                    # VOXEL_SIZE, world/chunk.rs:20
    ext_x, ext_z, ext_y = nx * s, nz * s, ny * s
    camera = dict(look_from=[-0.42 * ext_x, 0.95 * ext_y, -0.42 * ext_z], look_at=[0.1 * ext_x, 0.35 * ext_y, 0.1 * ext_z],
                  vfov=55.0, aperture=0.0)
    return dict(params=world_params(seed, nx, ny, nz), block_material=block_material, materials=md, voxel_size=s,
                camera=camera, sun_dir=[0.45, 0.8, 0.25], sun_irradiance=[3.2, 3.0, 2.7], width=1280, height=720,
                spp=8, max_depth=6, denoise=dict(radius=2, sigma_color=0.1, sigma_normal=0.2))


def world_views(world, seed: int = 1234, n: int = 16):
    """Seeded camera poses over a voxel world (the batched workload): n views of
    distinct, uneven sizes in [256, 1920] x [256, 1080], each looking from above
    the terrain at a point near the centre."""
    rng = np.random.default_rng(seed)
    p, s = world["params"], world["voxel_size"]
    ext_x, ext_y, ext_z = p["nx"] * s, p["ny"] * s, p["nz"] * s
    out, seen = [], set()
    while len(out) < n:
        w, h = int(rng.integers(256, 1921)), int(rng.integers(256, 1081))
        if (w, h) in seen:
            continue
        seen.add((w, h))
        ang = rng.uniform(0.0, 2.0 * np.pi)
        r = rng.uniform(0.25, 0.48) * ext_x
        look_from = [r * np.cos(ang), rng.uniform(0.75, 1.0) * ext_y, r * np.sin(ang) * ext_z / ext_x]
        look_at = [rng.uniform(-0.2, 0.2) * ext_x, rng.uniform(0.3, 0.5) * ext_y, rng.uniform(-0.2, 0.2) * ext_z]
        out.append(dict(width=w, height=h, look_from=[float(v) for v in look_from],
                        look_at=[float(v) for v in look_at], vfov=float(rng.uniform(40.0, 70.0))))
    return out


def icosphere(level: int):
    """Unit icosphere: (positions float64 (n,3), triangles int64 (m,3)), 20*4**level faces."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    p = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
                  (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], np.float64)
    p /= np.linalg.norm(p, axis=1, keepdims=True)
    f = np.array([(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
                  (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
                  (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)], np.int64)
    for _ in range(level):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = p[uniq[:, 0]] + p[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(p)
        p = np.concatenate([p, mid])
        m = inv.reshape(3, -1).T + base     # midpoints of edges (01, 12, 20)
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        m01, m12, m20 = m[:, 0], m[:, 1], m[:, 2]
        f = np.concatenate([np.stack([a, m01, m20], 1), np.stack([b, m12, m01], 1), np.stack([c, m20, m12], 1),
                            np.stack([m01, m12, m20], 1)])
    return p, f


def value_noise3(p: np.ndarray, seed: int, octaves: int = 5, lacunarity: float = 2.0, gain: float = 0.5,
                 base_freq: float = 2.0) -> np.ndarray:
    """Seeded fractal value noise in about [-1, 1]: trilinear smoothstep interpolation of lattice values."""
    rng = np.random.default_rng(seed)
    table = rng.uniform(-1.0, 1.0, size=4096)
    perm = rng.permutation(4096)
    out = np.zeros(len(p))
    amp, freq, norm = 1.0, base_freq, 0.0
    for _ in range(octaves):
        q = p * freq
        i = np.floor(q).astype(np.int64)
        fr = q - i
        w = fr * fr * (3.0 - 2.0 * fr)
        acc = 0.0
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    h = perm[(perm[(perm[(i[:, 0] + dx) & 4095] + i[:, 1] + dy) & 4095] + i[:, 2] + dz) & 4095]
                    wx = w[:, 0] if dx else 1 - w[:, 0]
                    wy = w[:, 1] if dy else 1 - w[:, 1]
                    wz = w[:, 2] if dz else 1 - w[:, 2]
                    acc = acc + table[h] * wx * wy * wz
        out += amp * acc
        norm += amp
        amp *= gain
        freq *= lacunarity
    return out / norm


def smooth_noise_env(seed: int, w: int = 512, h: int = 256) -> np.ndarray:
    """Seeded HDR equirectangular smooth-noise map (h, w, 3) float32, brighter sky above the horizon."""
    v = (np.arange(h) + 0.5) / h
    u = (np.arange(w) + 0.5) / w
    theta = (0.5 - v)[:, None] * np.pi
    phi = (u[None, :] - 0.5) * 2 * np.pi
    d = np.stack([np.cos(theta) * np.cos(phi), np.sin(theta) * np.ones_like(phi), np.cos(theta) * np.sin(phi)], -1)
    n = value_noise3(d.reshape(-1, 3), seed, octaves=4, base_freq=3.0).reshape(h, w)
    sky = np.clip(np.sin(theta), 0, 1) * np.ones_like(phi)
    base = 0.3 + 1.2 * sky + 0.1 * np.exp(3.0 * n)
    env = np.stack([base * 0.9, base * 0.95, base * 1.1], -1)
    return env.astype(np.float32)


def nearest_resize_rgba(env_rgb: np.ndarray, ow: int = 1024, oh: int = 512) -> np.ndarray:
    """texture.rs:124-148: nearest resize to 1024x512, clamp [0, 1e10], alpha 1."""
    h, w = env_rgb.shape[:2]
    ys = np.minimum(((np.arange(oh, dtype=np.float32) + np.float32(0.5)) * np.float32(h / oh)).astype(np.int64), h - 1)
    xs = np.minimum(((np.arange(ow, dtype=np.float32) + np.float32(0.5)) * np.float32(w / ow)).astype(np.int64), w - 1)
    out = np.ones((oh, ow, 4), np.float32)
    out[..., :3] = np.clip(env_rgb[ys][:, xs], 0, 1e10)
    return out


def displaced_icosphere(seed: int = 1234, level: int = 8, width: int = 1920, height: int = 1080):
    rng = np.random.default_rng(seed)
    p, f = icosphere(level)
    disp = 0.08 * value_noise3(p, seed + 1, octaves=5, base_freq=2.0)
    pos = p * (1.0 + disp)[:, None]
    pos[:, 1] += 1.2     # rest above the ground plane at y = 0
    # smooth normals: area-weighted face normals
    fn = np.cross(pos[f[:, 1]] - pos[f[:, 0]], pos[f[:, 2]] - pos[f[:, 0]])
    vn = np.zeros_like(pos)
    for k in range(3):
        np.add.at(vn, f[:, k], fn)
    vn /= np.maximum(np.linalg.norm(vn, axis=1, keepdims=True), 1e-12)
    nv = len(pos)
    V = np.zeros(nv + 4, VERTEX)
    V["position"][:nv, :3] = pos
    V["position"][:, 3] = 1.0
    V["normal"][:nv, :3] = vn
    G = 6.0
    V["position"][nv:, :3] = [(-G, 0, G), (G, 0, G), (G, 0, -G), (-G, 0, -G)]
    V["normal"][nv:, :3] = (0, 1, 0)
    V["uv"][nv:, :2] = [(0, 0), (1, 0), (1, 1), (0, 1)]
    # materials: 60 sphere materials (50 % Lambertian, 30 % GGX, 20 % dielectric) + ground
    md = np.zeros((), MATERIAL_DATA)
    n_l, n_g, n_d = 30, 18, 12
    k = 0
    for _ in range(n_l):
        _mat(md, k, MAT_LAMBERTIAN, rng.uniform(0.2, 0.8, 3)); k += 1
    for _ in range(n_g):
        _mat(md, k, MAT_GGX, rng.uniform(0.5, 0.95, 3), rng.uniform(0.05, 0.5)); k += 1
    for _ in range(n_d):
        _mat(md, k, MAT_DIELECTRIC, (1.0, 1.0, 1.0), 0.0, 1.5); k += 1
    _mat(md, k, MAT_LAMBERTIAN, (0.5, 0.5, 0.5))
    ground = k
    md["mat_count"] = k + 1
    # triangle groups = faces of the level-2 ancestor (320 groups); each group draws a material
    m = len(f)
    group = (np.arange(m) % (m // 320)) if level >= 2 else np.arange(m)
    group = np.arange(m) // max(1, m // 320)
    gkind = rng.choice(3, size=group.max() + 1, p=[0.5, 0.3, 0.2])
    gmat = np.where(gkind == 0, rng.integers(0, n_l, group.max() + 1),
                    np.where(gkind == 1, n_l + rng.integers(0, n_g, group.max() + 1),
                             n_l + n_g + rng.integers(0, n_d, group.max() + 1)))
    T = np.zeros(m + 2, TRIANGLE)
    T["v"][:m] = f
    T["mat_idx"][:m] = gmat[group]
    T["v"][m:] = [(nv, nv + 1, nv + 2), (nv, nv + 2, nv + 3)]
    T["mat_idx"][m:] = ground
    env = nearest_resize_rgba(smooth_noise_env(seed + 2))
    camera = dict(look_from=[0.0, 2.2, 4.2], look_at=[0.0, 1.1, 0.0], vfov=40.0, aperture=0.0)
    return dict(vertices=V, triangles=T, materials=md, spheres=np.zeros(0, SPHERE), env=env, camera=camera,
                width=width, height=height, spp=16, max_depth=12)


# ---------------------------------------------------------------------------- OBJ text

def _fixed_field(x: np.ndarray, width: int, decimals: int) -> np.ndarray:
    """Fixed-point decimal text of float values, right-aligned in `width` bytes
    (leading spaces): uint8 (n, width)."""
    x = np.asarray(x, np.float64)
    q = np.rint(np.abs(x) * 10.0 ** decimals).astype(np.int64)
    neg = (x < 0) & (q > 0)
    ip = q // 10 ** decimals
    n_int = np.maximum(1, np.floor(np.log10(np.maximum(ip, 1))).astype(np.int64) + 1)
    if (n_int + decimals + 1 + neg > width).any():
        raise ValueError("value too wide for the field")
    out = np.full((len(x), width), ord(" "), np.uint8)
    for c in range(width):                     # c: column from the right
        col = width - 1 - c
        if c < decimals:
            out[:, col] = ord("0") + (q // 10 ** c) % 10
        elif c == decimals:
            out[:, col] = ord(".")
        else:
            j = c - decimals - 1               # integer digit j
            dig = ord("0") + (ip // 10 ** min(j, 18)) % 10
            out[:, col] = np.where(j < n_int, dig, np.where((j == n_int) & neg, ord("-"), ord(" ")))
    return out


def _index_pair_field(a: np.ndarray, b: np.ndarray | None, width: int) -> np.ndarray:
    """Face tokens "a" or "a//b" (1-based indices) right-aligned in `width` bytes."""
    a = np.asarray(a, np.int64)
    nd = lambda v: np.floor(np.log10(np.maximum(v, 1))).astype(np.int64) + 1
    na = nd(a)
    nb = np.zeros_like(na) if b is None else nd(np.asarray(b, np.int64))
    tail = np.zeros_like(na) if b is None else nb + 2
    if (na + tail > width).any():
        raise ValueError("index too wide for the field")
    out = np.full((len(a), width), ord(" "), np.uint8)
    for c in range(width):
        col = width - 1 - c
        ja = c - tail
        da = ord("0") + (a // 10 ** np.clip(ja, 0, 18)) % 10
        ch = np.where((ja >= 0) & (ja < na), da, ord(" "))
        if b is not None:
            db = ord("0") + (np.asarray(b, np.int64) // 10 ** min(c, 18)) % 10
            ch = np.where(c < nb, db, np.where((c >= nb) & (c < nb + 2), ord("/"), ch))
        out[:, col] = ch
    return out


def obj_text(positions: np.ndarray, faces: np.ndarray, normals: np.ndarray | None = None,
             face_normals: np.ndarray | None = None, decimals: int = 6) -> bytes:
    """Wavefront OBJ text: ``v`` lines of positions (n, 3), ``vn`` lines of
    normals (m, 3) if given, then one ``f`` line per row of faces (k, c)
    (0-based vertex indices, c >= 3) with tokens ``a`` or ``a//n`` (normal
    indices from face_normals (k, c), or the vertex index when normals has one
    row per position).  Coordinates are fixed-point with `decimals` places;
    fields are space-padded to a fixed width (valid OBJ: tokens are split at
    whitespace)."""
    P = np.asarray(positions)
    F = np.asarray(faces, np.int64)
    w = 6 + decimals
    def lines(tag, cols):
        n = len(cols[0])
        parts = [np.frombuffer(tag, np.uint8)[None, :].repeat(n, 0)]
        for c in cols:
            parts.append(np.full((n, 1), ord(" "), np.uint8))
            parts.append(c)
        parts.append(np.full((n, 1), ord("\n"), np.uint8))
        return np.concatenate(parts, 1).tobytes()
    out = [lines(b"v", [_fixed_field(P[:, k], w, decimals) for k in range(3)])]
    if normals is not None:
        Nn = np.asarray(normals)
        out.append(lines(b"vn", [_fixed_field(Nn[:, k], w, decimals) for k in range(3)]))
        FN = F if face_normals is None else np.asarray(face_normals, np.int64)
        iw = 2 * len(str(max(len(P), len(Nn)))) + 2
        out.append(lines(b"f", [_index_pair_field(F[:, k] + 1, FN[:, k] + 1, iw) for k in range(F.shape[1])]))
    else:
        iw = len(str(len(P)))
        out.append(lines(b"f", [_index_pair_field(F[:, k] + 1, None, iw) for k in range(F.shape[1])]))
    return b"".join(out)


def displaced_icosphere_obj(seed: int = 1234, level: int = 8) -> bytes:
    """The displaced icosphere's sphere mesh (without the ground) as OBJ text:
    positions and smooth normals to 6 decimals, faces ``a//a b//b c//c``
    (20 * 4**level triangles sharing vertices through the OBJ loader's
    (position, uv, normal) cache)."""
    sc = displaced_icosphere(seed, level)
    nv = len(sc["vertices"]) - 4
    m = len(sc["triangles"]) - 2
    P = sc["vertices"]["position"][:nv, :3]
    Nn = sc["vertices"]["normal"][:nv, :3]
    return obj_text(P, sc["triangles"]["v"][:m], normals=Nn)


def world_mesh_obj(vertices: np.ndarray, triangles: np.ndarray) -> bytes:
    """The voxel world's face mesh (4 vertices per quad) as OBJ text: one ``v``
    per vertex, the six axis normals as ``vn``, and the mesh's own triangles as
    ``f a//n b//n c//n`` (the mesher flips the winding of some quads, so the
    triangles are written as they are rather than as quads)."""
    V = np.asarray(vertices)
    T = np.asarray(triangles)["v"].astype(np.int64)
    axes = np.array([(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)], np.float32)
    n = V["normal"][:, :3]
    nidx = np.argmax((n[:, None, :] * axes[None, :, :]).sum(-1), axis=1)
    return obj_text(V["position"][:, :3], T, normals=axes, face_normals=nidx[T])
