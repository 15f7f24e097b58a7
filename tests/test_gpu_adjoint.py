"""GPU: next-event estimation bit-exact against the oracle; the path-replay
adjoint against the oracle's brute-force gradient on the same samples, against
central finite differences at 4096 spp through the torch.autograd.Function
harness, and in a 200-iteration Adam inverse rendering of the GGX Cornell box."""
import numpy as np
import pytest

import mcrt_gb300 as M
from mcrt_gb300 import scenes

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _camera(sc, w, h):
    c = sc["camera"]
    return M.compute_camera(w, h, c["look_from"], c["look_at"], c["vfov"], 0.0)


def _textured_scene():
    from test_gpu_regression import SCENE_YAML
    s = M.load_scene_yaml_str(SCENE_YAML.format(), "<textured>")
    c = s.camera
    return dict(spheres=s.spheres, vertices=s.vertices, triangles=s.triangles, materials=s.materials,
                cam=lambda w, h: M.compute_camera(w, h, c["look_from"], c["look_at"], c["vfov"], c["aperture"],
                                                  c["focus_dist"]))


def _scene(name):
    if name == "textured":
        return _textured_scene()
    sc = scenes.cornell_box(7) if name == "cornell" else scenes.cornell_box_ggx(1234)
    return dict(spheres=None, vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"],
                cam=lambda w, h: _camera(sc, w, h))


@pytest.mark.parametrize("name", ["cornell", "cornell_ggx", "textured"])
def test_nee_render_bit_exact(ctx, oracle, name):
    s = _scene(name)
    w, h, spp = 48, 40, 4
    cam = s["cam"](w, h)
    env = M.gradient_env_map()
    ctx.upload_scene(spheres=s["spheres"], vertices=s["vertices"], triangles=s["triangles"],
                     materials=s["materials"], env=env)
    r = ctx.render(cam, w, h, spp, first_frame=3, max_depth=8, nee=True)
    o = oracle.OracleScene(materials=s["materials"], spheres=s["spheres"], vertices=s["vertices"],
                           triangles=s["triangles"], env=env).render(cam, w, h, spp, first_frame=3, max_depth=8,
                                                                     nee=True)
    assert np.array_equal(bits(r["rgba"]), bits(o["rgba"]))
    assert np.array_equal(r["sum"].view(np.uint64), o["sum"].view(np.uint64))


@pytest.mark.parametrize("name,nee", [("cornell_ggx", True), ("cornell_ggx", False), ("textured", True),
                                      ("cornell", True)])
def test_adjoint_matches_bruteforce_gradient(ctx, oracle, name, nee):
    """Path replay (reverse mode, float, per-block sums) against forward-mode
    differentiation of the same sampled paths in double precision."""
    s = _scene(name)
    w, h, spp = 40, 32, 6
    cam = s["cam"](w, h)
    env = M.gradient_env_map()
    ctx.upload_scene(spheres=s["spheres"], vertices=s["vertices"], triangles=s["triangles"],
                     materials=s["materials"], env=env)
    d_img = np.random.default_rng(2).standard_normal((h, w, 4)).astype(np.float32)
    g, img = ctx.adjoint(cam, w, h, spp, d_img, first_frame=11, max_depth=8, nee=nee, with_image=True)
    osc = oracle.OracleScene(materials=s["materials"], spheres=s["spheres"], vertices=s["vertices"],
                             triangles=s["triangles"], env=env)
    want, _ = osc.adjoint(cam, w, h, spp, d_img, first_frame=11, max_depth=8, nee=nee)
    # the primal pass is the forward render
    o = osc.render(cam, w, h, spp, first_frame=11, max_depth=8, nee=nee)
    assert np.array_equal(bits(img), bits(o["rgba"]))
    scale = np.abs(want).max()
    assert scale > 0
    assert np.all(np.abs(g - want) <= 2e-4 * scale + 2e-3 * np.abs(want)), np.abs(g - want).max() / scale
    assert np.array_equal(g != 0, want != 0)


def test_adjoint_against_finite_differences():
    """torch.autograd.Function harness at 256 x 256: d L2(image, target) / d params
    by the adjoint against central differences (h = 1e-3) of the same 4096-spp
    estimate, relative error <= 1e-2."""
    torch = pytest.importorskip("torch")
    from adjoint_harness import CornellRenderer, RenderImage, l2_loss
    with M.Context(0) as ctx:
        R = CornellRenderer(ctx)
        tg, st = R.sc["target"], R.sc["start"]
        R.set_params(tg["albedo"], tg["roughness"], tg["radiance"])
        target = torch.from_numpy(R.image(1024, 1 << 20))
        spp = 4096
        th = {k: torch.tensor(np.asarray(v, np.float64), requires_grad=True) for k, v in st.items()}
        img = RenderImage.apply(th["albedo"], th["roughness"], th["radiance"], R, spp, 0, spp, 0)
        loss = l2_loss(img, target)
        loss.backward()
        g_adj = np.concatenate([th["albedo"].grad.numpy().ravel(), th["roughness"].grad.numpy().ravel(),
                                th["radiance"].grad.numpy().ravel()])

        def loss_at(p):
            R.set_params(p["albedo"], p["roughness"], p["radiance"])
            return float(l2_loss(torch.from_numpy(R.image(spp, 0)), target))

        base = {k: np.asarray(v, np.float64) for k, v in st.items()}
        fd = []
        for key in ("albedo", "roughness", "radiance"):
            hstep = 1e-3 * (17.0 if key == "radiance" else 1.0)
            for idx in np.ndindex(base[key].shape):
                a = {k: v.copy() for k, v in base.items()}
                b = {k: v.copy() for k, v in base.items()}
                a[key][idx] += hstep
                b[key][idx] -= hstep
                fd.append((loss_at(a) - loss_at(b)) / (2 * hstep))
        fd = np.array(fd)
    err = np.linalg.norm(g_adj - fd) / np.linalg.norm(fd)
    err_alb = np.linalg.norm(g_adj[:15] - fd[:15]) / np.linalg.norm(fd[:15])
    print("adjoint", g_adj, "\nfd", fd, "\nrelative error", err, "albedo", err_alb)
    assert err <= 1e-2
    assert err_alb <= 1e-3


def test_inverse_rendering_adam():
    """200 Adam iterations from albedo 0.5 / roughness 0.5 / nominal radiance,
    32 spp forward + 32 spp adjoint per iteration at 256 x 256."""
    torch = pytest.importorskip("torch")
    from adjoint_harness import CornellRenderer, RenderImage, l2_loss
    with M.Context(0) as ctx:
        R = CornellRenderer(ctx)
        tg, st = R.sc["target"], R.sc["start"]
        R.set_params(tg["albedo"], tg["roughness"], tg["radiance"])
        target = torch.from_numpy(R.image(1024, 1 << 20))
        th = {k: torch.tensor(np.asarray(v, np.float64), requires_grad=True) for k, v in st.items()}
        opt = torch.optim.Adam([{"params": [th["albedo"], th["roughness"]], "lr": 0.02},
                                {"params": [th["radiance"]], "lr": 0.3}])
        losses = []
        for it in range(200):
            opt.zero_grad()
            img = RenderImage.apply(th["albedo"], th["roughness"], th["radiance"], R, 32, 64 * it, 32,
                                    64 * it + 32)
            loss = l2_loss(img, target)
            loss.backward()
            opt.step()
            with torch.no_grad():
                th["albedo"].clamp_(0.01, 0.99)
                th["roughness"].clamp_(0.05, 1.0)
                th["radiance"].clamp_(0.1, 100.0)
            losses.append(float(loss))
        R.set_params(th["albedo"].detach().numpy(), th["roughness"].detach().numpy(),
                     th["radiance"].detach().numpy())
        final = float(l2_loss(torch.from_numpy(R.image(1024, 1 << 21)), target))
        R.set_params(st["albedo"], st["roughness"], st["radiance"])
        initial = float(l2_loss(torch.from_numpy(R.image(1024, 1 << 21)), target))
    err0 = np.abs(st["albedo"] - tg["albedo"]).mean()
    err1 = np.abs(th["albedo"].detach().numpy() - tg["albedo"]).mean()
    print("loss", initial, "->", final, "albedo error", err0, "->", err1)
    assert final < 0.05 * initial
    assert err1 < 0.5 * err0
