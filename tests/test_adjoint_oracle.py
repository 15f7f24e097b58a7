"""CPU checks of the oracle's next-event estimator and of its brute-force
(forward-mode) gradient, the checkers of the kernels' NEE and adjoint paths."""
import numpy as np
import pytest

import mcrt_gb300 as M
from mcrt_gb300 import scenes


def _oracle_scene(oracle, sc, md=None):
    return oracle.OracleScene(materials=sc["materials"] if md is None else md, vertices=sc["vertices"],
                              triangles=sc["triangles"], env=M.gradient_env_map())


def _camera(sc, w, h):
    c = sc["camera"]
    return M.compute_camera(w, h, c["look_from"], c["look_at"], c["vfov"], 0.0)


def _relmse(x, ref):
    return float(np.mean((x - ref) ** 2 / (ref ** 2 + 1e-2)))


@pytest.mark.parametrize("ggx", [False, True])
def test_nee_and_plain_estimators_agree(oracle, ggx):
    """NEE with MIS and the reference estimator converge to the same image."""
    sc = scenes.cornell_box_ggx(7) if ggx else scenes.cornell_box(7)
    w = h = 12
    cam = _camera(sc, w, h)
    o = _oracle_scene(oracle, sc)
    plain = o.render(cam, w, h, 16384, max_depth=8)["sum"] / 16384
    nee = o.render(cam, w, h, 2048, max_depth=8, nee=True, first_frame=99)["sum"] / 2048
    assert _relmse(nee, plain) < 2e-3


def test_nee_flag_off_is_the_reference_estimator(oracle):
    sc = scenes.cornell_box(3)
    cam = _camera(sc, 16, 16)
    o = _oracle_scene(oracle, sc)
    a = o.render(cam, 16, 16, 4)
    b = oracle.OracleScene.render(o, cam, 16, 16, 4, nee=False)
    assert np.array_equal(a["rgba"].view(np.uint32), b["rgba"].view(np.uint32))


def test_ggx_alpha_derivative_matches_finite_differences(oracle):
    rng = np.random.default_rng(5)
    for _ in range(200):
        a = rng.uniform(0.02, 0.9)
        mz, co, ci = rng.uniform(0.05, 1.0, 3)
        d, _ = oracle.ggx_dg(a, mz, co, ci)
        h = 1e-6 * a
        fd = (oracle.ggx_dg(a + h, mz, co, ci)[1] - oracle.ggx_dg(a - h, mz, co, ci)[1]) / (2 * h)
        assert abs(d - fd) <= 1e-6 * max(1.0, abs(fd))


def _perturbed(params, key, idx, h):
    p = {k: np.array(v, dtype=np.float64, copy=True) for k, v in params.items()}
    p[key][idx] += h
    return scenes.ggx_materials(**{k: v.astype(np.float32) for k, v in p.items()})


@pytest.mark.parametrize("nee", [False, True])
def test_bruteforce_gradient_matches_finite_differences(oracle, nee):
    """Albedo and radiance enter every sample multiplicatively, so with common
    random numbers the forward-mode gradient equals the central difference of the
    same estimate up to rounding."""
    sc = scenes.cornell_box_ggx(1234)
    w = h = 16
    spp = 8
    cam = _camera(sc, w, h)
    d_img = np.random.default_rng(1).standard_normal((h, w, 4)).astype(np.float32)
    g, _ = _oracle_scene(oracle, sc).adjoint(cam, w, h, spp, d_img, nee=nee)

    def objective(md):
        s = _oracle_scene(oracle, sc, md).render(cam, w, h, spp, nee=nee)["sum"] / spp
        return float((s * d_img[..., :3]).sum())

    tg = sc["target"]
    checks = [("albedo", (k, c), (slot, c), 1e-3) for k, slot in enumerate(scenes.GGX_SLOTS) for c in range(3)]
    checks += [("radiance", (c,), (scenes.LIGHT_SLOT, c), 1e-2) for c in range(3)]
    scale = max(abs(g).max(), 1e-9)
    for key, idx, gi, hh in checks:
        fd = (objective(_perturbed(tg, key, idx, hh)) - objective(_perturbed(tg, key, idx, -hh))) / (2 * hh)
        assert abs(g[gi] - fd) <= 2e-4 * scale + 1e-3 * abs(fd), (key, idx, g[gi], fd)
    # roughness derivatives exist for every GGX slot the image sees
    assert all(g[slot, 3] != 0.0 for slot in scenes.GGX_SLOTS)
    # no gradient for slots the scene does not use
    assert not g[6:].any()
