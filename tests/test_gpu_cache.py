"""GPU: the radiance-cache MLP on the tensor cores — forward pass and training
gradients against the CPU oracle (same bf16 rounding points), and online
training that fits a smooth radiance field."""
import numpy as np
import pytest

import mcrt_gb300 as M

pytestmark = pytest.mark.gpu

LO, HI = np.array([-1.0, -0.5, -2.0], np.float32), np.array([1.0, 1.5, 0.0], np.float32)


def _unit(rng, n):
    v = rng.standard_normal((n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def _queries(rng, n):
    p = LO + (HI - LO) * rng.uniform(-0.05, 1.05, (n, 3))
    return np.concatenate([p, _unit(rng, n), _unit(rng, n), rng.uniform(0, 1, (n, 3))], 1).astype(np.float32)


def _field(q):
    """A smooth radiance field of position, direction and albedo."""
    p, w, a = q[:, 0:3], q[:, 3:6], q[:, 9:12]
    base = 0.6 + 0.3 * np.sin(2.5 * p[:, 0:1]) * np.cos(1.7 * p[:, 2:3]) + 0.2 * w[:, 1:2]
    return (base * (0.3 + a)).astype(np.float32)


@pytest.fixture
def cache_ctx():
    with M.Context(0) as ctx:
        ctx.cache_set_bounds(LO, HI)
        ctx.cache_init(seed=7)
        yield ctx


def test_cache_forward_matches_oracle(cache_ctx, oracle):
    rng = np.random.default_rng(1)
    q = _queries(rng, 1000)                        # 7 full tiles and a ragged one
    got = cache_ctx.cache_infer(q)
    want = oracle.mlp_forward(cache_ctx.cache_params(), LO, HI, q)
    scale = np.abs(want).max()
    assert scale > 1e-3
    assert np.abs(got - want).max() <= 2e-2 * scale, np.abs(got - want).max() / scale


def test_cache_gradients_match_oracle(cache_ctx, oracle):
    rng = np.random.default_rng(2)
    n = 700
    q = _queries(rng, n)
    s = np.zeros((n, 16), np.float32)
    s[:, :12] = q
    s[:, 12:15] = _field(q)
    s[:, 15] = 1.0
    s[-37:, 15] = 0.0                              # unweighted samples contribute nothing
    p = cache_ctx.cache_params()
    loss, grad = cache_ctx.cache_train(s, steps=0, want_grad=True)
    want, want_loss = oracle.mlp_grad(p, LO, HI, s)
    assert abs(loss[0] - want_loss) <= 1e-3 * want_loss
    # per layer: W then b, relative error in norm
    offs = [0]
    for l in range(6):
        nin, nout = (96 if l == 0 else 64), (16 if l == 5 else 64)
        offs += [offs[-1] + nout * nin, offs[-1] + nout * nin + nout]
    for a, b in zip(offs[:-1], offs[1:]):
        ref = want[a:b]
        if np.linalg.norm(ref) == 0:
            assert np.all(grad[a:b] == 0)
            continue
        assert np.linalg.norm(grad[a:b] - ref) <= 3e-2 * np.linalg.norm(ref), (a, b)
    # the unused output rows stay exactly zero
    w5 = grad[offs[10]:offs[11]].reshape(16, 64)
    assert not w5[3:].any()


def test_cache_learns_a_radiance_field(cache_ctx):
    rng = np.random.default_rng(3)
    n = 1 << 15
    q = _queries(rng, n)
    s = np.zeros((n, 16), np.float32)
    s[:, :12], s[:, 12:15], s[:, 15] = q, _field(q), 1.0
    q_test = _queries(rng, 4096)
    t_test = _field(q_test)

    def rel_err():
        y = cache_ctx.cache_infer(q_test)
        return float(np.mean((y - t_test) ** 2 / (t_test ** 2 + 1e-2)))

    before = rel_err()
    loss, _ = cache_ctx.cache_train(s, steps=400, batch=1 << 14, lr=1e-3)
    after = rel_err()
    print("held-out relative L2", before, "->", after, "train loss", loss[0], "->", loss[-1])
    assert np.all(np.isfinite(loss))
    assert loss[-1] < 0.1 * loss[0]
    assert after < 0.1 * before


def test_cache_stop_bit_exact(ctx, oracle):
    """Paths stopped into a cache that predicts a constant: the render equals the
    oracle's, bit for bit (training paths traced in full, the others ending at
    their second vertex with that vertex's next-event sample and throughput x
    prediction)."""
    from mcrt_gb300 import scenes
    sc = scenes.cornell_box(5)
    c = sc["camera"]
    cam = M.compute_camera(48, 40, c["look_from"], c["look_at"], c["vfov"], 0.0)
    ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"],
                     env=M.gradient_env_map())
    ctx.cache_config(query_vertex=1, train_stride=7, train_steps=0, lr=0.0)
    p = np.zeros(ctx.cache_params().size, np.float32)
    const = np.array([0.3, 0.2, 0.1], np.float32)
    p[-16:-13] = const                              # output bias
    ctx.cache_set_params(p)
    for nee in (False, True):
        r = ctx.render(cam, 48, 40, 6, max_depth=8, nee=nee, spp_per_pass=3, cache=True)
        o = oracle.OracleScene(materials=sc["materials"], vertices=sc["vertices"], triangles=sc["triangles"],
                               env=M.gradient_env_map()).render_cache_const(cam, 48, 40, 6, const, 3, 7, 1,
                                                                            max_depth=8, nee=nee)
        assert np.array_equal(r["rgba"].view(np.uint32), o["rgba"].view(np.uint32))
        assert np.array_equal(r["sum"].view(np.uint64), o["sum"].view(np.uint64))


def test_trained_cache_gains_over_untrained_and_nee(ctx):
    """Cornell box 128 x 128, relMSE against a 4096-spp NEE reference.  The
    tracer with the online-trained cache (next-event estimation, paths stopped
    at their third vertex) against the same tracer with an untrained network
    at equal spp, and against next-event estimation alone at an equal number of
    traced rays (closest-hit and shadow rays, the training paths' included; the
    warm-up training is not counted): the stopped paths are cheaper, and the
    trained network's prediction is accurate enough that the extra samples pay.
    (Counted with the warm-up, in wall time to relMSE 1e-3, the gain over NEE
    alone is small: bench.py's time_to_relmse.)"""
    from mcrt_gb300 import scenes
    sc = scenes.cornell_box(1234)
    c = sc["camera"]
    W = H = 128
    cam = M.compute_camera(W, H, c["look_from"], c["look_at"], c["vfov"], 0.0)
    ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"],
                     env=M.gradient_env_map())
    ref = ctx.render(cam, W, H, 4096, first_frame=1 << 20, max_depth=8, nee=True, outputs=("sum",))["sum"] / 4096

    def rel(x):
        return float(np.mean((x - ref) ** 2 / (ref ** 2 + 1e-2)))

    def rays():
        t = ctx.timings()
        return t["rays"] + t["shadow_rays"]

    spp = 32
    nee = rel(ctx.render(cam, W, H, spp, max_depth=8, nee=True, outputs=("sum",))["sum"] / spp)
    nee_rays = rays()
    ctx.cache_config(query_vertex=2, train_stride=16, train_steps=0, lr=0.0)
    ctx.cache_init(1)
    untrained = rel(ctx.render(cam, W, H, 256, max_depth=8, nee=True, cache=True, outputs=("sum",))["sum"] / 256)
    ctx.cache_config(query_vertex=2, train_stride=16, train_steps=4, lr=1e-3)
    ctx.cache_init(1)
    for i in range(40):
        ctx.render(cam, W, H, 4, first_frame=100000 + 4 * i, max_depth=8, nee=True, cache=True, outputs=())
    trained = rel(ctx.render(cam, W, H, 256, max_depth=8, nee=True, cache=True, outputs=("sum",))["sum"] / 256)
    per_spp = rays() / 256
    spp_c = int(nee_rays / per_spp)                 # the cached tracer's spp for NEE's rays
    cached = rel(ctx.render(cam, W, H, spp_c, first_frame=5000, max_depth=8, nee=True, cache=True,
                            outputs=("sum",))["sum"] / spp_c)
    assert rays() <= nee_rays
    print("relMSE NEE", nee, "cache at equal rays", cached, f"({spp_c} spp)", "untrained", untrained,
          "trained", trained)
    assert trained < untrained / 3
    assert spp_c > 1.3 * spp
    assert cached < nee


def test_cache_bias_judge_and_fallback(ctx):
    """The bias judge compares the cache with what the plain tracer's training
    paths gathered.  A cache that predicts far too much light is judged biased;
    with max_bias set, the next render falls back to the plain tracer (bit for
    bit the render without the cache) while the judge keeps measuring.  An
    online-trained cache is judged close to unbiased and stops paths again."""
    from mcrt_gb300 import scenes
    sc = scenes.cornell_box(1234)
    c = sc["camera"]
    W = H = 64
    cam = M.compute_camera(W, H, c["look_from"], c["look_at"], c["vfov"], 0.0)
    ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"],
                     env=M.gradient_env_map())
    ctx.cache_config(query_vertex=1, train_stride=4, train_steps=0, lr=0.0, max_bias=0.25)
    p = np.zeros(ctx.cache_params().size, np.float32)
    p[-16:-13] = 20.0                               # output bias: a constant far above the scene's radiance
    ctx.cache_set_params(p)
    ctx.render(cam, W, H, 8, max_depth=8, nee=True, cache=True, outputs=())
    judged = ctx.cache_stats()
    assert judged["stopped"] and judged["samples"] > 1000 and min(judged["bias"]) > 1.0, judged
    r = ctx.render(cam, W, H, 8, first_frame=8, max_depth=8, nee=True, cache=True, outputs=("sum",))
    fallback = ctx.cache_stats()
    assert not fallback["stopped"] and min(fallback["bias"]) > 1.0, fallback
    plain = ctx.render(cam, W, H, 8, first_frame=8, max_depth=8, nee=True, outputs=("sum",))
    assert np.array_equal(r["sum"].view(np.uint64), plain["sum"].view(np.uint64))

    ctx.cache_config(query_vertex=1, train_stride=16, train_steps=8, lr=1e-3, max_bias=0.25)
    ctx.cache_init(1)
    for i in range(40):
        ctx.render(cam, W, H, 16, first_frame=1000 + 16 * i, max_depth=8, nee=True, cache=True, outputs=())
    trained = ctx.cache_stats()
    print("judged bias: constant cache", judged["bias"], "trained cache", trained["bias"])
    assert trained["stopped"] and max(abs(b) for b in trained["bias"]) < 0.25, trained


def test_cached_passes_replay_as_a_graph(ctx):
    """Cached passes have no host round trip, so MCRT_RENDER_GRAPH replays them
    (training included).  With a learning rate of 0 the network stays fixed
    while the training kernels run, and the graph replay equals the pass-by-pass
    render bit for bit; with training on, the graph-replayed cache learns (the
    judge finds it close to unbiased)."""
    from mcrt_gb300 import scenes
    sc = scenes.cornell_box(1234)
    c = sc["camera"]
    W = H = 64
    cam = M.compute_camera(W, H, c["look_from"], c["look_at"], c["vfov"], 0.0)
    ctx.upload_scene(vertices=sc["vertices"], triangles=sc["triangles"], materials=sc["materials"],
                     env=M.gradient_env_map())
    ctx.cache_config(query_vertex=1, train_stride=8, train_steps=2, lr=0.0)
    ctx.cache_init(3)
    sums = []
    for graph in (False, True, True):
        r = ctx.render(cam, W, H, 6, first_frame=40, max_depth=8, nee=True, spp_per_pass=2, cache=True,
                       graph=graph, outputs=("sum",))
        sums.append(r["sum"].view(np.uint64))
    assert np.array_equal(sums[0], sums[1]) and np.array_equal(sums[0], sums[2])
    ctx.cache_config(query_vertex=1, train_stride=16, train_steps=8, lr=1e-3)
    ctx.cache_init(1)
    for i in range(40):
        ctx.render(cam, W, H, 16, first_frame=1000 + 16 * i, max_depth=8, nee=True, spp_per_pass=4, cache=True,
                   graph=True, outputs=())
    st = ctx.cache_stats()
    print("graph-trained cache: judged bias", st["bias"])
    assert st["samples"] > 0 and max(abs(b) for b in st["bias"]) < 0.25, st
