"""Radiance cache on the GPU against the CPU oracle (oracle/nrc.py): the tensor-core MMA layout
(exact, with permutation weights), the forward pass, the gradients and the Adam step, training
convergence, and the cache integrator against plain path tracing."""
import numpy as np
import pytest

from oracle import nrc
from verion_gb300 import pack, scenes
from verion_gb300.backend import Cache, Renderer

pytestmark = pytest.mark.gpu

BOX = ((-1.0, -1.0, -1.0), (1.0, 1.0, 1.0))
SMALL = dict(levels=8, log2_entries=14, base_resolution=4, max_resolution=128)


def grid_of(cache):
    c = cache.config
    return nrc.Grid.from_config(c.levels, c.log2_entries, c.base_resolution, c.max_resolution,
                                tuple(c.bounds_lo), tuple(c.bounds_hi))


def records(n, seed, target=None):
    rng = np.random.default_rng(seed)
    r = np.zeros((n, nrc.REC), np.float32)
    r[:, 0:3] = rng.uniform(-1.0, 1.0, (n, 3))
    for o in (3, 6):
        d = rng.normal(size=(n, 3))
        r[:, o:o + 3] = d / np.linalg.norm(d, axis=1, keepdims=True)
    r[:, 9:15] = rng.uniform(0.0, 1.0, (n, 6))
    if target is None:
        r[:, 16:19] = rng.uniform(0.0, 3.0, (n, 3))
    else:
        r[:, 16:19] = target(r)
    return r


def table16(cache, grid):
    _, g = cache.read_params()
    return g.reshape(grid.levels, grid.entries, 2).astype(np.float16)


@pytest.fixture(scope="module")
def small_cache(gpu_ctx):
    return Cache(gpu_ctx, bounds=BOX, **SMALL)


def test_mma_layout_exact_with_permutation_weights(small_cache):
    # Every layer a permutation: the prediction is a chosen input column, exactly (bf16).
    cache = small_cache
    g = grid_of(cache)
    rng = np.random.default_rng(7)
    m, gsize = cache.param_counts()
    grid = rng.uniform(0.05, 1.0, gsize).astype(np.float32)
    for trial in range(3):
        mlp = np.zeros(m, np.float32)
        src = np.arange(64)
        for l in range(4):
            p = rng.permutation(64)
            w = np.zeros((64, 64), np.float32)
            w[np.arange(64), p] = 1.0
            mlp[l * 4096:(l + 1) * 4096] = w.ravel()
            src = src[p]
        sel = rng.choice(45, 3, replace=False)  # columns 45-63 are zero
        pos = [int(np.nonzero(src == s)[0][0]) for s in sel]
        w4 = np.zeros((16, 64), np.float32)
        w4[np.arange(3), pos] = 1.0
        mlp[16384:] = w4.ravel()
        cache.write_params(mlp, grid)
        rec = records(1000 + 77 * trial, 10 + trial)
        x = nrc.inputs(g, table16(cache, g), rec)
        want = nrc.bf16(x[:, sel]).astype(np.float32)
        got = cache.infer(rec)
        assert np.array_equal(got, want), f"trial {trial}: {np.argwhere(got != want)[:5]}"


def test_forward_matches_oracle(small_cache):
    cache = small_cache
    g = grid_of(cache)
    rng = np.random.default_rng(8)
    m, gsize = cache.param_counts()
    mlp = (rng.normal(size=m) * 0.15).astype(np.float32)
    mlp[16384 + 3 * 64:] = 0.0
    cache.write_params(mlp, rng.uniform(-1, 1, gsize).astype(np.float32))
    rec = records(3000, 9)
    want = nrc.predict(mlp, g, table16(cache, g), rec)
    got = cache.infer(rec)
    # f32 tensor-core sums against f64; an activation that lands on a bf16 rounding boundary may
    # round the other way (one bf16 ulp, 2^-8 relative).
    scale = np.abs(want).max()
    err = np.abs(got - want)
    assert np.all(err <= 2e-2 * np.abs(want) + 2e-3 * scale), err.max()
    assert np.median(err / (np.abs(want) + 1e-3 * scale)) < 1e-4


def test_gradients_match_oracle(small_cache):
    cache = small_cache
    g = grid_of(cache)
    rng = np.random.default_rng(11)
    m, gsize = cache.param_counts()
    mlp = (rng.normal(size=m) * 0.15).astype(np.float32)
    mlp[16384 + 3 * 64:] = 0.0
    cache.write_params(mlp, rng.uniform(-1, 1, gsize).astype(np.float32))
    rec = records(2000, 12)
    gm, gg, loss = cache.gradients(rec)
    x = nrc.inputs(g, table16(cache, g), rec)
    l_ref, dws, gx = nrc.backward(nrc.layers(mlp), x, rec[:, 16:19])
    assert loss == pytest.approx(l_ref, rel=1e-3)
    ref = nrc.flat_mlp(dws)
    for l in range(5):
        a, b = (l * 4096, (l + 1) * 4096) if l < 4 else (16384, 17408)
        e = np.linalg.norm(gm[a:b] - ref[a:b]) / np.linalg.norm(ref[a:b])
        assert e < 2e-2, (l, e)
    assert np.all(gm[16384 + 3 * 64:] == 0.0)
    gref = nrc.grid_gradient(g, rec, gx).ravel()
    e = np.linalg.norm(gg - gref) / np.linalg.norm(gref)
    assert e < 2e-2, e


def test_adam_step_matches_oracle(small_cache):
    cache = small_cache
    rng = np.random.default_rng(13)
    m, gsize = cache.param_counts()
    mlp = (rng.normal(size=m) * 0.15).astype(np.float32)
    mlp[16384 + 3 * 64:] = 0.0
    grid = rng.uniform(-1, 1, gsize).astype(np.float32)
    cache.write_params(mlp, grid)
    rec = records(1500, 14)
    gm, gg, _ = cache.gradients(rec)
    cache.train(rec, batch=len(rec))
    mlp1, grid1 = cache.read_params()
    lr = cache.config.learning_rate
    for p0, g_sum, p1 in ((mlp, gm, mlp1), (grid, gg, grid1)):
        want, _, _ = nrc.adam_f32(p0, g_sum, np.zeros_like(p0), np.zeros_like(p0), used=len(rec), step=1, lr=lr)
        zero = g_sum == 0.0
        assert np.array_equal(p1[zero], p0[zero])
        big = np.abs(g_sum) > 1e-3 * np.abs(g_sum).max()
        assert np.abs((p1 - p0)[big] - (want - p0)[big]).max() <= 1e-3 * lr


def test_training_fits_a_smooth_function(gpu_ctx):
    cache = Cache(gpu_ctx, bounds=BOX, **SMALL)

    def target(r):
        return (r[:, 10:13] * (0.6 + 0.4 * r[:, 7:8]) + 0.3 * (r[:, 0:1] + 1.0)).astype(np.float32)

    train = records(65536, 21, target)
    test = records(4096, 22, target)

    def rel_l2(pred):
        y = test[:, 16:19]
        return float(np.mean((pred - y) ** 2 / (y ** 2 + 0.01)))

    before = rel_l2(cache.infer(test))
    for _ in range(8):
        cache.train(train, batch=4096)
    after = rel_l2(cache.infer(test))
    assert after < before / 10, (before, after)


def rmse(a, b):
    return float(np.sqrt(np.mean((a - b) ** 2)))


@pytest.mark.parametrize("integrator", ["megakernel", "wavefront"])
def test_cache_integrator_gains_over_no_cache(gpu_ctx, integrator):
    # Cornell box: the trained cache's image is far closer to the converged plain image than the
    # same spread-terminated paths with no trained cache (prediction 0), and its bias is small.
    from verion_gb300.backend import Integrator
    integ = Integrator.WAVEFRONT if integrator == "wavefront" else Integrator.MEGAKERNEL
    s = scenes.cornell()
    p = pack.pack(s)
    w = h = 64
    ref_r = Renderer(gpu_ctx, p)
    ref = ref_r.render(w, h, 8192)

    def run(train_steps, zero):
        r = Renderer(gpu_ctx, p)
        r.set_integrator(integ)
        cache = Cache(gpu_ctx, bounds=r.bounds())
        if zero:
            m, _ = cache.param_counts()
            cache.write_params(np.zeros(m, np.float32))
        r.set_cache(cache, spread=0.01, train_paths=1024, train_steps=train_steps, train_batch=4096)
        acc = r.new_accumulation(w, h)
        for _ in range(8):
            r.accumulate(acc, 64)
        st = acc.cache_stats()
        return acc.mean(), st

    img, st = run(4, False)
    zero_img, zst = run(0, True)
    assert st.queries > 0 and st.train_records > 0 and np.isfinite(st.loss)
    e_cache, e_zero = rmse(img, ref), rmse(zero_img, ref)
    assert e_cache < 0.5 * e_zero, (e_cache, e_zero)
    assert abs(img.mean() - ref.mean()) < 0.1 * ref.mean()


@pytest.mark.parametrize("scene", ["cornell", "feature_zoo"])
def test_cache_on_the_wavefront_matches_the_megakernel_cache(gpu_ctx, scene):
    # Without training the cache is fixed, so the query paths on the streaming wavefront leave the
    # image of the one-kernel query paths: same paths, same queries, same answers per pixel. One
    # sample per frame: bit for bit. Three per frame: the training pixels differ (one set per frame
    # instead of one per sample; with train_paths 0 at most one pixel per frame) and the cache's
    # answers are added after the frame's path sums rather than after each, so the other pixels
    # agree to rounding. The feature zoo has glass and cut-out surfaces (shadow rays in the
    # combined shadow stage), the Cornell box is opaque (any-hit stage).
    from verion_gb300.backend import Integrator
    if scene == "cornell":
        p = pack.pack(scenes.cornell())
    else:
        from . import analytic
        p = pack.pack(analytic.feature_zoo())
    w, h = 48, 40
    px = w * h

    def run(integ, frame, train_paths, calls):
        r = Renderer(gpu_ctx, p)
        r.set_integrator(integ)
        cache = Cache(gpu_ctx, bounds=r.bounds(), seed=7)
        r.set_cache(cache, spread=0.01, train_paths=train_paths, train_steps=0, train_batch=1024)
        if frame is not None:
            r.set_cache_frame(frame)
        acc = r.new_accumulation(w, h)
        queries = 0
        for n in calls:
            r.accumulate(acc, n)
            queries += acc.cache_stats().queries
        return acc.sums_f64(), queries

    want, wq = run(Integrator.MEGAKERNEL, None, 64, [1, 1, 1])
    assert wq > 0
    got, gq = run(Integrator.WAVEFRONT, 1, 64, [1, 1, 1])
    assert gq == wq
    assert np.array_equal(got, want), np.abs(got - want).max()

    want, wq = run(Integrator.MEGAKERNEL, None, 0, [1, 1, 1])
    got, gq = run(Integrator.WAVEFRONT, 3, 0, [3])
    train = set()
    for sample in range(3):
        off = (sample * 2654435761) % 2**32 % (px + 1)
        train.add((px + 1 - off) % (px + 1))
    keep = np.ones(px, bool)
    keep[[t for t in train if t < px]] = False
    assert abs(gq - wq) <= 3, (gq, wq)
    np.testing.assert_allclose(got.reshape(px, 3)[keep], want.reshape(px, 3)[keep], rtol=1e-12, atol=1e-12)


def test_cache_warmup_trains_without_touching_the_image(gpu_ctx):
    # Warm-up frames trace their training paths into a scratch buffer: with a learning rate of 0
    # (training changes no parameter) the image is the one without warm-up, bit for bit; with a
    # learning rate the warm-up frames train the cache before the first sample.
    from verion_gb300.backend import Integrator
    p = pack.pack(scenes.cornell())

    def run(warm, lr):
        r = Renderer(gpu_ctx, p)
        r.set_integrator(Integrator.WAVEFRONT)
        cache = Cache(gpu_ctx, bounds=r.bounds(), seed=3, learning_rate=lr)
        r.set_cache(cache, spread=0.01, train_paths=256, train_steps=2, train_batch=1024)
        r.set_cache_warmup(warm)
        acc = r.new_accumulation(40, 32)
        r.accumulate(acc, 2)
        assert acc.samples() == 2
        return acc.sums_f64(), cache.read_params()[0]

    img0, m0 = run(0, 0.0)
    img3, m3 = run(3, 0.0)
    assert np.array_equal(img0, img3)
    assert np.array_equal(m0, m3)
    _, t0 = run(0, 0.01)
    _, t3 = run(3, 0.01)
    assert not np.array_equal(t0, t3)
