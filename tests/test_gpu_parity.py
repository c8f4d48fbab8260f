"""GPU parity: the CUDA backend (through the C ABI) against the CPU oracle on the same seeded
inputs. Integer results (hit flags, instance and primitive ids, queue counts, sample counts) and,
with single-precision sums, the float sums themselves are compared bit for bit: the kernels and the
oracle evaluate the same IEEE single-precision operations in the same order.

Reference tests these follow: crates/verion-gpu-metal/tests/pathtrace.rs (analytic scenes,
wavefront == megakernel at :169-176, adaptive at :178-231), crates/verion-gpu-vulkan/tests/gpu.rs:50-67
(bit-for-bit integrator equality), crates/verion-gpu-metal/tests/trace.rs:95-121 (hit distances).
"""
import numpy as np
import pytest

import oracle
from verion_gb300 import pack, scenes
from verion_gb300 import scene as sc
from verion_gb300.backend import Error, Integrator, Renderer, WavefrontMode
from verion_gb300.readback import Adaptive, Restir

pytestmark = pytest.mark.gpu


def random_rays(n, seed, center=(0.0, 0.0, 0.0), spread=3.0):
    rng = np.random.default_rng(seed)
    o = rng.uniform(-spread, spread, (n, 3)) + np.asarray(center)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, d], axis=1).astype(np.float32)


def params(p, w, h, lighting=False, multiscatter=True, adaptive=None, restir=None, depth=8):
    return pack.base_params(p.info, p.view, (w, h), lighting, multiscatter, adaptive, restir, depth)


def gpu_render(ctx, p, w, h, spp, *, integrator=Integrator.MEGAKERNEL, precision=32, lighting=False,
               adaptive=None, restir=None, depth=8, chunks=None, mode=WavefrontMode.STREAMING):
    r = Renderer(ctx, p)
    r.set_accum_precision(precision)
    r.set_integrator(integrator)
    r.set_wavefront_mode(mode)
    r.set_max_depth(depth)
    r.set_adaptive(adaptive)
    r.set_restir(restir)
    acc = r.new_accumulation(w, h, lighting)
    for n in (chunks or [spp]):
        r.accumulate(acc, n)
    return r, acc


def oracle_render(p, w, h, spp, *, acc64=False, lighting=False, adaptive=None, restir=None, depth=8,
                  wavefront=False):
    o = oracle.OracleScene(p)
    a = oracle.OracleAccumulation(w, h, lighting=lighting, acc64=acc64, adaptive=adaptive is not None,
                                  restir=restir is not None)
    oracle.render(o, params(p, w, h, lighting, True, adaptive, restir, depth), a, spp, wavefront=wavefront)
    return a


def assert_same(got, want, what):
    got = np.asarray(got)
    want = np.asarray(want)
    bad = got != want
    if bad.any():
        i = np.flatnonzero(bad.ravel())[:5]
        raise AssertionError(f"{what}: {int(bad.sum())} of {bad.size} differ, first {i.tolist()}: "
                             f"{got.ravel()[i].tolist()} vs {want.ravel()[i].tolist()}")


def test_trace_closest_cornell_matches_oracle(gpu_ctx):
    p = pack.pack(scenes.cornell())
    r = Renderer(gpu_ctx, p)
    o = oracle.OracleScene(p)
    rays = random_rays(200_000, 1, spread=1.2)
    got = r.trace_closest(rays)
    assert_same(got, o.trace_closest(rays, brute=True), "closest hits vs brute force")
    assert got[:, 0].mean() > 0.5


def test_trace_closest_many_spheres_matches_oracle(gpu_ctx):
    p = pack.pack(scenes.many_spheres(hdri=None))
    r = Renderer(gpu_ctx, p)
    o = oracle.OracleScene(p)
    rays = random_rays(300_000, 2, center=(0.0, 1.0, 0.0), spread=8.0)
    got = r.trace_closest(rays)
    assert_same(got, o.trace_closest(rays), "closest hits vs oracle BVH")
    info = r.bvh_info()
    assert info.triangles == 1_014_274 and info.wide_depth <= 30


def test_trace_two_instances_hit_distances(gpu_ctx):
    # crates/verion-gpu-metal/tests/trace.rs:95-121: two instances of a triangle at z = -1 and
    # z = -2, rays from the origin down -z hit at distance 1; a ray beside them misses.
    s = sc.Scene()
    m = s.add_mesh(sc.Mesh(np.array([[-1, -1, 0], [1, -1, 0], [0, 1, 0]], np.float32), np.array([0, 1, 2])))
    mat = s.add_material(scenes.material((0.5, 0.5, 0.5)))
    s.add_instance(sc.Instance(m, mat, ((1, 0, 0, 0), (0, 1, 0, 0), (0, 0, 1, -1.0))))
    s.add_instance(sc.Instance(m, mat, ((1, 0, 0, 3.0), (0, 1, 0, 0), (0, 0, 1, -1.0))))
    r = Renderer(gpu_ctx, s)
    rays = np.array([[0, 0, 0, 0, 0, -1], [3, 0, 0, 0, 0, -1], [10, 0, 0, 0, 0, -1]], np.float32)
    h = r.trace_closest(rays)
    t = [h[i, 3:4].view(np.float32)[0] if h[i, 0] else -1.0 for i in range(3)]
    assert t == [1.0, 1.0, -1.0]
    assert h[0, 1] == 0 and h[1, 1] == 1


def test_occlusion_matches_oracle(gpu_ctx):
    p = pack.pack(scenes.cornell())
    r = Renderer(gpu_ctx, p)
    o = oracle.OracleScene(p)
    base = random_rays(100_000, 3, spread=0.9)
    tmax = np.random.default_rng(4).uniform(0.01, 3.0, (len(base), 1)).astype(np.float32)
    rays = np.concatenate([base, tmax], axis=1)
    assert_same(r.trace_occluded(rays), o.trace_occluded(rays), "occlusion")


def test_cornell_megakernel_bit_exact(gpu_ctx):
    p = pack.pack(scenes.cornell())
    w, h, spp = 96, 96, 8
    _, acc = gpu_render(gpu_ctx, p, w, h, spp)
    ref = oracle_render(p, w, h, spp)
    assert_same(acc.sums(), ref.sums, "cornell megakernel sums")


def test_cornell_wavefront_bit_exact_with_queue_counts(gpu_ctx):
    p = pack.pack(scenes.cornell())
    w, h = 80, 64
    r = Renderer(gpu_ctx, p)
    r.set_accum_precision(32)
    r.set_integrator(Integrator.WAVEFRONT)
    r.set_wavefront_mode(WavefrontMode.PER_SAMPLE)
    acc = r.new_accumulation(w, h)
    o = oracle.OracleScene(p)
    ref = oracle.OracleAccumulation(w, h)
    for k in range(4):
        r.accumulate(acc, 1)
        oracle.render(o, params(p, w, h), ref, 1, wavefront=True)
        assert_same(acc.queue_counts(8), np.array(ref.queue_counts[k], np.uint32), f"queue counts, sample {k}")
    assert_same(acc.sums(), ref.sums, "cornell wavefront sums")


def test_wavefront_equals_megakernel(gpu_ctx):
    # pathtrace.rs:169-176 and gpu.rs:50-67: both integrators give the same image, bit for bit.
    p = pack.pack(scenes.furnace_room(0.5, 1.0))
    _, mega = gpu_render(gpu_ctx, p, 16, 16, 8, precision=64)
    _, wave = gpu_render(gpu_ctx, p, 16, 16, 8, precision=64, integrator=Integrator.WAVEFRONT)
    assert_same(wave.sums_f64(), mega.sums_f64(), "wavefront vs megakernel")


def test_white_furnace_returns_the_sky(gpu_ctx):
    # pathtrace.rs:117-137
    r = Renderer(gpu_ctx, scenes.white_furnace())
    img = r.render(32, 32, 4)
    assert np.all(np.abs(img - 1.0) < 1e-4)


def test_closed_room_series_sum(gpu_ctx):
    # pathtrace.rs:103-115: L = E (1 - rho^8) / (1 - rho) within 1%.
    r = Renderer(gpu_ctx, scenes.furnace_room(0.5, 1.0))
    got = float(r.render(64, 64, 64)[:, 0].mean())
    want = (1 - 0.5 ** 8) / (1 - 0.5)
    assert abs(got - want) / want < 0.01


def test_f64_sums_bit_exact(gpu_ctx):
    p = pack.pack(scenes.cornell())
    _, acc = gpu_render(gpu_ctx, p, 64, 48, 8, precision=64)
    ref = oracle_render(p, 64, 48, 8, acc64=True)
    assert_same(acc.sums_f64(), ref.sums, "double sums")


@pytest.mark.parametrize("integrator", [Integrator.MEGAKERNEL, Integrator.WAVEFRONT])
def test_adaptive_counts_and_sums_bit_exact(gpu_ctx, integrator):
    p = pack.pack(scenes.furnace_room(0.5, 1.0))
    a = Adaptive(threshold=0.05, min_spp=4)
    _, acc = gpu_render(gpu_ctx, p, 16, 16, 32, integrator=integrator, adaptive=a, chunks=[8, 8, 8, 8])
    ref = oracle_render(p, 16, 16, 32, adaptive=a)
    assert_same(acc.sums(), ref.sums, "adaptive sums")
    assert_same(acc.raw_stats(), ref.stats, "adaptive statistics")
    counts = acc.sample_counts()
    assert (counts < 32).any() and (counts == 32).any()


def test_adaptive_switch_mid_accumulation_is_an_error(gpu_ctx):
    # pathtrace.rs:216-231
    r = Renderer(gpu_ctx, scenes.furnace_room(0.5, 1.0))
    r.set_adaptive(Adaptive(threshold=1e9, min_spp=4))
    acc = r.new_accumulation(16, 16)
    r.accumulate(acc, 8)
    assert (acc.sample_counts() == 4).all()
    assert acc.active_pixels() == 0
    r.set_adaptive(None)
    with pytest.raises(Error) as e:
        r.accumulate(acc, 1)
    assert e.value.kind == "Scene"


@pytest.mark.parametrize("integrator", [Integrator.MEGAKERNEL, Integrator.WAVEFRONT])
def test_lighting_split_bit_exact(gpu_ctx, integrator):
    s = scenes.cornell()
    s.add_light(sc.Point((0.3, 0.8, 0.2), (1.0, 0.9, 0.8), 2.0))
    s.add_light(sc.Directional((0.2, -1.0, -0.3), (0.5, 0.5, 0.6), 1.0))
    p = pack.pack(s)
    _, acc = gpu_render(gpu_ctx, p, 48, 40, 4, integrator=integrator, lighting=True)
    ref = oracle_render(p, 48, 40, 4, lighting=True)
    assert_same(acc.sums(), ref.sums, "sums with lighting split")
    assert_same(acc.raw_lighting(), ref.lighting, "lighting split")


@pytest.mark.parametrize("integrator", [Integrator.MEGAKERNEL, Integrator.WAVEFRONT])
def test_restir_di_bit_exact(gpu_ctx, integrator):
    p = pack.pack(scenes.cornell())
    rs = Restir(di=True, gi=False, candidates=4, history=4)
    _, acc = gpu_render(gpu_ctx, p, 48, 48, 6, integrator=integrator, restir=rs, chunks=[1, 2, 3])
    ref = oracle_render(p, 48, 48, 6, restir=rs)
    assert_same(acc.sums(), ref.sums, "ReSTIR DI sums")


@pytest.mark.parametrize("integrator", [Integrator.MEGAKERNEL, Integrator.WAVEFRONT])
@pytest.mark.parametrize("di", [False, True])
def test_restir_gi_bit_exact(gpu_ctx, integrator, di):
    # ReSTIR GI (pt_core.slang:897-981, 1566-1617): reservoirs reused across 6 frames, against the
    # oracle's reference-layout reservoirs; with the dispersive glass block and with DI on top.
    from . import analytic as an

    for s in (an.closed_room(0.9), an.room_with(0.9, True)):
        p = pack.pack(s)
        rs = Restir(di=di, gi=True, candidates=4, history=4)
        _, acc = gpu_render(gpu_ctx, p, 48, 48, 6, integrator=integrator, restir=rs, chunks=[1, 2, 3])
        ref = oracle_render(p, 48, 48, 6, restir=rs)
        assert_same(acc.sums(), ref.sums, "ReSTIR GI sums")


def _img(r, w, h, spp):
    acc = r.new_accumulation(w, h)
    r.accumulate(acc, spp)
    return acc.mean()


def test_restir_gi_converges_to_the_path_traced_image(gpu_ctx):
    # crates/verion-gpu-vulkan/tests/restir.rs:240-250
    from . import analytic as an

    r = Renderer(gpu_ctx, an.closed_room(0.9))
    plain = _img(r, 64, 64, 1024).mean()
    r.set_restir(Restir(di=False, gi=True))
    gi = _img(r, 64, 64, 1024).mean()
    assert abs(gi - plain) / plain < 0.03, (plain, gi)


def test_restir_gi_draws_the_same_image_with_both_integrators(gpu_ctx):
    # restir.rs:252-261
    from . import analytic as an

    r = Renderer(gpu_ctx, an.closed_room(0.9))
    r.set_restir(Restir(di=False, gi=True))
    mega = _img(r, 64, 64, 16)
    r.set_integrator(Integrator.WAVEFRONT)
    assert np.array_equal(mega, _img(r, 64, 64, 16))


def test_restir_gi_leaves_sharp_surfaces_alone(gpu_ctx):
    # restir.rs:263-271
    from . import analytic as an

    r = Renderer(gpu_ctx, an.closed_room(0.05))
    plain = _img(r, 64, 64, 8)
    r.set_restir(Restir(di=False, gi=True))
    assert np.array_equal(plain, _img(r, 64, 64, 8))


def test_restir_gi_leaves_no_stains_behind_dispersive_glass(gpu_ctx):
    # restir.rs:273-308: the largest relative difference of the 8x8 block means (per channel) of
    # GI against plain path tracing stays below 0.15 at 2048 spp.
    from . import analytic as an

    r = Renderer(gpu_ctx, an.room_with(0.9, True))
    plain = _img(r, 64, 64, 2048).reshape(8, 8, 8, 8, 3).sum(axis=(1, 3))
    r.set_restir(Restir(di=False, gi=True))
    gi = _img(r, 64, 64, 2048).reshape(8, 8, 8, 8, 3).sum(axis=(1, 3))
    worst = np.max(np.abs(gi - plain) / np.maximum(plain, 1e-3))
    assert worst < 0.15, worst


def test_many_spheres_depth16_env_bit_exact(gpu_ctx):
    s = scenes.many_spheres(hdri=(256, 128))
    p = pack.pack(s)
    w, h = 64, 36
    _, acc = gpu_render(gpu_ctx, p, w, h, 2, depth=16)
    ref = oracle_render(p, w, h, 2, depth=16)
    assert_same(acc.sums(), ref.sums, "1M-triangle scene, depth 16, environment map")


@pytest.mark.parametrize("mode,tail", [(WavefrontMode.PER_SAMPLE, 0), (WavefrontMode.STREAMING, 0),
                                       (WavefrontMode.STREAMING, 400), (WavefrontMode.STREAMING, 1 << 30)])
@pytest.mark.parametrize("adaptive", [None, Adaptive(threshold=0.05, min_spp=4)])
def test_wavefront_modes_match_the_oracle(gpu_ctx, mode, tail, adaptive):
    # Streaming with the tail off (waves only), on at a few hundred live slots, and on at once.
    s = scenes.many_spheres(hdri=(256, 128))
    p = pack.pack(s)
    w, h = 48, 27
    r = Renderer(gpu_ctx, p)
    r.set_accum_precision(32)
    r.set_integrator(Integrator.WAVEFRONT)
    r.set_wavefront_mode(mode)
    r.set_stream_tail(tail)
    r.set_max_depth(16)
    r.set_adaptive(adaptive)
    acc = r.new_accumulation(w, h)
    for n in (5, 7):
        r.accumulate(acc, n)
    ref = oracle_render(p, w, h, 12, depth=16, adaptive=adaptive)
    assert_same(acc.sums(), ref.sums, f"{mode.name} wavefront sums (tail {tail})")
    if adaptive is not None:
        assert_same(acc.raw_stats(), ref.stats, "adaptive statistics")
    if mode == WavefrontMode.STREAMING:
        assert 0 < acc.last_waves() <= 7 * 16 + 3


@pytest.mark.parametrize("deferred,dynamic,coop", [(False, False, False), (True, False, False), (True, True, False),
                                                  (True, True, True)])
def test_streaming_shadow_stage_matches_the_oracle(gpu_ctx, deferred, dynamic, coop):
    # The emitter / environment shadow ray traced inline in shade, or in the separate shadow stage;
    # with dynamic fetch the extend and shadow traversals refill idle lanes from the queue, with
    # coop their warps test the leaves' triangles one (ray, triangle) pair per lane.
    from . import analytic as an

    for s, depth in ((scenes.many_spheres(hdri=(256, 128)), 16), (an.feature_zoo(), 8)):
        p = pack.pack(s)
        r = Renderer(gpu_ctx, p)
        r.set_accum_precision(32)
        r.set_integrator(Integrator.WAVEFRONT)
        r.set_deferred_shadows(deferred)
        r.set_dynamic_fetch(dynamic)
        r.set_coop_triangles(coop)
        r.set_stream_tail(0)
        r.set_max_depth(depth)
        acc = r.new_accumulation(40, 30)
        r.accumulate(acc, 6)
        ref = oracle_render(p, 40, 30, 6, depth=depth)
        assert_same(acc.sums(), ref.sums, f"shadow stage {'deferred' if deferred else 'inline'}")


def test_streaming_lighting_split_bit_exact(gpu_ctx):
    s = scenes.cornell()
    s.add_light(sc.Spot((0.0, 0.9, 0.0), (0.0, -1.0, 0.1), (1.0, 0.8, 0.6), 3.0, 0.3, 0.6))
    p = pack.pack(s)
    _, acc = gpu_render(gpu_ctx, p, 40, 30, 6, integrator=Integrator.WAVEFRONT, lighting=True, chunks=[2, 4])
    ref = oracle_render(p, 40, 30, 6, lighting=True)
    assert_same(acc.sums(), ref.sums, "sums")
    assert_same(acc.raw_lighting(), ref.lighting, "lighting split")


@pytest.mark.parametrize("integrator", [Integrator.MEGAKERNEL, Integrator.WAVEFRONT])
@pytest.mark.parametrize("lighting", [False, True])
def test_feature_zoo_bit_exact(gpu_ctx, integrator, lighting):
    # Textures with mip chains, normal and opacity maps, IES, spot / point / directional lights with
    # light linking, sheen, clearcoat, dispersive and rough glass, textured emitters, instancing.
    from . import analytic as an

    p = pack.pack(an.feature_zoo())
    _, acc = gpu_render(gpu_ctx, p, 64, 48, 6, integrator=integrator, lighting=lighting, chunks=[2, 4])
    ref = oracle_render(p, 64, 48, 6, lighting=lighting)
    assert_same(acc.sums(), ref.sums, "feature zoo sums")
    if lighting:
        assert_same(acc.raw_lighting(), ref.lighting, "feature zoo lighting split")


def test_transparent_background_bit_exact(gpu_ctx):
    from . import analytic as an

    p = pack.pack(an.feature_zoo(transparent_background=True))
    _, acc = gpu_render(gpu_ctx, p, 48, 36, 4, integrator=Integrator.WAVEFRONT)
    ref = oracle_render(p, 48, 36, 4)
    assert_same(acc.sums(), ref.sums, "transparent background sums")


@pytest.mark.parametrize("restir", [None, Restir(di=True, gi=False, candidates=8, history=8)])
def test_material_sorted_shading_matches_the_oracle(gpu_ctx, restir):
    # Deferred shade stage with the wave's slots regrouped by shading class (missed, diffuse,
    # conductor, dielectric) and in queue order: the same sums as the oracle, waves only (tail off).
    s = scenes.many_spheres(hdri=(256, 128))
    p = pack.pack(s)
    out = {}
    for sort in (True, False):
        r = Renderer(gpu_ctx, p)
        r.set_accum_precision(32)
        r.set_integrator(Integrator.WAVEFRONT)
        r.set_max_depth(16)
        r.set_restir(restir)
        r.set_stream_tail(0)
        r.set_material_sort(sort)
        acc = r.new_accumulation(64, 36)
        for n in (2, 3):
            r.accumulate(acc, n)
        out[sort] = acc.sums()
    ref = oracle_render(p, 64, 36, 5, depth=16, restir=restir)
    assert_same(out[True], ref.sums, "material-sorted shading")
    assert_same(out[False], ref.sums, "queue-order shading")


def test_coop_leaf_testing_keeps_hits_and_counters(gpu_ctx):
    # Warp-cooperative leaf testing against each lane testing its own triangles: the same sums,
    # the same nodes visited and triangles tested (the walk's order is unchanged), the same number
    # of shadow rays, on the 1M-triangle scene with adaptive sampling.
    p = pack.pack(scenes.many_spheres(hdri=(256, 128)))
    out = {}
    for coop in (False, True):
        r = Renderer(gpu_ctx, p)
        r.set_accum_precision(32)
        r.set_integrator(Integrator.WAVEFRONT)
        r.set_max_depth(16)
        r.set_adaptive(Adaptive(threshold=0.05, min_spp=4))
        r.set_coop_triangles(coop)
        r.set_stream_tail(0)  # waves only: the tail launch traces each slot's path in one thread
        r.set_traversal_stats(True)
        acc = r.new_accumulation(160, 90)
        for n in (4, 4):
            r.accumulate(acc, n)
        out[coop] = (acc.sums(), acc.traversal_stats(), acc.shadow_rays())
    assert_same(out[True][0], out[False][0], "sums")
    assert out[True][1] == out[False][1]
    assert out[True][2] == out[False][2]
    assert out[True][1]["tests"] > 0


@pytest.mark.parametrize("integrator", [Integrator.MEGAKERNEL, Integrator.WAVEFRONT])
def test_first_sample_index_bit_exact(gpu_ctx, integrator):
    # An accumulation whose sample indices start at 1000 traces the oracle's samples 1000..1006
    # (per-pixel sequences seeded from the sample index), over two calls.
    p = pack.pack(scenes.cornell())
    r = Renderer(gpu_ctx, p)
    r.set_accum_precision(32)
    r.set_integrator(integrator)
    acc = r.new_accumulation(64, 48)
    acc.set_first_sample(1000)
    r.accumulate(acc, 4)
    r.accumulate(acc, 3)
    o = oracle.OracleScene(p)
    ref = oracle.OracleAccumulation(64, 48)
    ref.samples = 1000
    oracle.render(o, params(p, 64, 48), ref, 7)
    assert_same(acc.sums(), ref.sums, "sums from sample 1000")
    zero = r.new_accumulation(64, 48)
    r.accumulate(zero, 7)
    assert not np.array_equal(zero.sums(), acc.sums())
    with pytest.raises(Error):
        acc.set_first_sample(5)  # after the first sample
    r.set_restir(Restir(di=True, gi=False))
    other = r.new_accumulation(16, 16)
    other.set_first_sample(8)
    with pytest.raises(Error) as e:
        r.accumulate(other, 1)
    assert e.value.kind == "Scene"
