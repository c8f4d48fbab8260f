"""Batched rendering (vg_batch_render): requests of uneven size, scene and sample count in shared
launches (the persistent tile launch, the batch wavefront with its device-side bounce loop). Plain
requests add exactly what a megakernel accumulate adds on either; a cached request without
training adds exactly what the cache integrator adds; repeated batches replay the captured graphs;
the autotuner returns a setting that renders the same sums."""
import numpy as np
import pytest

from verion_gb300 import pack, scenes
from verion_gb300.backend import (BATCH_AS_GIVEN, BATCH_LONGEST_FIRST, BATCH_SHORTEST_FIRST, BatchRequest, Cache,
                                  Error, Integrator, Renderer)
from verion_gb300.readback import Adaptive

pytestmark = pytest.mark.gpu


def scenes_for_batch():
    return [pack.pack(scenes.cornell()), pack.pack(scenes.furnace_room(0.5, 1.0)),
            pack.pack(scenes.many_spheres(hdri=(64, 32)))]


TILES_ONLY = (1 << 64) - 1  # size threshold: every request on the tile launch

SPEC = [(0, 40, 30, 8, 32), (1, 17, 13, 3, 64), (2, 48, 27, 2, 32), (0, 96, 64, 4, 64), (2, 33, 71, 3, 64),
        (1, 128, 96, 1, 32)]


def make(ctx, packed):
    rs, accs = [], []
    for si, w, h, spp, prec in SPEC:
        r = Renderer(ctx, packed[si])
        r.set_accum_precision(prec)
        r.set_max_depth(16 if si == 2 else 8)
        rs.append(r)
        accs.append(r.new_accumulation(w, h))
    return rs, accs


@pytest.mark.parametrize("order", [BATCH_SHORTEST_FIRST, BATCH_AS_GIVEN, BATCH_LONGEST_FIRST])
def test_plain_requests_match_megakernel_accumulates(gpu_ctx, order):
    packed = scenes_for_batch()
    rs, accs = make(gpu_ctx, packed)
    gpu_ctx.set_batch_options(0, order, TILES_ONLY)
    reqs = [BatchRequest(r, a, spec[3]) for r, a, spec in zip(rs, accs, SPEC)]
    out = gpu_ctx.batch_render(reqs)
    again = gpu_ctx.batch_render(reqs)  # same shape: the captured graph is replayed
    assert again.graph_replayed
    assert all(t > 0 for t in out.seconds) and out.total_seconds >= max(out.seconds) * 0.5
    for (si, w, h, spp, prec), a in zip(SPEC, accs):
        r = Renderer(gpu_ctx, packed[si])
        r.set_accum_precision(prec)
        r.set_max_depth(16 if si == 2 else 8)
        r.set_integrator(Integrator.MEGAKERNEL)
        ref = r.new_accumulation(w, h)
        r.accumulate(ref, spp)
        r.accumulate(ref, spp)
        assert a.samples() == 2 * spp
        if prec == 64:
            assert np.array_equal(a.sums_f64(), ref.sums_f64())
        else:
            assert np.array_equal(a.sums(), ref.sums())
    gpu_ctx.set_batch_options(0, BATCH_SHORTEST_FIRST)


WAVE_SPEC = SPEC + [(3, 64, 48, 3, 32), (3, 37, 29, 2, 64)]


@pytest.mark.parametrize("slots,tail,device_loop", [(1 << 21, 32768, True), (1024, 64, True), (1024, 4096, True),
                                                   (1024, 64, False)])
def test_batch_wavefront_matches_megakernel_accumulates(gpu_ctx, slots, tail, device_loop):
    # Threshold 0: every plain request shares the batch wavefront. The feature zoo has opacity
    # cut-outs (shadow rays through translucent layers in the finish stage). With 1024 slots each
    # slot takes many pixels in turn, through the device-side loop (tail 64) or mostly through the
    # tail kernel (tail 4096, above the slot count); the host-driven loop gives the same sums.
    from . import analytic as an

    packed = scenes_for_batch() + [pack.pack(an.feature_zoo())]
    rs, accs = [], []
    for si, w, h, spp, prec in WAVE_SPEC:
        r = Renderer(gpu_ctx, packed[si])
        r.set_accum_precision(prec)
        r.set_max_depth(16 if si == 2 else 8)
        r.set_stream_tail(tail)
        rs.append(r)
        accs.append(r.new_accumulation(w, h))
    gpu_ctx.set_batch_options(0, BATCH_SHORTEST_FIRST, 0)
    gpu_ctx.set_batch_wave_slots(slots)
    gpu_ctx.set_batch_device_loop(device_loop)
    try:
        reqs = [BatchRequest(r, a, spec[3]) for r, a, spec in zip(rs, accs, WAVE_SPEC)]
        out = gpu_ctx.batch_render(reqs)
        again = gpu_ctx.batch_render(reqs)  # same shape: the captured graph is replayed
    finally:
        gpu_ctx.set_batch_options(0, BATCH_SHORTEST_FIRST)
        gpu_ctx.set_batch_wave_slots(1 << 21)
        gpu_ctx.set_batch_device_loop(True)
    assert again.graph_replayed and not out.graph_replayed
    assert all(t > 0 for t in again.seconds) and again.total_seconds >= max(again.seconds)
    for (si, w, h, spp, prec), a in zip(WAVE_SPEC, accs):
        r = Renderer(gpu_ctx, packed[si])
        r.set_accum_precision(prec)
        r.set_max_depth(16 if si == 2 else 8)
        r.set_integrator(Integrator.MEGAKERNEL)
        ref = r.new_accumulation(w, h)
        r.accumulate(ref, spp)
        r.accumulate(ref, spp)
        assert a.samples() == 2 * spp
        if prec == 64:
            assert np.array_equal(a.sums_f64(), ref.sums_f64())
        else:
            assert np.array_equal(a.sums(), ref.sums())


@pytest.mark.parametrize("slots", [1 << 21, 1024])
def test_batch_wavefront_cached_requests_match_the_cache_integrator(gpu_ctx, slots):
    # Threshold 0: cached requests share the batch wavefront with plain ones. Without training the
    # caches are fixed, so each cached request adds exactly what the megakernel cache integrator
    # adds (one sample per frame): the same paths, training pixels, queries and answers, in the
    # same order per pixel. Two caches answer in the same wave kernel; the feature zoo has
    # translucent surfaces; with 1024 slots the slots take many pixels each.
    from . import analytic as an

    packed = [pack.pack(scenes.cornell()), pack.pack(an.feature_zoo())]
    spec = [(0, 48, 40, 3, 64, 0), (1, 37, 29, 2, 64, 1), (0, 33, 20, 4, 32, 0), (0, 40, 30, 2, 32, None)]

    def renderer(si, prec, cached):
        r = Renderer(gpu_ctx, packed[si])
        r.set_accum_precision(prec)
        c = None
        if cached:
            c = Cache(gpu_ctx, bounds=r.bounds(), seed=7)
            r.set_cache(c, spread=0.01, train_paths=256, train_steps=0, train_batch=1024)
        return r, c

    shared = {}
    reqs, accs = [], []
    for si, w, h, spp, prec, ci in spec:
        if ci is None:
            r, c = renderer(si, prec, False)
        else:
            if ci not in shared:
                shared[ci] = renderer(si, prec, True)
            r, c = shared[ci]
            r.set_accum_precision(prec)
        a = r.new_accumulation(w, h)
        accs.append(a)
        reqs.append(BatchRequest(r, a, spp, c))
    gpu_ctx.set_batch_options(0, BATCH_SHORTEST_FIRST, 0)
    gpu_ctx.set_batch_wave_slots(slots)
    try:
        out = gpu_ctx.batch_render(reqs)
    finally:
        gpu_ctx.set_batch_options(0, BATCH_SHORTEST_FIRST)
        gpu_ctx.set_batch_wave_slots(1 << 21)
    assert len(out.seconds) == len(spec)
    for (si, w, h, spp, prec, ci), a in zip(spec, accs):
        r, _ = renderer(si, prec, ci is not None)
        ref = r.new_accumulation(w, h)
        r.accumulate(ref, spp)
        assert a.samples() == spp
        if prec == 64:
            assert np.array_equal(a.sums_f64(), ref.sums_f64()), (si, w, h)
        else:
            assert np.array_equal(a.sums(), ref.sums()), (si, w, h)


def test_batch_wavefront_trains_the_caches(gpu_ctx):
    p = pack.pack(scenes.cornell())
    r = Renderer(gpu_ctx, p)
    cache = Cache(gpu_ctx, bounds=r.bounds())
    r.set_cache(cache, spread=0.01, train_paths=1024, train_steps=2, train_batch=4096)
    before, _ = cache.read_params()
    gpu_ctx.set_batch_options(0, BATCH_SHORTEST_FIRST, 0)
    try:
        gpu_ctx.batch_render([BatchRequest(r, r.new_accumulation(64, 64), 2, cache)])
    finally:
        gpu_ctx.set_batch_options(0, BATCH_SHORTEST_FIRST)
    after, _ = cache.read_params()
    assert not np.array_equal(before, after)


def test_batch_wavefront_finishes_small_requests_early(gpu_ctx):
    packed = scenes_for_batch()
    r = Renderer(gpu_ctx, packed[2])
    r.set_max_depth(16)
    sizes = [(32, 32, 1), (256, 256, 4), (64, 64, 2), (512, 256, 4)]
    reqs = [BatchRequest(r, r.new_accumulation(w, h), spp) for w, h, spp in sizes]
    gpu_ctx.set_batch_options(0, BATCH_SHORTEST_FIRST, 0)
    try:
        out = gpu_ctx.batch_render(reqs)
    finally:
        gpu_ctx.set_batch_options(0, BATCH_SHORTEST_FIRST)
    assert out.seconds[0] < out.seconds[1] and out.seconds[0] < out.seconds[3]
    assert out.seconds[2] < out.seconds[3]


def test_shortest_first_finishes_small_requests_early(gpu_ctx):
    packed = scenes_for_batch()
    r = Renderer(gpu_ctx, packed[2])
    r.set_max_depth(16)
    sizes = [(32, 32, 1), (256, 256, 4), (64, 64, 2), (512, 256, 4)]
    reqs = [BatchRequest(r, r.new_accumulation(w, h), spp) for w, h, spp in sizes]
    gpu_ctx.set_batch_options(0, BATCH_SHORTEST_FIRST, TILES_ONLY)
    try:
        out = gpu_ctx.batch_render(reqs)
    finally:
        gpu_ctx.set_batch_options(0, BATCH_SHORTEST_FIRST)
    assert out.seconds[0] < out.seconds[1] and out.seconds[0] < out.seconds[3]
    assert max(out.seconds) == out.seconds[3]


def test_cached_request_matches_the_cache_integrator_without_training(gpu_ctx):
    p = pack.pack(scenes.cornell())
    w, h, spp = 48, 40, 4
    r1 = Renderer(gpu_ctx, p)
    c1 = Cache(gpu_ctx, bounds=r1.bounds())
    r1.set_cache(c1, spread=0.01, train_paths=256, train_steps=0, train_batch=1024)
    a1 = r1.new_accumulation(w, h)
    r1.accumulate(a1, spp)
    r2 = Renderer(gpu_ctx, p)
    c2 = Cache(gpu_ctx, bounds=r2.bounds())
    r2.set_cache(c2, spread=0.01, train_paths=256, train_steps=0, train_batch=1024)
    a2 = r2.new_accumulation(w, h)
    plain = r2.new_accumulation(w, h)
    gpu_ctx.set_batch_options(0, BATCH_SHORTEST_FIRST, TILES_ONLY)
    try:
        out = gpu_ctx.batch_render([BatchRequest(r2, a2, spp, c2), BatchRequest(r2, plain, 2)])
    finally:
        gpu_ctx.set_batch_options(0, BATCH_SHORTEST_FIRST)
    assert len(out.seconds) == 2
    assert np.array_equal(a2.sums_f64(), a1.sums_f64())


def test_cached_requests_train_their_cache(gpu_ctx):
    p = pack.pack(scenes.cornell())
    r = Renderer(gpu_ctx, p)
    cache = Cache(gpu_ctx, bounds=r.bounds())
    r.set_cache(cache, spread=0.01, train_paths=1024, train_steps=2, train_batch=4096)
    before, _ = cache.read_params()
    gpu_ctx.set_batch_options(0, BATCH_SHORTEST_FIRST, TILES_ONLY)
    try:
        gpu_ctx.batch_render([BatchRequest(r, r.new_accumulation(64, 64), 2, cache)])
    finally:
        gpu_ctx.set_batch_options(0, BATCH_SHORTEST_FIRST)
    after, _ = cache.read_params()
    assert not np.array_equal(before, after)


def test_tune_picks_a_setting_and_keeps_the_sums(gpu_ctx):
    packed = scenes_for_batch()
    rs, accs = make(gpu_ctx, packed)
    reqs = [BatchRequest(r, a, spec[3]) for r, a, spec in zip(rs, accs, SPEC)]
    t = gpu_ctx.batch_tune(reqs)
    assert t["trials"] >= 8 and t["blocks_per_sm"] >= 1 and t["p50_seconds"] > 0
    assert t["wave_slots"] in (1 << 20, 1 << 21)
    assert all(a.samples() == 0 for a in accs)  # the tuner used scratch accumulations
    gpu_ctx.batch_render(reqs)
    si, w, h, spp, prec = SPEC[0]
    r = Renderer(gpu_ctx, packed[si])
    r.set_accum_precision(prec)
    ref = r.new_accumulation(w, h)
    r.accumulate(ref, spp)
    assert np.array_equal(accs[0].sums(), ref.sums())
    gpu_ctx.set_batch_options(0, BATCH_SHORTEST_FIRST)
    gpu_ctx.set_batch_wave_slots(1 << 21)


def test_batch_rejects_adaptive_requests(gpu_ctx):
    r = Renderer(gpu_ctx, scenes.cornell())
    r.set_adaptive(Adaptive())
    with pytest.raises(Error):
        gpu_ctx.batch_render([BatchRequest(r, r.new_accumulation(16, 16), 1)])


def test_large_requests_leave_the_shared_launch(gpu_ctx):
    # Above the threshold a plain request runs on the batch wavefront after the tile launch; its
    # sums are still the megakernel's and it finishes after the small request.
    p = pack.pack(scenes.cornell())
    r = Renderer(gpu_ctx, p)
    r.set_accum_precision(32)
    small, big = r.new_accumulation(40, 40), r.new_accumulation(200, 150)
    gpu_ctx.set_batch_options(0, BATCH_SHORTEST_FIRST, 100 * 100)
    out = gpu_ctx.batch_render([BatchRequest(r, big, 3), BatchRequest(r, small, 5)])
    assert out.seconds[1] < out.seconds[0]
    for acc, (w, h, spp) in ((small, (40, 40, 5)), (big, (200, 150, 3))):
        ref_r = Renderer(gpu_ctx, p)
        ref_r.set_accum_precision(32)
        ref = ref_r.new_accumulation(w, h)
        ref_r.accumulate(ref, spp)
        assert np.array_equal(acc.sums(), ref.sums())
    gpu_ctx.set_batch_options(0, BATCH_SHORTEST_FIRST)
