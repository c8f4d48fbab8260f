"""The wave graph, the BVH8's SAH cost and the wavefront autotuner change speed, never sums."""
import numpy as np
import pytest

from verion_gb300 import pack, scenes
from verion_gb300.backend import Integrator, Renderer, WavefrontMode

pytestmark = pytest.mark.gpu


def render(r, w, h, spp, chunks=1):
    acc = r.new_accumulation(w, h)
    for _ in range(chunks):
        r.accumulate(acc, spp)
    return acc.sums()


def wave_renderer(ctx, p, depth=16):
    r = Renderer(ctx, p)
    r.set_accum_precision(32)
    r.set_integrator(Integrator.WAVEFRONT)
    r.set_wavefront_mode(WavefrontMode.STREAMING)
    r.set_max_depth(depth)
    return r


@pytest.mark.parametrize("tail", [0, 4000])
@pytest.mark.parametrize("waves", [2, 8])
def test_wave_graph_gives_the_same_sums(gpu_ctx, tail, waves):
    p = pack.pack(scenes.many_spheres(hdri=(256, 128)))
    ref = wave_renderer(gpu_ctx, p)
    ref.set_stream_tail(tail)
    want = render(ref, 96, 54, 3, chunks=2)
    r = wave_renderer(gpu_ctx, p)
    r.set_stream_tail(tail)
    r.set_wavefront_graph(waves)
    assert np.array_equal(render(r, 96, 54, 3, chunks=2), want)


def test_wave_graph_rejects_odd_counts(gpu_ctx):
    from verion_gb300.backend import Error

    r = Renderer(gpu_ctx, scenes.cornell())
    with pytest.raises(Error):
        r.set_wavefront_graph(3)


def test_bvh_traversal_cost_keeps_the_hits(gpu_ctx):
    p = pack.pack(scenes.many_spheres(hdri=None))
    r = wave_renderer(gpu_ctx, p)
    want = render(r, 64, 36, 2)
    nodes = r.bvh_info().wide_nodes
    r.set_bvh_traversal_cost(2.0)
    assert r.bvh_info().wide_nodes != nodes
    assert np.array_equal(render(r, 64, 36, 2), want)


def test_autotune_keeps_the_sums(gpu_ctx):
    p = pack.pack(scenes.many_spheres(hdri=(256, 128)))
    r = wave_renderer(gpu_ctx, p)
    t = r.autotune(160, 90, 2)
    assert t["trials"] >= 6 and t["mpaths_after"] >= t["mpaths_before"] > 0
    assert t["graph_waves"] in (0, 8) and t["bvh_traversal_cost"] in (0.25, 0.5, 1.0, 2.0)
    assert t["extend_blocks_per_sm"] >= 1
    assert t["coop_triangles"] in (0, 1) and t["fetch_refill"] in (4, 8, 16) and t["fetch_steps"] in (2, 4, 8)
    assert t["material_sort"] in (0, 1)
    fresh = wave_renderer(gpu_ctx, p)
    assert np.array_equal(render(r, 80, 45, 3), render(fresh, 80, 45, 3))


@pytest.mark.parametrize("refill,steps", [(1, 1), (4, 2), (16, 8), (32, 64)])
def test_traversal_fetch_settings_keep_the_sums(gpu_ctx, refill, steps):
    p = pack.pack(scenes.many_spheres(hdri=(256, 128)))
    want = render(wave_renderer(gpu_ctx, p), 64, 36, 2)
    for coop in (False, True):
        r = wave_renderer(gpu_ctx, p)
        r.set_stream_tail(0)  # waves only: small frames would otherwise go straight to the tail launch
        r.set_coop_triangles(coop)
        r.set_traversal_fetch(refill, steps)
        assert np.array_equal(render(r, 64, 36, 2), want), (refill, steps, coop)


def test_traversal_fetch_rejects_out_of_range(gpu_ctx):
    from verion_gb300.backend import Error

    r = Renderer(gpu_ctx, scenes.cornell())
    for bad in ((0, 4), (33, 4), (8, 0), (8, 65)):
        with pytest.raises(Error):
            r.set_traversal_fetch(*bad)


def test_traversal_counters_count_and_change_nothing(gpu_ctx):
    # The counting instantiations of the extend and shadow stages give the same sums; they count
    # every closest-hit ray (one per path vertex reached, at least one per camera path) and the
    # shadow rays of the deferred light samples (at most one per closest hit).
    p = pack.pack(scenes.many_spheres(hdri=(256, 128)))
    r = wave_renderer(gpu_ctx, p)
    want = render(r, 96, 54, 2)
    r.set_traversal_stats(True)
    acc = r.new_accumulation(96, 54)
    r.accumulate(acc, 2)
    st = acc.traversal_stats()
    shadow = acc.shadow_rays()
    assert np.array_equal(acc.sums(), want)
    assert st["rays"] >= 96 * 54 * 2 and st["nodes"] > st["rays"]
    assert 0 < shadow <= st["rays"]
