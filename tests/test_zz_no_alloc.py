"""vg_trace_closest_noalloc (static device scratch, no allocation) against vg_trace_closest.

Collected last so that it also runs after every other GPU test has used the device; it passes
alone in a fresh process too. Hit records are integers and bit patterns: compared exactly."""
import numpy as np
import pytest

from verion_gb300 import pack, scenes
from verion_gb300.backend import VG_TRACE_NOALLOC_MAX_RAYS, Error, Renderer, device_allocations

pytestmark = pytest.mark.gpu


def rays(n, seed, center=(0.0, 0.0, 0.0), spread=1.2):
    rng = np.random.default_rng(seed)
    o = rng.uniform(-spread, spread, (n, 3)) + np.asarray(center)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, d], axis=1).astype(np.float32)


@pytest.mark.parametrize("scene", ["cornell", "many_spheres"])
def test_noalloc_matches_trace_closest_twice(gpu_ctx, scene):
    if scene == "cornell":
        p, batches = pack.pack(scenes.cornell()), (rays(VG_TRACE_NOALLOC_MAX_RAYS, 11), rays(777, 12))
    else:
        p = pack.pack(scenes.many_spheres(hdri=None))
        batches = (rays(VG_TRACE_NOALLOC_MAX_RAYS, 13, (0.0, 1.0, 0.0), 8.0), rays(40_001, 14, (0.0, 1.0, 0.0), 8.0))
    r = Renderer(gpu_ctx, p)
    for b in batches:
        want = r.trace_closest(b)
        before = device_allocations()
        # Two calls in a row: the fetch counter and error flag are cleared per call.
        for call in range(2):
            got = r.trace_closest_noalloc(b)
            assert np.array_equal(got, want), f"{scene}: call {call}, {len(b)} rays"
        # The property the entry point exists for: no cudaMalloc and no cudaFree in either call.
        assert device_allocations() == before
        assert want[:, 0].any()


def test_noalloc_empty_and_oversized(gpu_ctx):
    r = Renderer(gpu_ctx, pack.pack(scenes.cornell()))
    assert r.trace_closest_noalloc(np.zeros((0, 6), np.float32)).shape == (0, 4)
    with pytest.raises(Error, match="static scratch"):
        r.trace_closest_noalloc(np.zeros((VG_TRACE_NOALLOC_MAX_RAYS + 1, 6), np.float32))
    one = rays(1, 15)
    assert np.array_equal(r.trace_closest_noalloc(one), r.trace_closest(one))
