"""GPU parity on the configurations the benchmark measures, against the CPU oracle.

1. The 1M-triangle workload exactly as the benchmark runs it: the full 1920 x 1080 frame, the
   2048 x 1024 HDRI, depth 16, adaptive sampling (threshold 0.02, 16 minimum samples), f64 sums, the
   streaming wavefront with its defaults (dynamic ray fetch, deferred shadow stage, tail launch),
   over five accumulate calls of 8 samples, so pixels stop at every sample count from 16 on and the
   adaptive state carries across calls. The oracle traces a sample of the frame's rows (the
   predicate reads a pixel's own statistics only, so those rows evolve as in the full frame); the
   f64 sums and the sample counts are compared bit for bit, the statistics after the same
   round-to-nearest cast to f32 the readback applies.
2. ReSTIR DI on the many-light workload (4,096 emissive triangles, 32 candidates, history 20,
   temporal and spatial reuse) under the benchmark's camera pan, both integrators, five frames of
   one sample with the camera moved between frames (the reservoirs of the previous frame are
   reused across the move), bit for bit on a 480 x 270 frame (the spatial reuse reads neighbours of
   the previous frame, so the oracle traces whole frames).

Reference tests these follow: crates/verion-gpu-metal/tests/pathtrace.rs:178-231 (adaptive
sampling), crates/verion-gpu-vulkan/tests/restir.rs:90-121 (ReSTIR DI).
"""
import math

import numpy as np
import pytest

import oracle
from verion_gb300 import pack, scenes
from verion_gb300.backend import Integrator, Renderer
from verion_gb300.pack import View
from verion_gb300.readback import Adaptive, Restir

pytestmark = pytest.mark.gpu

W, H, DEPTH, STEP = 1920, 1080, 16, 8
ADAPTIVE = Adaptive(threshold=0.02, min_spp=16)


def _same(got, want, what):
    bad = np.asarray(got) != np.asarray(want)
    if bad.any():
        i = np.flatnonzero(bad.ravel())[:5]
        raise AssertionError(f"{what}: {int(bad.sum())} of {bad.size} differ, first {i.tolist()}: "
                             f"{np.asarray(got).ravel()[i].tolist()} vs {np.asarray(want).ravel()[i].tolist()}")


def test_benchmark_configuration_bit_exact(gpu_ctx):
    p = pack.pack(scenes.many_spheres())
    assert p.info.env_width == 2048 and p.info.env_height == 1024
    r = Renderer(gpu_ctx, p)
    r.set_integrator(Integrator.WAVEFRONT)
    r.set_max_depth(DEPTH)
    r.set_adaptive(ADAPTIVE)
    r.set_accum_precision(64)
    acc = r.new_accumulation(W, H)
    rows = list(range(3, H, 90)) + [H - 1]
    o = oracle.OracleScene(p)
    ref = oracle.OracleAccumulation(W, H, acc64=True, adaptive=True)
    prm = pack.base_params(p.info, p.view, (W, H), False, True, adaptive=ADAPTIVE, max_depth=DEPTH)
    calls = 5
    for k in range(calls):
        r.accumulate(acc, STEP)
        oracle.render(o, prm, ref, STEP, rows=rows)
        got = acc.sums_f64().reshape(H, W, 3)[rows]
        _same(got, ref.sums.reshape(H, W, 3)[rows], f"f64 sums after call {k + 1}")
    stats = acc.raw_stats().reshape(H, W, 3)[rows]
    want = ref.stats.reshape(H, W, 3)[rows]
    _same(stats[..., 0], want[..., 0], "sample counts")
    _same(stats, want.astype(np.float32), "adaptive statistics")
    counts = stats[..., 0]
    # Pixels stopped at 16, between two calls' boundaries, and ran to the end.
    assert (counts == 16).any() and (counts == STEP * calls).any()
    assert ((counts > 16) & (counts < STEP * calls) & (counts % STEP != 0)).any()


def _pan(f):
    a = math.radians(0.5 * f)
    return View.new(scenes.look_at((14.0 * math.sin(a), 6.0, 14.0 * math.cos(a)), (0.0, 0.5, 0.0), fov=0.9))


@pytest.mark.parametrize("integrator", [Integrator.MEGAKERNEL, Integrator.WAVEFRONT])
def test_many_lights_restir_di_with_camera_pan_bit_exact(gpu_ctx, integrator):
    p = pack.pack(scenes.many_lights())
    assert p.info.emitter_count == 4096
    rs = Restir(di=True, gi=False, candidates=32, history=20)
    w, h = 480, 270
    r = Renderer(gpu_ctx, p)
    r.set_integrator(integrator)
    r.set_accum_precision(32)
    r.set_restir(rs)
    acc = r.new_accumulation(w, h)
    o = oracle.OracleScene(p)
    ref = oracle.OracleAccumulation(w, h, restir=True)
    for f in range(5):
        view = p.view if f == 0 else _pan(f)
        if f > 0:
            r.set_camera(view)
        r.accumulate(acc, 1)
        oracle.render(o, pack.base_params(p.info, view, (w, h), False, True, restir=rs), ref, 1)
        _same(acc.sums(), ref.sums, f"ReSTIR DI sums after frame {f}")
    assert float(ref.sums.mean()) > 0.0
