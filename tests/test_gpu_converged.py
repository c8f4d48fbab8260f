"""GPU images against the converged FP64 CPU oracle images (tests/golden/converged_fp64.npz, written
by tests/golden/make_converged.py: the oracle in double precision, samples from index 2^20, so no
sample is shared with these renders).

For an unbiased image of N samples the RMSE against the oracle image is predicted by the noise
alone: the oracle image's noise e (measured from its two halves) belongs to M samples, so the
per-sample standard deviation is e sqrt(M) and the expected RMSE is e sqrt(M / N + 1). Bounds, by
scene: the Cornell box within 0.8-1.25 of the prediction and the reference's exr_diff gates (worst
channel mean within 1%, worst 4 x 4 block mean within 2%: crates/verion-render-io/examples/exr_diff.rs);
the many-light scene's direct light within 0.8-1.25 and the channel gate; the 1M-triangle workload's
rows (a sun of radiance 1e4 behind glass: a heavy-tailed error) at most 1.5 times the prediction and
its mean within 3%.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from verion_gb300 import pack, scenes
from verion_gb300.backend import Integrator, Renderer
from verion_gb300.exr import diff

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def fixture(name):
    npz, js = GOLDEN / "converged_fp64.npz", GOLDEN / "converged_fp64.json"
    return np.load(npz)[name].astype(np.float64), json.loads(js.read_text())[name]


def render(ctx, p, w, h, spp, depth, integrator):
    r = Renderer(ctx, p)
    r.set_integrator(integrator)
    r.set_max_depth(depth)
    r.set_accum_precision(64)
    acc = r.new_accumulation(w, h)
    done = 0
    while done < spp:
        n = min(64, spp - done)
        r.accumulate(acc, n)
        done += n
    return acc.mean().astype(np.float64).reshape(h, w, 3)


def predicted(meta, n):
    return meta["noise_rmse"] * np.sqrt(meta["spp"] / n + 1.0)


@pytest.mark.parametrize("integrator", [Integrator.MEGAKERNEL, Integrator.WAVEFRONT])
def test_cornell_against_the_fp64_oracle(gpu_ctx, integrator):
    ref, meta = fixture("cornell_512_d8")
    img = render(gpu_ctx, pack.pack(scenes.cornell()), 512, 512, 256, 8, integrator)
    rmse = float(np.sqrt(np.mean((img - ref) ** 2)))
    want = predicted(meta, 256)
    assert 0.8 * want <= rmse <= 1.25 * want, (rmse, want)
    d = diff(ref.reshape(-1, 3), img.reshape(-1, 3), 512, 512)
    assert d["pass"], d


def test_many_lights_direct_light_against_the_fp64_oracle(gpu_ctx):
    ref, meta = fixture("many_lights_480x270_d1")
    img = render(gpu_ctx, pack.pack(scenes.many_lights()), 480, 270, 128, 1, Integrator.WAVEFRONT)
    rmse = float(np.sqrt(np.mean((img - ref) ** 2)))
    want = predicted(meta, 128)
    assert 0.8 * want <= rmse <= 1.25 * want, (rmse, want)
    # The channel gate only: the visible emitters (radiance up to 100) leave 4 x 4 block means
    # noisier than exr_diff's 2% at 128 samples.
    d = diff(ref.reshape(-1, 3), img.reshape(-1, 3), 480, 270)
    assert d["channel"] < 0.01, d


def test_benchmark_rows_against_the_fp64_oracle(gpu_ctx):
    ref, meta = fixture("many_spheres_1080p_d16_rows476_507")
    r0, r1 = meta["rows"]
    img = render(gpu_ctx, pack.pack(scenes.many_spheres()), 1920, 1080, 64, 16, Integrator.WAVEFRONT)[r0:r1]
    rmse = float(np.sqrt(np.mean((img - ref) ** 2)))
    assert rmse <= 1.5 * predicted(meta, 64), (rmse, predicted(meta, 64))
    assert abs(img.mean() / ref.mean() - 1.0) < 0.03
