"""Readback of the sums: with double-precision sums the f32 readback (converted on the device) is
the f64 readback rounded to nearest, bit for bit, into a pinned or a pageable buffer."""
import numpy as np
import pytest

from verion_gb300 import pack, scenes
from verion_gb300.backend import Integrator, Renderer

pytestmark = pytest.mark.gpu


def test_f32_readback_of_f64_sums_is_the_rounded_f64_readback(gpu_ctx):
    import torch

    r = Renderer(gpu_ctx, pack.pack(scenes.cornell()))
    r.set_integrator(Integrator.WAVEFRONT)
    r.set_accum_precision(64)
    acc = r.new_accumulation(67, 45)
    r.accumulate(acc, 5)
    want = acc.sums_f64().astype(np.float32)
    assert np.array_equal(acc.sums(), want)
    pinned = torch.empty(want.size, dtype=torch.float32).pin_memory().numpy()
    acc.sums(into=pinned)
    assert np.array_equal(pinned, want)
