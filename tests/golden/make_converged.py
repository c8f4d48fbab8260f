"""Renders the converged reference images of the benchmark's scenes with the CPU oracle in double
precision (FP64 arithmetic and FP64 sums) and writes them to tests/golden/converged_fp64.npz (float16
pixel means, (rows, width, 3) per image) with their settings and noise in converged_fp64.json.

`python tests/golden/make_converged.py [name ...]` (all images by default; minutes of CPU time).

* Samples start at index 2^20: the per-pixel random sequence is seeded from the sample index
  (pt_core.slang:645-682), so these images share no sample with a render of fewer than 2^20
  samples, and an RMSE against them is not lowered by correlated noise.
* Each image is rendered in two halves; `noise_rmse` = RMSE(half 1 - half 2) / 2 estimates the
  RMSE of the full image against the true solution, the floor under any RMSE measured against it.
* float16 keeps 11 significant bits (a relative rounding of 2^-12), far below the noise.
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

SAMPLE_OFFSET = 1 << 20

# name: scene, frame size, max depth, samples, rows of the frame (None: all)
IMAGES = {
    "cornell_512_d8": ("cornell", (512, 512), 8, 2048, None),
    "many_spheres_1080p_d16_rows476_507": ("many_spheres", (1920, 1080), 16, 1024, list(range(476, 508))),
    "many_lights_480x270_d8": ("many_lights", (480, 270), 8, 1024, None),
    "many_lights_480x270_d1": ("many_lights", (480, 270), 1, 1024, None),
}


def render(name: str):
    import oracle
    from verion_gb300 import pack, scenes

    scene, (w, h), depth, spp, rows = IMAGES[name]
    p = pack.pack(getattr(scenes, scene)())
    o = oracle.OracleScene(p)
    prm = pack.base_params(p.info, p.view, (w, h), False, True, max_depth=depth)
    acc = oracle.OracleAccumulation(w, h, acc64=True)
    acc.samples = SAMPLE_OFFSET
    sel = slice(None) if rows is None else rows
    t0 = time.perf_counter()
    oracle.render(o, prm, acc, spp // 2, double=True, rows=rows)
    first = acc.sums.reshape(h, w, 3)[sel].copy()
    oracle.render(o, prm, acc, spp - spp // 2, double=True, rows=rows)
    dt = time.perf_counter() - t0
    full = acc.sums.reshape(h, w, 3)[sel]
    m1 = first / (spp // 2)
    m2 = (full - first) / (spp - spp // 2)
    mean = full / spp
    noise = float(np.sqrt(np.mean((m1 - m2) ** 2)) / 2.0)
    meta = {"scene": scene, "width": w, "height": h, "max_depth": depth, "spp": spp,
            "rows": [rows[0], rows[-1] + 1] if rows else [0, h], "sample_offset": SAMPLE_OFFSET,
            "precision": "oracle double mode: f64 arithmetic, f64 sums", "noise_rmse": noise,
            "mean": float(mean.mean()), "seconds": dt, "threads": oracle.default_threads()}
    return mean.astype(np.float16), meta


def main(names) -> None:
    npz = HERE / "converged_fp64.npz"
    js = HERE / "converged_fp64.json"
    arrays = dict(np.load(npz)) if npz.exists() else {}
    metas = json.loads(js.read_text()) if js.exists() else {}
    for name in names:
        img, meta = render(name)
        arrays[name] = img
        metas[name] = meta
        print(name, json.dumps(meta), flush=True)
        np.savez_compressed(npz, **arrays)
        js.write_text(json.dumps(metas, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    main(sys.argv[1:] or list(IMAGES))
