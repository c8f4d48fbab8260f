"""Benchmark of the CUDA path-tracing backend on the 1M-triangle wavefront workload.

Workload (the 1M-triangle benchmark configuration): 64 subdivided spheres on a noise-displaced 512 x 512 grid
(1,014,274 triangles; GGX conductor / dielectric / Lambertian materials), a 2048 x 1024 float HDRI,
1920 x 1080, max depth 16, wavefront integrator with adaptive sampling (threshold 0.02, 16 minimum
samples), double-precision sums. All inputs are generated from seeds (`data: synthetic`).

One step = `accumulate(acc, 8)`: eight samples per pixel of the running render (the reference
session's 8-sample chunk, crates/verion-render/src/session.rs:244-248). `value` is camera paths
traced per second (Mpaths/s), counted exactly from the adaptive sample counts, over the device time
of the timed steps (CUDA events on the backend's stream); L2 is flushed (a 256 MiB write) between
steps. `e2e` is the same metric through the C ABI with host buffers: each step sets the camera
(host to device) and reads the pixel sums into pinned host memory (device to host), timed on the
host clock.

`--impl reference` times the CPU restatement of the reference's integrator (the oracle) on the host
cores instead: the reference itself (Rust + Slang on Metal / Vulkan hardware ray tracing) cannot run
on this machine.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WIDTH, HEIGHT, DEPTH, SPP_STEP = 1920, 1080, 16, 8
ADAPTIVE = (0.02, 16)
METRIC = "Mpaths/s (camera paths traced per second), 1M-triangle scene, 1920x1080, depth 16"
UNIT = "Mpaths/s"


def parse():
    global WIDTH, HEIGHT
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["cuda", "reference"], default="cuda")
    ap.add_argument("--integrator", choices=["wavefront", "megakernel"], default="wavefront")
    ap.add_argument("--cpu-seconds", type=float, default=16.0, help="target length of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-cache", action="store_true", help="skip the radiance-cache measurement")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-serving measurement")
    ap.add_argument("--no-restir", action="store_true", help="skip the ReSTIR DI many-light measurement")
    ap.add_argument("--batch-spp-scale", type=float, default=1.0,
                    help="batched serving: fraction of the 16-256 spp range to render (1 = the full workload)")
    ap.add_argument("--profile-extend", action="store_true",
                    help="profiling helper: one step with traversal counters inside the NVTX range 'traffic', "
                         "then print the counters (for an ncu capture of the extend kernels' DRAM bytes)")
    ap.add_argument("--profile-cache", action="store_true",
                    help="profiling helper: the radiance cache on this workload (the cache report's C2 settings), "
                         "--warmup frames of 4 samples, then one timed frame; prints its device time and split")
    ap.add_argument("--profile-mlp", action="store_true",
                    help="profiling helper: the cache's kernels on 2^20 synthetic records, one untimed and one "
                         "timed launch of each (encode, inference, training pass, scatter); prints their times")
    ap.add_argument("--profile-batch", action="store_true",
                    help="profiling helper: one small batch (16 requests of 128-256 px square, 4-16 spp, plain and "
                         "cached, scenes of the 1M-triangle kind) on the tile launch, rendered twice through "
                         "vg_batch_render")
    ap.add_argument("--profile-batch-wave", action="store_true",
                    help="profiling helper: the --profile-batch requests through the batch wavefront (size "
                         "threshold 0, host-driven loop), rendered twice through vg_batch_render")
    ap.add_argument("--profile-per-sample", action="store_true",
                    help="profiling helper: the benchmark scene at --width x --height on the per-sample wavefront "
                         "(the reference's depth-by-depth order: wf_begin / wf_select / wf_extend / wf_shade), "
                         "adaptive (0.02, 16), 20 samples in one accumulate call")
    ap.add_argument("--profile-restir", action="store_true",
                    help="profiling helper: the many-light scene with ReSTIR DI (32 candidates) at --width x --height "
                         "on the streaming wavefront, four frames of one sample")
    ap.add_argument("--width", type=int, default=WIDTH, help="smaller frames are for profiling runs only")
    ap.add_argument("--height", type=int, default=HEIGHT)
    a = ap.parse_args()
    WIDTH, HEIGHT = a.width, a.height
    return a


def workload():
    from verion_gb300 import pack, scenes

    s = scenes.many_spheres()
    return s, pack.pack(s)


def config(args, extra=None):
    c = {"workload": "many_spheres_1M_tris_hdri2048", "triangles": 1_014_274, "width": WIDTH, "height": HEIGHT,
         "max_depth": DEPTH, "spp_per_step": SPP_STEP, "integrator": args.integrator,
         "adaptive": {"threshold": ADAPTIVE[0], "min_spp": ADAPTIVE[1]}, "sums": "f64",
         "l2": "flushed between steps (256 MiB write)", "parallelism": f"replicas x{args.gpus}"}
    if extra:
        c.update(extra)
    return c


def dist_init(args, backend=None):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = backend or ("nccl" if args.impl == "cuda" else "gloo")
        dist.init_process_group(backend)
    return rank, world


def select_device() -> int:
    """CUDA ordinal of this process: LOCAL_RANK under torchrun (one process per GPU), else 0."""
    return int(os.environ.get("LOCAL_RANK", "0"))


def open_device(args, set_device=None, make_context=None, backend=None):
    """Makes this rank's GPU current (before the process group, so NCCL binds it), joins the
    group, builds the library once per node (local rank 0; the others wait at a barrier) and opens
    the backend's context on that GPU. Returns (rank, world, device, context)."""
    dev = select_device()
    if set_device is None:
        import torch

        set_device = torch.cuda.set_device
    set_device(dev)
    rank, world = dist_init(args, backend)
    if make_context is None:
        from verion_gb300 import build
        from verion_gb300.backend import Context

        if dev == 0:
            build.build()
        barrier(world)
        if dev != 0:
            build.build()  # finds the library up to date
        make_context = Context
    return rank, world, dev, make_context(device=dev)


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def allmax(world, v: float) -> float:
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(world, v: float) -> float:
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self._p = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                        "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except FileNotFoundError:
            self._p = None
        return self

    def _read(self):
        for line in self._p.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self._p:
            self._p.terminate()
            try:
                self._p.wait(timeout=5)
            except Exception:
                self._p.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[4 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_per_ray():
    """DRAM bytes per extend ray from the committed ncu summary of wf_extend, if present."""
    p = ROOT / "profiles" / "wf_extend_traffic.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["dram_bytes_per_ray"]), d.get("source", str(p.name))
    return None, None


def oracle_steps(packed, warmup: int, steps: int, step_seconds: float, threads: int = 0):
    """The oracle (the reference's integrator restated in single precision) on a row sample of the
    benchmark frame with the GPU arm's settings: adaptive sampling (0.02, 16), f64 sums, depth 16,
    8 samples per step. `warmup` untimed steps, then `steps` timed ones on the same accumulation,
    so the timed steps trace the pixels adaptive sampling left active, as the GPU arm's do (the
    predicate reads a pixel's own statistics only, so a row sample evolves exactly like those rows
    of the full frame). Every k-th row, k chosen so that a step with every pixel active takes about
    `step_seconds`. Returns (Mpaths/s over the timed steps, seconds per timed step, sample text)."""
    import oracle
    from verion_gb300 import pack
    from verion_gb300.readback import Adaptive

    o = oracle.OracleScene(packed)
    threads = threads or oracle.default_threads()
    prm = pack.base_params(packed.info, packed.view, (WIDTH, HEIGHT), False, True, adaptive=Adaptive(*ADAPTIVE),
                           max_depth=DEPTH)
    probe = list(range(0, HEIGHT, 135))[:8]
    acc = oracle.OracleAccumulation(WIDTH, HEIGHT, acc64=True, adaptive=True)
    t0 = time.perf_counter()
    oracle.render(o, prm, acc, SPP_STEP, threads=threads, rows=probe)
    per_row = (time.perf_counter() - t0) / len(probe)
    n = int(max(1, min(HEIGHT, step_seconds / max(per_row, 1e-6))))
    stride = max(1, HEIGHT // n)
    rows = list(range(stride // 2, HEIGHT, stride))[:n]
    acc = oracle.OracleAccumulation(WIDTH, HEIGHT, acc64=True, adaptive=True)

    def traced():
        return float(acc.stats.reshape(-1, 3)[:, 0].sum())

    for _ in range(warmup):
        oracle.render(o, prm, acc, SPP_STEP, threads=threads, rows=rows)
    p0 = traced()
    times = []
    for _ in range(steps):
        t = time.perf_counter()
        oracle.render(o, prm, acc, SPP_STEP, threads=threads, rows=rows)
        times.append(time.perf_counter() - t)
    paths = traced() - p0
    sample = (f"{len(rows)} of {HEIGHT} rows (every {stride}th) x {WIDTH} px, {warmup} untimed + {steps} timed "
              f"steps of {SPP_STEP} spp with adaptive sampling {ADAPTIVE} and f64 sums, {paths:.0f} paths timed")
    return paths / sum(times) / 1e6, times, sample, threads


def cpu_baseline(packed, seconds: float, warmup: int, threads: int = 0):
    """The oracle on a bounded row sample of the same workload (oracle_steps): the GPU arm's warm-up
    steps, then two timed steps, about `seconds` of CPU work in all."""
    per_step = seconds / (warmup + 2)
    value, times, sample, threads = oracle_steps(packed, warmup, 2, per_step, threads)
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample}, sum(times)


def run_reference(args):
    rank, world = dist_init(args)
    if rank != 0:
        return 0
    _, packed = workload()
    # Each step: a bounded row sample of the frame at 8 spp, about 1.5 s with every pixel active.
    value, times, sample, threads = oracle_steps(packed, args.warmup, args.steps, 1.5)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config(args, {"integrator": "megakernel (CPU)"}), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


CACHE_W = CACHE_H = 512
C2_ORACLE = "many_spheres_1080p_d16_rows476_507"  # converged FP64 oracle rows of the 1M-triangle frame
CACHE_REF_SPP = 8192
C2_REF_SPP = 2048
REF_FIRST_SAMPLE = 1 << 24  # reference images start here: no sample shared with a measured curve
CACHE_MLP_FLOP = 2 * (4 * 64 * 64 + 64 * 3)  # per record, inference (algorithmic, 3 outputs)


def _rmse(a, b):
    return float(np.sqrt(np.mean((a - b) ** 2)))


_CONVERGED = None


def converged(name):
    """A converged image of the CPU oracle in double precision (tests/golden/make_converged.py):
    (float64 (rows, width, 3) pixel means, its settings), or (None, None) if absent."""
    global _CONVERGED
    if _CONVERGED is None:
        npz, js = ROOT / "tests" / "golden" / "converged_fp64.npz", ROOT / "tests" / "golden" / "converged_fp64.json"
        _CONVERGED = (dict(np.load(npz)), json.loads(js.read_text())) if npz.exists() and js.exists() else ({}, {})
    img, meta = _CONVERGED[0].get(name), _CONVERGED[1].get(name)
    return (None, None) if img is None else (img.astype(np.float64), meta)


def rmse_vs_fp64(img, width, height, name):
    """RMSE of a (pixels, 3) mean image of `width` x `height` against the converged FP64 oracle image
    `name`, over that image's rows; with the oracle image's own noise (the floor of any such RMSE)."""
    ref, meta = converged(name)
    if ref is None or (meta["width"], meta["height"]) != (width, height):
        return None
    r0, r1 = meta["rows"]
    a = np.asarray(img, np.float64).reshape(height, width, 3)[r0:r1]
    return {"rmse": _rmse(a, ref), "oracle_image": name, "oracle_spp": meta["spp"],
            "oracle_noise_rmse": meta["noise_rmse"], "rows": [r0, r1],
            "mean_rel_error": float(a.mean() / ref.mean() - 1.0)}


def _time_at(curve, target):
    """First time (log-log interpolation between points) at which the curve's RMSE reaches target.
    Curve points are (seconds, rmse, samples)."""
    for (t0, e0, *_), (t1, e1, *_) in zip(curve, curve[1:]):
        if e1 <= target < e0 or (e0 <= target and t0 == curve[0][0]):
            if e0 <= target:
                return t0
            f = (math.log(e0) - math.log(target)) / (math.log(e0) - math.log(e1))
            return math.exp(math.log(t0) + f * (math.log(t1) - math.log(t0)))
    return None


def _cache_curve(r, acc, ref, chunks, limit_s=None):
    curve, n = [], 0
    for k in chunks:
        r.accumulate(acc, k)
        n += k
        curve.append((acc.gpu_seconds(), _rmse(acc.mean(), ref), n))
        if limit_s is not None and acc.gpu_seconds() > limit_s:
            break
    return curve, n


def _speedup(plains, curve, target):
    """Each plain curve's time to `target` RMSE, the cache curve's, and the speed-up against the
    fastest plain integrator."""
    t_plain = {name: _time_at(c, target) or c[-1][0] for name, c in plains.items()}
    best = min(t_plain, key=t_plain.get)
    t_cache = _time_at(curve, target)
    return {"target_rmse": target, "time_to_target_s": {**{"plain_" + k: v for k, v in t_plain.items()},
                                                         "cache": t_cache},
            "speedup": (t_plain[best] / t_cache) if t_cache else None, "speedup_against": "plain " + best,
            "reached": t_cache is not None}


def _cache_vs_plain(plains, curve, target_at):
    """_speedup at the RMSE the first plain curve has at its point `target_at`."""
    first = next(iter(plains.values()))
    return _speedup(plains, curve, first[target_at][1])


def _fit_noise(curve, points=3):
    """Least-squares fit of rmse^2 = B + S / N to a curve's last `points` points (N = samples): an
    unbiased estimate's squared error falls as S / N, so B is the floor (bias energy and the
    reference's own noise) and S the per-sample variance."""
    pts = curve[-points:]
    A = np.array([[1.0, 1.0 / n] for _, _, n in pts])
    y = np.array([e * e for _, e, _ in pts])
    (B, S), *_ = np.linalg.lstsq(A, y, rcond=None)
    return float(B), float(S)


def _at_spp_by_fit(plains, curve, spp, ref_spp):
    """Time to reach the RMSE plain path tracing has at `spp` samples, from the curves' noise fits:
    plain is unbiased, so against a reference of ref_spp independent plain samples its measured
    error is rmse^2 = S_p (1 / N + 1 / ref_spp) (S_p fitted to the fastest plain curve's last
    points), and at `spp` samples it is S_p (1 / spp + 1 / ref_spp); plain takes spp times its time
    per sample. The cache's fit rmse^2 = B + S / N gives the samples it needs, N = S / (target^2 - B),
    or none when its floor B is at or above the target (bias the network does not lose)."""
    best = min(plains, key=lambda k: plains[k][-1][0] / plains[k][-1][2])
    pc = plains[best]
    pts = pc[-3:]
    S_p = float(np.mean([e * e / (1.0 / n + 1.0 / ref_spp) for _, e, n in pts]))
    target2 = S_p * (1.0 / spp + 1.0 / ref_spp)
    t_plain = spp * pc[-1][0] / pc[-1][2]
    B, S = _fit_noise(curve)
    t_per = curve[-1][0] / curve[-1][2]
    n_cache = S / (target2 - B) if target2 > B and S > 0 else None
    t_cache = n_cache * t_per if n_cache else None
    return {"target_rmse": math.sqrt(target2), "plain_spp": spp, "method": "fit (see bench.py _at_spp_by_fit)",
            "time_to_target_s": {"plain_" + best: t_plain, "cache": t_cache},
            "cache_fit": {"floor_rmse": math.sqrt(max(B, 0.0)), "per_sample_sigma": math.sqrt(max(S, 0.0)),
                          "reference_noise_rmse": math.sqrt(S_p / ref_spp)},
            "cache_spp_needed": n_cache, "speedup": (t_plain / t_cache) if t_cache else None,
            "speedup_against": "plain " + best, "reached": t_cache is not None}


def mlp_kernel_seconds(ctx, nrec, reps):
    """Device seconds per launch of the cache's kernels (vg_cache_time: one untimed round, then
    `reps` launches of each) on nrec synthetic records: positions uniform in a unit box, unit
    directions, material features and targets uniform."""
    from verion_gb300.backend import Cache

    rng = np.random.default_rng(5)
    lo, hi = ((-1.0,) * 3, (1.0,) * 3)
    rec = np.zeros((nrec, 20), np.float32)
    rec[:, 0:3] = rng.uniform(lo, hi, (nrec, 3))
    for o in (3, 6):
        d = rng.normal(size=(nrec, 3))
        rec[:, o:o + 3] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rec[:, 9:15] = rng.uniform(0, 1, (nrec, 6))
    rec[:, 16:19] = rng.uniform(0, 2, (nrec, 3))
    return Cache(ctx, bounds=(lo, hi)).time_kernels(rec, reps=reps)


def cache_report(ctx, packed_c2, peak_tflops, peak_kind):
    """Radiance cache (cache query paths on the streaming wavefront) against plain path tracing:
    time to reach a plain image's RMSE (against a long plain reference, GPU time), the speed-up
    taken against the fastest plain integrator. C4: Cornell box 512 x 512, depth 8. C2: the
    1M-triangle workload at 1920 x 1080, depth 16, against plain wavefront with and without
    adaptive sampling. Then the MLP kernels' device time on 2^20 synthetic records against the
    tensor roofline."""
    from verion_gb300 import pack, scenes
    from verion_gb300.backend import Cache, Integrator, Renderer
    from verion_gb300.readback import Adaptive

    out = {}
    # C4: the Cornell box with the stated cache (2^19 entries, 2^16 training records per frame).
    p = pack.pack(scenes.cornell())
    ref_r = Renderer(ctx, p)
    ref_r.set_integrator(Integrator.WAVEFRONT)
    acc = ref_r.new_accumulation(CACHE_W, CACHE_H)
    acc.set_first_sample(REF_FIRST_SAMPLE)
    for _ in range(CACHE_REF_SPP // 512):
        ref_r.accumulate(acc, 512)
    ref = acc.mean()
    del acc, ref_r
    plains, plain_ms, plain_fp64 = {}, {}, {}
    for name, integ, chunks in (("megakernel", Integrator.MEGAKERNEL, (32, 32, 64, 128, 256, 512)),
                                ("wavefront", Integrator.WAVEFRONT, (32, 32, 64, 128, 256, 512, 1024, 2048))):
        plain_r = Renderer(ctx, p)
        plain_r.set_integrator(integ)
        acc = plain_r.new_accumulation(CACHE_W, CACHE_H)
        plains[name], n = _cache_curve(plain_r, acc, ref, chunks)
        plain_ms[name] = 1e3 * acc.gpu_seconds() / n
        plain_fp64[name] = rmse_vs_fp64(acc.mean(), CACHE_W, CACHE_H, "cornell_512_d8")
        del acc, plain_r
    r = Renderer(ctx, p)
    r.set_integrator(Integrator.WAVEFRONT)
    r.set_cache_frame(8)
    cache = Cache(ctx, bounds=r.bounds())
    r.set_cache(cache, spread=0.01, train_paths=8192, train_steps=2, train_batch=32768)
    r.set_stage_timing(True)
    acc = r.new_accumulation(CACHE_W, CACHE_H)
    curve, n = _cache_curve(r, acc, ref, (32, 32, 64, 128, 256, 512, 1024, 2048))
    st = acc.cache_stats()
    c4 = {"config": "Cornell box 512x512, depth 8; cache 16 levels x 2^19 entries x 2 fp16, MLP 64 x 4 hidden bf16; "
                    "frames of 8 samples, ~8192 training pixels, 2 Adam steps of 32768 records (2^16 per frame); "
                    f"reference {CACHE_REF_SPP} spp plain from sample index 2^24 (no sample shared with the curves); "
                    "targets: plain megakernel RMSE at 1024 spp, plain wavefront RMSE at 4096 spp (measured)",
          "plain_ms_per_spp": plain_ms, "cache_ms_per_spp": 1e3 * acc.gpu_seconds() / n,
          "cache_split_seconds": {"paths": st.path_seconds, "encode_and_infer": st.infer_seconds,
                                  "train": st.train_seconds},
          "bias_rel_mean": float((acc.mean().mean() - ref.mean()) / ref.mean()),
          "cache_curve": curve, "plain_curves": plains}
    c4.update(_cache_vs_plain({"megakernel": plains["megakernel"], "wavefront": plains["wavefront"]}, curve, -1))
    c4["at_4096spp"] = _speedup({"wavefront": plains["wavefront"]}, curve, plains["wavefront"][-1][1])
    c4["rmse_vs_fp64_oracle"] = {"cache": rmse_vs_fp64(acc.mean(), CACHE_W, CACHE_H, "cornell_512_d8"),
                                 **{"plain_" + k: v for k, v in plain_fp64.items()}}
    out["cornell_512"] = c4
    del acc, r
    # C2.
    def c2_renderer(adaptive=False):
        rr = Renderer(ctx, packed_c2)
        rr.set_integrator(Integrator.WAVEFRONT)
        rr.set_max_depth(DEPTH)
        if adaptive:
            rr.set_adaptive(Adaptive(*ADAPTIVE))
        return rr

    ref_r = c2_renderer()
    acc = ref_r.new_accumulation(WIDTH, HEIGHT)
    acc.set_first_sample(REF_FIRST_SAMPLE)
    for _ in range(C2_REF_SPP // 128):
        ref_r.accumulate(acc, 128)
    ref = acc.mean()
    del acc, ref_r
    plains, plain_fp64 = {}, {}
    for name, adaptive in (("wavefront", False), ("wavefront_adaptive", True)):
        rr = c2_renderer(adaptive)
        acc = rr.new_accumulation(WIDTH, HEIGHT)
        plains[name], _ = _cache_curve(rr, acc, ref, (8, 8, 16, 32, 64, 128))
        plain_fp64[name] = rmse_vs_fp64(acc.mean(), WIDTH, HEIGHT, C2_ORACLE)
        del acc, rr
    r = c2_renderer()
    cache = Cache(ctx, bounds=r.bounds())
    # Spread threshold 0.002 (the best of 0.001-0.1 on this scene; 0.01, the default, reaches the
    # 64-spp target 2.5x sooner instead of 3.7x); ~16384 training pixels, 4 Adam steps of 16384.
    r.set_cache(cache, spread=0.002)
    r.set_stage_timing(True)
    acc = r.new_accumulation(WIDTH, HEIGHT)
    curve, n = _cache_curve(r, acc, ref, (8, 8, 16, 32, 64, 128, 256))
    st = acc.cache_stats()
    c2 = {"config": "1M-triangle workload 1920x1080, depth 16; cache 16 levels x 2^19 entries, spread threshold "
                    "0.002, frames of 4 samples, ~16384 training pixels, 4 Adam steps of 16384 records per frame; "
                    f"reference {C2_REF_SPP} spp plain from sample index 2^24; the 4096-spp target is fitted "
                    "(plain: error^2 = S (1/N + 1/reference spp); cache: error^2 = B + S/N over its last points)",
          "cache_ms_per_spp": 1e3 * acc.gpu_seconds() / n,
          "cache_split_seconds": {"paths": st.path_seconds, "encode_and_infer": st.infer_seconds,
                                  "train": st.train_seconds},
          "bias_rel_mean": float((acc.mean().mean() - ref.mean()) / ref.mean()),
          "cache_curve": curve, "plain_curves": plains}
    for label, at in (("at_64spp", 3), ("at_256spp", 5)):
        c2[label] = _cache_vs_plain(plains, curve, at)
    c2["at_4096spp"] = _at_spp_by_fit(plains, curve, 4096, C2_REF_SPP)
    c2["rmse_vs_fp64_oracle"] = {"cache": rmse_vs_fp64(acc.mean(), WIDTH, HEIGHT, C2_ORACLE),
                                 **{"plain_" + k: v for k, v in plain_fp64.items()}}
    out["many_spheres_1080p"] = c2
    del acc, r
    # MLP kernels on synthetic records.
    nrec = 1 << 20
    kt = mlp_kernel_seconds(ctx, nrec, reps=10)
    infer_tf = CACHE_MLP_FLOP * nrec / kt["infer"] / 1e12
    train_tf = 3 * CACHE_MLP_FLOP * nrec / kt["train"] / 1e12
    out["mlp_kernels"] = {"records": nrec, "seconds_per_launch": kt,
                          "infer_tflops": infer_tf, "train_tflops": train_tf,
                          "peak_tflops": peak_tflops, "peak_kind": peak_kind,
                          "infer_frac": infer_tf / peak_tflops, "train_frac": train_tf / peak_tflops,
                          "flop_per_record": {"infer": CACHE_MLP_FLOP, "train": 3 * CACHE_MLP_FLOP}}
    return out


BATCH_SCENES = [(4, 15, 48), (16, 21, 160), (48, 31, 400), (128, 31, 724)]  # spheres, sphere resolution, grid


def _pct(v, q):
    v = sorted(v)
    return v[min(len(v) - 1, max(0, int(math.ceil(q * len(v))) - 1))]


def batch_report(ctx, spp_scale, side_range=(256, 2048), spp_range=(16, 256)):
    """Batched serving (64 requests): resolution log-uniform 256^2-2048^2 (square), scenes of ~10k-2M
    triangles generated like the 1M-triangle workload, spp log-uniform 16-256 (times spp_scale),
    depth 16, every second request with a radiance cache. One batch (vg_batch_render: the tile
    launch below the tuned size threshold, the batch wavefront from it up, each a replayed CUDA
    graph) against the same requests rendered one at a time with accumulate (each on the faster of
    the wavefront and the megakernel), shortest first; latency = device time from the start until
    the request's last tile or pixel. The batch is first autotuned (vg_batch_tune: threshold,
    order, tile CTAs per SM, wavefront slots) at a quarter of the sample counts."""
    from verion_gb300 import pack, scenes
    from verion_gb300.backend import BatchRequest, Cache, Integrator, Renderer

    rng = np.random.default_rng(0x5EED5EED)
    plain_r, cached_r, tris = [], [], []
    for sph, n, grid in BATCH_SCENES:
        p = pack.pack(scenes.many_spheres(spheres=sph, sphere_n=n, grid=grid))
        r = Renderer(ctx, p)
        r.set_max_depth(DEPTH)
        r.set_accum_precision(32)
        rc = Renderer(ctx, p)
        rc.set_max_depth(DEPTH)
        rc.set_accum_precision(32)
        cache = Cache(ctx, bounds=rc.bounds())
        rc.set_cache(cache, spread=0.01, train_paths=16384, train_steps=4, train_batch=16384)
        rc._batch_cache = cache
        plain_r.append(r)
        cached_r.append(rc)
        tris.append(r.bvh_info().triangles)
    spec = []
    for i in range(64):
        side = int(round(math.exp(rng.uniform(math.log(side_range[0]), math.log(side_range[1])))))
        spp = max(1, int(round(math.exp(rng.uniform(math.log(spp_range[0]), math.log(spp_range[1]))) * spp_scale)))
        spec.append((side, spp, int(rng.integers(len(BATCH_SCENES))), i % 2 == 1))

    def requests():
        out = []
        for side, spp, si, cached in spec:
            r = cached_r[si] if cached else plain_r[si]
            out.append(BatchRequest(r, r.new_accumulation(side, side), spp, r._batch_cache if cached else None))
        return out

    paths = float(sum(side * side * spp for side, spp, _, _ in spec))
    reqs = requests()
    tune_reqs = [BatchRequest(q.renderer, q.accum, max(1, q.samples // 4), q.cache) for q in reqs]
    tuned = ctx.batch_tune(tune_reqs)
    ctx.batch_render(reqs)  # captures the graph
    out = ctx.batch_render(reqs)  # replays it
    # One at a time, shortest first, through accumulate, each request on the faster of the two
    # integrators: both are timed on requests below 512 x 512 pixels; from there up the streaming
    # wavefront is the faster on these scenes (the megakernel traces the same paths at about a
    # quarter of its rate), so only it is timed.
    order = sorted(range(64), key=lambda i: spec[i][0] ** 2 * spec[i][1])
    seq_t, now, lat = [], 0.0, [0.0] * 64
    for i in order:
        side, spp, si, cached = spec[i]
        r = cached_r[si] if cached else plain_r[si]
        best = None
        for integ in ((Integrator.WAVEFRONT, Integrator.MEGAKERNEL) if side * side < 512 * 512
                      else (Integrator.WAVEFRONT,)):
            r.set_integrator(integ)
            acc = r.new_accumulation(side, side)
            r.accumulate(acc, spp)
            best = acc.gpu_seconds() if best is None else min(best, acc.gpu_seconds())
            del acc
        now += best
        lat[i] = now
    for r in plain_r + cached_r:
        r.set_integrator(Integrator.MEGAKERNEL)
    big = tuned["wavefront_pixels"]
    launches = {"tile_launch": sum(1 for s in spec if s[0] * s[0] < big),
                "batch_wavefront": sum(1 for s in spec if s[0] * s[0] >= big and not (s[3] and s[0] * s[0] > 1 << 22)),
                "one_at_a_time": sum(1 for s in spec if s[0] * s[0] >= big and s[3] and s[0] * s[0] > 1 << 22)}
    return {
        "config": f"64 requests, square {min(s[0] for s in spec)}-{max(s[0] for s in spec)} px, "
                  f"spp {min(s[1] for s in spec)}-{max(s[1] for s in spec)} ({spp_range[0]}-{spp_range[1]} x {spp_scale}), "
                  f"depth {DEPTH}, "
                  f"scenes of {min(tris)}-{max(tris)} triangles, 32 requests with a radiance cache",
        "paths": paths,
        "batch": {"p50_s": _pct(out.seconds, 0.5), "p99_s": _pct(out.seconds, 0.99), "total_s": out.total_seconds,
                  "mpaths_s": paths / out.total_seconds / 1e6, "graph_replayed": out.graph_replayed,
                  "requests_by_launch": launches, "tuned": tuned},
        "one_at_a_time": {"p50_s": _pct(lat, 0.5), "p99_s": _pct(lat, 0.99), "total_s": now,
                          "mpaths_s": paths / now / 1e6},
    }


def restir_report(ctx):
    """ReSTIR DI on the many-light scene (~205k triangles, 4096 emissive triangles of radiance
    log-uniform in [0.1, 100]): 1920 x 1080, 1 spp per frame, 32 RIS candidates, temporal and spatial
    reuse, over an 8-frame camera pan; device time per frame with and without ReSTIR for both
    integrators. Quality: a static camera at 480 x 270, RMSE after 8 frames (8 spp) with and
    without ReSTIR against a 1024-spp plain image, for full paths (depth 8) and for direct light
    alone (depth 1), over all pixels and over the pixels that do not see an emitter ("lit")."""
    from verion_gb300 import pack, scenes
    from verion_gb300.backend import Integrator, Renderer
    from verion_gb300.readback import Restir

    s = scenes.many_lights()
    p = pack.pack(s)
    rs = Restir(di=True, gi=False, candidates=32, history=20)
    out = {"config": "many_lights: 205,248 triangles, 4096 emitters; 1920x1080, 1 spp/frame, 32 candidates, "
                     "temporal + spatial reuse, 8-frame pan (camera orbits 0.5 degrees per frame)"}
    for integ, name in ((Integrator.MEGAKERNEL, "megakernel"), (Integrator.WAVEFRONT, "wavefront")):
        for on in (False, True):
            r = Renderer(ctx, p)
            r.set_integrator(integ)
            r.set_accum_precision(32)
            r.set_restir(rs if on else None)
            acc = r.new_accumulation(WIDTH, HEIGHT)
            r.accumulate(acc, 1)
            g0 = acc.gpu_seconds()
            for f in range(8):
                a = math.radians(0.5 * (f + 1))
                r.set_camera(scenes.look_at((14.0 * math.sin(a), 6.0, 14.0 * math.cos(a)), (0.0, 0.5, 0.0), fov=0.9))
                r.accumulate(acc, 1)
            out[f"{name}_{'restir' if on else 'plain'}_ms_per_frame"] = 1e3 * (acc.gpu_seconds() - g0) / 8
    w, h = 480, 270
    # Full paths (depth 8), and direct light only (depth 1), where ReSTIR DI does all the work.
    for depth, tag in ((8, ""), (1, "_direct")):
        ref_r = Renderer(ctx, p)
        ref_r.set_max_depth(depth)
        ref = ref_r.render(w, h, 1024)
        for on in (False, True):
            r = Renderer(ctx, p)
            r.set_max_depth(depth)
            r.set_restir(rs if on else None)
            acc = r.new_accumulation(w, h)
            for _ in range(8):
                r.accumulate(acc, 1)
            img = acc.mean()
            out[f"rmse_8_frames{tag}_{'restir' if on else 'plain'}"] = _rmse(img, ref)
            out[f"rmse_vs_fp64_oracle_8_frames{tag}_{'restir' if on else 'plain'}"] = rmse_vs_fp64(
                img, w, h, f"many_lights_480x270_d{depth}")
            # Without the pixels that see an emitter (reference luminance above its 95th percentile):
            # their error is edge aliasing of the bright triangles, which no light sampling changes.
            lum = ref @ np.array([0.2126, 0.7152, 0.0722])
            keep = lum <= np.percentile(lum, 95)
            out[f"rmse_8_frames{tag}_lit_{'restir' if on else 'plain'}"] = _rmse(img[keep], ref[keep])
        for k in ("", "_lit"):
            out[f"rmse_ratio{tag}{k}_plain_over_restir"] = (out[f"rmse_8_frames{tag}{k}_plain"] /
                                                           out[f"rmse_8_frames{tag}{k}_restir"])
    return out


def run_cuda(args):
    rank, world, device, ctx = open_device(args)
    import torch

    from verion_gb300.backend import Integrator, Renderer
    from verion_gb300.readback import Adaptive

    _, packed = workload()
    r = Renderer(ctx, packed)
    r.set_integrator(Integrator.WAVEFRONT if args.integrator == "wavefront" else Integrator.MEGAKERNEL)
    r.set_max_depth(DEPTH)
    r.set_adaptive(Adaptive(*ADAPTIVE))
    r.set_accum_precision(64)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    total = args.warmup + args.steps

    if args.profile_batch or args.profile_batch_wave:
        from verion_gb300 import pack, scenes
        from verion_gb300.backend import BATCH_SHORTEST_FIRST, BatchRequest, Cache

        if args.profile_batch_wave:
            # The host-driven loop: a profiler cannot look into a graph with a conditional node.
            ctx.set_batch_options(0, BATCH_SHORTEST_FIRST, 0)
            ctx.set_batch_device_loop(False)
        else:
            ctx.set_batch_options(0, BATCH_SHORTEST_FIRST, (1 << 64) - 1)  # the tile launch

        pb = pack.pack(scenes.many_spheres(spheres=16, sphere_n=21, grid=160))
        rb, rcb = Renderer(ctx, pb), Renderer(ctx, pb)
        for x in (rb, rcb):
            x.set_max_depth(DEPTH)
            x.set_accum_precision(32)
        cb = Cache(ctx, bounds=rcb.bounds(), log2_entries=17)
        rcb.set_cache(cb, spread=0.01)
        rng = np.random.default_rng(7)
        for _ in range(2):
            reqs = []
            for i in range(16):
                side, spp = int(rng.integers(128, 257)), int(rng.integers(4, 17))
                rr = rcb if i % 2 else rb
                reqs.append(BatchRequest(rr, rr.new_accumulation(side, side), spp, cb if i % 2 else None))
            out = ctx.batch_render(reqs)
        print(json.dumps({"batch_total_s": out.total_seconds}), flush=True)
        return

    if args.profile_per_sample:
        from verion_gb300.backend import WavefrontMode

        rp = Renderer(ctx, packed)
        rp.set_integrator(Integrator.WAVEFRONT)
        rp.set_wavefront_mode(WavefrontMode.PER_SAMPLE)
        rp.set_max_depth(DEPTH)
        rp.set_adaptive(Adaptive(*ADAPTIVE))
        rp.set_accum_precision(64)
        acc_p = rp.new_accumulation(WIDTH, HEIGHT)
        rp.accumulate(acc_p, 20)
        print(json.dumps({"per_sample_ms": 1e3 * acc_p.gpu_seconds()}), flush=True)
        return

    if args.profile_restir:
        from verion_gb300 import pack, scenes
        from verion_gb300.readback import Restir

        pr = pack.pack(scenes.many_lights())
        rr = Renderer(ctx, pr)
        rr.set_integrator(Integrator.WAVEFRONT)
        rr.set_accum_precision(32)
        rr.set_restir(Restir(di=True, gi=False, candidates=32, history=20))
        acc_r = rr.new_accumulation(WIDTH, HEIGHT)
        for _ in range(4):
            rr.accumulate(acc_r, 1)
        print(json.dumps({"restir_ms_per_frame": 1e3 * acc_r.gpu_seconds() / 4}), flush=True)
        return

    if args.profile_mlp:
        print(json.dumps(mlp_kernel_seconds(ctx, 1 << 20, reps=1)), flush=True)
        return

    if args.profile_cache:
        from verion_gb300.backend import Cache

        rc = Renderer(ctx, packed)
        rc.set_integrator(Integrator.WAVEFRONT)
        rc.set_max_depth(DEPTH)
        cache = Cache(ctx, bounds=rc.bounds())
        rc.set_cache(cache, spread=0.002)
        rc.set_stage_timing(True)
        acc_c = rc.new_accumulation(WIDTH, HEIGHT)
        for _ in range(args.warmup):
            rc.accumulate(acc_c, 4)
        g0, st0 = acc_c.gpu_seconds(), acc_c.cache_stats()
        rc.accumulate(acc_c, 4)
        st1 = acc_c.cache_stats()
        print(json.dumps({"frame_ms": 1e3 * (acc_c.gpu_seconds() - g0),
                          "paths_ms": 1e3 * (st1.path_seconds - st0.path_seconds),
                          "encode_and_infer_ms": 1e3 * (st1.infer_seconds - st0.infer_seconds),
                          "train_ms": 1e3 * (st1.train_seconds - st0.train_seconds),
                          "queries": st1.queries, "train_records": st1.train_records}), flush=True)
        return

    if args.profile_extend:
        acc_p = r.new_accumulation(WIDTH, HEIGHT)
        for _ in range(args.warmup):
            r.accumulate(acc_p, SPP_STEP)
        r.set_traversal_stats(True)
        s0 = acc_p.traversal_stats()
        flush.zero_()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("traffic")
        r.accumulate(acc_p, SPP_STEP)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        s1 = acc_p.traversal_stats()
        print(json.dumps({k: s1[k] - s0[k] for k in s1}), flush=True)
        return

    def paths_of(acc):
        st = acc.raw_stats()
        return float(st.reshape(-1, 3)[:, 0].astype(np.float64).sum())

    # Device-timed run.
    r.set_stage_timing(False)
    acc = r.new_accumulation(WIDTH, HEIGHT)
    for _ in range(args.warmup):
        flush.zero_()
        torch.cuda.synchronize()
        r.accumulate(acc, SPP_STEP)
    p0 = paths_of(acc)
    launches0 = acc.launches()
    r.set_stage_timing(True)
    step_times = []
    with Clocks(device) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            barrier(world)
            g0 = acc.gpu_seconds()
            r.accumulate(acc, SPP_STEP)
            torch.cuda.synchronize()
            step_times.append(acc.gpu_seconds() - g0)
        barrier(world)
    paths = paths_of(acc) - p0
    gpu_launches = acc.launches() - launches0
    fp64 = rmse_vs_fp64(acc.mean(), WIDTH, HEIGHT, C2_ORACLE)
    if fp64 is not None:
        fp64["mean_spp"] = paths_of(acc) / (WIDTH * HEIGHT)
    stage = acc.stage_seconds() or (0.0, 0.0)
    extend_launch_s = acc.extend_launch_seconds()
    t_local = sum(step_times)
    t = allmax(world, t_local)
    paths_all = allsum(world, paths)
    value = paths_all / t / 1e6

    # Traversal counters for the same steps (deterministic replay with counting on, untimed).
    r.set_stage_timing(False)
    r.set_traversal_stats(True)
    acc_s = r.new_accumulation(WIDTH, HEIGHT)
    for _ in range(args.warmup):
        r.accumulate(acc_s, SPP_STEP)
    s0 = acc_s.traversal_stats() if args.integrator == "wavefront" else None
    sh0 = acc_s.shadow_rays() if args.integrator == "wavefront" else 0
    for _ in range(args.steps):
        r.accumulate(acc_s, SPP_STEP)
    s1 = acc_s.traversal_stats() if args.integrator == "wavefront" else None
    sh1 = acc_s.shadow_rays() if args.integrator == "wavefront" else 0
    # Rays (closest-hit + shadow) per camera path: the replay traces the timed steps' paths.
    rays_per_path = ((s1["rays"] - s0["rays"] + sh1 - sh0) / max(paths, 1.0)) if s0 is not None else None
    r.set_traversal_stats(False)
    del acc_s

    # End to end through the C ABI with host buffers.
    pinned = torch.empty(3 * WIDTH * HEIGHT, dtype=torch.float32, pin_memory=True)
    host_sums = pinned.numpy()
    view = packed.view
    acc_e = r.new_accumulation(WIDTH, HEIGHT)
    for _ in range(args.warmup):
        r.accumulate(acc_e, SPP_STEP)
    pe0 = paths_of(acc_e)
    wall = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r.set_camera(view)
        r.accumulate(acc_e, SPP_STEP)
        acc_e.sums(into=host_sums)
        wall.append(time.perf_counter() - t0)
    pe = paths_of(acc_e) - pe0
    e2e_t = allmax(world, sum(wall))
    e2e_value = allsum(world, pe) / e2e_t / 1e6
    del acc_e

    # Megakernel on the same steps, for comparison (device time).
    mega = None
    if args.integrator == "wavefront":
        r.set_integrator(Integrator.MEGAKERNEL)
        acc_m = r.new_accumulation(WIDTH, HEIGHT)
        for _ in range(args.warmup):
            r.accumulate(acc_m, SPP_STEP)
        pm0 = paths_of(acc_m)
        g0 = acc_m.gpu_seconds()
        for _ in range(min(args.steps, 4)):
            flush.zero_()
            torch.cuda.synchronize()
            r.accumulate(acc_m, SPP_STEP)
        mega = (paths_of(acc_m) - pm0) / (acc_m.gpu_seconds() - g0) / 1e6
        r.set_integrator(Integrator.WAVEFRONT)
        del acc_m

    roofline = None
    peak, peak_kind = peaks()
    if s0 is not None and extend_launch_s > 0:
        rays = s1["rays"] - s0["rays"]
        nodes = s1["nodes"] - s0["nodes"]
        tests = s1["tests"] - s0["tests"]
        rays1 = s1["rays_after_depth0"] - s0["rays_after_depth0"]
        node_b, tri_b = 80, 48
        alg_bytes = 20 * rays + 24 * rays1 + node_b * nodes + tri_b * tests
        extend_launches = max(1, int(round(stage[0] / extend_launch_s)))  # launches in the timed steps
        per_launch_bytes = alg_bytes / extend_launches
        achieved = per_launch_bytes / extend_launch_s / 1e9
        tpr, tsrc = traffic_per_ray()
        roofline = {"kernel": "wf_extend", "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "peak_kind": f"{peak_kind} (hbm_gbs)",
                    "traffic": (tpr * rays / extend_launches) if tpr else None,
                    "traffic_source": tsrc,
                    "algorithmic_bytes_per_launch": per_launch_bytes,
                    "avg_launch_ms": extend_launch_s * 1e3,
                    "per_ray": {"nodes": nodes / max(rays, 1), "triangle_tests": tests / max(rays, 1),
                                "bytes": alg_bytes / max(rays, 1)},
                    "formula": "20 B/ray (queue id + hit record) + 24 B/ray past depth 0 (origin, direction) "
                               "+ 80 B/node visited + 48 B/triangle tested"}

    cache = None
    if rank == 0 and not args.no_cache:
        bf = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("bf16_tflops") \
            if (ROOT / "MEASURED_PEAKS.json").exists() else None
        cache = cache_report(ctx, packed, bf or 1900.0, "measured (bf16_tflops, burst)" if bf else "fallback")

    restir = None
    if rank == 0 and not args.no_restir:
        restir = restir_report(ctx)

    batch = None
    if rank == 0 and not args.no_batch:
        batch = batch_report(ctx, args.batch_spp_scale)
        # Small requests (128-512 px square, 4-32 spp): the shared persistent launch's case.
        batch["small_requests"] = batch_report(ctx, 1.0, side_range=(128, 512), spp_range=(4, 32))

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu, _ = cpu_baseline(packed, args.cpu_seconds, args.warmup)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": config(args), "impl": "cuda",
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 80,
                        "d2h_bytes_per_step": 3 * 4 * WIDTH * HEIGHT},
                "roofline": roofline, "cpu_baseline": cpu, "gpu_launches": gpu_launches,
                "clocks": clk.summary(),
                "stage_seconds": {"extend": stage[0], "shade": stage[1]},
                "paths_per_step": paths_all / args.steps,
                "mrays_per_s": value * rays_per_path if rays_per_path else None,
                "rays_per_path": rays_per_path,
                "rmse_vs_fp64_oracle": fp64,
                "megakernel_value": mega, "radiance_cache": cache, "batched_serving": batch,
                "restir_many_lights": restir}
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_cuda(args)


if __name__ == "__main__":
    sys.exit(main())
