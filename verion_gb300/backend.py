"""Python face of the CUDA backend: `Renderer` and `Accumulation` with the methods of Verion's
`RayTracingBackend` and `Accumulation` traits (crates/verion-gpu/src/lib.rs:12-93), over the C ABI
of include/vgcuda.h (libvgcuda.so, built in-tree by verion_gb300.build).

There is no CPU fallback: without the library or a GB300 every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from enum import IntEnum
from pathlib import Path
from typing import Optional

import numpy as np

from . import readback as rb
from .pack import Packed, View, pack
from .readback import Adaptive, Restir

LIB_PATH = Path(os.environ.get("VGCUDA_LIB", Path(__file__).resolve().parent / "_build" / "libvgcuda.so"))

VG_OK, VG_ERR_NO_DEVICE, VG_ERR_UNSUPPORTED, VG_ERR_OOM, VG_ERR_RESOURCE, VG_ERR_KERNEL, VG_ERR_SCENE, \
    VG_ERR_TIMEOUT, VG_ERR_INVALID = range(9)
VG_TRACE_NOALLOC_MAX_RAYS = 65536  # include/vgcuda.h
_KIND = {VG_ERR_NO_DEVICE: "NoDevice", VG_ERR_UNSUPPORTED: "Unsupported", VG_ERR_OOM: "OutOfMemory",
         VG_ERR_RESOURCE: "Resource", VG_ERR_KERNEL: "Kernel", VG_ERR_SCENE: "Scene", VG_ERR_TIMEOUT: "Timeout",
         VG_ERR_INVALID: "Invalid"}


class Error(RuntimeError):
    """A backend error: `kind` is the reference's error variant (crates/verion-gpu-metal/src/lib.rs:25-41)."""

    def __init__(self, status: int, message: str, needed: int = 0, available: int = 0):
        super().__init__(f"{_KIND.get(status, status)}: {message}")
        self.status = status
        self.kind = _KIND.get(status, str(status))
        self.needed = needed
        self.available = available


class Integrator(IntEnum):
    MEGAKERNEL = 0
    WAVEFRONT = 1


class WavefrontMode(IntEnum):
    """PER_SAMPLE: the reference's depth-by-depth order (per-depth queue counts readable).
    STREAMING: path regeneration, the same sums with far fewer, fuller launches."""
    PER_SAMPLE = 0
    STREAMING = 1


class MemoryUsage(C.Structure):
    _fields_ = [("budget", C.c_uint64), ("allocated", C.c_uint64), ("uploaded", C.c_uint64)]


class _MeshRange(C.Structure):
    _fields_ = [("vertex_offset", C.c_uint32), ("vertex_count", C.c_uint32), ("index_offset", C.c_uint32),
                ("index_count", C.c_uint32)]


class _SceneInfo(C.Structure):
    _fields_ = [("light_count", C.c_uint32), ("emitter_count", C.c_uint32), ("env_width", C.c_uint32),
                ("env_height", C.c_uint32), ("env_pdf_scale", C.c_float), ("sky", C.c_float * 3),
                ("virtual_light", C.c_uint32), ("transparent_background", C.c_uint32)]


class _View(C.Structure):
    _fields_ = [("camera", C.c_float * 16), ("aperture", C.c_float), ("focus", C.c_float), ("shift", C.c_float * 2)]


_P = C.c_void_p
_S = C.c_size_t


class _Packed(C.Structure):
    _fields_ = [(n, t) for pair in [
        (("positions", _P), ("positions_len", _S)), (("indices", _P), ("indices_len", _S)),
        (("uvs", _P), ("uvs_len", _S)), (("vnormals", _P), ("vnormals_len", _S)),
        (("instances", _P), ("instances_len", _S)), (("materials", _P), ("materials_len", _S)),
        (("lights", _P), ("lights_len", _S)), (("emitters", _P), ("emitters_len", _S)),
        (("emit_cdf", _P), ("emit_cdf_len", _S)), (("env_pixels", _P), ("env_pixels_len", _S)),
        (("env_marginal", _P), ("env_marginal_len", _S)), (("env_conditional", _P), ("env_conditional_len", _S)),
        (("texels", _P), ("texels_len", _S)), (("tex_info", _P), ("tex_info_len", _S)),
        (("meshes", _P), ("mesh_count", _S)), (("tlas_mesh", _P),),
        (("tlas_transform", _P), ("instance_count", _S)),
        (("info", _SceneInfo), ("view", _View))] for n, t in pair]


class BvhInfo(C.Structure):
    _fields_ = [("triangles", C.c_uint32), ("wide_nodes", C.c_uint32), ("wide_depth", C.c_uint32),
                ("binary_nodes", C.c_uint32), ("binary_depth", C.c_uint32), ("node_bytes", C.c_uint64),
                ("triangle_bytes", C.c_uint64), ("build_seconds", C.c_double)]


class CacheConfig(C.Structure):
    """Radiance-cache configuration (include/vgcuda.h VgCacheConfig)."""
    _fields_ = [("levels", C.c_uint32), ("log2_entries", C.c_uint32), ("base_resolution", C.c_uint32),
                ("max_resolution", C.c_uint32), ("learning_rate", C.c_float), ("beta1", C.c_float),
                ("beta2", C.c_float), ("epsilon", C.c_float), ("seed", C.c_uint32),
                ("bounds_lo", C.c_float * 3), ("bounds_hi", C.c_float * 3)]


class CacheStats(C.Structure):
    _fields_ = [("queries", C.c_uint32), ("train_records", C.c_uint32), ("loss", C.c_double),
                ("path_seconds", C.c_double), ("infer_seconds", C.c_double), ("train_seconds", C.c_double)]


class _TuneResult(C.Structure):
    _fields_ = [("dynamic_fetch", C.c_int), ("deferred_shadows", C.c_int), ("stream_tail", C.c_uint32),
                ("graph_waves", C.c_uint32), ("bvh_traversal_cost", C.c_float), ("mpaths_before", C.c_double),
                ("mpaths_after", C.c_double), ("trials", C.c_uint32), ("extend_blocks_per_sm", C.c_int),
                ("coop_triangles", C.c_int), ("fetch_refill", C.c_uint32), ("fetch_steps", C.c_uint32),
                ("material_sort", C.c_int)]


class _BatchRequest(C.Structure):
    _fields_ = [("renderer", C.c_void_p), ("accum", C.c_void_p), ("samples", C.c_uint32), ("cache", C.c_void_p)]


class _BatchTune(C.Structure):
    _fields_ = [("blocks_per_sm", C.c_int), ("order", C.c_int), ("wavefront_pixels", C.c_uint64),
                ("p50_seconds", C.c_double),
                ("p99_seconds", C.c_double), ("total_seconds", C.c_double), ("trials", C.c_uint32),
                ("wave_slots", C.c_uint32)]


BATCH_SHORTEST_FIRST, BATCH_AS_GIVEN, BATCH_LONGEST_FIRST = 0, 1, 2


@dataclass
class BatchRequest:
    """One request of vg_batch_render."""
    renderer: "Renderer"
    accum: "Accumulation"
    samples: int
    cache: Optional["Cache"] = None


@dataclass
class BatchOutcome:
    seconds: list          # per request, from the batch start to its last tile (device clock)
    total_seconds: float   # the whole batch, training included
    graph_replayed: bool


class _UpdatePlan(C.Structure):
    _fields_ = [("full", C.c_int), ("materials", C.c_int), ("lights", C.c_int), ("emitters", C.c_int),
                ("instances", C.c_int), ("vertices", C.c_int), ("blases", C.c_void_p), ("blas_count", C.c_size_t),
                ("tlas", C.c_int), ("camera", C.c_int)]


class _UpdateReport(C.Structure):
    _fields_ = [("blases_built", C.c_uint64), ("tlas_built", C.c_int), ("bytes_uploaded", C.c_uint64)]


@dataclass
class UpdateReport:
    """lib.rs:63-71"""
    blases_built: int = 0
    tlas_built: bool = False
    bytes_uploaded: int = 0


CACHE_RECORD_FLOATS = 20  # include/vgcuda.h VG_CACHE_RECORD_FLOATS
CACHE_MLP_PARAMS = 17408  # VG_CACHE_MLP_PARAMS

_lib = None


def lib() -> C.CDLL:
    """Loads libvgcuda.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise Error(VG_ERR_RESOURCE, f"{LIB_PATH} is missing: run `python -m verion_gb300.build`")
        L = C.CDLL(str(LIB_PATH))
        vp, u32, i32, f64 = C.c_void_p, C.c_uint32, C.c_int, C.c_double
        sig = {
            "vg_last_error": (_S, [C.c_char_p, _S]),
            "vg_last_oom": (None, [C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
            "vg_context_create": (i32, [C.POINTER(vp)]),
            "vg_context_create_on": (i32, [i32, C.POINTER(vp)]),
            "vg_debug_allocations": (None, [C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
            "vg_context_destroy": (None, [vp]),
            "vg_memory": (i32, [vp, C.POINTER(MemoryUsage)]),
            "vg_renderer_create": (i32, [vp, C.POINTER(_Packed), C.POINTER(vp)]),
            "vg_renderer_destroy": (None, [vp]),
            "vg_renderer_bvh_info": (i32, [vp, C.POINTER(BvhInfo)]),
            "vg_renderer_update": (i32, [vp, C.POINTER(_Packed), C.POINTER(_UpdatePlan), C.POINTER(_UpdateReport)]),
            "vg_set_camera": (i32, [vp, C.POINTER(_View)]),
            "vg_set_multiscatter": (i32, [vp, i32]),
            "vg_set_integrator": (i32, [vp, i32]),
            "vg_integrator": (i32, [vp]),
            "vg_set_stage_timing": (i32, [vp, i32]),
            "vg_set_adaptive": (i32, [vp, i32, C.c_float, u32]),
            "vg_set_restir": (i32, [vp, i32, i32, i32, u32, u32]),
            "vg_set_max_depth": (i32, [vp, u32]),
            "vg_set_traversal_stats": (i32, [vp, i32]),
            "vg_set_wavefront_mode": (i32, [vp, i32]),
            "vg_accum_last_waves": (u32, [vp]),
            "vg_accum_wave_profile": (_S, [vp, vp, _S]),
            "vg_set_stream_tail": (i32, [vp, u32]),
            "vg_accum_tail_seconds": (f64, [vp]),
            "vg_set_deferred_shadows": (i32, [vp, i32]),
            "vg_set_dynamic_fetch": (i32, [vp, i32]),
            "vg_set_coop_triangles": (i32, [vp, i32]),
            "vg_set_material_sort": (i32, [vp, i32]),
            "vg_set_traversal_fetch": (i32, [vp, u32, u32, u32, u32]),
            "vg_set_wavefront_graph": (i32, [vp, u32]),
            "vg_set_bvh_traversal_cost": (i32, [vp, C.POINTER(_Packed), C.c_float]),
            "vg_autotune": (i32, [vp, C.POINTER(_Packed), u32, u32, u32, C.POINTER(_TuneResult)]),
            "vg_accum_traversal_stats": (i32, [vp, C.POINTER(C.c_uint64)]),
            "vg_accum_shadow_rays": (i32, [vp, C.POINTER(C.c_uint64)]),
            "vg_set_accum_precision": (i32, [vp, i32]),
            "vg_accum_create": (i32, [vp, u32, u32, i32, C.POINTER(vp)]),
            "vg_accum_destroy": (None, [vp]),
            "vg_accumulate": (i32, [vp, vp, u32]),
            "vg_accum_samples": (u32, [vp]),
            "vg_accum_set_first_sample": (i32, [vp, u32]),
            "vg_accum_gpu_seconds": (f64, [vp]),
            "vg_accum_stage_seconds": (i32, [vp, C.POINTER(f64)]),
            "vg_accum_wavefront_bytes": (_S, [vp]),
            "vg_accum_restir_bytes": (_S, [vp]),
            "vg_accum_precision": (i32, [vp]),
            "vg_accum_read_sums": (i32, [vp, vp, _S]),
            "vg_accum_read_sums_f64": (i32, [vp, vp, _S]),
            "vg_accum_read_lighting": (i32, [vp, vp, _S]),
            "vg_accum_read_stats": (i32, [vp, vp, _S]),
            "vg_accum_launches": (C.c_uint64, [vp]),
            "vg_accum_read_queue_counts": (i32, [vp, vp, _S]),
            "vg_accum_extend_launch_seconds": (f64, [vp]),
            "vg_render_normals": (i32, [vp, u32, u32, vp]),
            "vg_render_aovs": (i32, [vp, u32, u32, vp, vp, vp, vp]),
            "vg_trace_closest": (i32, [vp, vp, _S, vp]),
            "vg_trace_occluded": (i32, [vp, vp, _S, vp]),
            "vg_trace_closest_device": (i32, [vp, vp, _S, vp, C.POINTER(f64)]),
            "vg_trace_closest_noalloc": (i32, [vp, vp, _S, vp]),
            "vg_cache_default_config": (None, [C.POINTER(CacheConfig)]),
            "vg_renderer_bounds": (i32, [vp, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
            "vg_cache_create": (i32, [vp, C.POINTER(CacheConfig), C.POINTER(vp)]),
            "vg_cache_destroy": (i32, [vp]),
            "vg_cache_param_counts": (i32, [vp, C.POINTER(_S), C.POINTER(_S)]),
            "vg_cache_read_params": (i32, [vp, vp, vp]),
            "vg_cache_write_params": (i32, [vp, vp, vp]),
            "vg_cache_infer": (i32, [vp, vp, _S, vp]),
            "vg_cache_gradients": (i32, [vp, vp, _S, vp, vp, C.POINTER(f64)]),
            "vg_cache_train": (i32, [vp, vp, _S, u32, C.POINTER(f64)]),
            "vg_set_cache": (i32, [vp, vp, C.c_float, u32, u32, u32]),
            "vg_set_cache_frame": (i32, [vp, u32]),
            "vg_set_cache_warmup": (i32, [vp, u32]),
            "vg_cache_time": (i32, [vp, vp, _S, u32, C.POINTER(f64)]),
            "vg_batch_render": (i32, [vp, vp, _S, vp, C.POINTER(f64), C.POINTER(C.c_int)]),
            "vg_set_batch_options": (i32, [vp, i32, i32, C.c_uint64]),
            "vg_set_batch_wave_slots": (i32, [vp, C.c_uint32]),
            "vg_set_batch_device_loop": (i32, [vp, i32]),
            "vg_batch_kernel_info": (i32, [vp, vp]),
            "vg_batch_tune": (i32, [vp, vp, _S, C.POINTER(_BatchTune)]),
            "vg_accum_cache_stats": (i32, [vp, C.POINTER(CacheStats)]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def device_allocations() -> tuple:
    """(cudaMalloc calls, cudaFree calls) the library has made since it was loaded."""
    m, f = C.c_uint64(), C.c_uint64()
    lib().vg_debug_allocations(C.byref(m), C.byref(f))
    return m.value, f.value


def _check(status: int) -> None:
    if status != VG_OK:
        L = lib()
        buf = C.create_string_buffer(1024)
        L.vg_last_error(buf, 1024)
        need, avail = C.c_uint64(), C.c_uint64()
        if status == VG_ERR_OOM:
            L.vg_last_oom(C.byref(need), C.byref(avail))
        raise Error(status, buf.value.decode(errors="replace"), need.value, avail.value)


def _ptr(a: np.ndarray) -> Optional[int]:
    return a.ctypes.data if a.size else None


def _view(v: View) -> _View:
    out = _View()
    out.camera[:] = [float(x) for x in v.camera]
    out.aperture = v.aperture
    out.focus = v.focus
    out.shift[:] = [float(v.shift[0]), float(v.shift[1])]
    return out


@dataclass
class Aovs:
    """lib.rs:165-181: primary-ray AOVs, row-major from the top-left; misses are zero."""
    albedo: np.ndarray       # (pixels, 3)
    depth: np.ndarray        # (pixels,) distance along the camera's forward axis
    object_id: np.ndarray    # instance index + 1
    material_id: np.ndarray  # material index + 1
    coverage: np.ndarray     # fraction of 16 stratified rays that hit


class Context:
    """The device and its stream (`RayTracingBackend::Context`). `device` is a CUDA ordinal; None
    opens the calling thread's current device (device 0 unless the caller selected another)."""

    def __init__(self, device: Optional[int] = None):
        h = C.c_void_p()
        if device is None:
            _check(lib().vg_context_create(C.byref(h)))
        else:
            _check(lib().vg_context_create_on(int(device), C.byref(h)))
        self._h = h
        self.device = device

    def memory(self) -> MemoryUsage:
        m = MemoryUsage()
        _check(lib().vg_memory(self._h, C.byref(m)))
        return m

    def batch_render(self, requests) -> "BatchOutcome":
        """vg_batch_render: `requests` are BatchRequest(renderer, accumulation, samples, cache)."""
        arr = (_BatchRequest * len(requests))()
        for i, q in enumerate(requests):
            arr[i].renderer = q.renderer._h
            arr[i].accum = q.accum._h
            arr[i].samples = q.samples
            arr[i].cache = q.cache._h if q.cache is not None else None
        out = (C.c_double * len(requests))()
        total = C.c_double()
        replayed = C.c_int()
        _check(lib().vg_batch_render(self._h, arr, len(requests), out, C.byref(total), C.byref(replayed)))
        return BatchOutcome(list(out), total.value, bool(replayed.value))

    def batch_kernel_info(self) -> dict:
        v = (C.c_int * 5)()
        _check(lib().vg_batch_kernel_info(self._h, v))
        return dict(zip(("blocks_per_sm", "registers", "local_bytes", "static_smem", "cuda_status"), list(v)))

    def set_batch_options(self, blocks_per_sm: int = 0, order: int = 0, wavefront_pixels: int = 0) -> None:
        _check(lib().vg_set_batch_options(self._h, blocks_per_sm, order, wavefront_pixels))

    def set_batch_wave_slots(self, slots: int) -> None:
        """vg_set_batch_wave_slots: path slots of the batch wavefront (pixels in flight at once)."""
        _check(lib().vg_set_batch_wave_slots(self._h, slots))

    def set_batch_device_loop(self, on: bool) -> None:
        """vg_set_batch_device_loop: the batch wavefront's bounce loop in the graph (True) or on the host."""
        _check(lib().vg_set_batch_device_loop(self._h, 1 if on else 0))

    def batch_tune(self, requests) -> dict:
        """vg_batch_tune: picks the tile launch's CTAs per SM, the item order, the size threshold and the
        batch wavefront's slots for these requests."""
        arr = (_BatchRequest * len(requests))()
        for i, q in enumerate(requests):
            arr[i].renderer = q.renderer._h
            arr[i].accum = q.accum._h
            arr[i].samples = q.samples
            arr[i].cache = q.cache._h if q.cache is not None else None
        t = _BatchTune()
        _check(lib().vg_batch_tune(self._h, arr, len(requests), C.byref(t)))
        return {"blocks_per_sm": t.blocks_per_sm, "order": t.order, "wavefront_pixels": t.wavefront_pixels,
                "p50_seconds": t.p50_seconds,
                "p99_seconds": t.p99_seconds, "total_seconds": t.total_seconds, "trials": t.trials,
                "wave_slots": t.wave_slots}

    def close(self):
        if self._h:
            lib().vg_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Accumulation:
    """Running radiance sums of one image (`Accumulation` trait, lib.rs:74-93)."""

    def __init__(self, renderer: "Renderer", width: int, height: int, lighting: bool):
        h = C.c_void_p()
        _check(lib().vg_accum_create(renderer._h, width, height, int(lighting), C.byref(h)))
        self._h = h
        self._r = renderer
        self.width, self.height, self.has_lighting = width, height, lighting
        self.adaptive: Optional[Adaptive] = None

    @property
    def pixels(self) -> int:
        return self.width * self.height

    def samples(self) -> int:
        return lib().vg_accum_samples(self._h)

    def gpu_seconds(self) -> float:
        return lib().vg_accum_gpu_seconds(self._h)

    def stage_seconds(self):
        out = (C.c_double * 2)()
        return (out[0], out[1]) if lib().vg_accum_stage_seconds(self._h, out) else None

    def wavefront_bytes(self) -> int:
        return lib().vg_accum_wavefront_bytes(self._h)

    def restir_bytes(self) -> int:
        return lib().vg_accum_restir_bytes(self._h)

    def precision(self) -> int:
        return lib().vg_accum_precision(self._h)

    def queue_counts(self, depth: int) -> np.ndarray:
        """Wavefront queue lengths of the last sample (depths 0..depth)."""
        out = np.empty(depth + 1, np.uint32)
        _check(lib().vg_accum_read_queue_counts(self._h, out.ctypes.data, out.size))
        return out

    def last_waves(self) -> int:
        return lib().vg_accum_last_waves(self._h)

    def tail_seconds(self) -> float:
        return lib().vg_accum_tail_seconds(self._h)

    def wave_profile(self) -> np.ndarray:
        """(waves, 4): live slots after each wave, extend, shade and shadow ms (last streaming call)."""
        n = lib().vg_accum_wave_profile(self._h, None, 0)
        out = np.zeros(4 * n, np.float32)
        lib().vg_accum_wave_profile(self._h, _ptr(out), n)
        return out.reshape(-1, 4)

    def traversal_stats(self) -> dict:
        out = (C.c_uint64 * 4)()
        _check(lib().vg_accum_traversal_stats(self._h, out))
        return {"rays": out[0], "nodes": out[1], "tests": out[2], "rays_after_depth0": out[3]}

    def shadow_rays(self) -> int:
        """Rays traced by the any-hit shadow stage (traversal stats on)."""
        out = C.c_uint64(0)
        _check(lib().vg_accum_shadow_rays(self._h, C.byref(out)))
        return out.value

    def launches(self) -> int:
        return lib().vg_accum_launches(self._h)

    def set_first_sample(self, first: int) -> None:
        """Sample indices start at `first` (before the first sample; plain path tracing only)."""
        _check(lib().vg_accum_set_first_sample(self._h, first))

    def extend_launch_seconds(self) -> float:
        return lib().vg_accum_extend_launch_seconds(self._h)

    def sums(self, into: Optional[np.ndarray] = None) -> np.ndarray:
        out = into if into is not None else np.empty(3 * self.pixels, np.float32)
        _check(lib().vg_accum_read_sums(self._h, out.ctypes.data, out.size))
        return out

    def sums_f64(self) -> np.ndarray:
        out = np.empty(3 * self.pixels, np.float64)
        _check(lib().vg_accum_read_sums_f64(self._h, out.ctypes.data, out.size))
        return out

    def raw_stats(self) -> Optional[np.ndarray]:
        if self.adaptive is None:
            return None
        out = np.empty(3 * self.pixels, np.float32)
        _check(lib().vg_accum_read_stats(self._h, out.ctypes.data, out.size))
        return out

    def raw_lighting(self) -> Optional[np.ndarray]:
        if not self.has_lighting:
            return None
        out = np.empty(rb.LIGHTING_STRIDE * self.pixels, np.float32)
        _check(lib().vg_accum_read_lighting(self._h, out.ctypes.data, out.size))
        return out

    def _inverse(self) -> np.ndarray:
        return rb.inverse_samples(self.raw_stats(), self.pixels, self.samples())

    def mean(self) -> np.ndarray:
        """Mean radiance per pixel, (pixels, 3), row-major from the top-left."""
        return rb.mean(self.sums(), self._inverse())

    def lighting(self) -> Optional[rb.LightingAovs]:
        data = self.raw_lighting()
        return None if data is None else rb.lighting(data, self._inverse())

    def sample_counts(self) -> Optional[np.ndarray]:
        st = self.raw_stats()
        return None if st is None else rb.sample_counts(st)

    def active_pixels(self) -> int:
        return rb.active_pixels(self.raw_stats(), self.adaptive, self.pixels)

    def cache_stats(self) -> CacheStats:
        st = CacheStats()
        _check(lib().vg_accum_cache_stats(self._h, C.byref(st)))
        return st

    def close(self):
        if self._h:
            lib().vg_accum_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Renderer:
    """A scene on the GPU (`RayTracingBackend` implementation, lib.rs:12-58)."""

    def __init__(self, ctx: Context, scene_or_packed):
        packed = scene_or_packed if isinstance(scene_or_packed, Packed) else pack(scene_or_packed)
        self.packed = packed
        pk = self._struct(packed)
        h = C.c_void_p()
        _check(lib().vg_renderer_create(ctx._h, C.byref(pk), C.byref(h)))
        self._h = h
        self._ctx = ctx
        self._keep = []
        self._adaptive: Optional[Adaptive] = None
        self._restir: Optional[Restir] = None

    def update(self, scene_or_packed, plan) -> "UpdateReport":
        """RayTracingBackend::update (lib.rs:23-27): applies `plan` (pack.UpdatePlan) from the
        edited scene's tables; returns what was rebuilt."""
        packed = scene_or_packed if isinstance(scene_or_packed, Packed) else pack(scene_or_packed)
        pk = self._struct(packed)
        blases = np.ascontiguousarray(plan.blases, np.uint32)
        up = _UpdatePlan(int(plan.full), int(plan.materials), int(plan.lights), int(plan.emitters),
                         int(plan.instances), int(plan.vertices), _ptr(blases) if blases.size else None,
                         blases.size, int(plan.tlas), int(plan.camera))
        rep = _UpdateReport()
        _check(lib().vg_renderer_update(self._h, C.byref(pk), C.byref(up), C.byref(rep)))
        self._keep = []
        self.packed = packed
        return UpdateReport(rep.blases_built, bool(rep.tlas_built), rep.bytes_uploaded)

    def _struct(self, packed: Packed) -> "_Packed":
        self._keep = []
        pk = _Packed()

        def put(name, arr, dtype):
            a = np.ascontiguousarray(arr, dtype=dtype).reshape(-1)
            self._keep.append(a)
            setattr(pk, name, _ptr(a))
            setattr(pk, name + "_len", a.size)

        put("positions", packed.positions, np.float32)
        put("indices", packed.indices, np.uint32)
        put("uvs", packed.uvs, np.float32)
        put("vnormals", packed.vnormals, np.float32)
        put("instances", packed.instances, np.uint32)
        put("materials", packed.materials, np.float32)
        put("lights", packed.lights, np.uint32)
        put("emitters", packed.emitters, np.float32)
        put("emit_cdf", packed.emit_cdf, np.float32)
        put("env_pixels", packed.env.pixels, np.float32)
        put("env_marginal", packed.env.marginal, np.float32)
        put("env_conditional", packed.env.conditional, np.float32)
        put("texels", packed.texels, np.float32)
        put("tex_info", packed.tex_info, np.uint32)
        meshes = np.ascontiguousarray(packed.meshes, np.uint32).reshape(-1, 4)
        tm = np.ascontiguousarray(packed.tlas_mesh, np.uint32)
        tt = np.ascontiguousarray(packed.tlas_transform, np.float32)
        self._keep += [meshes, tm, tt]
        pk.meshes, pk.mesh_count = _ptr(meshes), len(meshes)
        pk.tlas_mesh, pk.tlas_transform, pk.instance_count = _ptr(tm), _ptr(tt), len(tm)
        i = packed.info
        pk.info.light_count, pk.info.emitter_count = i.light_count, i.emitter_count
        pk.info.env_width, pk.info.env_height, pk.info.env_pdf_scale = i.env_width, i.env_height, i.env_pdf_scale
        pk.info.sky[:] = list(i.sky)
        pk.info.virtual_light, pk.info.transparent_background = int(i.virtual_light), int(i.transparent_background)
        pk.view = _view(packed.view)
        return pk

    # RayTracingBackend setters
    def set_camera(self, view_or_camera) -> None:
        v = view_or_camera if isinstance(view_or_camera, View) else View.new(view_or_camera)
        cv = _view(v)
        _check(lib().vg_set_camera(self._h, C.byref(cv)))

    def set_multiscatter(self, on: bool) -> None:
        _check(lib().vg_set_multiscatter(self._h, int(on)))

    def set_integrator(self, integrator: Integrator) -> None:
        _check(lib().vg_set_integrator(self._h, int(integrator)))

    def integrator(self) -> Integrator:
        return Integrator(lib().vg_integrator(self._h))

    def set_stage_timing(self, on: bool) -> None:
        _check(lib().vg_set_stage_timing(self._h, int(on)))

    def set_adaptive(self, adaptive: Optional[Adaptive]) -> None:
        a = adaptive
        _check(lib().vg_set_adaptive(self._h, int(a is not None), a.threshold if a else 0.0, a.min_spp if a else 0))
        self._adaptive = adaptive

    def set_restir(self, restir: Optional[Restir]) -> None:
        r = restir
        _check(lib().vg_set_restir(self._h, int(r is not None), int(r.di) if r else 0, int(r.gi) if r else 0,
                                   r.candidates if r else 0, r.history if r else 0))
        self._restir = restir

    def set_wavefront_mode(self, mode: "WavefrontMode") -> None:
        _check(lib().vg_set_wavefront_mode(self._h, int(mode)))

    def set_bvh_traversal_cost(self, cost: float) -> None:
        """Rebuilds the BVH8 with another SAH node-visit cost (needs the renderer's packed tables)."""
        pk = self._struct(self.packed)
        _check(lib().vg_set_bvh_traversal_cost(self._h, C.byref(pk), cost))
        self._keep = []

    def autotune(self, width: int, height: int, samples: int, bvh: bool = True) -> dict:
        """vg_autotune: picks the streaming-wavefront settings (and, with `bvh`, the BVH8's SAH cost)."""
        pk = self._struct(self.packed) if bvh else None
        t = _TuneResult()
        _check(lib().vg_autotune(self._h, C.byref(pk) if pk is not None else None, width, height, samples,
                                 C.byref(t)))
        self._keep = []
        return {k: getattr(t, k) for k, _ in _TuneResult._fields_}

    def set_wavefront_graph(self, waves: int) -> None:
        """Streaming mode: replay a captured CUDA graph of `waves` waves (even; 0 = off)."""
        _check(lib().vg_set_wavefront_graph(self._h, waves))

    def set_dynamic_fetch(self, on: bool) -> None:
        _check(lib().vg_set_dynamic_fetch(self._h, int(on)))

    def set_material_sort(self, on: bool) -> None:
        """Streaming wavefront: shade each wave's slots class by class (same sums)."""
        _check(lib().vg_set_material_sort(self._h, int(on)))

    def set_coop_triangles(self, on: bool) -> None:
        """Warp-cooperative leaf testing in the streaming traversal stages (same results)."""
        _check(lib().vg_set_coop_triangles(self._h, int(on)))

    def set_traversal_fetch(self, refill: int = 8, steps: int = 4, shadow_refill: int = None,
                            shadow_steps: int = None) -> None:
        """Dynamic fetch of the streaming traversal stages: idle lanes per refill, node visits
        between refills (the shadow stage's default to the extend stage's)."""
        _check(lib().vg_set_traversal_fetch(self._h, refill, steps, refill if shadow_refill is None else shadow_refill,
                                            steps if shadow_steps is None else shadow_steps))

    def set_deferred_shadows(self, on: bool) -> None:
        _check(lib().vg_set_deferred_shadows(self._h, int(on)))

    def set_stream_tail(self, threshold: int) -> None:
        _check(lib().vg_set_stream_tail(self._h, threshold))

    def set_traversal_stats(self, on: bool) -> None:
        _check(lib().vg_set_traversal_stats(self._h, int(on)))

    def set_max_depth(self, depth: int) -> None:
        _check(lib().vg_set_max_depth(self._h, depth))

    def set_accum_precision(self, bits: int) -> None:
        _check(lib().vg_set_accum_precision(self._h, bits))

    def bvh_info(self) -> BvhInfo:
        b = BvhInfo()
        _check(lib().vg_renderer_bvh_info(self._h, C.byref(b)))
        return b

    def new_accumulation(self, width: int, height: int, lighting: bool = False) -> Accumulation:
        return Accumulation(self, width, height, lighting)

    def accumulate(self, acc: Accumulation, samples: int) -> None:
        if acc.samples() == 0:
            acc.adaptive = self._adaptive
        _check(lib().vg_accumulate(self._h, acc._h, samples))

    def render(self, width: int, height: int, samples: int) -> np.ndarray:
        """One-shot mean radiance (the Metal renderer's `render`, renderer.rs:489-494)."""
        acc = self.new_accumulation(width, height, False)
        self.accumulate(acc, samples)
        return acc.mean()

    def render_normals(self, width: int, height: int) -> np.ndarray:
        """RayTracingBackend::render_normals: (pixels, 3) first-hit normals, misses zero."""
        out = np.empty(3 * width * height, np.float32)
        _check(lib().vg_render_normals(self._h, width, height, out.ctypes.data))
        return out.reshape(-1, 3)

    def render_aovs(self, width: int, height: int) -> "Aovs":
        """RayTracingBackend::render_aovs (lib.rs:165-181)."""
        n = width * height
        ad = np.empty(4 * n, np.float32)
        oi = np.empty(n, np.uint32)
        mi = np.empty(n, np.uint32)
        cv = np.empty(n, np.float32)
        _check(lib().vg_render_aovs(self._h, width, height, ad.ctypes.data, oi.ctypes.data, mi.ctypes.data,
                                    cv.ctypes.data))
        ad = ad.reshape(-1, 4)
        return Aovs(ad[:, :3].copy(), ad[:, 3].copy(), oi, mi, cv)

    # Traversal entry points
    def trace_closest(self, rays: np.ndarray) -> np.ndarray:
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        out = np.empty((len(r), 4), np.uint32)
        _check(lib().vg_trace_closest(self._h, _ptr(r), len(r), _ptr(out)))
        return out

    def trace_closest_noalloc(self, rays: np.ndarray) -> np.ndarray:
        """trace_closest through the library's static device scratch (no device allocation);
        at most VG_TRACE_NOALLOC_MAX_RAYS rays per call."""
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        out = np.empty((len(r), 4), np.uint32)
        _check(lib().vg_trace_closest_noalloc(self._h, _ptr(r), len(r), _ptr(out)))
        return out

    def trace_occluded(self, rays: np.ndarray) -> np.ndarray:
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 7)
        out = np.empty(len(r), np.uint32)
        _check(lib().vg_trace_occluded(self._h, _ptr(r), len(r), _ptr(out)))
        return out

    def bounds(self):
        """World-space box (lo, hi) of the scene's triangles."""
        lo, hi = (C.c_float * 3)(), (C.c_float * 3)()
        _check(lib().vg_renderer_bounds(self._h, lo, hi))
        return tuple(lo), tuple(hi)

    def set_cache(self, cache: Optional["Cache"], spread: float = 0.01, train_paths: int = 16384,
                  train_steps: int = 4, train_batch: int = 16384) -> None:
        """Radiance-cache integrator (None: off); the renderer keeps a reference to the cache."""
        _check(lib().vg_set_cache(self._h, cache._h if cache else None, spread, train_paths, train_steps,
                                  train_batch))
        self._cache = cache

    def set_cache_warmup(self, frames: int) -> None:
        """Radiance cache: training-only frames before the first sample of each accumulation."""
        _check(lib().vg_set_cache_warmup(self._h, frames))

    def set_cache_frame(self, samples_per_frame: int) -> None:
        """WAVEFRONT integrator with a cache: samples per cache frame (the cache is trained after
        each frame)."""
        _check(lib().vg_set_cache_frame(self._h, samples_per_frame))

    def close(self):
        if self._h:
            lib().vg_renderer_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Cache:
    """Radiance cache: hash-grid encoding + 64-wide MLP trained on the tensor cores (include/vgcuda.h,
    "Radiance cache"). Records are (n, CACHE_RECORD_FLOATS) float32 arrays."""

    def __init__(self, ctx: Context, config: Optional[CacheConfig] = None, bounds=None, **overrides):
        cfg = CacheConfig()
        lib().vg_cache_default_config(C.byref(cfg))
        if config is not None:
            C.memmove(C.byref(cfg), C.byref(config), C.sizeof(CacheConfig))
        for k, v in overrides.items():
            setattr(cfg, k, v)
        if bounds is not None:
            lo, hi = bounds
            for i in range(3):
                cfg.bounds_lo[i] = lo[i]
                cfg.bounds_hi[i] = hi[i]
        self.config = cfg
        self._ctx = ctx
        h = C.c_void_p()
        _check(lib().vg_cache_create(ctx._h, C.byref(cfg), C.byref(h)))
        self._h = h

    def param_counts(self):
        m, g = _S(), _S()
        _check(lib().vg_cache_param_counts(self._h, C.byref(m), C.byref(g)))
        return m.value, g.value

    def read_params(self):
        m, g = self.param_counts()
        mlp, grid = np.empty(m, np.float32), np.empty(g, np.float32)
        _check(lib().vg_cache_read_params(self._h, _ptr(mlp), _ptr(grid)))
        return mlp, grid

    def write_params(self, mlp: Optional[np.ndarray] = None, grid: Optional[np.ndarray] = None) -> None:
        m, g = self.param_counts()
        mp = np.ascontiguousarray(mlp, np.float32) if mlp is not None else None
        gp = np.ascontiguousarray(grid, np.float32) if grid is not None else None
        if mp is not None and mp.size != m or gp is not None and gp.size != g:
            raise ValueError("parameter vector of the wrong size")
        _check(lib().vg_cache_write_params(self._h, _ptr(mp) if mp is not None else None,
                                           _ptr(gp) if gp is not None else None))

    @staticmethod
    def _records(records: np.ndarray) -> np.ndarray:
        return np.ascontiguousarray(records, np.float32).reshape(-1, CACHE_RECORD_FLOATS)

    def infer(self, records: np.ndarray) -> np.ndarray:
        r = self._records(records)
        out = np.empty((len(r), 3), np.float32)
        _check(lib().vg_cache_infer(self._h, _ptr(r), len(r), _ptr(out)))
        return out

    def gradients(self, records: np.ndarray):
        """(mlp gradient sums, grid gradient sums, loss sum) over the records, not applied."""
        r = self._records(records)
        m, g = self.param_counts()
        gm, gg = np.empty(m, np.float32), np.empty(g, np.float32)
        loss = C.c_double()
        _check(lib().vg_cache_gradients(self._h, _ptr(r), len(r), _ptr(gm), _ptr(gg), C.byref(loss)))
        return gm, gg, loss.value

    def train(self, records: np.ndarray, batch: int) -> float:
        """Adam steps over consecutive batches; returns the last batch's mean loss per channel."""
        r = self._records(records)
        loss = C.c_double()
        _check(lib().vg_cache_train(self._h, _ptr(r), len(r), batch, C.byref(loss)))
        return loss.value

    def time_kernels(self, records: np.ndarray, reps: int = 10) -> dict:
        """Device seconds per launch of the encode, inference, training-pass and scatter kernels."""
        r = self._records(records)
        out = (C.c_double * 4)()
        _check(lib().vg_cache_time(self._h, _ptr(r), len(r), reps, out))
        return dict(zip(("encode", "infer", "train", "scatter"), list(out)))

    def close(self):
        if getattr(self, "_h", None):
            lib().vg_cache_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
