"""CPU ORACLE — test infrastructure only.

Only the tests, `__graft_entry__.smoke()` and the benchmark's CPU-baseline leg may load this
package, and only as the checker or as the timed CPU baseline; the CUDA backend never calls it.

`pt_oracle.cpp` restates Verion's path-tracing integrator (shaders/include/pt_core.slang,
shaders/include/wf_state.slang, shaders/pathtrace.slang, shaders/wf_*.slang) in C++; this module
compiles it (`build()`) and wraps its C interface with ctypes. Parity status: the albedo tables are
pinned byte for byte against the reference's; the BSDF/integrator arithmetic is a line-by-line
restatement checked against the reference's own analytic tests (white furnace, series sum, form
factors, Fresnel, GGX highlight); ray traversal has no reference counterpart (the reference uses
the driver's hardware ray tracing), so hit IDs are pinned by brute force and by the
two-instance distance test of crates/verion-gpu-metal/tests/trace.rs:95-121.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "pt_oracle.cpp"
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
DEPS = [SRC, HERE.parent / "verion_gb300" / "csrc" / "vg_math.h"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-fno-fast-math"]


def build(force: bool = False) -> Path:
    """Compiles liboracle.so (g++, no floating-point contraction)."""
    BUILD.mkdir(exist_ok=True)
    if not force and LIB.exists() and all(LIB.stat().st_mtime >= d.stat().st_mtime for d in DEPS):
        return LIB
    cxx = shutil.which("g++") or "g++"
    tmp = BUILD / f"liboracle.so.{os.getpid()}"
    r = subprocess.run([cxx] + CXX_FLAGS + [str(SRC), "-o", str(tmp)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


class _Tables(C.Structure):
    _fields_ = [(n, t) for pair in [
        (("positions", C.c_void_p), ("positions_len", C.c_size_t)),
        (("indices", C.c_void_p), ("indices_len", C.c_size_t)),
        (("uvs", C.c_void_p), ("uvs_len", C.c_size_t)),
        (("vnormals", C.c_void_p), ("vnormals_len", C.c_size_t)),
        (("instances", C.c_void_p), ("instances_len", C.c_size_t)),
        (("materials", C.c_void_p), ("materials_len", C.c_size_t)),
        (("lights", C.c_void_p), ("lights_len", C.c_size_t)),
        (("emitters", C.c_void_p), ("emitters_len", C.c_size_t)),
        (("emit_cdf", C.c_void_p), ("emit_cdf_len", C.c_size_t)),
        (("env_pixels", C.c_void_p), ("env_pixels_len", C.c_size_t)),
        (("env_marginal", C.c_void_p), ("env_marginal_len", C.c_size_t)),
        (("env_cond", C.c_void_p), ("env_cond_len", C.c_size_t)),
        (("texels", C.c_void_p), ("texels_len", C.c_size_t)),
        (("tex_info", C.c_void_p), ("tex_info_len", C.c_size_t)),
        (("tri_counts", C.c_void_p), ("instance_count", C.c_size_t))] for n, t in pair]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        L = C.CDLL(str(build()))
        vp, sz, u32p = C.c_void_p, C.c_size_t, C.c_void_p
        L.or_scene_create.restype = vp
        L.or_scene_create.argtypes = [C.POINTER(_Tables)]
        L.or_scene_destroy.argtypes = [vp]
        L.or_scene_triangles.restype = C.c_uint32
        L.or_scene_triangles.argtypes = [vp]
        L.or_trace_closest.argtypes = [vp, vp, sz, vp, C.c_int, C.c_int]
        L.or_trace_occluded.argtypes = [vp, vp, sz, vp, C.c_int]
        L.or_render.restype = C.c_int
        L.or_render.argtypes = [vp, vp, C.c_uint32, C.c_uint32, C.c_int, C.c_int, vp, vp, vp, vp, C.c_int, vp,
                                C.c_int, C.c_int, vp, C.c_uint32]
        for name in ("or_sinf", "or_cosf", "or_acosf", "or_log2f", "or_exp2f"):
            getattr(L, name).restype = C.c_float
            getattr(L, name).argtypes = [C.c_float]
        for name in ("or_atan2f", "or_powf"):
            getattr(L, name).restype = C.c_float
            getattr(L, name).argtypes = [C.c_float, C.c_float]
        L.or_render_normals.argtypes = [vp, vp, vp, C.c_int]
        L.or_render_aovs.argtypes = [vp, vp, vp, vp, vp, vp, C.c_int]
        L.or_pcg.restype = C.c_uint32
        L.or_pcg.argtypes = [C.c_uint32]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data if a is not None and a.size else None


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)


class OracleScene:
    """The packed tables of a scene on the CPU, with the oracle's own BVH."""

    def __init__(self, packed):
        self._keep = []

        def arr(a, t):
            x = np.ascontiguousarray(a, dtype=t).reshape(-1)
            self._keep.append(x)
            return x

        t = _Tables()
        for name, a, dt in [("positions", packed.positions, np.float32), ("indices", packed.indices, np.uint32),
                            ("uvs", packed.uvs, np.float32), ("vnormals", packed.vnormals, np.float32),
                            ("instances", packed.instances, np.uint32), ("materials", packed.materials, np.float32),
                            ("lights", packed.lights, np.uint32), ("emitters", packed.emitters, np.float32),
                            ("emit_cdf", packed.emit_cdf, np.float32), ("env_pixels", packed.env.pixels, np.float32),
                            ("env_marginal", packed.env.marginal, np.float32),
                            ("env_cond", packed.env.conditional, np.float32), ("texels", packed.texels, np.float32),
                            ("tex_info", packed.tex_info, np.uint32)]:
            x = arr(a, dt)
            setattr(t, name, _ptr(x))
            setattr(t, name + "_len", x.size)
        meshes = np.asarray(packed.meshes, np.uint32).reshape(-1, 4)
        counts = arr(meshes[np.asarray(packed.tlas_mesh, np.int64), 3] // 3, np.uint32)
        t.tri_counts, t.instance_count = _ptr(counts), counts.size
        self._h = lib().or_scene_create(C.byref(t))
        self.packed = packed

    def triangles(self) -> int:
        return lib().or_scene_triangles(self._h)

    def trace_closest(self, rays: np.ndarray, brute: bool = False, threads: int = 0) -> np.ndarray:
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        out = np.zeros((len(r), 4), np.uint32)
        lib().or_trace_closest(self._h, _ptr(r), len(r), _ptr(out), int(brute), threads or default_threads())
        return out

    def trace_occluded(self, rays: np.ndarray, threads: int = 0) -> np.ndarray:
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 7)
        out = np.zeros(len(r), np.uint32)
        lib().or_trace_occluded(self._h, _ptr(r), len(r), _ptr(out), threads or default_threads())
        return out

    def render_normals(self, camera18: np.ndarray, threads: int = 0) -> np.ndarray:
        """shaders/normals.slang: (pixels, 3) first-hit normals facing the viewer."""
        cam = np.ascontiguousarray(camera18, np.float32)
        n = int(cam[0]) * int(cam[1])
        out = np.zeros(3 * n, np.float32)
        lib().or_render_normals(self._h, _ptr(cam), _ptr(out), threads or default_threads())
        return out.reshape(-1, 3)

    def render_aovs(self, camera18: np.ndarray, threads: int = 0):
        """shaders/aov.slang: albedo + depth (pixels, 4), object ids, material ids, coverage."""
        cam = np.ascontiguousarray(camera18, np.float32)
        n = int(cam[0]) * int(cam[1])
        ad = np.zeros(4 * n, np.float32)
        oi = np.zeros(n, np.uint32)
        mi = np.zeros(n, np.uint32)
        cv = np.zeros(n, np.float32)
        lib().or_render_aovs(self._h, _ptr(cam), _ptr(ad), _ptr(oi), _ptr(mi), _ptr(cv), threads or default_threads())
        return ad.reshape(-1, 4), oi, mi, cv

    def __del__(self):
        try:
            if self._h:
                lib().or_scene_destroy(self._h)
        except Exception:
            pass


class OracleAccumulation:
    """Running sums like the backend's accumulation, filled by the oracle."""

    def __init__(self, width: int, height: int, lighting: bool = False, acc64: bool = False,
                 adaptive: bool = False, restir: bool = False):
        n = width * height
        self.width, self.height = width, height
        self.acc64 = acc64
        dt = np.float64 if acc64 else np.float32
        self.sums = np.zeros(3 * n, dt)
        self.stats = np.zeros(3 * n, dt) if adaptive else None
        self.lighting = np.zeros(65 * n, np.float32) if lighting else None
        self.restir = np.zeros(80 * n, np.float32) if restir else None
        self.samples = 0
        self.queue_counts = []


def render(scene: OracleScene, params: np.ndarray, acc: OracleAccumulation, samples: int, *,
           double: bool = False, wavefront: bool = False, threads: int = 0, brute: bool = False,
           rows=None) -> None:
    """Adds `samples` samples to `acc` with the parameter block `params` (43 words)."""
    p = np.ascontiguousarray(params, np.uint32).copy()
    depth = int(p[7])
    qc = np.zeros(samples * (depth + 1), np.uint32) if wavefront else None
    rows_a = None if rows is None else np.ascontiguousarray(rows, np.uint32)
    lib().or_render(scene._h, _ptr(p), acc.samples, samples, int(double), int(acc.acc64), _ptr(acc.sums),
                    _ptr(acc.stats), _ptr(acc.lighting), _ptr(acc.restir), int(wavefront), _ptr(qc),
                    threads or default_threads(), int(brute), _ptr(rows_a),
                    0 if rows_a is None else rows_a.size)
    if wavefront:
        acc.queue_counts.extend(qc.reshape(samples, depth + 1).tolist())
    acc.samples += samples
