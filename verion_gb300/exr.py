"""EXR output and comparison.

`write_exr` writes a frame through the C ABI (`vg_write_exr`, the reference's
crates/verion-render-io/src/exr_out.rs). `read_exr` reads scanline OpenEXR files (uncompressed,
RLE, ZIPS and ZIP; FLOAT, HALF and UINT channels) into numpy planes and header attributes, and
`beauty_rec709` applies the reference's `load_hdri` reading of a file's Beauty
(crates/verion-render-io/src/hdri.rs:61-77). `diff` computes the reference's `exr_diff` gates
(crates/verion-render-io/examples/exr_diff.rs): worst channel-mean ratio and worst 4x4 block-mean
ratio against a reference image, plus relative mean absolute error and PSNR.
"""
from __future__ import annotations

import ctypes as C
import math
import struct
import zlib
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

COLOR_LINEAR_REC709, COLOR_ACESCG = 0, 1
TONEMAP_NONE, TONEMAP_REINHARD = 0, 1
OETF_LINEAR, OETF_SRGB = 0, 1

# crates/verion-scene/src/color.rs:18-28
ACESCG_TO_REC709 = np.array([[1.705052, -0.621792, -0.083258], [-0.130257, 1.140805, -0.010548],
                             [-0.024004, -0.128969, 1.152972]], np.float32)


class _Transform(C.Structure):
    _fields_ = [("target", C.c_int), ("tone_map", C.c_int), ("oetf", C.c_int)]


class _Frame(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("working_space", C.c_int),
                ("beauty", C.c_void_p), ("normal", C.c_void_p), ("albedo", C.c_void_p), ("depth", C.c_void_p),
                ("object_id", C.c_void_p), ("material_id", C.c_void_p), ("sample_count", C.c_void_p),
                ("lighting", C.c_void_p * 5), ("visibility", C.c_void_p), ("physical", C.c_int),
                ("samples", C.c_uint32), ("stylization_revision", C.c_uint64), ("has_grade", C.c_int),
                ("exposure", C.c_float), ("saturation", C.c_float), ("white_balance", C.c_float * 3),
                ("denoiser", C.c_char_p), ("has_adaptive_threshold", C.c_int), ("adaptive_threshold", C.c_float),
                ("restir", C.c_char_p)]


@dataclass
class RenderInfo:
    """exr_out.rs:19-37"""
    physical: bool = True
    samples: int = 0
    stylization_revision: int = 0
    grade: Optional[tuple] = None  # (exposure, saturation, (r, g, b))
    denoiser: Optional[str] = None
    adaptive_threshold: Optional[float] = None
    restir: Optional[str] = None


def write_exr(path, width: int, height: int, beauty, *, normal=None, albedo=None, depth=None, object_id=None,
              material_id=None, sample_count=None, lighting=None, visibility=None,
              info: RenderInfo = RenderInfo(), working_space: int = COLOR_LINEAR_REC709,
              target: int = COLOR_LINEAR_REC709, tone_map: int = TONEMAP_NONE, oetf: int = OETF_LINEAR) -> None:
    """Writes one frame (pixels row-major from the top-left). `lighting` is the five radiance
    parts (direct diffuse, indirect diffuse, specular, transmission, emission); raises
    backend.Error for a malformed frame. Arrays whose size does not match width x height are
    rejected here, as the reference's writer does (exr_out.rs:111-140)."""
    from .backend import Error, _check, lib

    n = width * height
    keep = []

    def arr(a, dtype, per):
        if a is None:
            return None
        x = np.ascontiguousarray(a, dtype).reshape(-1)
        if x.size != n * per:
            raise Error(8, "invalid frame: pixel count does not match width x height")
        keep.append(x)
        return x.ctypes.data

    f = _Frame()
    f.width, f.height, f.working_space = width, height, working_space
    f.beauty = arr(beauty, np.float32, 3)
    f.normal = arr(normal, np.float32, 3)
    f.albedo = arr(albedo, np.float32, 3)
    f.depth = arr(depth, np.float32, 1)
    f.object_id = arr(object_id, np.uint32, 1)
    f.material_id = arr(material_id, np.uint32, 1)
    f.sample_count = arr(sample_count, np.uint32, 1)
    if lighting is not None:
        for k in range(5):
            f.lighting[k] = arr(lighting[k], np.float32, 3)
    f.visibility = arr(visibility, np.float32, 1)
    f.physical = int(info.physical)
    f.samples = min(int(info.samples), 0xFFFFFFFF)
    f.stylization_revision = int(info.stylization_revision)
    if info.grade is not None:
        f.has_grade = 1
        f.exposure, f.saturation = info.grade[0], info.grade[1]
        f.white_balance[:] = list(info.grade[2])
    f.denoiser = info.denoiser.encode() if info.denoiser else None
    if info.adaptive_threshold is not None:
        f.has_adaptive_threshold, f.adaptive_threshold = 1, info.adaptive_threshold
    f.restir = info.restir.encode() if info.restir else None
    t = _Transform(target, tone_map, oetf)
    L = lib()
    L.vg_write_exr.restype = C.c_int
    L.vg_write_exr.argtypes = [C.c_char_p, C.POINTER(_Frame), C.POINTER(_Transform)]
    _check(L.vg_write_exr(str(path).encode(), C.byref(f), C.byref(t)))


# ---- reading ---------------------------------------------------------------------------------------

@dataclass
class ExrImage:
    width: int
    height: int
    channels: dict = field(default_factory=dict)    # name -> (height, width) array (uint32, float16 or float32)
    attributes: dict = field(default_factory=dict)  # name -> decoded value (or raw bytes for unknown types)


_LINES = {0: 1, 1: 1, 2: 1, 3: 16}  # NONE, RLE, ZIPS, ZIP
_PIXEL = {0: (np.dtype("<u4"), 4), 1: (np.dtype("<f2"), 2), 2: (np.dtype("<f4"), 4)}


def _cstr(b: bytes, at: int):
    end = b.index(b"\0", at)
    return b[at:end].decode("latin-1"), end + 1


def _attr_value(t: str, v: bytes):
    if t == "int":
        return struct.unpack("<i", v)[0]
    if t == "float":
        return struct.unpack("<f", v)[0]
    if t == "string":
        return v.decode("utf-8")
    if t == "v2f":
        return struct.unpack("<2f", v)
    if t == "v3f":
        return struct.unpack("<3f", v)
    if t == "box2i":
        return struct.unpack("<4i", v)
    if t in ("compression", "lineOrder"):
        return v[0]
    if t == "chromaticities":
        return struct.unpack("<8f", v)
    if t == "chlist":
        out, at = [], 0
        while v[at] != 0:
            name, at = _cstr(v, at)
            ptype, _, _, xs, ys = struct.unpack("<iB3sii", v[at:at + 16])
            out.append((name, ptype, xs, ys))
            at += 16
        return out
    return v


def _undo_predictor_and_interleave(t: bytes) -> bytes:
    """OpenEXR's byte predictor (d[i] = d[i-1] + t[i] - 128) and even/odd split, used by RLE and
    ZIP compression."""
    tv = np.frombuffer(t, np.uint8)
    if tv.size == 0:
        return b""
    d = np.empty(tv.size, np.uint8)
    d[0] = tv[0]
    d[1:] = ((np.cumsum(tv[1:].astype(np.int64) - 128) + int(tv[0])) & 0xFF).astype(np.uint8)
    half = (tv.size + 1) // 2
    out = np.empty(tv.size, np.uint8)
    out[0::2] = d[:half]
    out[1::2] = d[half:]
    return out.tobytes()


def _rle_decode(b: bytes) -> bytes:
    out = bytearray()
    i = 0
    while i < len(b):
        c = struct.unpack("b", b[i:i + 1])[0]
        i += 1
        if c < 0:
            out += b[i:i - c]
            i += -c
        else:
            out += bytes([b[i]]) * (c + 1)
            i += 1
    return bytes(out)


def read_exr(path) -> ExrImage:
    """Reads a single-part scanline OpenEXR file."""
    b = open(path, "rb").read()
    magic, version = struct.unpack("<II", b[:8])
    if magic != 20000630:
        raise ValueError(f"{path}: not an OpenEXR file")
    if version & 0x200 or version & 0x800 or version & 0x1000:
        raise ValueError(f"{path}: tiled, deep or multi-part files are not supported")
    at = 8
    attrs = {}
    while b[at] != 0:
        name, at = _cstr(b, at)
        typ, at = _cstr(b, at)
        size = struct.unpack("<i", b[at:at + 4])[0]
        at += 4
        attrs[name] = _attr_value(typ, b[at:at + size])
        at += size
    at += 1
    x0, y0, x1, y1 = attrs["dataWindow"]
    w, h = x1 - x0 + 1, y1 - y0 + 1
    comp = attrs["compression"]
    if comp not in _LINES:
        raise ValueError(f"{path}: compression {comp} is not supported")
    lines = _LINES[comp]
    chunks = (h + lines - 1) // lines
    offsets = struct.unpack(f"<{chunks}Q", b[at:at + 8 * chunks])
    chl = attrs["channels"]
    img = ExrImage(w, h, {name: np.zeros((h, w), _PIXEL[p][0]) for name, p, _, _ in chl}, attrs)
    for off in offsets:
        y, size = struct.unpack("<ii", b[off:off + 8])
        data = b[off + 8:off + 8 + size]
        nl = min(lines, y0 + h - y)
        raw_size = sum(_PIXEL[p][1] for _, p, _, _ in chl) * w * nl
        if comp != 0 and size < raw_size:
            data = _undo_predictor_and_interleave(_rle_decode(data) if comp == 1 else zlib.decompress(data))
        pos = 0
        for ln in range(nl):
            row = y - y0 + ln
            for name, p, _, _ in chl:
                dt, sz = _PIXEL[p]
                img.channels[name][row] = np.frombuffer(data, dt, w, pos)
                pos += w * sz
    return img


def beauty_rec709(img: ExrImage) -> np.ndarray:
    """(height * width, 3) float32 Beauty, converted to linear Rec.709 when the file declares ACEScg
    chromaticities (hdri.rs:61-77)."""
    rgb = np.stack([img.channels[c].astype(np.float32).reshape(-1) for c in "RGB"], axis=1)
    ch = img.attributes.get("chromaticities")
    if ch is not None and abs(ch[0] - 0.713) < 0.01:
        rgb = (rgb @ ACESCG_TO_REC709.T).astype(np.float32)
    return rgb


# ---- exr_diff --------------------------------------------------------------------------------------

def diff(ref: np.ndarray, test: np.ndarray, width: int, height: int, gate_channel: float = 0.01,
         gate_block: float = 0.02) -> dict:
    """exr_diff.rs:40-97 on (pixels, 3) Beauty arrays: worst relative channel-mean error, worst
    relative 4x4 block-mean error (blocks whose larger mean is above 5% of the image mean), MAE over
    the mean, PSNR against the reference's peak; pass = both gates hold."""
    r = np.asarray(ref, np.float32).reshape(height, width, 3).astype(np.float64)
    t = np.asarray(test, np.float32).reshape(height, width, 3).astype(np.float64)
    worst = max(abs(t[..., c].mean() / r[..., c].mean() - 1.0) for c in range(3))
    allm = r.mean()
    n = 4
    bw, bh = width // n, height // n
    worst_block = 0.0
    for by in range(n):
        for bx in range(n):
            a = r[by * bh:(by + 1) * bh, bx * bw:(bx + 1) * bw].mean() if bw and bh else 0.0
            b = t[by * bh:(by + 1) * bh, bx * bw:(bx + 1) * bw].mean() if bw and bh else 0.0
            if max(a, b) > 0.05 * allm:
                worst_block = max(worst_block, abs(b / a - 1.0) if a > 0.0 else math.inf)
    d = (t - r).reshape(-1)
    mae = float(np.abs(d).mean()) / allm
    mse = float((d * d).mean())
    peak = float(r.max())
    psnr = 10.0 * math.log10(peak * peak / mse) if mse > 0 else math.inf
    return {"channel": worst, "block": worst_block, "mae_over_mean": mae, "psnr_db": psnr,
            "pass": bool(worst <= gate_channel and worst_block <= gate_block)}
