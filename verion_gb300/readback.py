"""Turns an accumulation's running sums into images: the arithmetic of Verion's
crates/verion-gpu/src/readback.rs, shared by every backend because the sums are plain float arrays.
Also `Adaptive` (crates/verion-gpu/src/lib.rs:110-162) and the lighting split (`LightingAovs`,
lib.rs:183-236)."""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import numpy as np

LIGHTING_STRIDE = 65  # readback.rs:7
SLOT_WORDS = 12       # readback.rs:9
LIGHT_SLOTS = 4       # crates/verion-scene/src/shading.rs


@dataclass(frozen=True)
class Adaptive:
    """lib.rs:110-162: a pixel stops once it has `min_spp` samples and the standard error of its
    luminance mean is at most `threshold` times the mean (floor 0.05)."""
    threshold: float = 0.02
    min_spp: int = 16

    def active(self, n: float, s: float, s2: float) -> bool:
        n, s, s2 = np.float32(n), np.float32(s), np.float32(s2)
        if n < np.float32(self.min_spp):
            return True
        mean = s / n
        var = max(s2 / n - mean * mean, np.float32(0.0)) * n / (n - np.float32(1.0))
        return bool(np.sqrt(np.float32(var / n)) > np.float32(self.threshold) * max(mean, np.float32(0.05)))


@dataclass(frozen=True)
class Restir:
    """lib.rs:119-146"""
    di: bool = True
    gi: bool = False
    candidates: int = 4
    history: int = 4


def inverse_samples(stats: Optional[np.ndarray], pixels: int, samples: int) -> np.ndarray:
    """readback.rs:18-31"""
    if stats is not None:
        return (np.float32(1.0) / np.maximum(stats.reshape(-1, 3)[:, 0], np.float32(1.0))).astype(np.float32)
    return np.full(pixels, np.float32(1.0) / np.float32(max(samples, 1)), np.float32)


def mean(sums: np.ndarray, inverse: np.ndarray) -> np.ndarray:
    """readback.rs:34-40: (pixels, 3) means."""
    return (sums.reshape(-1, 3).astype(np.float32) * inverse[:, None]).astype(np.float32)


def sample_counts(stats: np.ndarray) -> np.ndarray:
    """readback.rs:43-50"""
    return stats.reshape(-1, 3)[:, 0].astype(np.uint32)


def active_pixels(stats: Optional[np.ndarray], adaptive: Optional[Adaptive], pixels: int) -> int:
    """readback.rs:53-62"""
    if stats is None or adaptive is None:
        return pixels
    return sum(1 for r in stats.reshape(-1, 3) if adaptive.active(r[0], r[1], r[2]))


@dataclass
class LightingAovs:
    direct_diffuse: np.ndarray
    indirect_diffuse: np.ndarray
    specular: np.ndarray
    transmission: np.ndarray
    emission: np.ndarray
    visibility: np.ndarray
    light_u: np.ndarray         # (pixels, 4, 3)
    light_response: np.ndarray  # (pixels, 4)
    light_s: np.ndarray         # (pixels, 4, 3)
    light_dir: np.ndarray       # (pixels, 4, 3)
    light_lit: np.ndarray       # (pixels, 4)


def lighting(data: np.ndarray, inverse: np.ndarray) -> LightingAovs:
    """readback.rs:65-137"""
    r = data.reshape(-1, LIGHTING_STRIDE).astype(np.float32)
    inv = inverse[:, None]
    part = lambda k: (r[:, 3 * k:3 * k + 3] * inv).astype(np.float32)
    slots = r[:, 17:].reshape(-1, LIGHT_SLOTS, SLOT_WORDS)
    w = slots[:, :, 3] + np.float32(0.2126) * slots[:, :, 5] + np.float32(0.7152) * slots[:, :, 6] + \
        np.float32(0.0722) * slots[:, :, 7]
    with np.errstate(divide="ignore", invalid="ignore"):
        response = np.where(slots[:, :, 3] > 0, slots[:, :, 4] / slots[:, :, 3], 0.0).astype(np.float32)
        ldir = np.where(w[:, :, None] > 0, slots[:, :, 8:11] / w[:, :, None], 0.0).astype(np.float32)
        lit = np.where(w > 0, slots[:, :, 11] / w, 0.0).astype(np.float32)
        vis = np.where(r[:, 16] > 0, r[:, 15] / r[:, 16], 1.0).astype(np.float32)
    return LightingAovs(part(0), part(1), part(2), part(3), part(4), vis,
                        (slots[:, :, 0:3] * inv[:, :, None]).astype(np.float32), response,
                        (slots[:, :, 5:8] * inv[:, :, None]).astype(np.float32), ldir, lit)
