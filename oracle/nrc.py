"""CPU oracle of the radiance cache (test infrastructure only; never product code).

Restates in numpy what the cache kernels compute (verion_gb300/csrc/kern_nrc.cu, layout in
verion_gb300/csrc/nrc.cuh), so tests can check the GPU forward pass, gradients and Adam step.
There is no reference counterpart (the reference has no radiance cache), so parity here is the
oracle's own: the encoding is computed in float32 with the kernels' operation order (so network
inputs agree bit for bit), the MLP in float64 with bf16 rounding at the points where the kernels
round (weights, hidden activations, back-propagated gradients), and Adam in float32 with the
kernel's operation order. Methods restated: multi-resolution hash encoding (Mueller, Evans,
Schied and Keller 2022), the spatial hash of Teschner et al. 2003, neural radiance caching's
relative L2 loss (Mueller, Rousselle, Novak and Keller 2021), Adam (Kingma and Ba 2015).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

REC = 20
WIDTH = 64
OUT_ROWS = 16
MLP_PARAMS = 4 * WIDTH * WIDTH + OUT_ROWS * WIDTH
P1, P2 = 2654435761, 805459861


def bf16(x) -> np.ndarray:
    """Round to bfloat16 (round to nearest even, through float32), returned as float64."""
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)
    return np.where(np.isfinite(f), out, f).astype(np.float64)


@dataclass
class Grid:
    """The grid geometry of a cache configuration (cache.cu vg_cache_create)."""
    levels: int
    log2_t: int
    res: list
    dense: list
    lo: np.ndarray
    inv_extent: np.float32

    @staticmethod
    def from_config(levels, log2_entries, base_resolution, max_resolution, bounds_lo, bounds_hi) -> "Grid":
        growth = math.exp((math.log(max_resolution) - math.log(base_resolution)) / (levels - 1)) if levels > 1 else 1.0
        t = 1 << log2_entries
        res, dense = [], []
        for l in range(levels):
            r = max(int(math.floor(base_resolution * growth ** l + 1e-9)), 2)
            res.append(r)
            dense.append((r + 1) ** 3 <= t)
        lo = np.asarray(bounds_lo, np.float32)
        ext = np.float32(max(np.float32(bounds_hi[k]) - np.float32(bounds_lo[k]) for k in range(3)))
        return Grid(levels, log2_entries, res, dense, lo, np.float32(1.0) / ext)

    @property
    def entries(self) -> int:
        return 1 << self.log2_t

    def corners(self, pos: np.ndarray, l: int):
        """Entry indices (n, 8) and trilinear weights (n, 8, float32) of level l."""
        x = np.clip((pos.astype(np.float32) - self.lo) * self.inv_extent, np.float32(0), np.float32(1))
        r = self.res[l]
        s = x * np.float32(r)
        i = np.minimum(s.astype(np.uint32), r - 1)
        f = s - i.astype(np.float32)
        one = np.float32(1)
        idx = np.empty((len(pos), 8), np.int64)
        w = np.empty((len(pos), 8), np.float32)
        mask = self.entries - 1
        for k in range(8):
            c = [i[:, a].astype(np.uint64) + ((k >> a) & 1) for a in range(3)]
            if self.dense[l]:
                idx[:, k] = (c[0] + (r + 1) * (c[1] + (r + 1) * c[2])).astype(np.int64)
            else:
                h = (c[0] ^ ((c[1] * P1) & 0xFFFFFFFF) ^ ((c[2] * P2) & 0xFFFFFFFF)) & mask
                idx[:, k] = h.astype(np.int64)
            wx = f[:, 0] if k & 1 else one - f[:, 0]
            wy = f[:, 1] if k & 2 else one - f[:, 1]
            wz = f[:, 2] if k & 4 else one - f[:, 2]
            w[:, k] = (wx * wy) * wz
        return idx, w


def inputs(grid: Grid, table16: np.ndarray, rec: np.ndarray) -> np.ndarray:
    """Network inputs (n, 64) as the kernels form them (float32, before the bf16 rounding).
    table16 is the fp16 grid table, shape (levels, entries, 2)."""
    rec = np.asarray(rec, np.float32)
    n = len(rec)
    v = np.zeros((n, WIDTH), np.float32)
    for l in range(grid.levels):
        idx, w = grid.corners(rec[:, 0:3], l)
        tab = table16[l].astype(np.float32)
        a0 = np.zeros(n, np.float32)
        a1 = np.zeros(n, np.float32)
        for k in range(8):
            a0 = a0 + w[:, k] * tab[idx[:, k], 0]
            a1 = a1 + w[:, k] * tab[idx[:, k], 1]
        v[:, 2 * l] = a0
        v[:, 2 * l + 1] = a1
    v[:, 32:38] = rec[:, 3:9] * np.float32(0.5) + np.float32(0.5)
    v[:, 38:44] = rec[:, 9:15]
    v[:, 44] = 1.0
    return v


def layers(mlp: np.ndarray, rounded: bool = True):
    """The five weight matrices (out x in), bf16-rounded as the kernels use them."""
    mlp = np.asarray(mlp, np.float32)
    ws = [mlp[l * 4096:(l + 1) * 4096].reshape(64, 64) for l in range(4)] + [mlp[16384:].reshape(16, 64)]
    return [bf16(w) if rounded else w.astype(np.float64) for w in ws]


def forward(ws, x, rounded: bool = True):
    """(pre-activations, activations [x, h1..h4], output (n, 16))."""
    rnd = bf16 if rounded else (lambda a: np.asarray(a, np.float64))
    hs = [rnd(x)]
    zs = []
    for l in range(4):
        z = hs[-1] @ ws[l].T
        zs.append(z)
        hs.append(rnd(np.maximum(z, 0.0)))
    return zs, hs, hs[-1] @ ws[4].T


def predict(mlp, grid: Grid, table16, rec) -> np.ndarray:
    _, _, out = forward(layers(mlp), inputs(grid, table16, rec))
    return out[:, :3]


def backward(ws, x, target, rounded: bool = True, valid=None):
    """Loss sum and gradient sums: ([dW0..dW4], d loss / d input (n, 64)), the loss's denominator
    held constant, bf16 rounding where the kernels round."""
    rnd = bf16 if rounded else (lambda a: np.asarray(a, np.float64))
    zs, hs, out = forward(ws, x, rounded)
    p = out[:, :3]
    y = np.asarray(target, np.float64)
    d = p - y
    den = p * p + 0.01
    if valid is None:
        valid = np.ones(len(x), bool)
    loss = float(np.sum((d * d / den)[valid]))
    g = np.zeros((len(x), OUT_ROWS))
    g[:, :3] = np.where(valid[:, None], 2.0 * d / den, 0.0)
    G = rnd(g)
    dws = [None] * 5
    dws[4] = G.T @ hs[4]
    gh = G @ ws[4]
    for l in range(4, 0, -1):
        G = rnd(gh * (zs[l - 1] > 0))
        dws[l - 1] = G.T @ hs[l - 1]
        gh = G @ ws[l - 1]
    return loss, dws, gh


def grid_gradient(grid: Grid, rec, gx) -> np.ndarray:
    """Scatter of the input gradient's grid columns to the table (levels, entries, 2)."""
    out = np.zeros((grid.levels, grid.entries, 2))
    rec = np.asarray(rec, np.float32)
    for l in range(grid.levels):
        idx, w = grid.corners(rec[:, 0:3], l)
        for f in range(2):
            np.add.at(out[l, :, f], idx.ravel(), (w.astype(np.float64) * gx[:, 2 * l + f][:, None]).ravel())
    return out


def flat_mlp(dws) -> np.ndarray:
    return np.concatenate([dw.ravel() for dw in dws])


def adam_f32(p, g_sum, m, v, used, step, lr=0.01, beta1=0.9, beta2=0.99, eps=1e-8):
    """One Adam step in float32 with the kernel's operation order; returns (p, m, v)."""
    f = np.float32
    p, m, v = (np.asarray(a, np.float32).copy() for a in (p, m, v))
    scale = f(1.0) / (f(3.0) * f(used))
    b1, b2 = f(beta1), f(beta2)
    bc1 = f(1.0 - beta1 ** step)
    bc2 = f(1.0 - beta2 ** step)
    gi = np.asarray(g_sum, np.float32) * scale
    m = b1 * m + (f(1) - b1) * gi
    v = b2 * v + (f(1) - b2) * gi * gi
    p = p - f(lr) * (m / bc1) / (np.sqrt(v / bc2) + f(eps))
    return p, m, v


def loss_fixed_den(ws, x, target, den):
    """The relative L2 loss with a given denominator (for finite-difference checks), no rounding."""
    _, _, out = forward(ws, x, rounded=False)
    d = out[:, :3] - np.asarray(target, np.float64)
    return float(np.sum(d * d / den))
