"""Generates the three directional-albedo tables the BSDF reads after the light table.

The tables are data of Verion's packer (crates/verion-gpu/tables/*.f32, embedded by
crates/verion-gpu/src/pack.rs:20-27 and read by `ggxAlbedo`, `sheenAlbedo` and `dielectricAlbedo`
in shaders/include/pt_core.slang:384-445). This script restates the integrals they hold, with the
same quadrature nodes and the same rounding of the stored values, vectorised with numpy:

* ggx_albedo.f32 (32 x 32, [r][mu], alpha = r^2): single-scattering GGX albedo for F = 1 with
  separable Smith G, integrated over the GGX half-vector distribution on a 256 x 256 midpoint grid
  (u uniform in the half-vector CDF, phi uniform); rounded to 6 decimals.
* sheen_albedo.f32 (16 x 16, [r][mu], r >= 0.07): albedo of the Charlie sheen lobe with the
  Neubelt visibility, midpoint rule over 1024 polar x 64 azimuth cells; 6 decimals.
* dielectric_albedo.f32 (2 x 9 x 16 x 16, [side][ior][r][mu]): rough dielectric interface,
  mean over a 96 x 96 stratified grid of visible-normal samples (Heitz 2018) of
  F G1(reflected) + (1 - F) G1(transmitted); 5 decimals.

Usage: python -m verion_gb300.tables.gen_albedo [OUT_DIR]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def _g1(c, a):
    return 2.0 / (1.0 + np.sqrt(1.0 + a * a * (1.0 - c * c) / (c * c)))


def ggx_table(n: int = 32, cells: int = 256) -> np.ndarray:
    out = np.empty((n, n))
    u = (np.arange(cells) + 0.5) / cells
    phi = (np.arange(cells) + 0.5) / cells * (2.0 * np.pi)
    for r in range(n):
        a = (r / (n - 1)) ** 2
        for m in range(n):
            mu = max(m / (n - 1), 0.01)
            if a == 0.0:
                out[r, m] = 1.0
                continue
            wo = np.array([np.sqrt(1.0 - mu * mu), 0.0, mu])
            tan2 = a * a * u / (1.0 - u)
            cos_h = 1.0 / np.sqrt(1.0 + tan2)
            sin_h = np.sqrt(1.0 - cos_h * cos_h)
            hx = sin_h[:, None] * np.cos(phi)[None, :]
            hy = sin_h[:, None] * np.sin(phi)[None, :]
            hz = np.broadcast_to(cos_h[:, None], hx.shape)
            woh = wo[0] * hx + wo[1] * hy + wo[2] * hz
            wiz = 2.0 * woh * hz - wo[2]
            ok = (woh > 0.0) & (wiz > 0.0)
            with np.errstate(divide="ignore", invalid="ignore"):
                val = _g1(mu, a) * woh / (mu * hz) * _g1(np.where(ok, wiz, 1.0), a)
            # Row-major accumulation order of the original double loop.
            total = 0.0
            for row in np.where(ok, val, 0.0):
                for v in row:
                    total += v
            out[r, m] = min(total / (cells * cells), 1.0)
    return out


def sheen_table(n: int = 16, nu: int = 1024, nphi: int = 64) -> np.ndarray:
    out = np.empty((n, n))
    theta = (np.arange(nu) + 0.5) / nu * (np.pi / 2)
    ci, si = np.cos(theta), np.sin(theta)
    phi = (np.arange(nphi) + 0.5) / nphi * (2.0 * np.pi)
    for r_i in range(n):
        r = max(r_i / (n - 1), 0.07)
        a = r * r
        for m in range(n):
            mu = max(m / (n - 1), 0.01)
            wo = (np.sqrt(1.0 - mu * mu), 0.0, mu)
            wix = si[:, None] * np.cos(phi)[None, :]
            wiy = si[:, None] * np.sin(phi)[None, :]
            wiz = np.broadcast_to(ci[:, None], wix.shape)
            hx, hy, hz = wo[0] + wix, wo[1] + wiy, wo[2] + wiz
            nrm = np.sqrt(hx * hx + hy * hy + hz * hz)
            hzn = hz / nrm
            sin_h = np.sqrt(np.maximum(1.0 - hzn * hzn, 0.0))
            d = (2.0 + 1.0 / a) * sin_h ** (1.0 / a) / (2.0 * np.pi)
            v = 1.0 / (4.0 * (wiz + mu - wiz * mu))
            val = d * v * wiz * si[:, None]
            total = 0.0
            for row in val:
                for x in row:
                    total += x
            out[r_i, m] = min(total * (np.pi / 2 / nu) * (2.0 * np.pi / nphi), 1.0)
    return out


def _fresnel(cosi, eta):
    s2 = (1.0 - cosi * cosi) / (eta * eta)
    cost = np.sqrt(np.maximum(1.0 - s2, 0.0))
    rs = (cosi - eta * cost) / (cosi + eta * cost)
    rp = (eta * cosi - cost) / (eta * cosi + cost)
    return np.where(s2 >= 1.0, 1.0, 0.5 * (rs * rs + rp * rp))


def _vndf(wo, alpha, u1, u2):
    vh = np.array([alpha * wo[0], alpha * wo[1], wo[2]])
    vh = vh / np.sqrt((vh * vh).sum())
    lensq = vh[0] ** 2 + vh[1] ** 2
    if lensq > 0.0:
        k = 1.0 / np.sqrt(lensq)
        t1 = np.array([-vh[1] * k, vh[0] * k, 0.0])
    else:
        t1 = np.array([1.0, 0.0, 0.0])
    t2 = np.cross(vh, t1)
    r = np.sqrt(u1)
    phi = 2.0 * np.pi * u2
    a, b = r * np.cos(phi), r * np.sin(phi)
    s = 0.5 * (1.0 + vh[2])
    b = (1.0 - s) * np.sqrt(1.0 - a * a) + s * b
    c = np.sqrt(np.maximum(0.0, 1.0 - a * a - b * b))
    nh = [a * t1[i] + b * t2[i] + c * vh[i] for i in range(3)]
    x, y, z = alpha * nh[0], alpha * nh[1], np.maximum(0.0, nh[2])
    nn = np.sqrt(x * x + y * y + z * z)
    return x / nn, y / nn, z / nn


def dielectric_table(n: int = 16, n_ior: int = 9, ns: int = 96) -> np.ndarray:
    out = np.empty((2, n_ior, n, n))
    g = (np.arange(ns) + 0.5) / ns
    u1 = np.repeat(g, ns)
    u2 = np.tile(g, ns)
    for side in range(2):
        for i_ior in range(n_ior):
            ior = 1.0 + 0.25 * i_ior
            eta = ior if side == 0 else 1.0 / ior
            for i_r in range(n):
                alpha = max((i_r / (n - 1)) ** 2, 1.0e-3)
                for i_mu in range(n):
                    mu = max(i_mu / (n - 1), 0.01)
                    wo = (np.sqrt(1.0 - mu * mu), 0.0, mu)
                    hx, hy, hz = _vndf(wo, alpha, u1, u2)
                    woh = wo[0] * hx + wo[1] * hy + wo[2] * hz
                    f = _fresnel(woh, eta)
                    wiz = 2.0 * woh * hz - wo[2]
                    refl = np.where(wiz > 0.0, f * _g1(np.where(wiz > 0.0, wiz, 1.0), alpha), 0.0)
                    r = 1.0 / eta
                    k = 1.0 - r * r * (1.0 - woh * woh)
                    cc = r * woh - np.sqrt(np.maximum(k, 0.0))
                    wtz = -wo[2] * r + cc * hz
                    tok = (k > 0.0) & (wtz < 0.0)
                    trans = np.where(tok, (1.0 - f) * _g1(np.where(tok, -wtz, 1.0), alpha), 0.0)
                    total = 0.0
                    for a_, b_ in zip(refl, trans):
                        total += a_
                        total += b_
                    out[side, i_ior, i_r, i_mu] = min(total / (ns * ns), 1.0)
    return out


def _rounded(values: np.ndarray, decimals: int) -> np.ndarray:
    return np.array([float(f"{v:.{decimals}f}") for v in values.ravel()], dtype="<f4")


def generate(out_dir: Path = HERE) -> dict[str, Path]:
    out_dir.mkdir(parents=True, exist_ok=True)
    files = {
        "ggx_albedo.f32": _rounded(ggx_table(), 6),
        "sheen_albedo.f32": _rounded(sheen_table(), 6),
        "dielectric_albedo.f32": _rounded(dielectric_table(), 5),
    }
    paths = {}
    for name, data in files.items():
        p = out_dir / name
        p.write_bytes(data.tobytes())
        paths[name] = p
    return paths


def load_tables(directory: Path = HERE) -> np.ndarray:
    """The three tables concatenated as the packer appends them (GGX, sheen, dielectric)."""
    parts = [np.fromfile(directory / n, dtype="<f4") for n in ("ggx_albedo.f32", "sheen_albedo.f32",
                                                               "dielectric_albedo.f32")]
    return np.concatenate(parts)


if __name__ == "__main__":
    target = Path(sys.argv[1]) if len(sys.argv) > 1 else HERE
    for k, v in generate(target).items():
        print(k, v)
