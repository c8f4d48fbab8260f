"""Flattens a scene into the tables the kernels read, in the layouts of Verion's host packer
(crates/verion-gpu/src/pack.rs). The CUDA backend receives exactly these tables through
`vg_renderer_create`, as the Rust packer would hand them over.

Arithmetic follows pack.rs: world-space emitter vertices, areas and the selection CDF in single
precision with the reference's summation order, environment CDFs in double precision.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import scene as sc
from .tables.gen_albedo import load_tables

MAX_DEPTH = 8            # pack.rs:13
PARAM_WORDS = 43         # pack.rs:15
MATERIAL_WORDS = 24      # pack.rs:16
LIGHT_WORDS = 16         # pack.rs:17
ALBEDO_WORDS = 1024 + 256 + 4608  # pack.rs:29
EMITTER_WORDS = 16       # pack.rs:31
INSTANCE_WORDS = 16      # pack.rs:33
KIND_VIRTUAL = 3         # pack.rs:488

F32 = np.float32


def _f32(x) -> np.float32:
    return np.float32(x)


def _bits(x) -> int:
    return int(np.array([x], dtype=np.float32).view(np.uint32)[0])


def luminance(c) -> np.float32:
    c = np.asarray(c, dtype=np.float32)
    return F32(0.2126) * c[..., 0] + F32(0.7152) * c[..., 1] + F32(0.0722) * c[..., 2]


@dataclass
class Env:
    pixels: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    marginal: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    conditional: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    width: int = 0
    height: int = 0
    pdf_scale: float = 0.0


@dataclass
class SceneInfo:
    light_count: int
    emitter_count: int
    env_width: int
    env_height: int
    env_pdf_scale: float
    sky: tuple
    virtual_light: bool
    transparent_background: bool


@dataclass
class View:
    camera: np.ndarray  # 16 floats: [2] = tan(fov/2), [4..16] camera-to-world rows
    aperture: float
    focus: float
    shift: tuple

    @staticmethod
    def new(cam: sc.Camera) -> "View":
        c = np.zeros(16, np.float32)
        c[2] = np.float32(math.tan(np.float32(cam.vertical_fov) * np.float32(0.5)))
        c[4:16] = np.asarray(cam.transform, np.float32).reshape(12)
        return View(c, float(cam.aperture_radius), float(cam.focus_distance), tuple(cam.shift))


def camera_record(view: "View", width: int, height: int) -> np.ndarray:
    """pack.rs:97-108: the camera record of the normal and AOV kernels."""
    rec = np.zeros(18, np.float32)
    rec[:16] = view.camera
    rec[0], rec[1] = width, height
    rec[16:] = view.shift
    return rec


@dataclass
class Packed:
    positions: np.ndarray
    indices: np.ndarray
    uvs: np.ndarray
    vnormals: np.ndarray
    instances: np.ndarray
    materials: np.ndarray
    lights: np.ndarray
    emitters: np.ndarray
    emit_cdf: np.ndarray
    env: Env
    texels: np.ndarray
    tex_info: np.ndarray
    meshes: np.ndarray   # (n, 4) uint32: vertex offset, vertex count, index offset, index count
    tlas_mesh: np.ndarray
    tlas_transform: np.ndarray  # (n, 12) float32
    info: SceneInfo
    view: View


def world(t, p: np.ndarray) -> np.ndarray:
    """pack.rs:135-137: rows of the 3x4 transform applied to (n, 3) points in single precision."""
    t = np.asarray(t, np.float32).reshape(3, 4)
    out = np.empty_like(p, dtype=np.float32)
    for r in range(3):
        out[:, r] = ((t[r, 0] * p[:, 0] + t[r, 1] * p[:, 1]) + t[r, 2] * p[:, 2]) + t[r, 3]
    return out


def build_env(s: sc.Scene) -> Env:
    """pack.rs:144-211: sampling tables over luminance * sin(theta)."""
    maps = [l for l in s.lights if isinstance(l, sc.EnvironmentMap)]
    if len(maps) > 1:
        raise ValueError("only one environment map is supported")
    if not maps:
        return Env()
    m = maps[0]
    if not (0 <= m.image < len(s.images)):
        raise ValueError("environment map refers to a missing image")
    img = s.images[m.image]
    w, h = img.width, img.height
    pixels = (img.pixels * np.float32(m.scale)).astype(np.float32)
    lum = luminance(pixels).astype(np.float64).reshape(h, w)
    sin_theta = np.sin((np.arange(h, dtype=np.float64) + 0.5) / h * math.pi)
    weights = lum * sin_theta[:, None]
    running = np.cumsum(weights, axis=1)
    rows = running[:, -1].copy()
    cond = np.empty((h, w), np.float32)
    nz = rows > 0.0
    cond[nz] = (running[nz] / rows[nz, None]).astype(np.float32)
    cond[~nz] = ((np.arange(w) + 1) / np.float32(w)).astype(np.float32)[None, :]
    cond[:, w - 1] = 1.0
    total = float(np.cumsum(rows)[-1])
    if total <= 0.0:
        return Env()
    marginal = np.cumsum(rows / total).astype(np.float32)
    marginal[h - 1] = 1.0
    pdf_scale = float(np.float32((w * h) / (2.0 * math.pi ** 2 * total)))
    return Env(pixels.reshape(-1), marginal, cond.reshape(-1), w, h, pdf_scale)


def mip_chain(img: sc.Image):
    """pack.rs:214-242: box-filtered mip chain, level 0 first."""
    w, h = img.width, img.height
    level = img.pixels.reshape(h, w, 3).astype(np.float32)
    out = []
    levels = 0
    while True:
        out.append(level.reshape(-1))
        levels += 1
        if w == 1 and h == 1:
            return np.concatenate(out).astype(np.float32), levels
        nw, nh = max(w // 2, 1), max(h // 2, 1)
        ys = np.arange(nh)
        xs = np.arange(nw)
        acc = np.zeros((nh, nw, 3), np.float32)
        for dx, dy in ((0, 0), (1, 0), (0, 1), (1, 1)):
            yy = np.minimum(2 * ys + dy, h - 1)
            xx = np.minimum(2 * xs + dx, w - 1)
            acc = acc + level[yy][:, xx]
        level = (acc / np.float32(4.0)).astype(np.float32)
        w, h = nw, nh


def pack_geometry(s: sc.Scene):
    """pack.rs:254-285"""
    pos, idx, uvs, nrm, meshes = [], [], [], [], []
    voff = ioff = 0
    for m in s.meshes:
        n = len(m.positions)
        meshes.append((voff, n, ioff, m.indices.size))
        pos.append(m.positions.reshape(-1))
        uvs.append(m.uvs.reshape(-1) if m.uvs is not None else np.zeros(2 * n, np.float32))
        nrm.append(m.normals.reshape(-1) if m.normals is not None else np.zeros(3 * n, np.float32))
        idx.append(m.indices)
        voff += n
        ioff += m.indices.size
    cat = lambda a, t: np.concatenate(a).astype(t) if a else np.zeros(0, t)
    return (cat(pos, np.float32), cat(idx, np.uint32), cat(uvs, np.float32), cat(nrm, np.float32),
            np.array(meshes, np.uint32).reshape(-1, 4))


def pack_emitters(s: sc.Scene):
    """pack.rs:302-355: emissive world-space triangles, power-proportional selection CDF."""
    words, powers, bases = [], [], []
    count = 0
    for i, inst in enumerate(s.instances):
        b = s.materials[inst.material]
        le = np.asarray(b.emission, np.float32)
        radiance = (le[0] + le[1]) + le[2]
        if radiance <= 0.0 or b.emission_texture is not None:
            bases.append(0)
            continue
        mesh = s.meshes[inst.mesh]
        bases.append(count + 1)
        tri = mesh.indices.reshape(-1, 3)
        a = world(inst.transform, mesh.positions[tri[:, 0]])
        bb = world(inst.transform, mesh.positions[tri[:, 1]])
        c = world(inst.transform, mesh.positions[tri[:, 2]])
        e1 = bb - a
        e2 = c - a
        cr = np.stack([e1[:, 1] * e2[:, 2] - e1[:, 2] * e2[:, 1],
                       e1[:, 2] * e2[:, 0] - e1[:, 0] * e2[:, 2],
                       e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]], axis=1).astype(np.float32)
        area = (np.float32(0.5) * np.sqrt((cr[:, 0] * cr[:, 0] + cr[:, 1] * cr[:, 1]) + cr[:, 2] * cr[:, 2])).astype(np.float32)
        powers.append((area * radiance).astype(np.float32))
        rec = np.zeros((len(tri), EMITTER_WORDS), np.float32)
        rec[:, 0:3], rec[:, 3:6], rec[:, 6:9] = a, bb, c
        rec[:, 9:12] = le
        rec[:, 12] = area
        rec[:, 14] = np.array([s.instance_emit_mask(i)], np.uint32).view(np.float32)[0]
        words.append(rec)
        count += len(tri)
    if not words:
        return np.zeros(0, np.float32), np.zeros(0, np.float32), np.array(bases, np.uint32)
    rec = np.concatenate(words)
    p = np.concatenate(powers)
    total = np.float32(0.0)
    for v in p:  # sequential single-precision sum, as iter().sum()
        total = np.float32(total + v)
    sel = (p / total).astype(np.float32)
    rec[:, 13] = sel
    cdf = np.empty(len(p), np.float32)
    running = np.float32(0.0)
    for k, v in enumerate(sel):
        running = np.float32(running + v)
        cdf[k] = running
    cdf[-1] = 1.0
    return rec.reshape(-1), cdf, np.array(bases, np.uint32)


def pack_instances(s: sc.Scene, meshes: np.ndarray, bases: np.ndarray):
    """pack.rs:358-381"""
    n = len(s.instances)
    table = np.zeros((n, INSTANCE_WORDS), np.uint32)
    tmesh = np.zeros(n, np.uint32)
    tform = np.zeros((n, 12), np.float32)
    for i, inst in enumerate(s.instances):
        r = meshes[inst.mesh]
        table[i, 0] = r[0]
        table[i, 1] = r[2]
        table[i, 2] = inst.material
        table[i, 3] = bases[i]
        t = np.asarray(inst.transform, np.float32).reshape(12)
        table[i, 4:16] = t.view(np.uint32)
        tmesh[i] = inst.mesh
        tform[i] = t
    return table.reshape(-1), tmesh, tform


def pack_materials(s: sc.Scene):
    """pack.rs:395-467: material records (24 words) and mip-mapped textures."""
    slot_of, texels, tex_info = {}, [], []
    ntex = [0]

    def texture(img):
        if img is None:
            return 0.0
        if img not in slot_of:
            if not (0 <= img < len(s.images)):
                raise ValueError("material refers to a missing image")
            chain, levels = mip_chain(s.images[img])
            offset = sum(t.size for t in texels) // 3
            tex_info.extend([offset, s.images[img].width, s.images[img].height, levels])
            texels.append(chain)
            slot_of[img] = len(slot_of)
        return float(slot_of[img] + 1)

    mats = []
    for b in s.materials:
        tex = [texture(b.base_color_texture), texture(b.metallic_roughness_texture), texture(b.emission_texture)]
        nt = texture(b.normal_texture)
        ot = texture(b.opacity_texture)
        mats.append([*b.base_color, *b.emission, b.metallic, b.roughness, b.transmission, b.ior, *tex, nt,
                     b.normal_scale, b.clearcoat, b.clearcoat_roughness, b.sheen_roughness, *b.sheen_color,
                     b.dispersion, b.opacity, ot])
    m = np.array(mats, np.float32).reshape(-1)
    tx = np.concatenate(texels).astype(np.float32) if texels else np.zeros(0, np.float32)
    return m, tx, np.array(tex_info, np.uint32)


def virtual_light(s: sc.Scene):
    """pack.rs:494-588: direction toward the brightest part of the environment map and the
    irradiance it delivers, or None."""
    world_ = s.stylization_world
    if not world_.virtual_light:
        return None
    maps = [l for l in s.lights if isinstance(l, sc.EnvironmentMap)]
    if not maps or not (0 <= maps[0].image < len(s.images)):
        return None
    img = s.images[maps[0].image]
    w, h = img.width, img.height
    pi = np.float32(math.pi)
    rgb = (img.pixels * np.float32(maps[0].scale)).astype(np.float32).reshape(h, w, 3)
    j = np.arange(h, dtype=np.float32)[:, None]
    i = np.arange(w, dtype=np.float32)[None, :]
    theta = ((j + np.float32(0.5)) / np.float32(h) * pi) * np.ones_like(i)
    phi = (((i + np.float32(0.5)) / np.float32(w) - np.float32(0.5)) * np.float32(2.0) * pi) * np.ones_like(j)
    st = np.sin(theta).astype(np.float32)
    omega = (np.float32(2.0) * pi * pi / np.float32(w * h) * st).astype(np.float32)
    d = np.stack([st * np.sin(phi), np.cos(theta), -st * np.cos(phi)], axis=-1).astype(np.float32)
    lums = luminance(rgb).astype(np.float32)
    total = float((lums.astype(np.float64) * omega.astype(np.float64)).sum())
    area = float(omega.astype(np.float64).sum())
    mean = total / area
    flat = lums.reshape(-1)
    cut = max(flat.size // 100, 1)
    threshold = np.partition(-flat, cut - 1)[cut - 1] * -1
    sel = (lums >= threshold) & (lums.astype(np.float64) > mean)
    e = (lums * omega).astype(np.float64)[sel]
    energy = float(e.sum())
    if energy <= 0.0:
        return None
    solid = float(omega.astype(np.float64)[sel].sum())
    dvec = (e[:, None] * d[sel].astype(np.float64)).sum(axis=0)
    length = math.sqrt(float((dvec * dvec).sum())) / energy
    cluster_mean = energy / solid
    auto = length >= 0.5 and cluster_mean >= 1.5 * mean
    if world_.direction is not None:
        dd = np.asarray(world_.direction, np.float32)
        n = float(np.sqrt((dd * dd).sum()))
        if n <= 0.0:
            return None
        toward = (dd / np.float32(n)).astype(np.float32)
    elif auto:
        toward = (dvec / (length * energy)).astype(np.float32)
    else:
        return None
    cos = np.maximum((d * toward[None, None, :]).sum(axis=-1).astype(np.float64), 0.0)
    irr = ((rgb * omega[..., None]).astype(np.float64) * cos[..., None]).reshape(-1, 3).sum(axis=0)
    irr = (irr.astype(np.float32) * np.float32(world_.strength)).astype(np.float32)
    return toward, irr


def pack_lights(s: sc.Scene):
    """pack.rs:590-693: delta lights (16 words), slot ranking, the virtual main light, the albedo
    tables, the light-link masks per instance, then the IES profiles."""
    sky = np.zeros(3, np.float32)
    recs, strengths, profiles = [], [], []
    for k, l in enumerate(s.lights):
        cone = [0.0, 0.0, 0.0, 0.0]
        offset = 0.0
        if isinstance(l, sc.Point):
            kind, color, intensity, vec = 0, l.color, l.intensity, l.position
        elif isinstance(l, sc.Directional):
            kind, color, intensity, vec = 1, l.color, l.intensity, l.direction
        elif isinstance(l, sc.Spot):
            d = np.asarray(l.direction, np.float32)
            ln = np.float32(np.sqrt((d * d).sum()))
            axis = (d / ln).astype(np.float32)
            scale = np.float32(1.0) / max(np.float32(math.cos(l.inner_cone)) - np.float32(math.cos(l.outer_cone)),
                                          np.float32(1.0e-3))
            cone = [axis[0], axis[1], axis[2], scale]
            offset = -np.float32(math.cos(l.outer_cone)) * scale
            kind, color, intensity, vec = 2, l.color, l.intensity, l.position
        elif isinstance(l, sc.EnvironmentMap):
            continue
        elif isinstance(l, sc.Environment):
            sky = (sky + np.asarray(l.color, np.float32)).astype(np.float32)
            continue
        else:
            raise TypeError(f"unknown light {l!r}")
        extra = s.light_extra(k)
        if extra.ies is not None and kind != 1:
            profiles.append((len(recs), extra.ies))
        w = np.zeros(LIGHT_WORDS, np.uint32)
        w[0] = kind
        w[1:4] = np.asarray(color, np.float32).view(np.uint32)
        w[4] = _bits(intensity)
        w[5:8] = np.asarray(vec, np.float32).view(np.uint32)
        w[8:12] = np.asarray(cone, np.float32).view(np.uint32)
        w[12] = _bits(offset)
        w[14] = extra.link_mask & 0xFFFFFFFF
        recs.append(w)
        strengths.append(float(luminance(np.asarray(color, np.float32)) * np.float32(intensity)))
    ranked = sorted(range(len(strengths)), key=lambda i: -strengths[i])
    for rank, i in enumerate(ranked):
        recs[i][13] = min(rank, 2)
    vl = virtual_light(s)
    if vl is not None:
        toward, irr = vl
        w = np.zeros(LIGHT_WORDS, np.uint32)
        w[0] = KIND_VIRTUAL
        w[1:4] = irr.astype(np.float32).view(np.uint32)
        w[4] = _bits(1.0)
        w[5:8] = (-toward).astype(np.float32).view(np.uint32)
        w[13] = 3
        w[14] = 0xFFFFFFFF
        recs.append(w)
    count = len(recs)
    parts = [np.concatenate(recs) if recs else np.zeros(0, np.uint32), load_tables().view(np.uint32)]
    masks = np.zeros(2 * len(s.instances), np.uint32)
    for i in range(len(s.instances)):
        masks[2 * i] = s.instance_light_mask(i)
        masks[2 * i + 1] = s.instance_emit_mask(i)
    parts.append(masks)
    lights = np.concatenate(parts).astype(np.uint32)
    for li, (profile, axes) in profiles:
        lights[li * LIGHT_WORDS + 15] = lights.size + 1
        extra_words = np.concatenate([np.asarray(axes, np.float32).reshape(9), profile.table]).view(np.uint32)
        lights = np.concatenate([lights, extra_words]).astype(np.uint32)
    return lights, count, tuple(float(x) for x in sky), vl is not None


def pack(s: sc.Scene) -> Packed:
    """pack.rs:726-756"""
    if not s.instances:
        raise ValueError("scene has no instances")
    pos, idx, uvs, nrm, meshes = pack_geometry(s)
    ew, cdf, bases = pack_emitters(s)
    inst, tmesh, tform = pack_instances(s, meshes, bases)
    mats, texels, tex_info = pack_materials(s)
    lights, count, sky, vl = pack_lights(s)
    env = build_env(s)
    info = SceneInfo(count, int(cdf.size), env.width, env.height, env.pdf_scale, sky, vl, s.transparent_background)
    return Packed(pos, idx, uvs, nrm, inst, mats, lights, ew, cdf, env, texels, tex_info, meshes, tmesh, tform,
                  info, View.new(s.camera))


@dataclass
class UpdatePlan:
    """pack.rs:758-784: what a batch of scene edits makes a backend redo."""
    full: bool = False
    materials: bool = False
    lights: bool = False
    emitters: bool = False
    instances: bool = False
    vertices: bool = False
    blases: tuple = ()
    tlas: bool = False
    camera: bool = False

    @staticmethod
    def new(camera: bool = False, lights: bool = False, materials=(), instances=(), deformed=(),
            geometry: bool = False) -> "UpdatePlan":
        """pack.rs:786-823 (`UpdatePlan::new` over `verion_scene::Changes`): `materials`,
        `instances` and `deformed` are the edited material, instance and mesh indices."""
        p = UpdatePlan(camera=camera, lights=lights)
        if geometry:
            return UpdatePlan(True, True, True, True, True, True, (), True, camera)
        if materials:
            p.materials = True
            p.emitters = True
        if instances:
            p.instances = True
            p.tlas = True
            p.emitters = True
        if deformed:
            p.vertices = True
            p.blases = tuple(int(m) for m in deformed)
            p.tlas = True
            p.emitters = True
        # Emitters carry the instance table's emitter bases.
        p.instances |= p.emitters
        return p

    def is_empty(self) -> bool:
        return self == UpdatePlan()


def base_params(info: SceneInfo, view: View, size, lighting: bool, multiscatter: bool, adaptive=None,
                restir=None, max_depth: int = MAX_DEPTH) -> np.ndarray:
    """pack.rs:828-874: the parameter block with the per-dispatch words (6, 30, 31, 35) zero."""
    w, h = size
    p = np.zeros(PARAM_WORDS, np.uint32)
    p[0], p[1] = w, h
    p[2] = _bits(view.camera[2])
    p[3] = _bits(view.aperture)
    p[4] = _bits(view.focus)
    p[5] = info.light_count
    p[7] = max_depth
    p[8:20] = np.asarray(view.camera[4:16], np.float32).view(np.uint32)
    p[20:23] = np.asarray(info.sky, np.float32).view(np.uint32)
    p[23] = info.emitter_count
    p[24], p[25] = info.env_width, info.env_height
    p[26] = _bits(info.env_pdf_scale)
    p[27] = _bits(np.float32(2.0) * np.float32(view.camera[2]) / np.float32(h))
    p[41] = int(info.virtual_light)
    p[42] = int(info.transparent_background)
    p[39] = _bits(view.shift[0])
    p[40] = _bits(view.shift[1])
    p[28] = int(lighting)
    p[29] = int(multiscatter)
    if adaptive is not None:
        p[32] = 1
        p[33] = _bits(adaptive.threshold)
        p[34] = adaptive.min_spp
    if restir is not None:
        p[36] = int(restir.di) | (int(restir.gi) << 1)
        p[37] = restir.candidates
        p[38] = restir.history
    return p
