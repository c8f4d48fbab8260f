"""Scenes with known answers, ported from Verion's GPU tests
(crates/verion-gpu-metal/tests/pathtrace.rs); shared by the oracle tests and the GPU tests."""
import math

import numpy as np

from verion_gb300 import scene as sc
from verion_gb300 import scenes

IDENTITY = sc.IDENTITY


def up(z):
    return ((1.0, 0.0, 0.0, 0.0), (0.0, 1.0, 0.0, 0.0), (0.0, 0.0, 1.0, z))


def floor_scene(light, occluder: bool) -> sc.Scene:
    """pathtrace.rs:233-264: albedo-1 floor lit by one light, seen from z = 3."""
    s = sc.Scene()
    f = s.add_mesh(scenes.plane(5.0, 0.0))
    m = s.add_material(scenes.material((1.0, 1.0, 1.0)))
    s.add_instance(sc.Instance(f, m))
    if occluder:
        tri = sc.Mesh(np.array([[0.4, -0.3, 0.5], [0.6, -0.3, 0.5], [0.5, 0.3, 0.5]], np.float32), np.array([0, 1, 2]))
        t = s.add_mesh(tri)
        black = s.add_material(scenes.material((0.0, 0.0, 0.0)))
        s.add_instance(sc.Instance(t, black))
    s.add_light(light)
    s.camera = scenes.camera_at_z(3.0)
    return s


def point_light():
    """pathtrace.rs:275-289: L = rho/pi I cos / d^2 = 1 at the origin."""
    return sc.Point((1.0, 0.0, 1.0), (1.0, 1.0, 1.0), math.pi * 2.0 * math.sqrt(2.0))


def spot_at(off: float):
    """pathtrace.rs:292-304"""
    a = math.pi / 4 + off
    return sc.Spot((1.0, 0.0, 1.0), (-3.0 * math.sin(a), 0.0, -3.0 * math.cos(a)), (1.0, 1.0, 1.0),
                   math.pi * 2.0 * math.sqrt(2.0), 0.1, 0.5)


def sky_scene(mesh, material, camera_z: float) -> sc.Scene:
    """pathtrace.rs:547-560: one object under a uniform sky of 1."""
    s = sc.Scene()
    m = s.add_mesh(mesh)
    mat = s.add_material(material)
    s.add_instance(sc.Instance(m, mat))
    s.add_light(sc.Environment((1.0, 1.0, 1.0)))
    s.camera = scenes.camera_at_z(camera_z)
    return s


def floor_with_emitter(floor_material, light_mesh, light_transform, le: float) -> sc.Scene:
    """pathtrace.rs:851-876: floor at z = 0, emitter above, camera at z = 0.5."""
    s = sc.Scene()
    f = s.add_mesh(scenes.plane(25.0, 0.0))
    fm = s.add_material(floor_material)
    s.add_instance(sc.Instance(f, fm))
    l = s.add_mesh(light_mesh)
    lm = s.add_material(scenes.material((0.0, 0.0, 0.0), (le, le, le)))
    s.add_instance(sc.Instance(l, lm, light_transform))
    s.camera = scenes.camera_at_z(0.5)
    return s


def highlight_scene() -> sc.Scene:
    """pathtrace.rs:798-837: rough metal under a point light on the view axis."""
    alpha, d = 0.25, 2.0
    s = sc.Scene()
    f = s.add_mesh(scenes.plane(5.0, 0.0))
    m = s.add_material(sc.BaseBsdf(base_color=(1.0, 1.0, 1.0), metallic=1.0, roughness=0.5))
    s.add_instance(sc.Instance(f, m))
    s.add_light(sc.Point((0.0, 0.0, d), (1.0, 1.0, 1.0), 4.0 * math.pi * alpha * alpha * d * d))
    s.camera = scenes.camera_at_z(3.0)
    return s


def env_furnace() -> sc.Scene:
    """pathtrace.rs:937-962: constant lat-long map around an albedo-1 cube."""
    s = sc.Scene()
    m = s.add_mesh(scenes.cube(0.5))
    mat = s.add_material(scenes.material((1.0, 1.0, 1.0)))
    s.add_instance(sc.Instance(m, mat))
    img = s.add_image(sc.Image(32, 16, np.ones((32 * 16, 3), np.float32)))
    s.add_light(sc.EnvironmentMap(img, 1.0))
    s.camera = scenes.camera_at_z(3.0)
    return s


def metal_plane(roughness: float, cos_o: float) -> sc.Scene:
    """pathtrace.rs:1266-1310: metal plane seen at cos_o under a uniform sky of 1."""
    sin_o = math.sqrt(1.0 - cos_o * cos_o)
    t1, t2, f = (cos_o, 0.0, -sin_o), (0.0, 1.0, 0.0), 5.0

    def p(a, b):
        return [a * t1[k] + b * t2[k] for k in range(3)]

    s = sc.Scene()
    mesh = s.add_mesh(sc.Mesh(np.array([p(-f, -f), p(f, -f), p(f, f), p(-f, f)], np.float32),
                              np.array([0, 1, 2, 0, 2, 3])))
    mat = s.add_material(sc.BaseBsdf(base_color=(1.0, 1.0, 1.0), metallic=1.0, roughness=roughness))
    s.add_instance(sc.Instance(mesh, mat))
    s.add_light(sc.Environment((1.0, 1.0, 1.0)))
    s.camera = scenes.camera_at_z(3.0)
    return s


def ggx_albedo_quadrature(cos_o: float, alpha: float, n: int = 600) -> float:
    """pathtrace.rs:1240-1264: f64 midpoint quadrature of single-scatter GGX albedo (F = 1)."""
    def g1(c):
        return 2.0 / (1.0 + np.sqrt(1.0 + alpha * alpha * (1.0 - c * c) / (c * c)))

    theta = (np.arange(n) + 0.5) / n * (math.pi / 2)
    phi = (np.arange(n) + 0.5) / n * (2 * math.pi)
    st, ct = np.sin(theta)[:, None], np.cos(theta)[:, None]
    wi = np.stack([st * np.cos(phi)[None, :], st * np.sin(phi)[None, :], ct * np.ones((1, n))], axis=-1)
    wo = np.array([math.sqrt(1 - cos_o * cos_o), 0.0, cos_o])
    h = wo + wi
    hz = h[..., 2] / np.linalg.norm(h, axis=-1)
    a2 = alpha * alpha
    d = a2 / (math.pi * (hz * hz * (a2 - 1.0) + 1.0) ** 2)
    val = d * g1(cos_o) * g1(wi[..., 2]) / (4.0 * cos_o) * st
    return float(val.sum() * (math.pi / 2 / n) * (2 * math.pi / n))


def center_mean(img: np.ndarray, w: int, size: int) -> float:
    """pathtrace.rs:536-545 (red channel)."""
    lo = (w - size) // 2
    im = img.reshape(-1, w, 3)
    return float(im[lo:lo + size, lo:lo + size, 0].mean())


def textured_plane(half: float, z: float, repeat: float = 1.0) -> sc.Mesh:
    """A square with uvs spanning [0, repeat] and +z vertex normals."""
    h = half
    pos = np.array([[-h, -h, z], [h, -h, z], [h, h, z], [-h, h, z]], np.float32)
    uv = np.array([[0, 0], [repeat, 0], [repeat, repeat], [0, repeat]], np.float32)
    nrm = np.tile(np.array([[0.0, 0.0, 1.0]], np.float32), (4, 1))
    return sc.Mesh(pos, np.array([0, 1, 2, 0, 2, 3]), normals=nrm, uvs=uv)


def _rot_y(a, s=1.0, t=(0.0, 0.0, 0.0)):
    c, n = math.cos(a) * s, math.sin(a) * s
    return ((c, 0.0, n, t[0]), (0.0, s, 0.0, t[1]), (-n, 0.0, c, t[2]))


def feature_zoo(transparent_background: bool = False) -> sc.Scene:
    """Every shading feature of pt_core.slang in one small scene: textures with mip chains (base
    colour, metallic-roughness, emission, normal map, opacity cut-out), sheen, clearcoat, dispersive
    glass, rough dielectric, IES, spot, point and directional lights, light linking, a uniform sky,
    and rotated / scaled instances with interpolated normals."""
    rng = np.random.default_rng(5)
    s = sc.Scene()
    checker = np.array([[0.9, 0.2, 0.1] if (i // 4 + j // 4) % 2 else [0.1, 0.6, 0.9]
                        for j in range(16) for i in range(16)], np.float32)
    t_base = s.add_image(sc.Image(16, 16, checker))
    t_mr = s.add_image(sc.Image(8, 8, rng.uniform(0.1, 1.0, (64, 3)).astype(np.float32)))
    nm = np.zeros((32 * 32, 3), np.float32)
    for j in range(32):
        for i in range(32):
            nx, ny = 0.4 * math.sin(i * 0.6), 0.4 * math.cos(j * 0.5)
            nm[j * 32 + i] = [0.5 + 0.5 * nx, 0.5 + 0.5 * ny, 0.5 + 0.5 * math.sqrt(max(0.0, 1 - nx * nx - ny * ny))]
    t_nrm = s.add_image(sc.Image(32, 32, nm))
    t_em = s.add_image(sc.Image(4, 4, rng.uniform(0.5, 3.0, (16, 3)).astype(np.float32)))
    t_op = s.add_image(sc.Image(4, 4, np.array([[1.0] * 3, [0.0] * 3, [0.5] * 3, [1.0] * 3] * 4, np.float32)))

    floor = s.add_mesh(textured_plane(4.0, 0.0, repeat=3.0))
    m_floor = s.add_material(sc.BaseBsdf(base_color=(1.0, 1.0, 1.0), roughness=0.6, metallic=0.3,
                                         base_color_texture=t_base, metallic_roughness_texture=t_mr,
                                         normal_texture=t_nrm, normal_scale=0.8))
    s.add_instance(sc.Instance(floor, m_floor, ((1, 0, 0, 0), (0, 0, -1, -0.5), (0, 1, 0, 0))))  # floor at y = -0.5
    sp, sn, si = scenes.octasphere(6)
    ball = s.add_mesh(sc.Mesh(sp, si, normals=sn))
    m_velvet = s.add_material(sc.BaseBsdf(base_color=(0.6, 0.1, 0.3), roughness=0.7, sheen_color=(0.9, 0.8, 0.7),
                                          sheen_roughness=0.4, clearcoat=0.7, clearcoat_roughness=0.2))
    m_prism = s.add_material(sc.BaseBsdf(base_color=(1.0, 1.0, 1.0), transmission=1.0, roughness=0.0, dispersion=3.0))
    m_frost = s.add_material(sc.BaseBsdf(base_color=(0.9, 1.0, 0.9), transmission=1.0, roughness=0.35, ior=1.4))
    m_gold = s.add_material(sc.BaseBsdf(base_color=(1.0, 0.8, 0.4), metallic=1.0, roughness=0.25))
    s.add_instance(sc.Instance(ball, m_velvet, _rot_y(0.4, 0.35, (-0.6, -0.15, 0.2))))
    s.add_instance(sc.Instance(ball, m_prism, _rot_y(1.1, 0.3, (0.3, -0.2, 0.5))))
    s.add_instance(sc.Instance(ball, m_frost, ((0.3, 0.0, 0.0, 0.8), (0.0, 0.2, 0.0, -0.3), (0.0, 0.0, 0.35, -0.3))))
    gold = s.add_instance(sc.Instance(ball, m_gold, _rot_y(-0.3, 0.25, (-0.1, -0.25, -0.6))))
    lamp = s.add_mesh(textured_plane(0.3, 0.0))
    m_lamp = s.add_material(sc.BaseBsdf(base_color=(0.0, 0.0, 0.0), emission=(2.0, 2.0, 2.0), emission_texture=t_em))
    s.add_instance(sc.Instance(lamp, m_lamp, ((1, 0, 0, -1.2), (0, 1, 0, 0.6), (0, 0, 1, -1.5))))
    m_glow = s.add_material(scenes.material((0.2, 0.2, 0.2), (6.0, 5.0, 4.0)))
    s.add_instance(sc.Instance(lamp, m_glow, ((0.5, 0, 0, 0.9), (0, 0, -0.5, 1.4), (0, 0.5, 0, 0.0))))
    cut = s.add_mesh(textured_plane(0.4, 0.0, repeat=2.0))
    m_cut = s.add_material(sc.BaseBsdf(base_color=(0.2, 0.7, 0.2), opacity=0.9, opacity_texture=t_op))
    s.add_instance(sc.Instance(cut, m_cut, _rot_y(0.7, 1.0, (0.2, 0.3, 0.9))))
    ies = sc.IesProfile(np.array([[1.0 + 0.5 * math.cos(math.radians(v)) * (1 + 0.3 * math.sin(math.radians(h)))
                                   for v in range(181)] for h in range(361)], np.float32))
    s.add_light(sc.Point((0.5, 1.2, 0.8), (1.0, 0.9, 0.8), 3.0),
                sc.LightExtra(ies=(ies, ((1.0, 0.0, 0.0), (0.0, 0.0, 1.0), (0.0, -1.0, 0.0)))))
    s.add_light(sc.Spot((-0.8, 1.5, 0.5), (0.5, -1.0, -0.3), (0.6, 0.7, 1.0), 4.0, 0.2, 0.5))
    s.add_light(sc.Directional((0.3, -1.0, -0.5), (1.0, 1.0, 0.9), 1.5), sc.LightExtra(link_mask=0b10))
    s.instance_masks[gold] = 0b01  # the directional light does not reach the gold ball
    s.add_light(sc.Environment((0.1, 0.12, 0.15)))
    s.camera = scenes.look_at((0.0, 0.8, 3.2), (0.0, -0.1, 0.0), fov=0.8)
    s.transparent_background = transparent_background
    return s


def quads(cells) -> sc.Mesh:
    """crates/verion-gpu-vulkan/tests/restir.rs:8-22: squares in z planes, (centre, half size)."""
    p, i = [], []
    for (x, y, z), h in cells:
        b = len(p)
        p += [[x - h, y - h, z], [x + h, y - h, z], [x + h, y + h, z], [x - h, y + h, z]]
        i += [b, b + 1, b + 2, b, b + 2, b + 3]
    return sc.Mesh(np.array(p, np.float32), np.array(i, np.uint32))


def room_with(roughness: float, glass: bool) -> sc.Scene:
    """restir.rs:152-231: a closed room of rough walls lit by 16 small ceiling panels and a rough
    ball, seen from inside (mostly indirect light); with `glass`, a strongly dispersive glass block."""
    s = sc.Scene()
    room = s.add_mesh(scenes.cube(1.5))
    ball = s.add_mesh(scenes.cube(0.4))
    pos, idx = [], []
    for k in range(16):
        gx, gz = float(k % 4), float(k // 4)
        q = quads([([-0.6 + gx * 0.4, -0.6 + gz * 0.4, 0.0], 0.06)])
        b = len(pos)
        pos += [[v[0], 1.45, v[1]] for v in q.positions]
        idx += [int(j) + b for j in q.indices]
    lamps = s.add_mesh(sc.Mesh(np.array(pos, np.float32), np.array(idx, np.uint32)))
    walls = s.add_material(sc.BaseBsdf(base_color=(0.7, 0.65, 0.6), roughness=roughness, ior=1.0))
    glow = s.add_material(sc.BaseBsdf(base_color=(0.0, 0.0, 0.0), emission=(30.0, 30.0, 30.0), roughness=roughness))
    parts = [(room, walls, sc.IDENTITY), (ball, walls, sc.IDENTITY), (lamps, glow, sc.IDENTITY)]
    if glass:
        block = s.add_mesh(scenes.cube(0.35))
        dispersive = s.add_material(sc.BaseBsdf(base_color=(1.0, 1.0, 1.0), transmission=1.0, roughness=0.0, ior=1.6,
                                                dispersion=8.0))
        parts.append((block, dispersive, ((1, 0, 0, -0.7), (0, 1, 0, -0.9), (0, 0, 1, 0.0))))
    for mesh, material, t in parts:
        s.add_instance(sc.Instance(mesh, material, t))
    s.camera = sc.Camera(transform=((1, 0, 0, 0), (0, 1, 0, 0), (0, 0, 1, 1.4)))
    return s


def closed_room(roughness: float) -> sc.Scene:
    """restir.rs:152-157"""
    return room_with(roughness, False)
