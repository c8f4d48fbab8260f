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
