"""Synthetic scenes: the small analytic scenes of Verion's GPU tests
(crates/verion-gpu-metal/tests/pathtrace.rs) and the benchmark workloads, generated from seeds.

Workloads (no dataset is involved; every scene is generated here):
* `cornell`: Cornell box of 32 triangles — five walls of a unit box (10), two axis-aligned boxes
  without bottoms (2 x 10) and a light quad of radiance 15 (2); red (0.63, 0.06, 0.05),
  green (0.14, 0.45, 0.09), white 0.73; Lambertian (ior 1, as the reference tests' `material`).
* `many_spheres`: 64 subdivided spheres (octahedron subdivided 31 times: 7688 triangles each) on a
  512 x 512 grid (2 x 511^2 triangles) displaced by seeded value noise: 1,014,274 triangles.
  Materials uniform among GGX conductor (roughness U[0.05, 1]), dielectric (IOR 1.5, smooth) and
  Lambertian; a 2048 x 1024 float HDRI of a sky gradient and a sun disk of peak 1e4.
* `many_lights`: a 317 x 317 floor grid (200,312 triangles) with 120 random boxes and 4096 small
  emissive triangles at uniform random positions, radiance log-uniform in [0.1, 100].
"""
from __future__ import annotations

import math

import numpy as np

from . import scene as sc

GLOBAL_SEED = 0x5EED5EED


def pcg(v: int) -> int:
    """The reference's PCG hash (shaders/include/pt_core.slang:69-74)."""
    v &= 0xFFFFFFFF
    s = (v * 747796405 + 2891336453) & 0xFFFFFFFF
    w = (((s >> ((s >> 28) + 4)) ^ s) * 277803737) & 0xFFFFFFFF
    return ((w >> 22) ^ w) & 0xFFFFFFFF


def config_seed(config_id: int) -> int:
    return pcg(GLOBAL_SEED ^ config_id)


def material(base_color, emission=(0.0, 0.0, 0.0)) -> sc.BaseBsdf:
    """Pure Lambert: ior 1 switches the dielectric specular layer off (pathtrace.rs:21-31)."""
    return sc.BaseBsdf(base_color=tuple(base_color), emission=tuple(emission), ior=1.0)


def cube(half: float) -> sc.Mesh:
    """pathtrace.rs:40-62: axis-aligned cube, 12 triangles."""
    h = half
    pos = [[-h, -h, -h], [h, -h, -h], [h, h, -h], [-h, h, -h], [-h, -h, h], [h, -h, h], [h, h, h], [-h, h, h]]
    idx = [0, 1, 2, 0, 2, 3, 4, 5, 6, 4, 6, 7, 0, 1, 5, 0, 5, 4, 2, 3, 7, 2, 7, 6, 1, 2, 6, 1, 6, 5, 0, 3, 7, 0, 7, 4]
    return sc.Mesh(np.array(pos, np.float32), np.array(idx, np.uint32))


def plane(half: float, z: float) -> sc.Mesh:
    """pathtrace.rs:64-74: square in a z plane."""
    h = half
    return sc.Mesh(np.array([[-h, -h, z], [h, -h, z], [h, h, z], [-h, h, z]], np.float32),
                   np.array([0, 1, 2, 0, 2, 3], np.uint32))


def camera_at_z(z: float) -> sc.Camera:
    t = [list(r) for r in sc.IDENTITY]
    t[2][3] = z
    return sc.Camera(transform=tuple(tuple(r) for r in t))


def look_at(eye, target, up=(0.0, 1.0, 0.0), fov: float = 0.8) -> sc.Camera:
    eye, target, up = (np.asarray(v, np.float64) for v in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, up)
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    # camera-to-world columns: x = right, y = up, z = -forward
    m = np.stack([r, u, -f], axis=1)
    t = tuple(tuple(float(x) for x in list(m[i]) + [eye[i]]) for i in range(3))
    return sc.Camera(transform=t, vertical_fov=fov)


def furnace_room(rho: float, e: float) -> sc.Scene:
    """pathtrace.rs:88-100: camera inside a closed cube whose walls emit e and reflect rho."""
    s = sc.Scene()
    m = s.add_mesh(cube(1.0))
    mat = s.add_material(material([rho] * 3, [e] * 3))
    s.add_instance(sc.Instance(m, mat))
    return s


def white_furnace() -> sc.Scene:
    """pathtrace.rs:117-137: convex albedo-1 cube under a uniform sky of 1."""
    s = sc.Scene()
    m = s.add_mesh(cube(0.5))
    mat = s.add_material(material([1.0] * 3))
    s.add_instance(sc.Instance(m, mat))
    s.add_light(sc.Environment((1.0, 1.0, 1.0)))
    s.camera = camera_at_z(3.0)
    return s


def _quad(p0, p1, p2, p3):
    return [p0, p1, p2, p3], [0, 1, 2, 0, 2, 3]


def _box_no_bottom(lo, hi):
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    pos = [[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0], [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]]
    idx = [4, 5, 6, 4, 6, 7,  # front (+z)
           1, 0, 3, 1, 3, 2,  # back (-z)
           0, 4, 7, 0, 7, 3,  # left (-x)
           5, 1, 2, 5, 2, 6,  # right (+x)
           3, 7, 6, 3, 6, 2]  # top (+y)
    return sc.Mesh(np.array(pos, np.float32), np.array(idx, np.uint32))


def cornell() -> sc.Scene:
    """Cornell box, 32 triangles (see the module docstring)."""
    s = sc.Scene()
    white = s.add_material(material([0.73] * 3))
    red = s.add_material(material([0.63, 0.06, 0.05]))
    green = s.add_material(material([0.14, 0.45, 0.09]))
    light = s.add_material(material([0.78] * 3, [15.0] * 3))

    def add(pos, idx, mat):
        s.add_instance(sc.Instance(s.add_mesh(sc.Mesh(np.array(pos, np.float32), np.array(idx, np.uint32))), mat))

    a = 1.0
    add(*_quad([-a, -a, a], [a, -a, a], [a, -a, -a], [-a, -a, -a]), white)   # floor
    add(*_quad([-a, a, -a], [a, a, -a], [a, a, a], [-a, a, a]), white)       # ceiling
    add(*_quad([-a, -a, -a], [a, -a, -a], [a, a, -a], [-a, a, -a]), white)   # back
    add(*_quad([-a, -a, a], [-a, -a, -a], [-a, a, -a], [-a, a, a]), red)     # left
    add(*_quad([a, -a, -a], [a, -a, a], [a, a, a], [a, a, -a]), green)       # right
    tall = s.add_mesh(_box_no_bottom((-0.65, -1.0, -0.55), (-0.05, 0.2, 0.05)))
    short = s.add_mesh(_box_no_bottom((0.05, -1.0, -0.05), (0.65, -0.4, 0.55)))
    s.add_instance(sc.Instance(tall, white))
    s.add_instance(sc.Instance(short, white))
    q = 0.25
    add(*_quad([-q, 0.999, -q], [q, 0.999, -q], [q, 0.999, q], [-q, 0.999, q]), light)
    s.camera = sc.Camera(transform=((1.0, 0.0, 0.0, 0.0), (0.0, 1.0, 0.0, 0.0), (0.0, 0.0, 1.0, 3.4)),
                         vertical_fov=0.75)
    return s


def octasphere(n: int, radius: float = 1.0):
    """Sphere from an octahedron whose faces are subdivided n times per edge: 8 n^2 triangles,
    vertices projected to the sphere, smooth normals."""
    faces = []
    axes = [np.array(v, np.float64) for v in ([1, 0, 0], [0, 1, 0], [0, 0, 1])]
    verts, index = [], {}

    def vid(p):
        key = tuple(np.round(p, 9))
        if key not in index:
            index[key] = len(verts)
            verts.append(p)
        return index[key]

    for sx in (1, -1):
        for sy in (1, -1):
            for sz in (1, -1):
                a, b, c = axes[0] * sx, axes[1] * sy, axes[2] * sz
                if sx * sy * sz < 0:
                    b, c = c, b
                grid = {}
                for i in range(n + 1):
                    for j in range(n + 1 - i):
                        k = n - i - j
                        p = (a * i + b * j + c * k) / n
                        p = p / np.linalg.norm(p)
                        grid[(i, j)] = vid(p)
                for i in range(n):
                    for j in range(n - i):
                        faces.append((grid[(i, j)], grid[(i + 1, j)], grid[(i, j + 1)]))
                        if i + j + 1 < n:
                            faces.append((grid[(i + 1, j)], grid[(i + 1, j + 1)], grid[(i, j + 1)]))
    v = np.array(verts, np.float64)
    return (v * radius).astype(np.float32), v.astype(np.float32), np.array(faces, np.uint32).reshape(-1)


def _value_noise(rng: np.random.Generator, size: int, cells: int) -> np.ndarray:
    lattice = rng.random((cells + 2, cells + 2))
    t = np.linspace(0.0, cells, size)
    i = np.floor(t).astype(int)
    f = t - i
    f = f * f * (3.0 - 2.0 * f)
    a = lattice[i][:, i]
    b = lattice[i][:, i + 1]
    c = lattice[i + 1][:, i]
    d = lattice[i + 1][:, i + 1]
    fx, fy = f[None, :], f[:, None]
    return (a * (1 - fx) + b * fx) * (1 - fy) + (c * (1 - fx) + d * fx) * fy


def sky_hdri(width: int = 2048, height: int = 1024, sun_peak: float = 1.0e4, seed: int = 0) -> sc.Image:
    """Latitude-longitude sky: a vertical gradient (zenith blue to a bright horizon, dim ground) and
    a sun disk whose centre reaches `sun_peak`."""
    j = (np.arange(height) + 0.5) / height
    theta = j * math.pi
    elev = math.pi / 2 - theta
    zen = np.array([0.15, 0.3, 0.8])
    hor = np.array([0.8, 0.85, 0.95])
    gnd = np.array([0.12, 0.1, 0.08])
    up = np.clip(np.sin(elev), 0.0, 1.0)[:, None]
    sky = np.where(elev[:, None] >= 0.0, hor * (1 - up) + zen * up, gnd)
    img = np.repeat(sky[:, None, :], width, axis=1)
    i = (np.arange(width) + 0.5) / width
    phi = (i - 0.5) * 2.0 * math.pi
    th = theta[:, None]
    d = np.stack([np.sin(th) * np.sin(phi)[None, :], np.cos(th) * np.ones((1, width)),
                  -np.sin(th) * np.cos(phi)[None, :]], axis=-1)
    sun_el, sun_az = math.radians(35.0), math.radians(-40.0)
    s = np.array([math.cos(sun_el) * math.sin(sun_az), math.sin(sun_el), -math.cos(sun_el) * math.cos(sun_az)])
    ang = np.arccos(np.clip(d @ s, -1.0, 1.0))
    radius = math.radians(1.0)
    disk = sun_peak * np.exp(-(ang / radius) ** 2 * 4.0)
    img = img + disk[..., None] * np.array([1.0, 0.95, 0.85])
    return sc.Image(width, height, img.reshape(-1, 3).astype(np.float32))


def many_spheres(seed: int = None, spheres: int = 64, sphere_n: int = 31, grid: int = 512,
                 hdri=(2048, 1024)) -> sc.Scene:
    """The 1M-triangle wavefront workload (see the module docstring)."""
    seed = config_seed(2) if seed is None else seed
    rng = np.random.default_rng(seed)
    s = sc.Scene()
    mats = []
    for k in range(spheres):
        kind = k % 3
        if kind == 0:
            mats.append(s.add_material(sc.BaseBsdf(base_color=tuple(rng.uniform(0.5, 1.0, 3)), metallic=1.0,
                                                   roughness=float(rng.uniform(0.05, 1.0)))))
        elif kind == 1:
            mats.append(s.add_material(sc.BaseBsdf(base_color=(1.0, 1.0, 1.0), transmission=1.0, ior=1.5,
                                                   roughness=0.0)))
        else:
            mats.append(s.add_material(material(tuple(rng.uniform(0.2, 0.9, 3)))))
    ground = s.add_material(material((0.6, 0.58, 0.55)))
    # Ground grid with value-noise displacement.
    half = 12.0
    hgt = 0.6 * (_value_noise(rng, grid, 8) - 0.5) + 0.15 * (_value_noise(rng, grid, 32) - 0.5)
    xs = np.linspace(-half, half, grid)
    gx, gz = np.meshgrid(xs, xs)
    pos = np.stack([gx, hgt, gz], axis=-1).reshape(-1, 3).astype(np.float32)
    ii = np.arange(grid - 1)
    a = (ii[:, None] * grid + ii[None, :]).reshape(-1)
    b, c, d = a + 1, a + grid, a + grid + 1
    idx = np.stack([a, c, b, b, c, d], axis=1).reshape(-1).astype(np.uint32)
    # smooth normals from the height field
    gy, gxd = np.gradient(hgt, xs, xs)
    nrm = np.stack([-gxd, np.ones_like(hgt), -gy], axis=-1)
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    gm = s.add_mesh(sc.Mesh(pos, idx, normals=nrm.reshape(-1, 3).astype(np.float32)))
    s.add_instance(sc.Instance(gm, ground))
    sp, sn, si = octasphere(sphere_n)
    sm = s.add_mesh(sc.Mesh(sp, si, normals=sn))
    placed = []
    while len(placed) < spheres:
        r = float(rng.uniform(0.5, 1.1))
        x, z = rng.uniform(-half * 0.7, half * 0.7, 2)
        if any((x - px) ** 2 + (z - pz) ** 2 < (r + pr) ** 2 for px, pz, pr in placed):
            continue
        gi = int((z + half) / (2 * half) * (grid - 1))
        gj = int((x + half) / (2 * half) * (grid - 1))
        y = float(hgt[gi, gj]) + r
        placed.append((x, z, r))
        t = ((r, 0.0, 0.0, float(x)), (0.0, r, 0.0, y), (0.0, 0.0, r, float(z)))
        s.add_instance(sc.Instance(sm, mats[len(placed) - 1], t))
    if hdri:
        img = s.add_image(sky_hdri(hdri[0], hdri[1]))
        s.add_light(sc.EnvironmentMap(img, 1.0))
    s.camera = look_at((0.0, 5.5, 15.0), (0.0, 0.3, 0.0), fov=0.75)
    return s


def many_lights(seed: int = None, floor: int = 317, boxes: int = 120, emitters: int = 4096) -> sc.Scene:
    """The many-light ReSTIR workload: a floor grid of 2 x (floor - 1)^2 triangles (200k at 317) with
    random boxes standing on it, and `emitters` small emissive triangles at uniform random positions
    above it, radiance log-uniform in [0.1, 100]. Seeded from config 3."""
    seed = config_seed(3) if seed is None else seed
    rng = np.random.default_rng(seed)
    s = sc.Scene()
    half = 10.0
    xs = np.linspace(-half, half, floor)
    gx, gz = np.meshgrid(xs, xs)
    pos = np.stack([gx, np.zeros_like(gx), gz], axis=-1).reshape(-1, 3).astype(np.float32)
    ii = np.arange(floor - 1)
    a = (ii[:, None] * floor + ii[None, :]).reshape(-1)
    idx = np.stack([a, a + floor, a + 1, a + 1, a + floor, a + floor + 1], axis=1).reshape(-1).astype(np.uint32)
    ground = s.add_mesh(sc.Mesh(pos, idx))
    s.add_instance(sc.Instance(ground, s.add_material(material((0.7, 0.7, 0.7)))))
    box = s.add_mesh(cube(0.5))
    for _ in range(boxes):
        sx, sy, sz = rng.uniform(0.2, 1.2, 3)
        x, z = rng.uniform(-half * 0.9, half * 0.9, 2)
        m = s.add_material(material(tuple(rng.uniform(0.2, 0.9, 3))))
        s.add_instance(sc.Instance(box, m, ((sx, 0, 0, x), (0, sy, 0, sy * 0.5), (0, 0, sz, z))))
    tri = np.array([[-0.05, 0.0, -0.05], [0.05, 0.0, -0.05], [0.0, 0.0, 0.05]], np.float32)
    pos, idx, mats = [], [], []
    lights = s.add_mesh(sc.Mesh(tri, np.array([0, 1, 2], np.uint32)))
    for _ in range(emitters):
        p = rng.uniform((-half, 0.2, -half), (half, 4.0, half))
        le = float(math.exp(rng.uniform(math.log(0.1), math.log(100.0))))
        m = s.add_material(material((0.0, 0.0, 0.0), (le, le, le)))
        # Face down, tilted at random.
        t = rng.normal(size=3) * 0.3
        s.add_instance(sc.Instance(lights, m, ((1.0, t[0], 0.0, p[0]), (0.0, -1.0, 0.0, p[1]), (0.0, t[1], 1.0, p[2]))))
    s.camera = look_at((0.0, 6.0, 14.0), (0.0, 0.5, 0.0), fov=0.9)
    return s


def scene_triangles(s: sc.Scene) -> int:
    return sum(s.meshes[i.mesh].indices.size // 3 for i in s.instances)
