"""The CPU oracle against the reference's known answers (crates/verion-gpu-metal/tests/pathtrace.rs
and trace.rs) and against itself (its BVH against brute force, wavefront against megakernel).
These pin the oracle before it is used to check the CUDA backend."""
import math

import numpy as np
import pytest

import oracle
from verion_gb300 import pack, scenes
from verion_gb300 import scene as sc
from verion_gb300.readback import Adaptive, Restir

from . import analytic as an


def render(s, w, h, spp, *, multiscatter=True, lighting=False, adaptive=None, restir=None, depth=8,
           double=False, wavefront=False, rows=None, acc64=False):
    p = s if isinstance(s, pack.Packed) else pack.pack(s)
    o = oracle.OracleScene(p)
    a = oracle.OracleAccumulation(w, h, lighting=lighting, acc64=acc64, adaptive=adaptive is not None,
                                  restir=restir is not None)
    prm = pack.base_params(p.info, p.view, (w, h), lighting, multiscatter, adaptive, restir, depth)
    oracle.render(o, prm, a, spp, double=double, wavefront=wavefront, rows=rows)
    return a


def image(a):
    return (a.sums.reshape(-1, 3) / a.samples).astype(np.float64)


def test_white_furnace_returns_the_sky_exactly(oracle_lib):
    img = image(render(scenes.white_furnace(), 32, 32, 4))
    assert np.all(np.abs(img - 1.0) < 1e-4)


def test_closed_emissive_room_matches_the_series_sum(oracle_lib):
    got = image(render(scenes.furnace_room(0.5, 1.0), 64, 64, 64))[:, 0].mean()
    want = (1 - 0.5 ** 8) / (1 - 0.5)
    assert abs(got - want) / want < 0.01


def test_variance_decreases_with_samples(oracle_lib):
    v = [image(render(scenes.furnace_room(0.5, 1.0), 64, 64, n))[:, 0].var() for n in (4, 16, 64)]
    assert v[0] > v[1] > v[2]


def test_point_light_direct_lighting_matches_lambert(oracle_lib):
    lit = image(render(an.floor_scene(an.point_light(), False), 65, 65, 64))[32 * 65 + 32, 0]
    assert abs(lit - 1.0) < 0.01
    shadowed = image(render(an.floor_scene(an.point_light(), True), 65, 65, 64))[32 * 65 + 32, 0]
    assert shadowed < 1e-3


def test_spot_light_falls_off_between_its_cone_angles(oracle_lib):
    def lit(off):
        return image(render(an.floor_scene(an.spot_at(off), False), 65, 65, 64))[32 * 65 + 32, 0]

    assert abs(lit(0.0) - 1.0) < 0.01
    c, i, o = math.cos(0.3), math.cos(0.1), math.cos(0.5)
    assert abs(lit(0.3) - ((c - o) / (i - o)) ** 2) < 0.01
    assert lit(0.6) < 1e-3


def test_directional_light_matches_lambert(oracle_lib):
    light = sc.Directional((0.0, 0.0, -1.0), (1.0, 1.0, 1.0), math.pi)
    lit = image(render(an.floor_scene(light, False), 65, 65, 64))[32 * 65 + 32, 0]
    assert abs(lit - 1.0) < 0.01


def test_smooth_dielectric_reflects_the_normal_incidence_fresnel(oracle_lib):
    m = sc.BaseBsdf(base_color=(0.0, 0.0, 0.0), roughness=0.0)
    img = image(render(an.sky_scene(scenes.plane(5.0, 0.0), m, 3.0), 32, 32, 64))
    assert abs(an.center_mean(img, 32, 16) - 0.04) < 0.003


def test_metal_furnace_conserves_energy(oracle_lib):
    for roughness, lo in [(0.0, 0.99), (0.3, 0.96), (0.5, 0.9)]:
        m = sc.BaseBsdf(base_color=(1.0, 1.0, 1.0), metallic=1.0, roughness=roughness)
        img = image(render(an.sky_scene(scenes.cube(0.5), m, 3.0), 32, 32, 64))
        got = an.center_mean(img, 32, 16)
        assert lo < got < 1.005, (roughness, got)


def test_rough_metal_highlight_matches_ggx(oracle_lib):
    s = an.highlight_scene()
    single = image(render(s, 65, 65, 64, multiscatter=False))[32 * 65 + 32, 0]
    assert abs(single - 1.0) < 0.02
    comp = image(render(s, 65, 65, 64, multiscatter=True))[32 * 65 + 32, 0]
    assert abs(comp / single - 1.09) < 0.02


def test_large_area_light_over_a_floor_gives_rho_times_radiance(oracle_lib):
    s = an.floor_with_emitter(scenes.material((0.5, 0.5, 0.5)), scenes.plane(25.0, 0.0), an.up(1.0), 2.0)
    got = an.center_mean(image(render(s, 65, 65, 64)), 65, 5)
    assert abs(got - 0.5 * 2.0 * 0.999) < 0.015


def test_small_area_light_matches_the_square_form_factor(oracle_lib):
    a = 0.1
    root = math.sqrt(1 + a * a)
    corner = (a / root) * math.atan(a / root) / math.pi
    rho, le = 1.0, 50.0
    want = rho * 4.0 * corner * le
    s = an.floor_with_emitter(scenes.material((rho,) * 3), scenes.plane(0.1, 0.0), an.up(1.0), le)
    got = an.center_mean(image(render(s, 65, 65, 64)), 65, 5)
    assert abs(got - want) / want < 0.03


def test_glossy_metal_reflects_a_large_area_light_without_gain_or_loss(oracle_lib):
    for roughness, lo in [(0.0, 0.995), (0.3, 0.95), (0.5, 0.9)]:
        metal = sc.BaseBsdf(base_color=(1.0, 1.0, 1.0), metallic=1.0, roughness=roughness)
        s = an.floor_with_emitter(metal, scenes.plane(25.0, 0.0), an.up(1.0), 1.0)
        got = an.center_mean(image(render(s, 65, 65, 64)), 65, 5)
        assert lo < got < 1.005, (roughness, got)


def test_constant_environment_map_is_a_white_furnace(oracle_lib):
    img = image(render(an.env_furnace(), 32, 32, 64))
    assert abs(an.center_mean(img, 32, 16) - 1.0) < 0.015
    assert abs(img[:, 0].mean() - 1.0) < 0.015


def test_rough_metal_furnace_matches_ggx_single_scatter_albedo(oracle_lib):
    # pathtrace.rs:1312-1327 (4 x 4 centre pixels; rows 14..17 traced only)
    for roughness in (0.1, 0.3, 0.5, 1.0):
        for cos_o in (1.0, 0.5):
            a = render(an.metal_plane(roughness, cos_o), 32, 32, 1024, multiscatter=False, rows=[14, 15, 16, 17])
            img = (a.sums.reshape(32, 32, 3) / a.samples)[14:18, 14:18, 0]
            want = an.ggx_albedo_quadrature(cos_o, roughness * roughness)
            assert abs(float(img.mean()) - want) < 0.01, (roughness, cos_o, float(img.mean()), want)


def test_wavefront_matches_the_megakernel_bit_for_bit(oracle_lib):
    s = scenes.cornell()
    s.add_light(sc.Point((0.3, 0.8, 0.2), (1.0, 0.9, 0.8), 2.0))
    mega = render(s, 40, 32, 4, lighting=True)
    wave = render(s, 40, 32, 4, lighting=True, wavefront=True)
    assert np.array_equal(mega.sums, wave.sums)
    assert np.array_equal(mega.lighting, wave.lighting)
    counts = np.array(wave.queue_counts)
    assert (counts[:, 0] == 40 * 32).all() and (np.diff(counts, axis=1) <= 0).all()


def test_adaptive_gives_the_same_image_with_both_integrators(oracle_lib):
    a = Adaptive(threshold=0.05, min_spp=4)
    mega = render(scenes.furnace_room(0.5, 1.0), 16, 16, 32, adaptive=a)
    wave = render(scenes.furnace_room(0.5, 1.0), 16, 16, 32, adaptive=a, wavefront=True)
    assert np.array_equal(mega.sums, wave.sums) and np.array_equal(mega.stats, wave.stats)
    n = mega.stats.reshape(-1, 3)[:, 0]
    assert (n < 32).any() and (n == 32).any()


def test_adaptive_with_a_zero_threshold_samples_every_pixel(oracle_lib):
    uniform = render(scenes.furnace_room(0.5, 1.0), 16, 16, 8)
    acc = render(scenes.furnace_room(0.5, 1.0), 16, 16, 8, adaptive=Adaptive(0.0, 2))
    assert np.array_equal(acc.sums, uniform.sums)
    assert (acc.stats.reshape(-1, 3)[:, 0] == 8).all()


def test_restir_converges_to_the_plain_image(oracle_lib):
    # crates/verion-gpu-vulkan/tests/restir.rs:90-100: within 3% of plain sampling.
    plain = image(render(scenes.cornell(), 32, 32, 64))
    re = image(render(scenes.cornell(), 32, 32, 64, restir=Restir()))
    assert abs(re.mean() - plain.mean()) / plain.mean() < 0.03


def test_restir_gi_leaves_sharp_surfaces_alone(oracle_lib):
    # crates/verion-gpu-vulkan/tests/restir.rs:263-271: walls of roughness 0.05 are too sharp for
    # reuse, so the image is the plain one bit for bit.
    from .analytic import closed_room

    plain = render(closed_room(0.05), 24, 24, 4)
    gi = render(closed_room(0.05), 24, 24, 4, restir=Restir(di=False, gi=True))
    assert np.array_equal(plain.sums, gi.sums)


def test_restir_gi_converges_to_the_plain_image(oracle_lib):
    # restir.rs:240-250 (3% at 64x64 and 1024 spp on the GPU); a smaller run here.
    from .analytic import closed_room

    plain = image(render(closed_room(0.9), 24, 24, 96))
    gi = image(render(closed_room(0.9), 24, 24, 96, restir=Restir(di=False, gi=True)))
    assert abs(gi.mean() - plain.mean()) / plain.mean() < 0.06


def test_double_precision_agrees_with_single(oracle_lib):
    f = image(render(scenes.cornell(), 24, 24, 16))
    d = image(render(scenes.cornell(), 24, 24, 16, double=True, acc64=True))
    assert abs(f.mean() - d.mean()) / d.mean() < 0.01


def test_bvh_matches_brute_force(oracle_lib):
    rng = np.random.default_rng(11)
    s = sc.Scene()
    v = rng.uniform(-2, 2, (3000, 3)).astype(np.float32)
    tri = (v[:, None, :] + rng.normal(scale=0.2, size=(3000, 3, 3))).astype(np.float32).reshape(-1, 3)
    m = s.add_mesh(sc.Mesh(tri, np.arange(tri.shape[0], dtype=np.uint32)))
    mat = s.add_material(scenes.material((0.5,) * 3))
    s.add_instance(sc.Instance(m, mat))
    s.add_instance(sc.Instance(m, mat, ((0.0, 1.0, 0.0, 0.5), (1.0, 0.0, 0.0, 0.0), (0.0, 0.0, 1.0, 0.2))))
    o = oracle.OracleScene(pack.pack(s))
    o_ = rng.uniform(-3, 3, (20000, 3))
    d = rng.normal(size=(20000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([o_, d], axis=1).astype(np.float32)
    assert np.array_equal(o.trace_closest(rays), o.trace_closest(rays, brute=True))


def test_two_instances_hit_at_distance_one(oracle_lib):
    # crates/verion-gpu-metal/tests/trace.rs:95-121
    s = sc.Scene()
    m = s.add_mesh(sc.Mesh(np.array([[-1, -1, 0], [1, -1, 0], [0, 1, 0]], np.float32), np.array([0, 1, 2])))
    mat = s.add_material(scenes.material((0.5,) * 3))
    s.add_instance(sc.Instance(m, mat, ((1, 0, 0, 0), (0, 1, 0, 0), (0, 0, 1, -1.0))))
    s.add_instance(sc.Instance(m, mat, ((1, 0, 0, 3.0), (0, 1, 0, 0), (0, 0, 1, -1.0))))
    o = oracle.OracleScene(pack.pack(s))
    h = o.trace_closest(np.array([[0, 0, 0, 0, 0, -1], [3, 0, 0, 0, 0, -1], [10, 0, 0, 0, 0, -1]], np.float32))
    t = [h[i, 3:4].view(np.float32)[0] if h[i, 0] else -1.0 for i in range(3)]
    assert t == [1.0, 1.0, -1.0]


def test_edge_rays_hit_exactly_one_of_two_adjacent_triangles(oracle_lib):
    # Watertightness: rays through the shared diagonal of a quad never slip between its triangles.
    s = sc.Scene()
    m = s.add_mesh(scenes.plane(1.0, 0.0))
    mat = s.add_material(scenes.material((0.5,) * 3))
    s.add_instance(sc.Instance(m, mat))
    o = oracle.OracleScene(pack.pack(s))
    u = np.linspace(-0.99, 0.99, 2001, dtype=np.float32)
    rays = np.stack([u, u, np.full_like(u, 1.0), np.zeros_like(u), np.zeros_like(u), -np.ones_like(u)], axis=1)
    h = o.trace_closest(rays, brute=True)
    assert h[:, 0].all()


def test_clearcoat_adds_a_second_fresnel_layer(oracle_lib):
    # pathtrace.rs:600-617: coat F0 0.04 plus 0.04 of the 0.96 it lets through.
    m = sc.BaseBsdf(base_color=(0.0, 0.0, 0.0), roughness=0.0, clearcoat=1.0)
    img = image(render(an.sky_scene(scenes.plane(5.0, 0.0), m, 3.0), 32, 32, 128))
    assert abs(an.center_mean(img, 32, 16) - 0.0784) < 0.004


def test_clearcoat_and_sheen_furnaces_conserve_energy(oracle_lib):
    # pathtrace.rs:619-640, 662-683
    for m in (sc.BaseBsdf(base_color=(1.0,) * 3, roughness=0.5, clearcoat=1.0, clearcoat_roughness=0.0),
              sc.BaseBsdf(base_color=(1.0,) * 3, roughness=0.5, clearcoat=1.0, clearcoat_roughness=0.3)):
        got = an.center_mean(image(render(an.sky_scene(scenes.cube(0.5), m, 3.0), 32, 32, 64)), 32, 16)
        assert 0.95 < got < 1.01
    for r in (0.3, 1.0):
        m = sc.BaseBsdf(base_color=(1.0,) * 3, roughness=0.5, sheen_color=(1.0,) * 3, sheen_roughness=r)
        got = an.center_mean(image(render(an.sky_scene(scenes.cube(0.5), m, 3.0), 32, 32, 64)), 32, 16)
        assert 0.95 < got < 1.02


def test_sheen_adds_its_directional_albedo_to_a_black_base(oracle_lib):
    # pathtrace.rs:642-660
    m = sc.BaseBsdf(base_color=(0.0,) * 3, roughness=0.0, sheen_color=(1.0,) * 3, sheen_roughness=1.0)
    got = an.center_mean(image(render(an.sky_scene(scenes.plane(5.0, 0.0), m, 3.0), 32, 32, 128)), 32, 16)
    assert abs(got - (0.137 + (1.0 - 0.137) * 0.04)) < 0.01


def test_dispersion_gives_each_channel_its_own_fresnel_reflection(oracle_lib):
    # pathtrace.rs:700-738
    s = sc.Scene()
    glass = s.add_material(sc.BaseBsdf(base_color=(1.0,) * 3, roughness=0.0, transmission=1.0, dispersion=4.0))
    floor = s.add_material(sc.BaseBsdf(base_color=(0.0,) * 3, metallic=1.0, roughness=1.0))
    for mesh, mat in ((scenes.plane(5.0, 0.0), glass), (scenes.plane(5.0, -1.0), floor)):
        s.add_instance(sc.Instance(s.add_mesh(mesh), mat))
    s.add_light(sc.Environment((1.0, 1.0, 1.0)))
    s.camera = scenes.camera_at_z(3.0)
    img = image(render(s, 32, 32, 512)).reshape(32, 32, 3)[8:24, 8:24].reshape(-1, 3).mean(axis=0)
    for c, want in enumerate((0.0293, 0.04, 0.0465)):
        assert abs(img[c] - want) < 0.006
    assert img[0] < img[1] < img[2]


def test_metal_tints_by_base_color(oracle_lib):
    # pathtrace.rs:760-774
    m = sc.BaseBsdf(base_color=(0.5,) * 3, metallic=1.0, roughness=0.0)
    got = an.center_mean(image(render(an.sky_scene(scenes.plane(5.0, 0.0), m, 3.0), 32, 32, 16)), 32, 16)
    assert abs(got - 0.5) < 0.01


def test_glass_furnace_conserves_energy(oracle_lib):
    # pathtrace.rs:776-797 (a subdivided octahedron stands in for the icosphere)
    sp, _, si = scenes.octasphere(8)
    for roughness, lo in ((0.0, 0.98), (0.3, 0.9)):
        m = sc.BaseBsdf(base_color=(1.0,) * 3, roughness=roughness, transmission=1.0)
        got = image(render(an.sky_scene(sc.Mesh(sp, si), m, 4.0), 48, 48, 64))[:, 0].mean()
        assert lo < got < 1.01, (roughness, got)


def test_opacity_lets_rays_and_shadows_through(oracle_lib):
    # pathtrace.rs:1651-1672
    def lit(opacity):
        s = an.floor_scene(an.point_light(), True)
        s.materials[1] = sc.BaseBsdf(base_color=(0.0,) * 3, ior=1.0, opacity=opacity)
        return image(render(s, 65, 65, 64))[32 * 65 + 32, 0]

    full = image(render(an.floor_scene(an.point_light(), False), 65, 65, 64))[32 * 65 + 32, 0]
    assert abs(lit(0.0) - full) < 0.02 * full
    assert lit(1.0) < 0.02 * full
    assert abs(lit(0.5) - 0.5 * full) < 0.08 * full


def test_oracle_bvh_finds_the_brute_force_hits_on_a_floor_grid(oracle_lib):
    # The many-light scene's floor is a grid of coplanar triangles: the computed t of two
    # neighbours sharing an edge can differ by an ulp, and the box test must not cull the nearer
    # one's flat box against the farther one's t. The ray below once hit triangle 141917 at
    # t = 0x41380a7b instead of 142548 at 0x41380a7a through the oracle's BVH.
    import struct

    p = pack.pack(scenes.many_lights())
    o = oracle.OracleScene(p)
    f = lambda h: struct.unpack("<f", struct.pack("<I", h))[0]  # noqa: E731
    one = np.array([[0.0, 6.0, 14.0, f(0x3DB768F6), f(0xBF058916), f(0xBF5934DC)]], np.float32)
    assert o.trace_closest(one)[0].tolist() == [1, 0, 142548, 0x41380A7A]
    rng = np.random.default_rng(3)
    n = 20000
    org = np.array([0.0, 6.0, 14.0]) + rng.normal(scale=0.5, size=(n, 3))
    d = rng.normal(size=(n, 3))
    d[:, 1] = -np.abs(d[:, 1])
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([org, d], 1).astype(np.float32)
    assert np.array_equal(o.trace_closest(rays), o.trace_closest(rays, brute=True))
