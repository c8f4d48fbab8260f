"""Host-side known answers, ported from the reference's CPU unit tests:
crates/verion-gpu/src/lib.rs:251-270 (adaptive predicate), wavefront.rs:66-87 (buffer sizes and
stage order), readback.rs:139-166 (means, sample counts, empty lighting slots), pack.rs:879-1011
(albedo-table placement, virtual light, mip chain, parameter block), plus the albedo tables pinned
byte for byte against the reference's and the portable elementary functions' error bounds."""
import hashlib
import json
import math
from pathlib import Path

import numpy as np
import pytest

from verion_gb300 import pack, readback, scenes, wavefront
from verion_gb300 import scene as sc
from verion_gb300.readback import Adaptive, Restir
from verion_gb300.tables import gen_albedo

GOLDEN = Path(__file__).resolve().parent / "golden"
TABLES = Path(gen_albedo.__file__).resolve().parent


def test_albedo_tables_are_the_references():
    want = json.loads((GOLDEN / "albedo_sha256.json").read_text())
    for name, w in want.items():
        data = (TABLES / name).read_bytes()
        assert len(data) == w["bytes"]
        assert hashlib.sha256(data).hexdigest() == w["sha256"], name


def test_albedo_generator_reproduces_the_tables(tmp_path):
    gen_albedo.generate(tmp_path)
    for name in ("ggx_albedo.f32", "sheen_albedo.f32", "dielectric_albedo.f32"):
        assert (tmp_path / name).read_bytes() == (TABLES / name).read_bytes(), name


def test_adaptive_stops_after_the_minimum_once_the_error_is_small():
    # lib.rs:255-269
    a = Adaptive(threshold=0.1, min_spp=4)
    assert a.active(3.0, 3.0, 3.0)
    assert not a.active(4.0, 4.0, 4.0)
    assert a.active(4.0, 4.0, 8.0)
    assert not a.active(16.0, 0.0, 0.0)


def test_wavefront_sizes_follow_the_path_count():
    # wavefront.rs:70-78
    s = wavefront.Sizes.new(100, False)
    assert s.state == 100 * 16 * 4
    assert wavefront.Sizes.new(100, True).state == 100 * 33 * 4
    assert s.total() == 6400 + 1600 + 800 + 36 + 96


def test_adaptive_sampling_adds_select_at_depth_zero_only():
    # wavefront.rs:80-86
    assert len(wavefront.Stage.of_depth(0, True)) == 4
    assert len(wavefront.Stage.of_depth(0, False)) == 3
    assert len(wavefront.Stage.of_depth(3, True)) == 3


def test_mean_divides_by_the_pixels_own_sample_count():
    # readback.rs:144-156
    stats = np.array([4.0, 0.0, 0.0, 2.0, 0.0, 0.0], np.float32)
    inv = readback.inverse_samples(stats, 2, 99)
    assert inv.tolist() == [0.25, 0.5]
    m = readback.mean(np.array([4.0, 8.0, 12.0, 2.0, 2.0, 2.0], np.float32), inv)
    assert m.tolist() == [[1.0, 2.0, 3.0], [1.0, 1.0, 1.0]]
    assert readback.inverse_samples(None, 2, 4).tolist() == [0.25, 0.25]
    assert readback.sample_counts(stats).tolist() == [4, 2]


def test_lighting_reads_parts_and_defaults_empty_slots():
    # readback.rs:158-165
    rec = np.zeros(65, np.float32)
    rec[3:6] = [2.0, 4.0, 6.0]
    l = readback.lighting(rec, np.array([0.5], np.float32))
    assert l.indirect_diffuse.tolist() == [[1.0, 2.0, 3.0]]
    assert l.visibility.tolist() == [1.0]
    assert l.light_response.tolist() == [[0.0] * 4]


def test_albedo_tables_follow_the_light_table_and_precede_the_masks():
    # pack.rs:942-957
    s = sc.Scene()
    s.add_light(sc.Point((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), 1.0))
    lights, count, _, _ = pack.pack_lights(s)
    at = count * pack.LIGHT_WORDS
    assert lights.size == at + pack.ALBEDO_WORDS
    assert lights[at:at + 1].view(np.float32)[0] == 1.0  # GGX albedo at cos = 0, alpha = 0


def _env_scene(f):
    w, h = 64, 32
    px = np.array([[f(i, j)] * 3 for j in range(h) for i in range(w)], np.float32)
    s = sc.Scene()
    img = s.add_image(sc.Image(w, h, px))
    s.add_light(sc.EnvironmentMap(img, 1.0))
    return s


def test_virtual_light_follows_the_brightest_patch():
    # pack.rs:960-1000
    s = _env_scene(lambda i, j: 50.0 if (0 <= i < 4 and 8 <= j < 12) else 0.1)
    d, e = pack.virtual_light(s)
    phi = ((2.0 + 0.5) / 64.0 - 0.5) * 2.0 * math.pi
    theta = 10.0 / 32.0 * math.pi
    want = [math.sin(theta) * math.sin(phi), math.cos(theta), -math.sin(theta) * math.cos(phi)]
    assert float(np.dot(d, want)) > 0.99
    assert e[0] > 0.1 and e[0] == e[1]
    assert pack.virtual_light(_env_scene(lambda i, j: 1.0)) is None
    s.stylization_world = sc.StylizationWorld(virtual_light=False)
    assert pack.virtual_light(s) is None
    s.stylization_world = sc.StylizationWorld(direction=(0.0, 0.0, 2.0))
    assert pack.virtual_light(s)[0].tolist() == [0.0, 0.0, 1.0]


def test_mip_chain_ends_at_one_texel_and_averages():
    # pack.rs:1002-1009
    img = sc.Image(2, 2, np.array([[1.0] * 3, [3.0] * 3, [5.0] * 3, [7.0] * 3], np.float32))
    texels, levels = pack.mip_chain(img)
    assert levels == 2
    assert texels.size == (4 + 1) * 3
    assert texels[12:].tolist() == [4.0] * 3


def test_base_params_carry_the_view_and_leave_dispatch_words_clear():
    # pack.rs:1011-1040
    info = pack.SceneInfo(2, 5, 0, 0, 0.0, (0.1, 0.2, 0.3), False, False)
    view = pack.View.new(sc.Camera())
    p = pack.base_params(info, view, (64, 32), True, False, Adaptive(), Restir())
    assert (p[0], p[1], p[5], p[23]) == (64, 32, 2, 5)
    assert (p[28], p[29], p[32], p[34]) == (1, 0, 1, 16)
    assert (p[6], p[30], p[31], p[35]) == (0, 0, 0, 0)
    assert (p[36], p[37], p[38]) == (1, 4, 4)
    p = pack.base_params(info, view, (64, 32), False, False, None, Restir(gi=True))
    assert p[36] == 3
    assert p[21:22].view(np.float32)[0] == np.float32(0.2)


def test_empty_scene_is_rejected():
    # pack.rs:727-729
    with pytest.raises(ValueError):
        pack.pack(sc.Scene())


def test_emitter_cdf_is_power_proportional():
    p = pack.pack(scenes.cornell())
    assert p.info.emitter_count == 2
    e = p.emitters.reshape(-1, 16)
    assert np.allclose(e[:, 13], 0.5) and p.emit_cdf[-1] == 1.0
    assert np.allclose(e[:, 12], 0.125)  # two halves of a 0.5 x 0.5 quad


def test_pcg_matches_the_oracle(oracle_lib):
    L = oracle_lib.lib()
    for v in [0, 1, 2, 0x7F4A7C15, 0xFFFFFFFF, 123456789]:
        assert scenes.pcg(v) == L.or_pcg(v)


def _ulp_err(got, want):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    ulp = np.spacing(np.abs(want).astype(np.float32)).astype(np.float64)
    return np.abs(got - want) / np.maximum(ulp, np.finfo(np.float32).tiny)


def test_elementary_functions_are_accurate(oracle_lib):
    L = oracle_lib.lib()
    rng = np.random.default_rng(7)
    x = rng.uniform(-2 * math.pi, 2 * math.pi, 4000).astype(np.float32)
    s = np.array([L.or_sinf(float(v)) for v in x])
    c = np.array([L.or_cosf(float(v)) for v in x])
    assert np.abs(s - np.sin(x.astype(np.float64))).max() < 2.5e-7
    assert np.abs(c - np.cos(x.astype(np.float64))).max() < 2.5e-7
    u = rng.uniform(-1, 1, 4000).astype(np.float32)
    a = np.array([L.or_acosf(float(v)) for v in u])
    assert np.abs(a - np.arccos(u.astype(np.float64))).max() < 1e-6
    yx = rng.normal(size=(4000, 2)).astype(np.float32)
    t = np.array([L.or_atan2f(float(y), float(xx)) for y, xx in yx])
    assert np.abs(t - np.arctan2(yx[:, 0].astype(np.float64), yx[:, 1].astype(np.float64))).max() < 1e-6
    assert L.or_atan2f(0.0, -0.0) == np.float32(math.pi) and L.or_atan2f(-0.0, 1.0) == 0.0
    p = rng.uniform(1e-6, 1e6, 4000).astype(np.float32)
    lg = np.array([L.or_log2f(float(v)) for v in p])
    assert np.abs(lg - np.log2(p.astype(np.float64))).max() < 4e-6
    e = rng.uniform(-30, 30, 4000).astype(np.float32)
    ex = np.array([L.or_exp2f(float(v)) for v in e])
    assert _ulp_err(ex, np.exp2(e.astype(np.float64))).max() <= 4
    base = rng.uniform(0, 1, 2000).astype(np.float32)
    expo = rng.uniform(1, 200, 2000).astype(np.float32)
    pw = np.array([L.or_powf(float(b), float(q)) for b, q in zip(base, expo)])
    want = np.power(base.astype(np.float64), expo.astype(np.float64))
    # exp2(y log2 x): the relative error grows with |y log2 x| (a few ulp of the exponent).
    bound = 2.0 ** -21 * (1.0 + np.abs(expo * np.log2(base.astype(np.float64)))) * want + 1e-37
    assert np.all(np.abs(pw - want) <= bound)
    assert L.or_powf(0.0, 2.0) == 0.0
