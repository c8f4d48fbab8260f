"""GPU parity of the primary-hit AOV kernels (shaders/normals.slang, shaders/aov.slang) against the
oracle, bit for bit, and the reference's AOV known answers (crates/verion-gpu-metal/tests/normals.rs,
aov.rs): normals face the viewer, ids are instance / material + 1, misses are zero."""
import numpy as np
import pytest

import oracle
from verion_gb300 import pack, scenes
from verion_gb300.backend import Error, Renderer

from . import analytic as an

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("scene", ["zoo", "cornell"])
def test_normals_and_aovs_match_the_oracle(gpu_ctx, scene):
    s = an.feature_zoo() if scene == "zoo" else scenes.cornell()
    p = pack.pack(s)
    w, h = 72, 40
    r = Renderer(gpu_ctx, p)
    o = oracle.OracleScene(p)
    cam = pack.camera_record(p.view, w, h)
    n = r.render_normals(w, h)
    assert np.array_equal(n, o.render_normals(cam))
    a = r.render_aovs(w, h)
    ad, oi, mi, cv = o.render_aovs(cam)
    assert np.array_equal(a.albedo, ad[:, :3]) and np.array_equal(a.depth, ad[:, 3])
    assert np.array_equal(a.object_id, oi) and np.array_equal(a.material_id, mi)
    assert np.array_equal(a.coverage, cv)


def test_normals_face_the_viewer_and_misses_are_zero(gpu_ctx):
    s = scenes.white_furnace()
    r = Renderer(gpu_ctx, s)
    n = r.render_normals(32, 32).reshape(32, 32, 3)
    assert np.allclose(n[16, 16], [0.0, 0.0, 1.0], atol=1e-6)  # the cube's front face, toward the camera
    assert np.all(n[0, 0] == 0.0)  # a corner ray misses
    a = r.render_aovs(32, 32)
    assert a.object_id.reshape(32, 32)[16, 16] == 1 and a.object_id.reshape(32, 32)[0, 0] == 0
    assert abs(a.depth.reshape(32, 32)[16, 16] - 2.5) < 1e-5  # camera at z = 3, face at z = 0.5
    assert a.coverage.reshape(32, 32)[16, 16] == 1.0 and a.coverage.reshape(32, 32)[0, 0] == 0.0


def test_zero_size_is_a_scene_error(gpu_ctx):
    r = Renderer(gpu_ctx, scenes.white_furnace())
    with pytest.raises(Error) as e:
        r.render_normals(0, 4)
    assert e.value.kind == "Scene"
