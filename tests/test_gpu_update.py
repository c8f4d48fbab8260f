"""Scene updates (RayTracingBackend::update): an updated renderer draws exactly what a renderer built
from scratch on the edited scene draws, and rebuilds only what the edit needs. The room scene and the
six edits restate crates/verion-gpu-metal/tests/update.rs:67-208; the plan logic is pack.rs:948-967."""

import numpy as np
import pytest

from verion_gb300 import pack, scenes
from verion_gb300 import scene as sc
from verion_gb300.backend import Integrator, Renderer
from verion_gb300.pack import UpdatePlan


def test_plan_follows_the_reuse_table():
    p = UpdatePlan.new(camera=True)
    assert p.camera and not p.materials and not p.tlas and not p.blases and not p.full
    p = UpdatePlan.new(lights=True)
    assert p.lights and not p.emitters and not p.tlas and not p.vertices
    p = UpdatePlan.new(geometry=True)
    assert p.full and p.tlas and p.vertices
    assert UpdatePlan.new().is_empty()
    p = UpdatePlan.new(materials=[0])
    assert p.materials and p.emitters and p.instances and not p.tlas
    p = UpdatePlan.new(instances=[1])
    assert p.instances and p.tlas and p.emitters and not p.vertices
    p = UpdatePlan.new(deformed=[1])
    assert p.vertices and p.blases == (1,) and p.tlas and p.instances


def cube_at(half, y=0.0):
    m = scenes.cube(half)
    m.positions[:, 1] += y
    return m


def room():
    """update.rs:67-108: a closed room lit by a small emissive cube and a point light."""
    s = sc.Scene()
    room_mesh = s.add_mesh(cube_at(1.0))
    lamp_mesh = s.add_mesh(cube_at(0.1))
    walls = s.add_material(scenes.material((0.6, 0.6, 0.6)))
    glow = s.add_material(scenes.material((0.0, 0.0, 0.0), (8.0, 8.0, 8.0)))
    s.add_instance(sc.Instance(room_mesh, walls))
    lamp = s.add_instance(sc.Instance(lamp_mesh, glow, ((1, 0, 0, 0), (0, 1, 0, 0.7), (0, 0, 1, 0))))
    s.add_light(sc.Point((0.0, -0.5, 0.0), (1.0, 1.0, 1.0), 0.5))
    s.camera = sc.Camera(transform=((1, 0, 0, 0), (0, 1, 0, 0), (0, 0, 1, 0.95)))
    return s, walls, lamp_mesh, lamp


def render(r):
    acc = r.new_accumulation(48, 48)
    r.accumulate(acc, 8)
    return acc.sums()


def update_matches_fresh(ctx, r, scene, plan):
    before = render(r)
    report = r.update(scene, plan)
    after = render(r)
    fresh = render(Renderer(ctx, scene))
    assert np.array_equal(after, fresh), "the update differs from a rebuild"
    assert not np.array_equal(before, after), "the edit changed nothing"
    return report


pytestmark_gpu = pytest.mark.gpu


@pytestmark_gpu
@pytest.mark.parametrize("integrator", [Integrator.MEGAKERNEL, Integrator.WAVEFRONT])
def test_a_material_edit_reuses_the_acceleration_structure(gpu_ctx, integrator):
    s, walls, _, _ = room()
    r = Renderer(gpu_ctx, s)
    r.set_integrator(integrator)
    s.materials[walls] = scenes.material((0.9, 0.1, 0.1))
    rep = update_matches_fresh(gpu_ctx, r, s, UpdatePlan.new(materials=[walls]))
    assert (rep.blases_built, rep.tlas_built) == (0, False)
    assert rep.bytes_uploaded > 0


@pytestmark_gpu
def test_a_light_edit_reuses_the_acceleration_structure(gpu_ctx):
    s, _, _, _ = room()
    r = Renderer(gpu_ctx, s)
    s.lights[0] = sc.Point((0.0, -0.5, 0.0), (1.0, 0.5, 0.2), 2.0)
    rep = update_matches_fresh(gpu_ctx, r, s, UpdatePlan.new(lights=True))
    assert (rep.blases_built, rep.tlas_built) == (0, False)


@pytestmark_gpu
def test_moving_an_instance_rebuilds_only_the_instance_level(gpu_ctx):
    s, _, _, lamp = room()
    r = Renderer(gpu_ctx, s)
    inst = s.instances[lamp]
    s.instances[lamp] = sc.Instance(inst.mesh, inst.material, ((1, 0, 0, 0.4), (0, 1, 0, 0.7), (0, 0, 1, 0)))
    rep = update_matches_fresh(gpu_ctx, r, s, UpdatePlan.new(instances=[lamp]))
    assert (rep.blases_built, rep.tlas_built) == (0, True)


@pytestmark_gpu
def test_deforming_a_mesh_rewrites_only_its_vertices(gpu_ctx):
    s, _, lamp_mesh, _ = room()
    r = Renderer(gpu_ctx, s)
    s.meshes[lamp_mesh] = cube_at(0.3)
    rep = update_matches_fresh(gpu_ctx, r, s, UpdatePlan.new(deformed=[lamp_mesh]))
    assert (rep.blases_built, rep.tlas_built) == (1, True)
    assert rep.bytes_uploaded >= 8 * 32


@pytestmark_gpu
def test_a_camera_edit_rebuilds_nothing(gpu_ctx):
    s, _, _, _ = room()
    r = Renderer(gpu_ctx, s)
    s.camera = sc.Camera(transform=((1, 0, 0, 0.3), (0, 1, 0, 0), (0, 0, 1, 0.95)))
    rep = update_matches_fresh(gpu_ctx, r, s, UpdatePlan.new(camera=True))
    assert (rep.blases_built, rep.tlas_built, rep.bytes_uploaded) == (0, False, 0)


@pytestmark_gpu
def test_a_new_instance_rebuilds_everything_but_keeps_the_settings(gpu_ctx):
    s, walls, _, _ = room()
    r = Renderer(gpu_ctx, s)
    r.set_integrator(Integrator.WAVEFRONT)
    mesh = s.add_mesh(cube_at(0.2))
    s.add_instance(sc.Instance(mesh, walls, ((1, 0, 0, -0.5), (0, 1, 0, 0), (0, 0, 1, 0))))
    rep = update_matches_fresh(gpu_ctx, r, s, UpdatePlan.new(geometry=True))
    assert (rep.blases_built, rep.tlas_built) == (3, True)
    assert r.integrator() == Integrator.WAVEFRONT


@pytestmark_gpu
def test_a_vertex_count_change_needs_a_full_update(gpu_ctx):
    from verion_gb300.backend import Error

    s, _, lamp_mesh, _ = room()
    r = Renderer(gpu_ctx, s)
    m = scenes.cube(0.2)
    s.meshes[lamp_mesh] = sc.Mesh(np.concatenate([m.positions, m.positions[:1]]), m.indices)
    with pytest.raises(Error):
        r.update(s, UpdatePlan.new(deformed=[lamp_mesh]))


@pytestmark_gpu
def test_an_environment_map_edit_redraws_like_a_rebuild(gpu_ctx):
    # A new HDRI (its texels, CDFs and the sampling guide tables) through a lights update: the image
    # is the one of a renderer built on the edited scene.
    s = scenes.many_spheres(spheres=4, sphere_n=7, grid=16, hdri=None)
    first = s.add_image(scenes.sky_hdri(64, 32, sun_peak=200.0, seed=1))
    env = s.add_light(sc.EnvironmentMap(first, 1.0))
    r = Renderer(gpu_ctx, s)
    r.set_integrator(Integrator.WAVEFRONT)
    second = s.add_image(scenes.sky_hdri(128, 64, sun_peak=800.0, seed=2))
    s.lights[env] = sc.EnvironmentMap(second, 1.0)
    update_matches_fresh(gpu_ctx, r, s, UpdatePlan.new(lights=True))
