"""A rendered frame with its AOVs and lighting split written as EXR and read back bit for bit, and
exr_diff between two renders of the same scene (GPU)."""
import numpy as np
import pytest

from verion_gb300 import exr, pack, scenes
from verion_gb300.backend import Integrator, Renderer

pytestmark = pytest.mark.gpu


def test_render_to_exr_round_trip(gpu_ctx, tmp_path):
    w, h = 48, 32
    r = Renderer(gpu_ctx, pack.pack(scenes.cornell()))
    acc = r.new_accumulation(w, h, lighting=True)
    r.accumulate(acc, 16)
    beauty = acc.mean()
    light = acc.lighting()
    normals = r.render_normals(w, h)
    aovs = r.render_aovs(w, h)
    parts = [light.direct_diffuse, light.indirect_diffuse, light.specular, light.transmission, light.emission]
    p = tmp_path / "frame.exr"
    exr.write_exr(p, w, h, beauty, normal=normals, albedo=aovs.albedo, depth=aovs.depth, object_id=aovs.object_id,
                  material_id=aovs.material_id, lighting=parts, visibility=light.visibility,
                  info=exr.RenderInfo(samples=acc.samples()))
    img = exr.read_exr(p)
    got = np.stack([img.channels[c].reshape(-1) for c in "RGB"], axis=1)
    assert np.array_equal(got, beauty.astype(np.float32))
    assert np.array_equal(np.stack([img.channels["N." + c].reshape(-1) for c in "XYZ"], axis=1), normals)
    assert np.array_equal(img.channels["ObjectId"].reshape(-1), aovs.object_id)
    assert np.array_equal(img.channels["Z"].reshape(-1), aovs.depth)
    assert np.array_equal(img.channels["Emission.G"].reshape(-1), np.asarray(light.emission, np.float32)[:, 1])
    assert img.attributes["verion/samples"] == 16 and img.attributes["verion/physical"] == "true"


def test_exr_diff_passes_megakernel_against_wavefront(gpu_ctx, tmp_path):
    # The two integrators give the same image; a different sample count stays within the gates.
    w, h = 64, 64
    p = pack.pack(scenes.cornell())
    imgs = []
    for integ, spp in ((Integrator.MEGAKERNEL, 256), (Integrator.WAVEFRONT, 256), (Integrator.WAVEFRONT, 512)):
        r = Renderer(gpu_ctx, p)
        r.set_integrator(integ)
        imgs.append(r.render(w, h, spp))
    d = exr.diff(imgs[0], imgs[1], w, h)
    assert d["channel"] == 0.0 and d["block"] == 0.0
    files = []
    for i, img in enumerate(imgs):
        files.append(tmp_path / f"{i}.exr")
        exr.write_exr(files[-1], w, h, img, info=exr.RenderInfo(samples=256))
    from verion_gb300.exr_diff import main

    assert main([str(files[0]), str(files[1]), str(files[2])]) == 0
