"""SciVis over worlds with surfaces: b200_render_scivis against the oracle's
restatement of SciVis_renderSample (render/scivis/SciVis.ispc:24-222) with
SciVis_computeShading / directIllumination (render/scivis/surfaces.ispc),
evalMaterial (render/scivis/surfaces.ih:44-84), lightAlpha
(render/scivis/lightAlpha.ispc) and SciVis_computeAO, on a seeded height
field with spheres, OBJ materials (one translucent), a quad and an ambient
light, and optionally a volume over the surfaces.

Both sides trace the same rays with the same watertight/sphere tests (IDs and
depth bit-exact) and draw the same random numbers; they differ only in float
contraction and transcendental rounding of the shading, so colours agree to
1e-3 relative on nearly every pixel."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

W, H = 96, 80
CAM = dict(position=(0.5, 0.9, -0.35), direction=(0.0, -0.6, 0.8), up=(0.0, 1.0, 0.0), fovy=60.0, aspect=W / H)
LIGHTS = [dict(type="quad", position=(0.2, 0.9, 0.2), edge1=(0.4, 0.0, 0.0), edge2=(0.0, 0.0, 0.4), intensity=4.0,
               visible=True),
          dict(type="ambient", intensity=0.35, color=(0.9, 0.95, 1.0), visible=True)]
MATS = [dict(kd=(0.7, 0.6, 0.5), ks=(0.25, 0.25, 0.25), ns=24.0),
        dict(kd=(0.2, 0.4, 0.8), ks=(0.1, 0.1, 0.1), ns=8.0, d=0.55, tf=(0.3, 0.3, 0.1))]


@pytest.fixture(scope="module")
def world(b200_device):
    import ospray_gb300 as og
    from ospray_gb300 import scenes
    d = scenes.ao_heightfield_scene(n=64, nspheres=150)
    v = scenes.volume_scene(n=24)
    out = {}
    for with_volume in (False, True):
        g = og.Scene(b200_device)
        o = oracle.Scene()
        for s in (g, o):
            gm = s.add_mesh(d["vertex"], d["index"])
            gs = s.add_spheres(d["spheres"])
            s.add_instance(gm, 0, 0, material=0)
            s.add_instance(gs, 0, 1, material=1)
            s.commit()
        g.set_lights([og.quad_light(L["position"], L["edge1"], L["edge2"], L["intensity"], visible=L["visible"])
                      if L["type"] == "quad" else og.ambient_light(L["intensity"], L["color"], visible=L["visible"])
                      for L in LIGHTS])
        ov = None
        if with_volume:
            g.set_volume(v["volume"], v["origin"], v["spacing"], v["color"], v["opacity"], v["value_range"])
            ov = oracle.VolumeModel(v["volume"], v["origin"], v["spacing"], v["color"], v["opacity"],
                                    v["value_range"])
        out[with_volume] = (g, o, ov)
    return out


def render_both(world, b200_device, with_volume=False, spp=2, frames=1, **kw):
    import ospray_gb300 as og
    g, o, ov = world[with_volume]
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_DEPTH | og.FB_ID_PRIMITIVE | og.FB_ID_OBJECT | og.FB_ACCUM)
    cam = og.camera_desc(CAM["position"], CAM["direction"], CAM["up"], fovy=CAM["fovy"], aspect=CAM["aspect"])
    params = og.scivis_params(spp=spp, shadows=kw.get("shadows", False), visible_lights=kw.get("visible_lights", False),
                              ao_samples=kw.get("ao_samples", 0), bg=kw.get("bg", (0, 0, 0, 0)))
    for _ in range(frames):
        og.render_scivis(g, cam, params, fb, og.scivis_materials_array(MATS))
    gpu = dict(color=fb.read(og.FB_COLOR), depth=fb.read(og.FB_DEPTH), primID=fb.read(og.FB_ID_PRIMITIVE))
    ocam = oracle.camera(CAM["position"], CAM["direction"], CAM["up"], fovy=CAM["fovy"], aspect=CAM["aspect"])
    ref = oracle.render_scivis(o, ov, ocam, LIGHTS, MATS, W, H, spp=spp, frames=frames,
                               shadows=kw.get("shadows", False), visible_lights=kw.get("visible_lights", False),
                               ao_samples=kw.get("ao_samples", 0), bg=kw.get("bg", (0, 0, 0, 0)))
    return gpu, ref


def assert_close(gpu, ref, frac=0.995):
    hit = ref["primID"] != 0xFFFFFFFF
    assert hit.mean() > 0.3, hit.mean()  # the surfaces fill the view
    assert (gpu["primID"] == ref["primID"]).mean() >= 0.999
    same_depth = gpu["depth"].view(np.uint32) == ref["depth"].view(np.uint32)
    assert same_depth.mean() >= 0.999
    c, r = gpu["color"], ref["color"]
    assert np.isfinite(c).all()
    close = np.all(np.abs(c - r) <= 1e-3 * np.maximum(1.0, np.abs(r)) + 1e-5, axis=2)
    assert close.mean() >= frac, close.mean()
    assert np.abs(c.mean(axis=(0, 1)) - r.mean(axis=(0, 1))).max() < 1e-4


@pytest.mark.parametrize("shadows,ao", [(False, 0), (True, 0), (True, 2)])
def test_scivis_surfaces_match_oracle(world, b200_device, shadows, ao):
    gpu, ref = render_both(world, b200_device, shadows=shadows, ao_samples=ao)
    assert ref["color"][..., :3].max() > 0.05  # lit
    assert_close(gpu, ref)


def test_scivis_shadows_and_ao_darken(world, b200_device):
    """Shadows and AO only remove light: the lit image without them is
    brighter pixel by pixel (both renders on the GPU, same samples)."""
    plain, _ = render_both(world, b200_device, shadows=False, ao_samples=0)
    shaded, _ = render_both(world, b200_device, shadows=True, ao_samples=2)
    p, s = plain["color"][..., :3], shaded["color"][..., :3]
    assert (s <= p + 1e-5).mean() >= 0.999
    assert s.mean() < p.mean()


def test_scivis_surfaces_with_volume(world, b200_device):
    gpu, ref = render_both(world, b200_device, with_volume=True, shadows=True, ao_samples=1, bg=(0.1, 0.1, 0.2, 1.0))
    assert_close(gpu, ref, frac=0.99)


def test_scivis_visible_lights_and_accumulation(world, b200_device):
    gpu, ref = render_both(world, b200_device, spp=1, frames=3, visible_lights=True, shadows=True)
    assert_close(gpu, ref)


@pytest.mark.parametrize("shadows,ao", [(False, 0), (True, 1)])
def test_scivis_gradient_shading_with_surfaces(world, b200_device, shadows, ao):
    """Gradient-shaded volume (integrateVolumeIntervalsGradient with
    gradientShadingScale 0.75) in front of the surfaces: each opaque sample
    is lit like a material-less surface with normal -grad, shadow and AO
    rays through the surfaces and the volume."""
    g, o, ov = world[True]
    g.set_volume_gradient_shading(0.75)
    ov.set_gradient_shading(0.75)
    try:
        gpu, ref = render_both(world, b200_device, with_volume=True, shadows=shadows, ao_samples=ao,
                               bg=(0.1, 0.1, 0.2, 1.0))
    finally:
        g.set_volume_gradient_shading(0.0)
        ov.set_gradient_shading(0.0)
    assert_close(gpu, ref, frac=0.99)
    unshaded, _ = render_both(world, b200_device, with_volume=True, shadows=shadows, ao_samples=ao,
                              bg=(0.1, 0.1, 0.2, 1.0))
    # the shading changes the volume's colour where it is seen
    assert np.abs(unshaded["color"] - gpu["color"]).max() > 1e-2


def test_scivis_gradient_shading_volume_only(b200_device):
    """A volume-only world with gradient shading and lights renders through
    the shaded integrator (no surfaces traced) and matches the oracle."""
    import ospray_gb300 as og
    from ospray_gb300 import scenes
    v = scenes.volume_scene(n=24, width=W, height=H)
    g = og.Scene(b200_device)
    g.set_volume(v["volume"], v["origin"], v["spacing"], v["color"], v["opacity"], v["value_range"])
    lights = [dict(type="quad", position=(-1.0, 2.5, -1.0), edge1=(0.5, 0.0, 0.0), edge2=(0.0, 0.0, 0.5),
                   intensity=6.0, visible=False),
              dict(type="ambient", intensity=0.25, color=(1.0, 1.0, 1.0), visible=False)]
    g.set_lights([og.quad_light(L["position"], L["edge1"], L["edge2"], L["intensity"], visible=L["visible"])
                  if L["type"] == "quad" else og.ambient_light(L["intensity"], L["color"], visible=L["visible"])
                  for L in lights])
    g.set_volume_gradient_shading(1.0)
    ov = oracle.VolumeModel(v["volume"], v["origin"], v["spacing"], v["color"], v["opacity"], v["value_range"])
    ov.set_gradient_shading(1.0)
    c = v["camera"]
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_ACCUM)
    cam = og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=W / H)
    params = og.scivis_params(spp=2, shadows=True, ao_samples=1, bg=(0, 0, 0, 0))
    og.render_scivis(g, cam, params, fb)
    col = fb.read(og.FB_COLOR)
    ocam = oracle.camera(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=W / H)
    ref = oracle.render_scivis(None, ov, ocam, lights, [], W, H, spp=2, shadows=True, ao_samples=1)["color"]
    assert np.isfinite(col).all()
    assert ref[..., 3].max() > 0.3  # the volume is in view
    close = np.all(np.abs(col - ref) <= 1e-3 * np.maximum(1.0, np.abs(ref)) + 1e-5, axis=2)
    assert close.mean() >= 0.99, close.mean()
    assert np.abs(col.mean(axis=(0, 1)) - ref.mean(axis=(0, 1))).max() < 1e-4


def test_ao_renderer_composites_the_volume(world, b200_device):
    """The AO renderer over a world with surfaces and a volume
    (AORenderer_renderSample with integrateVolumeIntervals,
    render/ao/AORenderer.ispc:59-80, render/ao/volumes.ispc:251-352): the
    volume's colour and opacity in front of each layer, against the oracle."""
    import ospray_gb300 as og
    g, o, ov = world[True]
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_DEPTH | og.FB_ID_PRIMITIVE)
    cam = og.camera_desc(CAM["position"], CAM["direction"], CAM["up"], fovy=CAM["fovy"], aspect=CAM["aspect"])
    og.render_ao(g, cam, og.ao_params(spp=2, ao_samples=1, volume_sampling_rate=0.5, bg=(0.1, 0.1, 0.2, 1.0)), fb)
    ocam = oracle.camera(CAM["position"], CAM["direction"], CAM["up"], fovy=CAM["fovy"], aspect=CAM["aspect"])
    with oracle.AOVolume(ov, 0.5):
        ref = oracle.render_ao(o, ocam, 2, W, H, spp=2, ao_samples=1, bg=(0.1, 0.1, 0.2, 1.0))
    plain = oracle.render_ao(o, ocam, 2, W, H, spp=2, ao_samples=1, bg=(0.1, 0.1, 0.2, 1.0))
    assert np.abs(ref["color"] - plain["color"]).max() > 0.05  # the volume is seen
    assert np.mean(fb.read(og.FB_ID_PRIMITIVE) == ref["primID"]) >= 0.999
    c, r = fb.read(og.FB_COLOR), ref["color"]
    close = np.all(np.abs(c - r) <= 1e-3 * np.maximum(1.0, np.abs(r)) + 1e-5, axis=2)
    assert close.mean() >= 0.99, close.mean()
    assert np.abs(c.mean(axis=(0, 1)) - r.mean(axis=(0, 1))).max() < 1e-4


def test_transformed_volume_matches_oracle(world, b200_device):
    """A volume placed by an instance transform (rotation about y, scale 0.8,
    translation): rays go to volume space by the inverse transform, gradient
    normals come back by its transpose; SciVis with gradient shading and
    shadows, and the AO renderer, against the oracle."""
    import ospray_gb300 as og
    g, o, ov = world[True]
    a = np.radians(30.0)
    xfm = np.array([[0.8 * np.cos(a), 0.0, 0.8 * np.sin(a), 0.15],
                    [0.0, 0.8, 0.0, 0.05],
                    [-0.8 * np.sin(a), 0.0, 0.8 * np.cos(a), 0.2]], np.float32)
    for s in (g, ov):
        s.set_volume_transform(xfm) if s is g else s.set_transform(xfm)
    g.set_volume_gradient_shading(0.5)
    ov.set_gradient_shading(0.5)
    try:
        gpu, ref = render_both(world, b200_device, with_volume=True, shadows=True, ao_samples=1,
                               bg=(0.1, 0.1, 0.2, 1.0))
        fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_ID_PRIMITIVE)
        cam = og.camera_desc(CAM["position"], CAM["direction"], CAM["up"], fovy=CAM["fovy"], aspect=CAM["aspect"])
        og.render_ao(g, cam, og.ao_params(spp=2, ao_samples=1, bg=(0.1, 0.1, 0.2, 1.0)), fb)
        ocam = oracle.camera(CAM["position"], CAM["direction"], CAM["up"], fovy=CAM["fovy"], aspect=CAM["aspect"])
        with oracle.AOVolume(ov, 1.0):
            aref = oracle.render_ao(o, ocam, 2, W, H, spp=2, ao_samples=1, bg=(0.1, 0.1, 0.2, 1.0))
        g.set_volume_transform(None)
        ov.set_transform(None)
        untransformed, _ = render_both(world, b200_device, with_volume=True, shadows=True, ao_samples=1,
                                       bg=(0.1, 0.1, 0.2, 1.0))
    finally:
        g.set_volume_transform(None)
        ov.set_transform(None)
        g.set_volume_gradient_shading(0.0)
        ov.set_gradient_shading(0.0)
    assert np.abs(gpu["color"] - untransformed["color"]).max() > 0.05  # the transform moves the volume
    assert_close(gpu, ref, frac=0.99)
    c, r = fb.read(og.FB_COLOR), aref["color"]
    close = np.all(np.abs(c - r) <= 1e-3 * np.maximum(1.0, np.abs(r)) + 1e-5, axis=2)
    assert close.mean() >= 0.99, close.mean()
