"""Orthographic and panoramic cameras (OrthographicCamera_initRay
camera/OrthographicCamera.ispc:11-49, PanoramicCamera_initRay
camera/PanoramicCamera.ispc:12-90, mono) against the oracle: the
orthographic rays are bit-exact (plain products and sums), so AO IDs and
depth agree exactly; the panoramic rays go through sin/cos, whose last ulp
differs between CUDA and the host libm, so IDs agree on nearly every pixel."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

W, H = 128, 96


@pytest.fixture(scope="module")
def ao_world(b200_device):
    import ospray_gb300 as og
    from ospray_gb300 import scenes
    d = scenes.ao_heightfield_scene(n=96, nspheres=300)
    g = og.Scene(b200_device)
    scenes.build_ao_scene(g, d)
    o = oracle.Scene()
    scenes.build_ao_scene(o, d)
    return g, o


def _ao_both(b200_device, world, kind, pos, dirn, height=1.0, spp=1, pf=0):
    import ospray_gb300 as og
    g, o = world
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_DEPTH | og.FB_ID_PRIMITIVE | og.FB_ID_OBJECT)
    cam = og.camera_desc(pos, dirn, (0, 1, 0), aspect=W / H, kind=kind, height=height)
    og.render_ao(g, cam, og.ao_params(spp=spp, pixel_filter=pf), fb)
    ref = oracle.render_ao(o, oracle.camera(pos, dirn, (0, 1, 0), aspect=W / H, kind=kind, height=height), pf, W, H,
                           spp=spp)
    return fb, ref


def test_orthographic_camera_matches_oracle(b200_device, ao_world):
    import ospray_gb300 as og
    fb, ref = _ao_both(b200_device, ao_world, og.CAMERA_ORTHOGRAPHIC, (0.5, 1.5, 0.5), (0.0, -1.0, 0.3), height=1.2)
    prim, depth = fb.read(og.FB_ID_PRIMITIVE), fb.read(og.FB_DEPTH)
    assert np.mean(ref["primID"] != 0xFFFFFFFF) > 0.3
    assert np.mean(prim == ref["primID"]) >= 0.9999
    assert np.mean(depth.view(np.uint32) == ref["depth"].view(np.uint32)) >= 0.9999
    assert np.mean(np.all(fb.read(og.FB_COLOR) == ref["color"], axis=2)) >= 0.999


def test_panoramic_camera_matches_oracle(b200_device, ao_world):
    import ospray_gb300 as og
    fb, ref = _ao_both(b200_device, ao_world, og.CAMERA_PANORAMIC, (0.5, 0.25, 0.5), (1.0, 0.0, 0.0), spp=2, pf=2)
    prim = fb.read(og.FB_ID_PRIMITIVE)
    hit = ref["primID"] != 0xFFFFFFFF
    assert 0.2 < hit.mean() < 0.9  # the ground below, the sky above
    assert np.mean(prim == ref["primID"]) >= 0.995
    c, r = fb.read(og.FB_COLOR), ref["color"]
    assert np.mean(np.all(np.abs(c - r) <= 1e-3, axis=2)) >= 0.99
    assert abs(c.mean() - r.mean()) < 1e-3


def test_architectural_perspective_camera_matches_oracle(b200_device, ao_world):
    """"architectural": the image plane parallel to up (PerspectiveCamera::commit,
    camera/PerspectiveCamera.cpp:82-85); plain products and sums, so exact."""
    import ospray_gb300 as og
    g, o = ao_world
    pos, dirn = (0.5, 1.2, -1.4), (0.0, -0.8, 2.0)
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_DEPTH | og.FB_ID_PRIMITIVE)
    og.render_ao(g, og.camera_desc(pos, dirn, (0, 1, 0), aspect=W / H, architectural=True),
                 og.ao_params(pixel_filter=0), fb)
    ref = oracle.render_ao(o, oracle.camera(pos, dirn, (0, 1, 0), aspect=W / H, architectural=True), 0, W, H)
    np.testing.assert_array_equal(fb.read(og.FB_ID_PRIMITIVE), ref["primID"])
    np.testing.assert_array_equal(fb.read(og.FB_DEPTH), ref["depth"])


def test_depth_of_field_path_tracer_matches_oracle(b200_device):
    """A perspective camera with an aperture: the path tracer draws each camera
    sample's lens position from its sample stream (PathTracer.ispc:172-175,
    PerspectiveCamera.ispc:44-52); the lens disk goes through sin/cos, so the
    rays agree to an ulp and the images within the path-tracer tolerance;
    the out-of-focus background is blurred relative to the pinhole image."""
    import ospray_gb300 as og
    from test_motion_gpu import _pt, _pt_oracle, CAM
    import test_motion_gpu as tm
    dev = b200_device
    kw = dict(aperture_radius=0.25, focus_distance=6.0)
    g = og.Scene(dev)
    tm._build(g, True)
    g.set_lights([og.quad_light(L["position"], L["edge1"], L["edge2"], L["intensity"]) if L["type"] == "quad"
                  else og.ambient_light(L["intensity"]) for L in tm.LIGHTS])
    fb = og.Frame(dev, tm.W, tm.H, og.FB_COLOR | og.FB_ACCUM | og.FB_ID_PRIMITIVE)
    cam = og.camera_desc(CAM["position"], CAM["direction"], CAM["up"], fovy=CAM["fovy"], aspect=tm.W / tm.H, **kw)
    og.render_pt(g, cam, og.pt_params(spp=4, max_path_length=4, roulette_path_length=3), tm._materials(og), fb)
    o = oracle.Scene()
    tm._build(o, True)
    ref = oracle.render_pt(o, oracle.PtWorld(tm._material_dicts(), tm.LIGHTS),
                           oracle.camera(CAM["position"], CAM["direction"], CAM["up"], fovy=CAM["fovy"],
                                         aspect=tm.W / tm.H, **kw),
                           oracle.pt_params(spp=4, max_path_length=4, roulette_path_length=3), tm.W, tm.H)
    gpu = fb.read(og.FB_ACCUM)
    assert np.mean(fb.read(og.FB_ID_PRIMITIVE) == ref["primID"]) >= 0.99
    d = (gpu[..., :3] - ref["color"][..., :3]).reshape(-1)
    se = d.std() / np.sqrt(d.size)
    assert abs(d.mean()) <= 3 * se + 1e-6, (d.mean(), se)
    assert np.mean(np.all(np.abs(gpu[..., :3] - ref["color"][..., :3]) <= 2e-3 * np.maximum(1.0, np.abs(ref["color"][..., :3])), axis=2)) >= 0.97
    pin = _pt(og, dev, (0.5, 0.5))
    assert np.abs(pin["color"] - gpu).max() > 0.05
