"""Stereo cameras and sub-images on the GPU against the oracle: the AO
renderer's first hits (IDs bit for bit, depth too for the perspective
camera) and its colours to 1e-5 for
every stereo mode of the perspective and panoramic cameras and a sub-image;
the path tracer with a side-by-side camera over a sub-image to the usual
pixel tolerance (PerspectiveCamera.cpp:37-91, .ispc:28-41;
PanoramicCamera.cpp:45-52, .ispc:24-45; Camera_subRegion Camera.ih:28-31)."""
import numpy as np
import pytest

import oracle
from test_motion_gpu import CAM, LIGHTS, _build, _material_dicts

pytestmark = pytest.mark.gpu

W, H = 128, 64


def _kw(kind, mode, sub):
    kw = dict(fovy=CAM["fovy"], aspect=W / H, kind=kind, stereo_mode=mode, interpupillary_distance=0.3)
    if sub:
        kw.update(image_start=(0.125, 0.25), image_end=(0.875, 0.9))
    return kw


@pytest.mark.parametrize("kind", [0, 2])
@pytest.mark.parametrize("mode,sub", [(1, False), (2, False), (3, False), (4, False), (3, True), (0, True)])
def test_stereo_ao_matches_oracle(b200_device, kind, mode, sub):
    import ospray_gb300 as og
    dev = b200_device
    g, o = og.Scene(dev), oracle.Scene()
    _build(g, False)
    _build(o, False)
    kw = _kw(kind, mode, sub)
    fb = og.Frame(dev, W, H, og.FB_COLOR | og.FB_ACCUM | og.FB_DEPTH | og.FB_ID_PRIMITIVE | og.FB_ID_INSTANCE)
    og.render_ao(g, og.camera_desc(CAM["position"], CAM["direction"], CAM["up"], **kw),
                 og.ao_params(spp=2, ao_samples=2), fb)
    ref = oracle.render_ao(o, oracle.camera(CAM["position"], CAM["direction"], CAM["up"], **kw), 2, W, H, spp=2,
                           ao_samples=2)
    np.testing.assert_array_equal(fb.read(og.FB_ID_PRIMITIVE), ref["primID"])
    np.testing.assert_array_equal(fb.read(og.FB_ID_INSTANCE), ref["instID"])
    if kind == 0:
        np.testing.assert_array_equal(fb.read(og.FB_DEPTH), ref["depth"])
    else:  # the panoramic eye offset follows the direction's sin / cos, a few ulp apart on the two sides
        np.testing.assert_allclose(fb.read(og.FB_DEPTH), ref["depth"], rtol=4e-6, atol=0)
    close = np.all(np.abs(fb.read(og.FB_ACCUM) - ref["color"]) <= 1e-5, axis=2)
    assert close.mean() >= 0.999, close.mean()


def test_stereo_path_tracer_matches_oracle(b200_device):
    import ospray_gb300 as og
    dev = b200_device
    kw = _kw(0, 3, True)
    g = og.Scene(dev)
    _build(g, False)
    g.set_lights([og.quad_light(L["position"], L["edge1"], L["edge2"], L["intensity"]) if L["type"] == "quad"
                  else og.ambient_light(L["intensity"]) for L in LIGHTS])
    fb = og.Frame(dev, W, H, og.FB_COLOR | og.FB_ACCUM | og.FB_ID_PRIMITIVE)
    params = dict(spp=4, max_path_length=4, roulette_path_length=3)
    og.render_pt(g, og.camera_desc(CAM["position"], CAM["direction"], CAM["up"], **kw), og.pt_params(**params),
                 og.materials_array(_material_dicts()), fb)
    o = oracle.Scene()
    _build(o, False)
    ref = oracle.render_pt(o, oracle.PtWorld(_material_dicts(), LIGHTS),
                           oracle.camera(CAM["position"], CAM["direction"], CAM["up"], **kw),
                           oracle.pt_params(**params), W, H)
    assert np.mean(fb.read(og.FB_ID_PRIMITIVE) == ref["primID"]) >= 0.999
    gc, rc = fb.read(og.FB_ACCUM)[..., :3], ref["color"][..., :3]
    close = np.all(np.abs(gc - rc) <= 2e-3 * np.maximum(1.0, np.abs(rc)), axis=2)
    assert close.mean() >= 0.99, close.mean()
