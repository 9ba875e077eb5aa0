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
