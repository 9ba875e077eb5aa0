"""What the radiance cache gains: path tracing that ends paths in the
trained cache against the plain path tracer (the same method without it), on
the instanced-spheres scene at reduced size with maxPathLength 8.

Both are compared with a 1024-spp plain reference.  After the cache has
trained on 48 frames, 16 frames of 1 spp with the cache have a lower relMSE
than 16 frames of the plain path tracer (lower variance for a small bias),
and the cached image's mean stays within 10 % of the reference's.  Also:
with training off the cache changes nothing between frames (inference only),
and the frame counter and post-processing behave as for b200_render_pt."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W, H = 160, 90


@pytest.fixture(scope="module")
def world(b200_device):
    import ospray_gb300 as og
    from ospray_gb300 import scenes
    d = scenes.pt_instanced_scene(levels=4, width=W, height=H)
    g = og.Scene(b200_device)
    scenes.build_pt_scene(g, d)
    g.set_lights([og.quad_light(L["position"], L["edge1"], L["edge2"], L["intensity"]) if L["type"] == "quad"
                  else og.ambient_light(L["intensity"]) for L in d["lights"]])
    c = d["camera"]
    cam = og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
    mats = og.materials_array(d["materials"])
    ref = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_ACCUM)
    p16 = og.pt_params(spp=16, max_path_length=8)
    for _ in range(64):
        og.render_pt(g, cam, p16, mats, ref)
    return g, cam, mats, ref, g.bounds()


def test_cache_lowers_error_at_equal_samples(b200_device, world):
    import ospray_gb300 as og
    g, cam, mats, ref, b = world
    p1 = og.pt_params(spp=1, max_path_length=8)
    plain = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_ACCUM)
    for _ in range(16):
        og.render_pt(g, cam, p1, mats, plain)
    e_plain = og.relmse(plain, ref)
    cache = og.RadianceCache(b200_device, b[:3], b[3:], learning_rate=1e-2, seed=1)
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_ACCUM)
    for _ in range(48):  # training frames
        og.render_pt_nrc(g, cam, p1, mats, fb, cache, train_paths=2048, train_batch=4096)
    fb.reset()
    for _ in range(16):
        og.render_pt_nrc(g, cam, p1, mats, fb, cache, train_paths=2048, train_batch=4096)
    assert fb.frame_id == 16
    e_nrc = og.relmse(fb, ref)
    img, r = fb.read(og.FB_COLOR)[..., :3], ref.read(og.FB_COLOR)[..., :3]
    assert np.isfinite(img).all()
    assert abs(img.mean() / r.mean() - 1.0) < 0.1
    assert e_nrc < e_plain, (e_nrc, e_plain)


def test_inference_only_frames_are_repeatable(b200_device, world):
    import ospray_gb300 as og
    g, cam, mats, ref, b = world
    p1 = og.pt_params(spp=1, max_path_length=8)
    cache = og.RadianceCache(b200_device, b[:3], b[3:], seed=2)
    for _ in range(4):
        og.render_pt_nrc(g, cam, p1, mats, og.Frame(b200_device, W, H, og.FB_COLOR), cache, train_paths=1024,
                         train_batch=2048)
    a = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_ACCUM)
    c = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_ACCUM)
    og.render_pt_nrc(g, cam, p1, mats, a, cache, train=False, train_paths=1024)
    og.render_pt_nrc(g, cam, p1, mats, c, cache, train=False, train_paths=1024)
    np.testing.assert_allclose(a.read(og.FB_COLOR), c.read(og.FB_COLOR), rtol=1e-4, atol=1e-5)
