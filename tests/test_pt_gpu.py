"""Path-tracer parity: b200_render_pt against the oracle's restatement of
PathTracer_renderPixel / samplePath / nextEventEstimation on the instanced
displaced-sphere workload at reduced resolution.

Both sides draw the same Owen-scrambled Sobol samples (bit-exact
LDSampler), trace the same primary rays (bit-exact camera and
intersection) and evaluate the same BSDF and light formulas; transcendental
functions differ in the last ulp between CUDA and the host libm, which can
flip a Russian-roulette or occlusion decision in a small fraction of paths.
So: first-hit IDs and depth agree exactly, per-pixel colours agree to 1e-3
on >= 99.9 % of pixels (all of them in the runs so far; the margin is for a
rare flipped decision), and the image means agree within 3 standard errors
of the per-pixel difference."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

W, H = 192, 108


@pytest.fixture(scope="module")
def pt_setup(b200_device):
    import ospray_gb300 as og
    from ospray_gb300 import scenes
    d = scenes.pt_instanced_scene(levels=4, width=W, height=H)
    g = og.Scene(b200_device)
    scenes.build_pt_scene(g, d)
    lights = []
    for L in d["lights"]:
        if L["type"] == "quad":
            lights.append(og.quad_light(L["position"], L["edge1"], L["edge2"], L["intensity"]))
        else:
            lights.append(og.ambient_light(L["intensity"]))
    g.set_lights(lights)
    o = oracle.Scene()
    scenes.build_pt_scene(o, d)
    ow = oracle.PtWorld(d["materials"], d["lights"])
    return d, g, o, ow


def render_both(pt_setup, b200_device, spp=4, frames=1, pf=2, maxlen=5, rr=3):
    import ospray_gb300 as og
    d, g, o, ow = pt_setup
    c = d["camera"]
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_DEPTH | og.FB_ACCUM | og.FB_ID_PRIMITIVE |
                  og.FB_ID_INSTANCE)
    cam = og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
    p = og.pt_params(spp=spp, max_path_length=maxlen, roulette_path_length=rr, pixel_filter=pf)
    mats = og.materials_array(d["materials"])
    for _ in range(frames):
        og.render_pt(g, cam, p, mats, fb)
    gpu = dict(color=fb.read(og.FB_COLOR), depth=fb.read(og.FB_DEPTH), primID=fb.read(og.FB_ID_PRIMITIVE),
               instID=fb.read(og.FB_ID_INSTANCE))
    ocam = oracle.camera(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
    op = oracle.pt_params(spp=spp, max_path_length=maxlen, roulette_path_length=rr, pixel_filter=pf)
    ref = oracle.render_pt(o, ow, ocam, op, W, H, frames=frames)
    return gpu, ref


def test_pt_first_hit_and_image_match_oracle(pt_setup, b200_device):
    gpu, ref = render_both(pt_setup, b200_device)
    assert np.mean(gpu["primID"] == ref["primID"]) >= 0.9999
    assert np.mean(gpu["instID"] == ref["instID"]) >= 0.9999
    assert np.mean(gpu["depth"].view(np.uint32) == ref["depth"].view(np.uint32)) >= 0.9999
    g, r = gpu["color"][..., :3], ref["color"][..., :3]
    assert np.isfinite(g).all()
    close = np.all(np.abs(g - r) <= 1e-3 * np.maximum(1.0, np.abs(r)), axis=2)
    print("pixels within 1e-3: %.4f  mean gpu %.5f oracle %.5f" % (close.mean(), g.mean(), r.mean()))
    assert close.mean() >= 0.999, close.mean()
    diff = (g - r).reshape(-1)
    se = diff.std() / np.sqrt(diff.size)
    assert abs(diff.mean()) <= 3 * se + 1e-6, (diff.mean(), se)
    np.testing.assert_allclose(gpu["color"][..., 3], ref["color"][..., 3], atol=1e-5)


def test_pt_accumulation_matches_oracle(pt_setup, b200_device):
    gpu, ref = render_both(pt_setup, b200_device, spp=1, frames=3, pf=0, maxlen=3, rr=1)
    g, r = gpu["color"][..., :3], ref["color"][..., :3]
    close = np.all(np.abs(g - r) <= 1e-3 * np.maximum(1.0, np.abs(r)), axis=2)
    print("accumulated: pixels within 1e-3: %.4f  mean gpu %.5f oracle %.5f" % (close.mean(), g.mean(), r.mean()))
    assert close.mean() >= 0.999, close.mean()
    assert abs(g.mean() - r.mean()) <= 0.02 * r.mean() + 1e-4


def test_pt_statistics_converge(pt_setup, b200_device):
    """Independent estimators agree: the GPU image at 16 spp against a GPU
    image at 64 spp from other sample indices (accumulated frames), within
    the per-pixel standard error."""
    import ospray_gb300 as og
    d, g, _, _ = pt_setup
    c = d["camera"]
    cam = og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
    mats = og.materials_array(d["materials"])
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_ACCUM)
    og.render_pt(g, cam, og.pt_params(spp=16, max_path_length=5, roulette_path_length=3), mats, fb)
    a = fb.read(og.FB_COLOR)[..., :3]
    for _ in range(4):
        og.render_pt(g, cam, og.pt_params(spp=16, max_path_length=5, roulette_path_length=3), mats, fb)
    b = fb.read(og.FB_COLOR)[..., :3]
    assert np.isfinite(a).all() and np.isfinite(b).all()
    assert abs(a.mean() - b.mean()) <= 0.02 * b.mean()
