"""Material parity: the path tracer's material types on the GPU against the
oracle's restatement of the reference's materials and transparent shadows.

* every type on one scene: principled (opaque and cut-out), obj (Lambert +
  Blinn specular + transmission, d < 1), metal (specular and rough), glass
  (with an attenuating medium inside) and thin glass; the path tracer runs 6
  bounces so paths cross the glass and return (Principled.ispc:81-455,
  OBJ.ispc:29-126, Metal.ispc:16-48, Glass.ispc:16-60, ThinGlass.ispc:16-70,
  PathSampler.ispc:290-411);
* transparent shadows: cut-out and filtering surfaces between the quad light
  and the ground, whose shadow rays loop over closest hits and multiply the
  surfaces' transparency (TransparentShadow.ispc:18-85);
* the OSPRay API's "obj", "metal", "glass" and "thinGlass" materials render
  exactly what the b200 ABI renders for the same parameters.

Both sides draw the same samples and trace the same rays; transcendental
functions differ in the last ulp between CUDA and the host libm, which can
flip a Russian-roulette or Fresnel decision in a few paths, so colours are
compared per pixel to 1e-3 on nearly every pixel and by their means within
3 standard errors.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

W, H = 192, 108


def _materials(og, n):
    kinds = [og.principled((0.8, 0.35, 0.2), 0.3, 0.0, 1.0),
             og.principled((0.2, 0.6, 0.9), 0.5, 0.0, 0.35),
             og.obj_material(kd=(0.5, 0.4, 0.2), ks=(0.3, 0.3, 0.3), ns=25.0, d=0.7, tf=(0.2, 0.1, 0.0)),
             og.metal(roughness=0.0),
             og.metal(eta=(0.2, 0.9, 1.1), k=(3.9, 2.4, 2.2), roughness=0.25),
             og.glass(eta_inside=1.45, attenuation_color=(0.9, 0.6, 0.3), attenuation_distance=2.0),
             og.thin_glass(eta=1.5, attenuation_color=(0.6, 0.9, 0.7), thickness=0.3)]
    return [kinds[i % len(kinds)] for i in range(n)]


def _render(og, b200_device, g, o, d, mats, spp, frames=1, maxlen=6, rr=3, pf=2):
    c = d["camera"]
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_DEPTH | og.FB_ACCUM | og.FB_ID_PRIMITIVE |
                  og.FB_ID_INSTANCE)
    cam = og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
    p = og.pt_params(spp=spp, max_path_length=maxlen, roulette_path_length=rr, pixel_filter=pf)
    arr = og.materials_array(mats)
    for _ in range(frames):
        og.render_pt(g, cam, p, arr, fb)
    # the accumulated colour before the RGBA32F conversion (which clamps
    # alpha to [0, 1], ColorConversion.ispc:27-30): paths through thin glass
    # can carry a throughput above 1, so alpha may be negative here, as in the oracle
    gpu = dict(color=fb.read(og.FB_ACCUM), depth=fb.read(og.FB_DEPTH), primID=fb.read(og.FB_ID_PRIMITIVE),
               instID=fb.read(og.FB_ID_INSTANCE))
    ow = oracle.PtWorld(mats, d["lights"])
    ocam = oracle.camera(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
    ref = oracle.render_pt(o, ow, ocam, oracle.pt_params(spp=spp, max_path_length=maxlen, roulette_path_length=rr,
                                                         pixel_filter=pf), W, H, frames=frames)
    return gpu, ref


def _compare(gpu, ref, min_close):
    assert np.mean(gpu["primID"] == ref["primID"]) >= 0.9999
    assert np.mean(gpu["instID"] == ref["instID"]) >= 0.9999
    g, r = gpu["color"][..., :3], ref["color"][..., :3]
    assert np.isfinite(g).all()
    close = np.all(np.abs(g - r) <= 1e-3 * np.maximum(1.0, np.abs(r)), axis=2)
    diff = (g - r).reshape(-1)
    se = diff.std() / np.sqrt(diff.size)
    print("pixels within 1e-3: %.4f  mean gpu %.5f oracle %.5f (se %.2e)" % (close.mean(), g.mean(), r.mean(), se))
    assert close.mean() >= min_close, close.mean()
    assert abs(diff.mean()) <= 3 * se + 1e-6, (diff.mean(), se)
    np.testing.assert_allclose(gpu["color"][..., 3], ref["color"][..., 3], atol=2e-3)


@pytest.fixture(scope="module")
def mat_scene(b200_device):
    import ospray_gb300 as og
    from ospray_gb300 import scenes
    d = scenes.pt_instanced_scene(levels=4, width=W, height=H)
    g = og.Scene(b200_device)
    scenes.build_pt_scene(g, d)
    g.set_lights([og.quad_light(L["position"], L["edge1"], L["edge2"], L["intensity"]) if L["type"] == "quad"
                  else og.ambient_light(L["intensity"]) for L in d["lights"]])
    o = oracle.Scene()
    scenes.build_pt_scene(o, d)
    mats = _materials(og, len(d["xfm"])) + [(0.8, 0.8, 0.8, 1.0, 0.0)]
    return d, g, o, mats


def test_every_material_type_matches_oracle(mat_scene, b200_device):
    import ospray_gb300 as og
    d, g, o, mats = mat_scene
    gpu, ref = _render(og, b200_device, g, o, d, mats, spp=4)
    _compare(gpu, ref, 0.995)


def test_material_accumulation_matches_oracle(mat_scene, b200_device):
    import ospray_gb300 as og
    d, g, o, mats = mat_scene
    gpu, ref = _render(og, b200_device, g, o, d, mats, spp=1, frames=3, maxlen=8, rr=2, pf=0)
    _compare(gpu, ref, 0.995)


def test_transparent_shadows_match_oracle(b200_device):
    """Cut-out, filtering and thin-glass panels between the light and the
    ground: shadow rays continue through them, attenuated by each surface's
    transparency."""
    import ospray_gb300 as og
    quad_v = np.array([[-1, 0, -1], [1, 0, -1], [-1, 0, 1], [1, 0, 1]], np.float32)
    quad_i = np.array([[0, 2, 1], [1, 2, 3]], np.uint32)
    ground_v = np.array([[-6, 0, -6], [6, 0, -6], [-6, 0, 6], [6, 0, 6]], np.float32)
    panels = [(-2.2, 2.0), (0.0, 2.5), (2.2, 3.0)]

    def build(s):
        gq = s.add_mesh(quad_v, quad_i)
        for k, (x, y) in enumerate(panels):
            s.add_instance(gq, k, 0, np.array([[1.5, 0, 0, x], [0, 1, 0, y], [0, 0, 1.5, 0.0]], np.float32), k)
        s.add_instance(s.add_mesh(ground_v, quad_i), len(panels), 0, None, len(panels))
        s.commit()
    g, o = og.Scene(b200_device), oracle.Scene()
    build(g)
    build(o)
    lights = [dict(type="quad", position=(-3.0, 6.0, -1.0), edge1=(6.0, 0.0, 0.0), edge2=(0.0, 0.0, 2.0),
                   intensity=8.0), dict(type="ambient", intensity=0.05)]
    g.set_lights([og.quad_light(L["position"], L["edge1"], L["edge2"], L["intensity"]) if L["type"] == "quad"
                  else og.ambient_light(L["intensity"]) for L in lights])
    mats = [og.principled((0.9, 0.2, 0.2), 0.6, 0.0, 0.3),
            og.obj_material(kd=(0.1, 0.1, 0.1), d=0.5, tf=(0.2, 0.8, 0.3)),
            og.thin_glass(eta=1.4, attenuation_color=(0.5, 0.6, 0.95), thickness=0.5),
            (0.8, 0.8, 0.8, 1.0, 0.0)]
    d = dict(camera=dict(position=(0.0, 7.0, -7.0), direction=(0.0, -7.0, 6.0), up=(0, 1, 0), fovy=55.0,
                         aspect=W / H), lights=lights)
    gpu, ref = _render(og, b200_device, g, o, d, mats, spp=8, maxlen=4)
    _compare(gpu, ref, 0.995)
    # the panels' shadows are partial: the ground under them is lit, but less than in the open
    assert ref["color"][..., :3].mean() > 0.01


def test_ospray_api_materials_render_like_the_abi(b200_device):
    """"obj", "metal", "glass" and "thinGlass" objects made through
    libospray.so give the same image as the same parameters through
    b200_render_pt."""
    import ospray_gb300 as og
    from ospray_gb300 import osp, scenes
    L = osp.lib()
    cur = L.ospGetCurrentDevice()
    own = cur is None
    if own:
        assert L.ospInit(None, None) == 0
    else:
        L.ospDeviceRelease(cur)
    try:
        _api_vs_abi(og, osp, scenes, b200_device)
    finally:
        if own:
            L.ospShutdown()


def _api_vs_abi(og, osp, scenes, b200_device):
    d = scenes.pt_instanced_scene(levels=3, count=8, width=96, height=64)
    api_mats = [("obj", dict(kd=(0.5, 0.4, 0.2), ks=(0.3, 0.3, 0.3), ns=25.0, d=0.7, tf=(0.2, 0.1, 0.0))),
                ("metal", dict(roughness=0.25)), ("glass", dict(eta=1.45, attenuationColor=(0.9, 0.6, 0.3))),
                ("thinGlass", dict(eta=1.5, attenuationColor=(0.6, 0.9, 0.7), thickness=0.3))]
    abi_mats = [og.obj_material(kd=(0.5, 0.4, 0.2), ks=(0.3, 0.3, 0.3), ns=25.0, d=0.7, tf=(0.2, 0.1, 0.0)),
                og.metal(roughness=0.25), og.glass(eta_inside=1.45, attenuation_color=(0.9, 0.6, 0.3)),
                og.thin_glass(eta=1.5, attenuation_color=(0.6, 0.9, 0.7), thickness=0.3)]
    app = osp.PathTracerApp(d, spp=2, max_path_length=6, roulette_path_length=3, width=96, height=64,
                            materials=[api_mats[k % 4] for k in range(8)])
    app.frame()
    api_img = app.color.copy()
    app.release()
    g = og.Scene(b200_device)
    scenes.build_pt_scene(g, d)
    g.set_lights([og.quad_light(Lt["position"], Lt["edge1"], Lt["edge2"], Lt["intensity"]) if Lt["type"] == "quad"
                  else og.ambient_light(Lt["intensity"]) for Lt in d["lights"]])
    fb = og.Frame(b200_device, 96, 64, og.FB_COLOR | og.FB_ACCUM)
    c = d["camera"]
    og.render_pt(g, og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=96 / 64),
                 og.pt_params(spp=2, max_path_length=6, roulette_path_length=3),
                 og.materials_array([abi_mats[k % 4] for k in range(8)] + [d["materials"][-1]]), fb)
    abi_img = fb.read(og.FB_COLOR)
    assert abi_img[..., :3].mean() > 0.0
    np.testing.assert_allclose(api_img, abi_img, rtol=1e-5, atol=1e-6)


def test_principled_parameters_match_oracle(mat_scene, b200_device):
    """Principled's ior and specular (the dielectric coating), diffuse,
    edgeColor and specularMetallic, and roughness 0 (a smooth coating over
    Lambert and a smooth conductor: Dirac lobes, Principled.ispc:146-331,
    DielectricLayer.ih, Conductor.ih) against the oracle."""
    import ospray_gb300 as og
    d, g, o, _ = mat_scene
    kinds = [og.principled((0.7, 0.3, 0.2), 0.3, 0.0, ior=1.5, specular=0.7),
             og.principled((0.2, 0.5, 0.8), 0.0, 0.0, ior=1.45),
             og.principled((0.9, 0.6, 0.3), 0.0, 1.0, edge_color=(0.9, 0.5, 0.3)),
             og.principled((0.6, 0.6, 0.6), 0.25, 1.0, edge_color=(0.4, 0.8, 0.9), specular=0.4,
                           specular_metallic=False),
             og.principled((0.5, 0.8, 0.3), 0.5, 0.4, ior=2.0, diffuse=0.5),
             og.principled((0.8, 0.8, 0.2), 0.0, 0.0, ior=1.6, specular=0.0),
             og.principled((0.3, 0.7, 0.7), 0.15, 0.0, ior=1.3, opacity=0.6)]
    mats = [kinds[i % len(kinds)] for i in range(len(d["xfm"]))] + [(0.8, 0.8, 0.8, 1.0, 0.0)]
    gpu, ref = _render(og, b200_device, g, o, d, mats, spp=4)
    _compare(gpu, ref, 0.995)
