"""Normal and albedo framebuffer channels (OSP_FB_NORMAL / OSP_FB_ALBEDO,
accumulated like colour by LocalFB_accumulateSample fb/LocalFB.ispc:61-67)
against the oracle: AO (first hit's Ns and the surface colour, the ray
direction and background on a miss, render/ao/AORenderer.ispc:108-133),
SciVis (the first non-transparent hit's Ns and BSDF albedo,
render/scivis/SciVis.ispc:165-180) and the path tracer
(updateAuxilliaryData at the first smooth vertex,
render/pathtracer/PathTracerUtil.ih:48-60)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

W, H = 96, 64


def _chans():
    import ospray_gb300 as og
    return og.FB_COLOR | og.FB_ACCUM | og.FB_NORMAL | og.FB_ALBEDO | og.FB_ID_PRIMITIVE


@pytest.fixture(scope="module")
def pt_world(b200_device):
    import ospray_gb300 as og
    from ospray_gb300 import scenes
    d = scenes.pt_instanced_scene(levels=3, width=W, height=H)
    g = og.Scene(b200_device)
    scenes.build_pt_scene(g, d)
    g.set_lights([og.light_from_dict(L) for L in d["lights"]])
    o = oracle.Scene()
    scenes.build_pt_scene(o, d)
    return d, g, o


def _cams(d):
    import ospray_gb300 as og
    c = d["camera"]
    return (og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"]),
            oracle.camera(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"]))


def test_ao_normal_albedo_match_oracle(pt_world, b200_device):
    import ospray_gb300 as og
    d, g, o = pt_world
    cam, ocam = _cams(d)
    fb = og.Frame(b200_device, W, H, _chans())
    for _ in range(2):
        og.render_ao(g, cam, og.ao_params(spp=2, bg=(0.2, 0.3, 0.4, 1.0)), fb)
    with oracle.AuxOutput(W, H) as aux:
        oracle.render_ao(o, ocam, 2, W, H, spp=2, bg=(0.2, 0.3, 0.4, 1.0), frames=2)
    n, a = fb.read(og.FB_NORMAL), fb.read(og.FB_ALBEDO)
    assert np.abs(aux.normal).max() > 0.5 and (aux.albedo > 0.99).any() and (np.abs(aux.albedo - 0.3) < 1e-6).any()
    np.testing.assert_allclose(n, aux.normal, atol=1e-5)
    np.testing.assert_allclose(a, aux.albedo, atol=1e-5)


def test_pt_normal_albedo_match_oracle(pt_world, b200_device):
    import ospray_gb300 as og
    d, g, o = pt_world
    cam, ocam = _cams(d)
    fb = og.Frame(b200_device, W, H, _chans())
    p = og.pt_params(spp=4, max_path_length=3)
    for _ in range(2):
        og.render_pt(g, cam, p, og.materials_array(d["materials"]), fb)
    with oracle.AuxOutput(W, H) as aux:
        oracle.render_pt(o, oracle.PtWorld(d["materials"], d["lights"]), ocam,
                         oracle.pt_params(spp=4, max_path_length=3), W, H, frames=2)
    n, a = fb.read(og.FB_NORMAL), fb.read(og.FB_ALBEDO)
    assert np.abs(aux.normal).max() > 0.5 and aux.albedo.max() > 0.1
    close_n = np.all(np.abs(n - aux.normal) <= 1e-4, axis=2)
    close_a = np.all(np.abs(a - aux.albedo) <= 1e-4, axis=2)
    assert close_n.mean() >= 0.999 and close_a.mean() >= 0.999, (close_n.mean(), close_a.mean())


def test_scivis_normal_albedo_match_oracle(pt_world, b200_device):
    import ospray_gb300 as og
    d, g, o = pt_world
    cam, ocam = _cams(d)
    mats = [dict(kd=(0.7, 0.6, 0.5), ks=(0.2, 0.2, 0.2), ns=16.0)]
    fb = og.Frame(b200_device, W, H, _chans())
    og.render_scivis(g, cam, og.scivis_params(spp=2), fb, og.scivis_materials_array(mats))
    with oracle.AuxOutput(W, H) as aux:
        oracle.render_scivis(o, None, ocam, d["lights"], mats, W, H, spp=2)
    n, a = fb.read(og.FB_NORMAL), fb.read(og.FB_ALBEDO)
    assert np.abs(aux.normal).max() > 0.5 and aux.albedo.max() > 0.5
    np.testing.assert_allclose(n, aux.normal, atol=1e-5)
    np.testing.assert_allclose(a, aux.albedo, atol=1e-5)
