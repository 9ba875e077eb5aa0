"""Instance motion blur and the camera shutter on the GPU against the oracle.

A key-framed instance (MotionTransform "motion.transform" / "time",
common/MotionTransform.cpp:10-66) is seen by each ray under the two keys
around the ray's time blended component-wise; the path tracer draws the
camera sample's time from its own sample stream over an open shutter
(PathTracer.ispc:177-180, Camera_shutterTime camera/Camera.ih:33-42), the
AO renderer takes the shutter time of 0.5, which a rolling shutter spreads
over the screen.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

W, H = 128, 96
CAM = dict(position=(0.0, 2.5, -8.0), direction=(0.0, -1.0, 7.0), up=(0.0, 1.0, 0.0), fovy=50.0)


def _sphere(nu=24, nv=14):
    th, ph = np.meshgrid(np.linspace(0, np.pi, nv + 1), np.linspace(0, 2 * np.pi, nu + 1), indexing="ij")
    v = np.stack([np.sin(th) * np.cos(ph), np.cos(th), np.sin(th) * np.sin(ph)], -1).reshape(-1, 3)
    idx = []
    for i in range(nv):
        for j in range(nu):
            a, b = i * (nu + 1) + j, i * (nu + 1) + j + 1
            idx += [[a, a + nu + 1, b], [b, a + nu + 1, b + nu + 1]]
    return v.astype(np.float32), np.asarray(idx, np.uint32)


def _keys():
    # three keys: moving right and up, turning about y, growing
    ks = []
    for k, (tx, ty, ang, s) in enumerate([(-1.5, 1.0, 0.0, 1.0), (0.0, 1.6, 0.6, 1.2), (1.6, 1.1, 1.3, 0.9)]):
        c, sn = np.cos(ang), np.sin(ang)
        ks.append(np.array([[s * c, 0, s * sn, tx], [0, s, 0, ty], [-s * sn, 0, s * c, 1.0]], np.float32))
    return np.stack(ks)


def _build(scene, motion, static_key=None):
    ground_v = np.array([[-8, 0, -8], [8, 0, -8], [-8, 0, 8], [8, 0, 8]], np.float32)
    quad_i = np.array([[0, 2, 1], [1, 2, 3]], np.uint32)
    sv, si = _sphere()
    g0 = scene.add_mesh(ground_v, quad_i)
    g1 = scene.add_mesh(sv, si)
    g2 = scene.add_spheres(np.array([[2.5, 0.6, 2.0, 0.6], [-2.6, 0.5, 1.5, 0.5]], np.float32))
    scene.add_instance(g0, 0, 0, None, 0)
    if static_key is not None:
        scene.add_instance(g1, 1, 0, _keys()[static_key], 1)
    elif motion:
        scene.add_instance_motion(g1, 1, 0, _keys(), (0.0, 1.0), 1)
    scene.add_instance_motion(g2, 2, 0, _keys()[:2] * np.array([1, 1, 1, 0.5], np.float32), (0.2, 0.8), 2)
    scene.commit()


MATS = [((0.8, 0.8, 0.75), 1.0, 0.0), ((0.9, 0.3, 0.2), 0.4, 0.0), ((0.2, 0.6, 0.9), 0.3, 1.0)]
LIGHTS = [dict(type="quad", position=(-1.0, 7.0, -2.0), edge1=(3.0, 0.0, 0.0), edge2=(0.0, 0.0, 3.0),
               intensity=6.0), dict(type="ambient", intensity=0.2)]


def _material_dicts():
    import ospray_gb300 as og
    return [og.principled(c, r, m) for c, r, m in MATS]


def _materials(og):
    return og.materials_array(_material_dicts())


def _pt(og, dev, shutter, spp=4, static_key=None, shutter_type=0, duration=0.0):
    g = og.Scene(dev)
    _build(g, True, static_key)
    g.set_lights([og.quad_light(L["position"], L["edge1"], L["edge2"], L["intensity"]) if L["type"] == "quad"
                  else og.ambient_light(L["intensity"]) for L in LIGHTS])
    fb = og.Frame(dev, W, H, og.FB_COLOR | og.FB_ACCUM | og.FB_ID_PRIMITIVE | og.FB_ID_INSTANCE | og.FB_DEPTH)
    cam = og.camera_desc(CAM["position"], CAM["direction"], CAM["up"], fovy=CAM["fovy"], aspect=W / H,
                         shutter=shutter, shutter_type=shutter_type, rolling_shutter_duration=duration)
    og.render_pt(g, cam, og.pt_params(spp=spp, max_path_length=4, roulette_path_length=3), _materials(og), fb)
    return dict(color=fb.read(og.FB_ACCUM), primID=fb.read(og.FB_ID_PRIMITIVE),
                instID=fb.read(og.FB_ID_INSTANCE), depth=fb.read(og.FB_DEPTH))


def _pt_oracle(shutter, spp=4, shutter_type=0, duration=0.0):
    o = oracle.Scene()
    _build(o, True)
    world = oracle.PtWorld(_material_dicts(), LIGHTS)
    cam = oracle.camera(CAM["position"], CAM["direction"], CAM["up"], fovy=CAM["fovy"], aspect=W / H,
                        shutter=shutter, shutter_type=shutter_type, rolling_shutter_duration=duration)
    return oracle.render_pt(o, world, cam, oracle.pt_params(spp=spp, max_path_length=4, roulette_path_length=3),
                            W, H)


def test_motion_blurred_path_tracer_matches_oracle(b200_device):
    import ospray_gb300 as og
    gpu = _pt(og, b200_device, (0.0, 1.0))
    ref = _pt_oracle((0.0, 1.0))
    assert np.mean(gpu["primID"] == ref["primID"]) >= 0.999
    g, r = gpu["color"][..., :3], ref["color"][..., :3]
    close = np.all(np.abs(g - r) <= 2e-3 * np.maximum(1.0, np.abs(r)), axis=2)
    diff = (g - r).reshape(-1)
    se = diff.std() / np.sqrt(diff.size)
    assert close.mean() >= 0.99, close.mean()
    assert abs(diff.mean()) <= 3 * se + 1e-6, (diff.mean(), se)
    # the blur is there: the moving sphere shows in pixels where the middle key does not put it
    still = _pt(og, b200_device, (0.5, 0.5))["instID"] == 1
    assert np.sum((gpu["instID"] == 1) & ~still) > 10


@pytest.mark.parametrize("t,key", [(0.0, 0), (1.0, 2), (0.5, 1)])
def test_closed_shutter_at_a_key_renders_the_static_key(b200_device, t, key):
    """At a key's time the blend is that key exactly, so the image equals the
    one of a static instance under that key (bit for bit)."""
    import ospray_gb300 as og
    a = _pt(og, b200_device, (t, t))
    b = _pt(og, b200_device, (t, t), static_key=key)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.parametrize("shutter_type", [1, 4])
def test_rolling_shutter_ao_matches_oracle(b200_device, shutter_type):
    import ospray_gb300 as og
    dev = b200_device
    g, o = og.Scene(dev), oracle.Scene()
    _build(g, True)
    _build(o, True)
    cam = dict(CAM, aspect=W / H)
    kw = dict(shutter=(0.1, 0.9), shutter_type=shutter_type, rolling_shutter_duration=0.3)
    fb = og.Frame(dev, W, H, og.FB_COLOR | og.FB_ACCUM | og.FB_DEPTH | og.FB_ID_PRIMITIVE | og.FB_ID_INSTANCE)
    og.render_ao(g, og.camera_desc(cam["position"], cam["direction"], cam["up"], fovy=cam["fovy"],
                                   aspect=cam["aspect"], **kw), og.ao_params(spp=2, ao_samples=2), fb)
    ref = oracle.render_ao(o, oracle.camera(cam["position"], cam["direction"], cam["up"], fovy=cam["fovy"],
                                            aspect=cam["aspect"], **kw), 2, W, H, spp=2, ao_samples=2)
    np.testing.assert_array_equal(fb.read(og.FB_ID_PRIMITIVE), ref["primID"])
    np.testing.assert_array_equal(fb.read(og.FB_ID_INSTANCE), ref["instID"])
    np.testing.assert_array_equal(fb.read(og.FB_DEPTH), ref["depth"])
    close = np.all(np.abs(fb.read(og.FB_ACCUM) - ref["color"]) <= 1e-5, axis=2)
    assert close.mean() >= 0.999, close.mean()
