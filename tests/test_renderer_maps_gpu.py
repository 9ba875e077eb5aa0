"""The AO and SciVis renderers with surface attributes and renderer maps,
and the path tracer's maxDepth texture, on the GPU against the oracle.

* SciVis (render/scivis/surfaces.ih:44-84, lightAlpha.ispc:19-122): vertex
  colours as the default diffuse colour and opacity, vertex normals, obj
  map_kd (rgb x kd, alpha x d) looked up with the ray cone's footprint, and
  shadow / AO rays through surfaces whose map or vertex alpha lets light
  through;
* AO (AORenderer.ispc:23-149, surfaces.ispc:17-77): obj kd x map_kd x the
  vertex colour, opacity d x map alpha x vertex alpha, rays continuing
  through surfaces that are not opaque;
* every renderer: map_backplate behind the scene and map_maxDepth limiting
  the camera rays (Renderer.ispc:19-40, RendererRenderTaskFn.inl:40-72,
  PathTracer.ispc:189-192).
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

W, H = 128, 96
CAM = dict(position=(0.0, 2.2, -7.5), direction=(0.0, -0.9, 6.0), up=(0.0, 1.0, 0.0), fovy=50.0)


def _checker(n, cells, alpha, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:n, 0:n]
    on = ((x // (n // cells)) + (y // (n // cells))) % 2 == 0
    img = np.zeros((n, n, 4), np.uint8)
    img[..., 0] = np.where(on, 230, 40)
    img[..., 1] = np.where(on, 190, 90)
    img[..., 2] = np.where(on, 60, 200)
    img[..., :3] = np.clip(img[..., :3].astype(np.int64) + rng.integers(-20, 21, (n, n, 3)), 0, 255)
    img[..., 3] = np.where(on, 255, 70) if alpha else 255
    return img


def _sphere(nu=16, nv=10):
    th, ph = np.meshgrid(np.linspace(0, np.pi, nv + 1), np.linspace(0, 2 * np.pi, nu + 1), indexing="ij")
    n = np.stack([np.sin(th) * np.cos(ph), np.cos(th), np.sin(th) * np.sin(ph)], -1).reshape(-1, 3)
    idx = []
    for i in range(nv):
        for j in range(nu):
            a, b = i * (nu + 1) + j, i * (nu + 1) + j + 1
            idx += [[a, a + nu + 1, b], [b, a + nu + 1, b + nu + 1]]
    uv = np.stack([ph.reshape(-1) / (2 * np.pi), 1.0 - th.reshape(-1) / np.pi], -1).astype(np.float32)
    col = np.stack([0.5 + 0.5 * n[:, 0], 0.5 + 0.5 * n[:, 1], 0.6 - 0.3 * n[:, 2],
                    np.where(n[:, 1] > 0.3, 0.45, 1.0)], -1).astype(np.float32)
    return n.astype(np.float32), np.asarray(idx, np.uint32), n.astype(np.float32), col, uv


def _build(og, dev):
    ground_v = np.array([[-8, 0, -8], [8, 0, -8], [-8, 0, 8], [8, 0, 8]], np.float32)
    quad_i = np.array([[0, 2, 1], [1, 2, 3]], np.uint32)
    ground_t = np.array([[0, 0], [8, 0], [0, 8], [8, 8]], np.float32)
    sv, si, sn, sc, su = _sphere()
    panel_v = np.array([[-1, 0, -1], [1, 0, -1], [-1, 0, 1], [1, 0, 1]], np.float32)
    panel_t = np.array([[0, 0], [2, 0], [0, 2], [2, 2]], np.float32)

    def build(s, set_attr):
        g0 = s.add_mesh(ground_v, quad_i)
        set_attr(s, g0, None, None, ground_t)
        g1 = s.add_mesh(sv, si)
        set_attr(s, g1, sn, sc, su)
        g2 = s.add_mesh(panel_v, quad_i)
        set_attr(s, g2, None, None, panel_t)
        s.add_instance(g0, 0, 0, None, 0)
        s.add_instance(g1, 1, 0, np.array([[1.2, 0, 0, -1.2], [0, 1.2, 0, 1.2], [0, 0, 1.2, 0.5]], np.float32), 1)
        s.add_instance(g2, 2, 0, np.array([[1.3, 0, 0, 1.8], [0, 1, 0, 2.4], [0, 0, 1.3, -0.4]], np.float32), 2)
        s.commit()
    g, o = og.Scene(dev), oracle.Scene()
    build(g, lambda s, k, n, c, t: s.set_mesh_attributes(k, normal=n, color=c, texcoord=t))
    build(o, lambda s, k, n, c, t: oracle.set_mesh_attributes(s, k, normal=n, color=c, texcoord=t))
    return g, o


def _textures(og, dev):
    imgs = [(_checker(64, 8, False, 3), 1, dict()), (_checker(32, 4, True, 9), 0, dict(filter=1)),
            (np.random.default_rng(4).uniform(0, 255, (12, 20, 3)).astype(np.uint8), 3, dict())]
    gt = [og.Texture(dev, a, f, **kw) for a, f, kw in imgs]
    ot = [oracle.OrTexture(a, f, **kw) for a, f, kw in imgs]
    depth = np.full((6, 8), 40.0, np.float32)
    depth[2:4, 2:6] = 7.5  # a window where the camera rays stop before the ground's far part
    gt.append(og.Texture(dev, depth, og.TEX_R32F, filter=og.TEX_FILTER_NEAREST))
    ot.append(oracle.OrTexture(depth, 7, filter=1))
    return gt, ot


def _mats(tex):
    return [dict(kd=(1.0, 1.0, 1.0), ks=(0.2, 0.2, 0.2), ns=20.0, d=1.0, tf=(0, 0, 0), map_kd=tex[0]),
            None,
            dict(kd=(0.8, 0.7, 0.9), ks=(0, 0, 0), ns=10.0, d=0.9, tf=(0.1, 0.3, 0.1), map_kd=tex[1])]


def _compare(gc, rc, tol, min_close):
    close = np.all(np.abs(gc - rc) <= tol * np.maximum(1.0, np.abs(rc)), axis=2)
    print("pixels within %g: %.4f" % (tol, close.mean()))
    assert close.mean() >= min_close, close.mean()


@pytest.mark.parametrize("shadows", [False, True])
def test_scivis_attributes_and_maps_match_oracle(b200_device, shadows):
    import ospray_gb300 as og
    g, o = _build(og, b200_device)
    gt, ot = _textures(og, b200_device)
    lights = [dict(type="distant", direction=(0.3, -1.0, 0.5), intensity=2.0, color=(1.0, 0.95, 0.9)),
              dict(type="ambient", intensity=0.3)]
    g.set_lights([og.distant_light(lights[0]["direction"], intensity=2.0, color=lights[0]["color"]),
                  og.ambient_light(0.3)])
    cam = og.camera_desc(CAM["position"], CAM["direction"], CAM["up"], fovy=CAM["fovy"], aspect=W / H)
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_DEPTH | og.FB_ID_PRIMITIVE)
    og.render_scivis(g, cam, og.scivis_params(spp=2, shadows=shadows, ao_samples=2, ao_distance=3.0,
                                              backplate=gt[2], max_depth=gt[3], mip_map_bias=0.5),
                     fb, og.scivis_materials_array(_mats(gt)))
    ref = oracle.render_scivis(o, None, oracle.camera(CAM["position"], CAM["direction"], CAM["up"],
                                                      fovy=CAM["fovy"], aspect=W / H), lights, _mats(ot), W, H,
                               spp=2, shadows=shadows, ao_samples=2, ao_radius=3.0, backplate=ot[2],
                               max_depth=ot[3], mip_map_bias=0.5)
    assert np.mean(fb.read(og.FB_ID_PRIMITIVE) == ref["primID"]) >= 0.999
    depth = fb.read(og.FB_DEPTH)
    assert np.any(depth == np.float32(7.5))  # the maxDepth window
    assert np.mean(depth.view(np.uint32) == ref["depth"].view(np.uint32)) >= 0.999
    _compare(fb.read(og.FB_COLOR)[..., :3], ref["color"][..., :3], 1e-3, 0.995)
    for t in gt:
        t.release()


def test_ao_surface_colours_and_maps_match_oracle(b200_device):
    import ospray_gb300 as og
    g, o = _build(og, b200_device)
    gt, ot = _textures(og, b200_device)
    cam = og.camera_desc(CAM["position"], CAM["direction"], CAM["up"], fovy=CAM["fovy"], aspect=W / H)
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_DEPTH | og.FB_ID_PRIMITIVE | og.FB_ALBEDO)
    og.render_ao(g, cam, og.ao_params(spp=2, ao_samples=2, ao_distance=3.0, backplate=gt[2], max_depth=gt[3],
                                      mip_map_bias=0.5, materials=og.scivis_materials_array(_mats(gt))), fb)
    ref = oracle.render_ao(o, oracle.camera(CAM["position"], CAM["direction"], CAM["up"], fovy=CAM["fovy"],
                                            aspect=W / H), 2, W, H, spp=2, ao_samples=2, ao_radius=3.0,
                           backplate=ot[2], max_depth=ot[3], mip_map_bias=0.5, materials=_mats(ot))
    assert np.mean(fb.read(og.FB_ID_PRIMITIVE) == ref["primID"]) >= 0.999
    assert np.mean(fb.read(og.FB_DEPTH).view(np.uint32) == ref["depth"].view(np.uint32)) >= 0.999
    _compare(fb.read(og.FB_COLOR), ref["color"], 1e-4, 0.998)
    for t in gt:
        t.release()


def test_path_tracer_max_depth_matches_oracle(b200_device):
    import ospray_gb300 as og
    g, o = _build(og, b200_device)
    gt, ot = _textures(og, b200_device)
    lights = [dict(type="ambient", intensity=0.8)]
    g.set_lights([og.ambient_light(0.8)])
    mats = [og.principled((0.8, 0.6, 0.4), 0.5, 0.0), og.principled((0.3, 0.6, 0.9), 0.3, 0.0),
            og.principled((0.9, 0.9, 0.9), 0.6, 0.0)]
    cam = og.camera_desc(CAM["position"], CAM["direction"], CAM["up"], fovy=CAM["fovy"], aspect=W / H)
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_ACCUM | og.FB_DEPTH | og.FB_ID_PRIMITIVE)
    og.render_pt(g, cam, og.pt_params(spp=2, max_path_length=3, max_depth=gt[3], backplate=gt[2]),
                 og.materials_array(mats), fb)
    ref = oracle.render_pt(o, oracle.PtWorld(mats, lights),
                           oracle.camera(CAM["position"], CAM["direction"], CAM["up"], fovy=CAM["fovy"],
                                         aspect=W / H),
                           oracle.pt_params(spp=2, max_path_length=3, max_depth=ot[3], backplate=ot[2]), W, H)
    assert np.mean(fb.read(og.FB_ID_PRIMITIVE) == ref["primID"]) >= 0.999
    depth = fb.read(og.FB_DEPTH)
    assert np.any(depth == np.float32(7.5))
    assert np.mean(depth.view(np.uint32) == ref["depth"].view(np.uint32)) >= 0.999
    _compare(fb.read(og.FB_ACCUM)[..., :3], ref["color"][..., :3], 1e-3, 0.995)
    for t in gt:
        t.release()
