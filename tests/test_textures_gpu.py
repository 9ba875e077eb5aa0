"""Textures and vertex attributes: the GPU against the oracle's restatement.

* MIP chains (MipMap_generate, texture/MipMapGeneration.ispc; level sizes
  Texture2D.cpp:97-135) for every supported format on odd, even and
  one-dimensional sizes: bit-identical texels, but for the sRGB formats,
  whose transfer curve goes through pow (CUDA and the host libm may differ in
  the last ulp, so a byte may round the other way);
* lookups (Texture2D_get, texture/Texture2D.ispc:13-164): wrap modes,
  nearest / bilinear filters, level selection from the pixel footprint with
  trilinear blending, at random texture coordinates;
* the path tracer with colour maps (principled map_baseColor, obj map_kd with
  alpha: cut-outs and transparent shadows), per-vertex normals, colours and
  texture coordinates (TriangleMesh_postIntersect geometry/Mesh.ispc:
  178-276), ray cones (World.ih:458-464) selecting MIP levels on a ground
  plane seen at a grazing angle, mipMapBias, and a backplate
  (Renderer.ispc:19-29) behind the scene.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

FORMATS = {  # format -> (channels, dtype)
    0: (4, np.uint8), 1: (4, np.uint8), 2: (4, np.float32), 3: (3, np.uint8), 4: (3, np.uint8),
    5: (3, np.float32), 6: (1, np.uint8), 7: (1, np.float32), 8: (1, np.uint8), 9: (2, np.uint8),
    10: (2, np.uint8), 11: (4, np.uint16), 12: (3, np.uint16), 13: (2, np.uint16), 14: (1, np.uint16),
    15: (2, np.float32)}
SRGB_FORMATS = {1, 4, 8, 10}


def _texels(rng, h, w, fmt):
    c, dt = FORMATS[fmt]
    shape = (h, w) if c == 1 else (h, w, c)
    if dt == np.float32:
        return rng.uniform(0.0, 2.0, shape).astype(np.float32)
    hi = 256 if dt == np.uint8 else 65536
    return rng.integers(0, hi, shape).astype(dt)


@pytest.mark.parametrize("fmt", sorted(FORMATS))
def test_mip_chain_matches_oracle(b200_device, fmt):
    import ospray_gb300 as og
    rng = np.random.default_rng(100 + fmt)
    for (h, w) in [(20, 37), (16, 16), (9, 1), (1, 6)]:
        data = _texels(rng, h, w, fmt)
        gt = og.Texture(b200_device, data, fmt)
        ot = oracle.OrTexture(data, fmt)
        assert gt.levels == ot.levels
        for lv in range(ot.levels):
            a, b = gt.read_level(lv), ot.read_level(lv)
            if fmt in SRGB_FORMATS:
                assert np.abs(a.astype(np.int64) - b.astype(np.int64)).max() <= 1, (fmt, h, w, lv)
            else:
                np.testing.assert_array_equal(a, b, err_msg="format %d size %dx%d level %d" % (fmt, w, h, lv))
        gt.release()


@pytest.mark.parametrize("filt", [0, 1])
@pytest.mark.parametrize("wrap", [(0, 0), (1, 2), (2, 1)])
def test_texture_lookups_match_oracle(b200_device, filt, wrap):
    import ospray_gb300 as og
    rng = np.random.default_rng(7)
    for fmt in (0, 2, 4, 11):
        data = _texels(rng, 24, 40, fmt)
        gt = og.Texture(b200_device, data, fmt, filter=filt, wrap=wrap)
        ot = oracle.OrTexture(data, fmt, filter=filt, wrap=wrap)
        st = rng.uniform(-2.0, 3.0, (4000, 2)).astype(np.float32)
        fp = np.where(rng.uniform(size=4000) < 0.3, 0.0, rng.uniform(0.0, 0.6, 4000)).astype(np.float32)
        a, b = gt.sample(st, fp), ot.sample(st, fp)
        err = np.abs(a - b).max(axis=1)
        # nearest lookups at a texel border may land on either side after a
        # last-ulp difference in the blend; everything else agrees to 1e-5
        scale = np.maximum(1.0, np.abs(b).max(axis=1))
        assert np.mean(err <= 1e-5 * scale) >= (0.999 if filt else 0.995), (fmt, filt, wrap)
        assert np.mean(err) < 1e-3
        gt.release()


W, H = 160, 96


def _checker(n=64, cells=8, alpha=False, seed=3):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:n, 0:n]
    on = ((x // (n // cells)) + (y // (n // cells))) % 2 == 0
    img = np.zeros((n, n, 4), np.uint8)
    img[..., 0] = np.where(on, 230, 40)
    img[..., 1] = np.where(on, 200, 90)
    img[..., 2] = np.where(on, 60, 180)
    img[..., :3] = np.clip(img[..., :3].astype(np.int64) + rng.integers(-20, 21, (n, n, 3)), 0, 255)
    img[..., 3] = np.where(on, 255, 60) if alpha else 255
    return img


def _sphere_mesh(nu=16, nv=10, r=1.0):
    th, ph = np.meshgrid(np.linspace(0, np.pi, nv + 1), np.linspace(0, 2 * np.pi, nu + 1), indexing="ij")
    n = np.stack([np.sin(th) * np.cos(ph), np.cos(th), np.sin(th) * np.sin(ph)], -1).reshape(-1, 3)
    v = (n * r).astype(np.float32)
    idx = []
    for i in range(nv):
        for j in range(nu):
            a, b = i * (nu + 1) + j, i * (nu + 1) + j + 1
            c, d = a + nu + 1, b + nu + 1
            idx += [[a, c, b], [b, c, d]]
    uv = np.stack([ph.reshape(-1) / (2 * np.pi), 1.0 - th.reshape(-1) / np.pi], -1).astype(np.float32)
    col = np.stack([0.5 + 0.5 * n[:, 0], 0.5 + 0.5 * n[:, 1], 0.6 - 0.3 * n[:, 2], np.ones(len(n))], -1)
    return v, np.asarray(idx, np.uint32), n.astype(np.float32), col.astype(np.float32), uv


def _scene(og, dev, obj_cutout):
    """A textured ground (texture coordinates repeating 8 times), a smooth
    sphere with vertex normals, colours and texture coordinates, and a cut-out
    panel (map with alpha) between the light and the ground."""
    ground_v = np.array([[-8, 0, -8], [8, 0, -8], [-8, 0, 8], [8, 0, 8]], np.float32)
    ground_i = np.array([[0, 2, 1], [1, 2, 3]], np.uint32)
    ground_t = np.array([[0, 0], [8, 0], [0, 8], [8, 8]], np.float32)
    sv, si, sn, sc, su = _sphere_mesh()
    panel_v = np.array([[-1, 0, -1], [1, 0, -1], [-1, 0, 1], [1, 0, 1]], np.float32)
    panel_t = np.array([[0, 0], [2, 0], [0, 2], [2, 2]], np.float32)

    def build(s, set_attr):
        g0 = s.add_mesh(ground_v, ground_i)
        set_attr(s, g0, None, None, ground_t)
        g1 = s.add_mesh(sv, si)
        set_attr(s, g1, sn, sc, su)
        g2 = s.add_mesh(panel_v, ground_i)
        set_attr(s, g2, None, None, panel_t)
        s.add_instance(g0, 0, 0, None, 0)
        s.add_instance(g1, 1, 0, np.array([[1.2, 0, 0, -1.2], [0, 1.2, 0, 1.2], [0, 0, 1.2, 0.5]], np.float32), 1)
        s.add_instance(g2, 2, 0, np.array([[1.3, 0, 0, 1.8], [0, 1, 0, 2.4], [0, 0, 1.3, -0.4]], np.float32), 2)
        s.commit()

    g, o = og.Scene(dev), oracle.Scene()
    build(g, lambda s, k, n, c, t: s.set_mesh_attributes(k, normal=n, color=c, texcoord=t))
    build(o, lambda s, k, n, c, t: oracle.set_mesh_attributes(s, k, normal=n, color=c, texcoord=t))
    lights = [dict(type="quad", position=(-1.0, 7.0, -2.5), edge1=(3.0, 0.0, 0.0), edge2=(0.0, 0.0, 3.0),
                   intensity=6.0), dict(type="ambient", intensity=0.15)]
    g.set_lights([og.quad_light(L["position"], L["edge1"], L["edge2"], L["intensity"]) if L["type"] == "quad"
                  else og.ambient_light(L["intensity"]) for L in lights])
    return g, o, lights


def _render_both(og, dev, g, o, lights, mats_g, mats_o, spp=4, maxlen=5, bias=0.0, backplate=None, fmt_bp=3):
    cam = dict(position=(0.0, 2.2, -7.5), direction=(0.0, -0.9, 6.0), up=(0, 1, 0), fovy=50.0, aspect=W / H)
    fb = og.Frame(dev, W, H, og.FB_COLOR | og.FB_ACCUM | og.FB_ID_PRIMITIVE)
    gbp = og.Texture(dev, backplate, fmt_bp) if backplate is not None else None
    obp = oracle.OrTexture(backplate, fmt_bp) if backplate is not None else None
    og.render_pt(g, og.camera_desc(cam["position"], cam["direction"], cam["up"], fovy=cam["fovy"], aspect=cam["aspect"]),
                 og.pt_params(spp=spp, max_path_length=maxlen, roulette_path_length=3, mip_map_bias=bias,
                              backplate=gbp), og.materials_array(mats_g), fb)
    gpu = dict(color=fb.read(og.FB_ACCUM), primID=fb.read(og.FB_ID_PRIMITIVE))
    ow = oracle.PtWorld(mats_o, lights)
    ref = oracle.render_pt(o, ow, oracle.camera(cam["position"], cam["direction"], cam["up"], fovy=cam["fovy"],
                                                 aspect=cam["aspect"]),
                           oracle.pt_params(spp=spp, max_path_length=maxlen, roulette_path_length=3,
                                            mip_map_bias=bias, backplate=obp), W, H)
    if gbp is not None:
        gbp.release()
    return gpu, ref


def _compare(gpu, ref, min_close=0.99):
    assert np.mean(gpu["primID"] == ref["primID"]) >= 0.9995
    g, r = gpu["color"][..., :3], ref["color"][..., :3]
    assert np.isfinite(g).all()
    close = np.all(np.abs(g - r) <= 2e-3 * np.maximum(1.0, np.abs(r)), axis=2)
    diff = (g - r).reshape(-1)
    se = diff.std() / np.sqrt(diff.size)
    print("pixels within 2e-3: %.4f  mean gpu %.5f oracle %.5f (se %.2e)" % (close.mean(), g.mean(), r.mean(), se))
    assert close.mean() >= min_close, close.mean()
    assert abs(diff.mean()) <= 3 * se + 1e-6, (diff.mean(), se)
    np.testing.assert_allclose(gpu["color"][..., 3], ref["color"][..., 3], atol=3e-3)


@pytest.mark.parametrize("bias", [0.0, 1.5])
def test_textured_principled_scene_matches_oracle(b200_device, bias):
    import ospray_gb300 as og
    g, o, lights = _scene(og, b200_device, False)
    img = _checker()
    gt_g, gt_o = og.Texture(b200_device, img, og.TEX_SRGBA), oracle.OrTexture(img, 1)
    sph = _checker(32, 4, seed=5)
    st_g, st_o = og.Texture(b200_device, sph, og.TEX_RGBA8, filter=og.TEX_FILTER_NEAREST), \
        oracle.OrTexture(sph, 0, filter=1)
    panel = _checker(32, 4, alpha=True, seed=9)
    pt_g, pt_o = og.Texture(b200_device, panel, og.TEX_RGBA8), oracle.OrTexture(panel, 0)
    mg = [og.principled((1.0, 1.0, 1.0), 0.4, 0.0, base_color_map=gt_g),
          og.principled((0.9, 0.9, 0.9), 0.3, 0.0, base_color_map=st_g),
          og.principled((1.0, 0.8, 0.8), 0.5, 0.0, base_color_map=pt_g)]
    mo = [dict(m, baseColorMap=t) for m, t in zip(mg, (gt_o, st_o, pt_o))]
    bp = (np.random.default_rng(4).uniform(0, 255, (12, 20, 3))).astype(np.uint8)
    gpu, ref = _render_both(og, b200_device, g, o, lights, mg, mo, bias=bias, backplate=bp)
    _compare(gpu, ref)
    # the backplate shows where the camera sees no geometry
    assert (ref["primID"] == 0xffffffff).mean() > 0.05
    for t in (gt_g, st_g, pt_g):
        t.release()


def test_textured_obj_cutout_scene_matches_oracle(b200_device):
    """obj map_kd with alpha: d follows the map's alpha (cut-out), shadow
    rays pass the transparent texels; the sphere's vertex colours scale kd."""
    import ospray_gb300 as og
    g, o, lights = _scene(og, b200_device, True)
    img = _checker(64, 8, alpha=True, seed=11)
    t_g, t_o = og.Texture(b200_device, img, og.TEX_RGBA8, wrap=og.TEX_WRAP_MIRRORED_REPEAT), \
        oracle.OrTexture(img, 0, wrap=1)
    mg = [og.obj_material(kd=(0.9, 0.9, 0.9), ks=(0.1, 0.1, 0.1), ns=20.0, map_kd=t_g),
          og.obj_material(kd=(0.8, 0.8, 0.8)),
          og.obj_material(kd=(0.7, 0.7, 0.9), d=0.9, tf=(0.1, 0.3, 0.1), map_kd=t_g)]
    mo = [dict(m, baseColorMap=(t_o if m.get("baseColorMap") is not None else None)) for m in mg]
    gpu, ref = _render_both(og, b200_device, g, o, lights, mg, mo, spp=6)
    _compare(gpu, ref)
    t_g.release()


def test_vertex_colour_alpha_makes_obj_shadows_transparent(b200_device):
    """Vertex colours with alpha < 1 under an obj material scale its d: the
    sphere's shadow lightens, as in the oracle."""
    import ospray_gb300 as og
    ground_v = np.array([[-8, 0, -8], [8, 0, -8], [-8, 0, 8], [8, 0, 8]], np.float32)
    ground_i = np.array([[0, 2, 1], [1, 2, 3]], np.uint32)
    sv, si, sn, sc, _ = _sphere_mesh()
    sc[:, 3] = 0.3 + 0.4 * (sv[:, 1] > 0)

    def build(s, set_attr):
        s.add_instance(s.add_mesh(ground_v, ground_i), 0, 0, None, 0)
        k = s.add_mesh(sv, si)
        set_attr(s, k, sn, sc)
        s.add_instance(k, 1, 0, np.array([[1, 0, 0, 0], [0, 1, 0, 1.5], [0, 0, 1, 0]], np.float32), 1)
        s.commit()
    g, o = og.Scene(b200_device), oracle.Scene()
    build(g, lambda s, k, n, c: s.set_mesh_attributes(k, normal=n, color=c))
    build(o, lambda s, k, n, c: oracle.set_mesh_attributes(s, k, normal=n, color=c))
    lights = [dict(type="quad", position=(-0.5, 6.0, -0.5), edge1=(1.0, 0.0, 0.0), edge2=(0.0, 0.0, 1.0),
                   intensity=20.0)]
    g.set_lights([og.quad_light(L["position"], L["edge1"], L["edge2"], L["intensity"]) for L in lights])
    mats = [og.obj_material(kd=(0.8, 0.8, 0.8)), og.obj_material(kd=(0.9, 0.6, 0.3))]
    gpu, ref = _render_both(og, b200_device, g, o, lights, mats, mats, spp=4, maxlen=3)
    _compare(gpu, ref)


def test_textures_refused_by_batch(b200_device):
    import ospray_gb300 as og
    g = og.Scene(b200_device)
    g.add_instance(g.add_mesh(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32),
                              np.array([[0, 1, 2]], np.uint32)), 0, 0, None, 0)
    g.commit()
    t = og.Texture(b200_device, _checker(8, 2), og.TEX_RGBA8)
    b = og.Batch(b200_device)
    fb = og.Frame(b200_device, 8, 8, og.FB_COLOR)
    cam = og.camera_desc((0, 0, -3), (0, 0, 1), (0, 1, 0))
    with pytest.raises(og.B200Error):
        b.add_pt(g, cam, og.pt_params(), og.materials_array([og.principled(base_color_map=t)]), fb)
    t.release()


def test_ospray_api_textures_render_like_the_abi(b200_device):
    """texture2d objects, map_baseColor / map_kd, vertex.normal / color /
    texcoord and the renderer's map_backplate / mipMapBias made through
    libospray.so give the image the same inputs give through the b200 ABI."""
    import ospray_gb300 as og
    from ospray_gb300 import osp
    L = osp.lib()
    cur = L.ospGetCurrentDevice()
    own = cur is None
    if own:
        assert L.ospInit(None, None) == 0
    else:
        L.ospDeviceRelease(cur)
    try:
        _api_textures(og, osp, b200_device)
    finally:
        if own:
            L.ospShutdown()


def _api_textures(og, osp, dev):
    L = osp.lib()
    keep = []
    w, h = 96, 64
    ground_v = np.array([[-8, 0, -8], [8, 0, -8], [-8, 0, 8], [8, 0, 8]], np.float32)
    ground_i = np.array([[0, 2, 1], [1, 2, 3]], np.uint32)
    ground_t = np.array([[0, 0], [8, 0], [0, 8], [8, 8]], np.float32)
    sv, si, sn, sc, su = _sphere_mesh()
    img, sph, bp = _checker(), _checker(32, 4, alpha=True, seed=5), _checker(16, 2, seed=8)[..., :3].copy()
    cam = dict(position=(0.0, 2.2, -7.5), direction=(0.0, -0.9, 6.0), up=(0.0, 1.0, 0.0), fovy=50.0)
    quad = dict(position=(-1.0, 7.0, -2.5), edge1=(3.0, 0.0, 0.0), edge2=(0.0, 0.0, 3.0), intensity=6.0)
    # ---- through libospray.so
    t_ground = osp.new_texture(img, 1, osp.OSP_VEC4UC, keep=keep)              # SRGBA
    t_sphere = osp.new_texture(sph, 0, osp.OSP_VEC4UC, filter=1, wrap=(1, 2), keep=keep)
    t_bp = osp.new_texture(bp, 3, osp.OSP_VEC3UC, keep=keep)                   # RGB8
    insts = []
    for k, (v, i, attrs, mtype) in enumerate([(ground_v, ground_i, dict(texcoord=ground_t), "principled"),
                                              (sv, si, dict(normal=sn, color=sc, texcoord=su), "obj")]):
        g = L.ospNewGeometry(b"mesh")
        osp.set_data(g, "vertex.position", v, osp.OSP_VEC3F, len(v), keep)
        osp.set_data(g, "index", i, osp.OSP_VEC3UI, len(i), keep)
        if "normal" in attrs:
            osp.set_data(g, "vertex.normal", attrs["normal"], osp.OSP_VEC3F, len(v), keep)
            osp.set_data(g, "vertex.color", attrs["color"], osp.OSP_VEC4F, len(v), keep)
        osp.set_data(g, "vertex.texcoord", attrs["texcoord"], osp.OSP_VEC2F, len(v), keep)
        L.ospCommit(g)
        m = L.ospNewMaterial(mtype.encode())
        if mtype == "principled":
            osp.set_param(m, "baseColor", osp.OSP_VEC3F, np.float32([1.0, 1.0, 1.0]))
            osp.set_param(m, "roughness", osp.OSP_FLOAT, np.float32(0.4))
            osp.set_param(m, "map_baseColor", osp.OSP_TEXTURE, t_ground)
        else:
            osp.set_param(m, "kd", osp.OSP_VEC3F, np.float32([0.8, 0.8, 0.8]))
            osp.set_param(m, "map_kd", osp.OSP_TEXTURE, t_sphere)
        L.ospCommit(m)
        model = osp._new_model(g, m)
        L.ospRelease(m)
        L.ospRelease(g)
        md = osp._object_data([model], osp.OSP_GEOMETRIC_MODEL)
        L.ospRelease(model)
        grp = L.ospNewGroup()
        osp.set_param(grp, "geometry", osp.OSP_DATA, md)
        L.ospRelease(md)
        L.ospCommit(grp)
        inst = L.ospNewInstance(grp)
        L.ospRelease(grp)
        if k == 1:
            osp.set_param(inst, "transform", osp.OSP_AFFINE3F,
                          np.float32([1.2, 0, 0, 0, 1.2, 0, 0, 0, 1.2, -1.2, 1.2, 0.5]))
        L.ospCommit(inst)
        insts.append(inst)
    lights = []
    for typ, params in (("quad", quad), ("ambient", dict(intensity=0.15))):
        lh = L.ospNewLight(typ.encode())
        for key, val in params.items():
            osp.set_param(lh, key, osp.OSP_FLOAT if key == "intensity" else osp.OSP_VEC3F, np.float32(val))
        L.ospCommit(lh)
        lights.append(lh)
    world = L.ospNewWorld()
    for name, hs, typ in (("instance", insts, osp.OSP_INSTANCE), ("light", lights, osp.OSP_LIGHT)):
        d = osp._object_data(hs, typ)
        osp.set_param(world, name, osp.OSP_DATA, d)
        L.ospRelease(d)
    for hd in insts + lights:
        L.ospRelease(hd)
    L.ospCommit(world)
    camh = L.ospNewCamera(b"perspective")
    for key in ("position", "direction", "up"):
        osp.set_param(camh, key, osp.OSP_VEC3F, np.float32(cam[key]))
    osp.set_param(camh, "fovy", osp.OSP_FLOAT, np.float32(cam["fovy"]))
    osp.set_param(camh, "aspect", osp.OSP_FLOAT, np.float32(w / h))
    L.ospCommit(camh)
    ren = L.ospNewRenderer(b"pathtracer")
    osp.set_param(ren, "pixelSamples", osp.OSP_INT, np.int32(2))
    osp.set_param(ren, "maxPathLength", osp.OSP_INT, np.int32(4))
    osp.set_param(ren, "roulettePathLength", osp.OSP_INT, np.int32(3))
    osp.set_param(ren, "mipMapBias", osp.OSP_FLOAT, np.float32(0.5))
    osp.set_param(ren, "map_backplate", osp.OSP_TEXTURE, t_bp)
    L.ospCommit(ren)
    for t in (t_ground, t_sphere, t_bp):
        L.ospRelease(t)
    fb = L.ospNewFrameBuffer(w, h, osp.OSP_FB_RGBA32F, osp.OSP_FB_COLOR | osp.OSP_FB_ACCUM)
    fut = L.ospRenderFrame(fb, ren, camh, world)
    assert fut, L.ospDeviceGetLastErrorMsg(L.ospGetCurrentDevice())
    L.ospWait(fut, osp.OSP_TASK_FINISHED)
    L.ospRelease(fut)
    api_img = osp.map_channel(fb, osp.OSP_FB_COLOR, (h, w, 4), np.float32)
    for hd in (fb, ren, camh, world):
        L.ospRelease(hd)
    # ---- the same through the b200 ABI
    g = og.Scene(dev)
    k0 = g.add_mesh(ground_v, ground_i)
    g.set_mesh_attributes(k0, texcoord=ground_t)
    k1 = g.add_mesh(sv, si)
    g.set_mesh_attributes(k1, normal=sn, color=sc, texcoord=su)
    g.add_instance(k0, 0, 0, None, 0)
    g.add_instance(k1, 1, 0, np.array([[1.2, 0, 0, -1.2], [0, 1.2, 0, 1.2], [0, 0, 1.2, 0.5]], np.float32), 1)
    g.commit()
    g.set_lights([og.quad_light(quad["position"], quad["edge1"], quad["edge2"], quad["intensity"]),
                  og.ambient_light(0.15)])
    tg = og.Texture(dev, img, og.TEX_SRGBA)
    ts = og.Texture(dev, sph, og.TEX_RGBA8, filter=og.TEX_FILTER_NEAREST, wrap=(1, 2))
    tb = og.Texture(dev, bp, og.TEX_RGB8)
    fbo = og.Frame(dev, w, h, og.FB_COLOR | og.FB_ACCUM)
    og.render_pt(g, og.camera_desc(cam["position"], cam["direction"], cam["up"], fovy=cam["fovy"], aspect=w / h),
                 og.pt_params(spp=2, max_path_length=4, roulette_path_length=3, mip_map_bias=0.5, backplate=tb),
                 og.materials_array([og.principled((1.0, 1.0, 1.0), 0.4, 0.0, base_color_map=tg),
                                     og.obj_material(kd=(0.8, 0.8, 0.8), map_kd=ts)]), fbo)
    abi_img = fbo.read(og.FB_COLOR)
    for t in (tg, ts, tb):
        t.release()
    assert abi_img[..., :3].mean() > 0.0
    np.testing.assert_allclose(api_img, abi_img, rtol=1e-5, atol=1e-6)
