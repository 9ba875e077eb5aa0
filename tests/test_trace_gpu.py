"""Ray-query parity: b200_trace (CUDA, quantised 8-wide BVH) against the CPU
oracle on identical rays.  Closest hits must agree on (primID, geomID,
instID) and on t bit for bit; any-hit queries must agree exactly."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def gpu_trace(scene, rays, occlusion=False):
    r = torch.from_numpy(np.ascontiguousarray(rays, np.float32)).cuda()
    n = r.shape[0]
    f = torch.zeros((max(n, 1), 6), dtype=torch.float32, device="cuda")
    ids = torch.zeros((max(n, 1), 3), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    scene.trace(r.data_ptr(), n, f.data_ptr(), ids.data_ptr(), occlusion=occlusion)
    scene.device.sync()
    return f[:n].cpu().numpy(), ids[:n].cpu().numpy().view(np.uint32)


def both(b200_device, build):
    import ospray_gb300 as og
    g = og.Scene(b200_device)
    o = oracle.Scene()
    build(g)
    build(o)
    return g, o


def assert_closest_parity(gf, gi, of, oi, min_agree=1.0):
    same_id = np.all(gi == oi, axis=1)
    same_t = (gf[:, 0].view(np.uint32) == of[:, 0].view(np.uint32))
    agree = np.mean(same_id & same_t)
    assert agree >= min_agree, (agree, np.flatnonzero(~(same_id & same_t))[:10])


@pytest.fixture(scope="module")
def ao_scene(b200_device):
    from ospray_gb300 import scenes
    d = scenes.ao_heightfield_scene()
    g, o = both(b200_device, lambda s: scenes.build_ao_scene(s, d))
    return d, g, o


def test_primary_rays_match_oracle(ao_scene):
    import ospray_gb300 as og
    d, g, o = ao_scene
    cam = oracle.camera(d["camera"]["position"], d["camera"]["direction"], d["camera"]["up"])
    rays = oracle.camera_rays(cam, og.PF_POINT, 512, 512).reshape(-1, 8)
    gf, gi = gpu_trace(g, rays)
    of, oi = o.trace(rays)
    assert np.isfinite(of[:, 0]).sum() > 10000
    assert_closest_parity(gf, gi, of, oi, min_agree=0.9999)
    np.testing.assert_array_equal(gf[:, 3:6], of[:, 3:6])


def test_random_rays_and_occlusion_match_oracle(ao_scene):
    d, g, o = ao_scene
    rng = np.random.default_rng(5)
    n = 200000
    org = rng.uniform([-0.2, -0.1, -0.2], [1.2, 0.4, 1.2], (n, 3))
    dirs = rng.normal(size=(n, 3))
    tfar = rng.choice([np.inf, 0.3], n)
    rays = np.concatenate([org, np.full((n, 1), 1e-4), dirs, tfar[:, None]], 1).astype(np.float32)
    gf, gi = gpu_trace(g, rays)
    of, oi = o.trace(rays)
    assert_closest_parity(gf, gi, of, oi, min_agree=0.9999)
    go, _ = gpu_trace(g, rays, occlusion=True)
    oo, _ = o.trace(rays, occlusion=True)
    assert np.mean(go[:, 0] == oo[:, 0]) >= 0.9999


def test_instanced_scene_matches_oracle(b200_device):
    from ospray_gb300 import scenes
    v, i = scenes.displaced_sphere(3)
    x, _ = scenes.instances(3, 12, box=4.0)

    def build(s):
        gm = s.add_mesh(v, i)
        gs = s.add_spheres(np.array([[1, 1, 1, 0.5], [3, 2, 1, 0.25]], np.float32))
        for k in range(12):
            s.add_instance(gm, k, 0, x[k])
        s.add_instance(gs, 12, 0, x[0])
        s.add_instance(gs, 13, 0)
        s.commit()

    g, o = both(b200_device, build)
    rng = np.random.default_rng(9)
    n = 100000
    org = rng.uniform(-3, 7, (n, 3))
    dirs = rng.uniform(0, 4, (n, 3)) - org
    rays = np.concatenate([org, np.zeros((n, 1)), dirs, np.full((n, 1), np.inf)], 1).astype(np.float32)
    gf, gi = gpu_trace(g, rays)
    of, oi = o.trace(rays)
    assert np.isfinite(of[:, 0]).mean() > 0.2
    assert_closest_parity(gf, gi, of, oi, min_agree=0.9999)
    go, _ = gpu_trace(g, rays, occlusion=True)
    oo, _ = o.trace(rays, occlusion=True)
    assert np.mean(go[:, 0] == oo[:, 0]) >= 0.9999


def test_edge_cases(b200_device):
    import ospray_gb300 as og
    # empty world: everything misses
    e = og.Scene(b200_device)
    e.commit()
    rays = np.array([[0, 0, 0, 0, 0, 0, 1, np.inf]], np.float32)
    f, ids = gpu_trace(e, rays)
    assert np.isinf(f[0, 0]) and ids[0, 0] == 0xffffffff
    # zero rays
    f, ids = gpu_trace(e, np.zeros((0, 8), np.float32))
    assert f.shape == (0, 6)
    # single triangle, axis-aligned rays through its vertices and edges
    tri_v = np.array([[0, 0, 0], [1, 0, 0], [0, 0, 1]], np.float32)

    def build(s):
        gm = s.add_mesh(tri_v, np.array([[0, 1, 2]], np.uint32))
        s.add_instance(gm, 0, 0)
        s.commit()

    g, o = both(b200_device, build)
    pts = np.array([[0, 0], [1, 0], [0, 1], [0.5, 0], [0, 0.5], [0.5, 0.5], [0.25, 0.25], [0.7, 0.7]], np.float32)
    rays = np.zeros((len(pts), 8), np.float32)
    rays[:, 0], rays[:, 1], rays[:, 2], rays[:, 5], rays[:, 7] = pts[:, 0], 2.0, pts[:, 1], -1.0, np.inf
    gf, gi = gpu_trace(g, rays)
    of, oi = o.trace(rays)
    assert_closest_parity(gf, gi, of, oi)
    assert np.isinf(gf[-1, 0]) and np.all(np.isfinite(gf[:-1, 0]))


def test_invalid_arguments_raise(b200_device):
    import ospray_gb300 as og
    s = og.Scene(b200_device)
    with pytest.raises(og.B200Error) as e:
        s.add_mesh(np.zeros((3, 3), np.float32), np.array([[0, 1, 5]], np.uint32))
    assert e.value.code == 2
    with pytest.raises(og.B200Error) as e:
        s.add_instance(7, 0, 0)
    assert e.value.code == 2
    with pytest.raises(og.B200Error) as e:
        s.trace(0, 0, 0, 0)  # not committed
    assert e.value.code == 3


def test_sah_and_lbvh_builds_agree_and_sah_visits_fewer_nodes(b200_device):
    """The binned-SAH hierarchy (default) and the plain LBVH (dynamic scenes)
    give identical closest hits; on the instanced displaced spheres the SAH
    one visits fewer nodes per ray."""
    import ospray_gb300 as og
    from ospray_gb300 import scenes
    d = scenes.pt_instanced_scene(levels=5, width=320, height=180)
    out = {}
    for dynamic in (False, True):
        g = og.Scene(b200_device)
        g.set_dynamic(dynamic)
        scenes.build_pt_scene(g, d)
        c = d["camera"]
        cam = oracle.camera(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
        rays = oracle.camera_rays(cam, og.PF_POINT, 320, 180, spp=2).reshape(-1, 8)
        out[dynamic] = gpu_trace(g, rays)
        # node visits of a stats-collecting render of the same scene
        fb = og.Frame(b200_device, 320, 180, og.FB_COLOR)
        g.set_lights([og.ambient_light(1.0)])
        g.counters(reset=True)
        og.render_pt(g, og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"]),
                     og.pt_params(spp=2, max_path_length=3, stats=True), og.materials_array(d["materials"]), fb)
        cnt = g.counters(reset=True)
        out[(dynamic, "visits")] = cnt[1] / max(cnt[0], 1)
    (f0, i0), (f1, i1) = out[False], out[True]
    np.testing.assert_array_equal(i0, i1)
    np.testing.assert_array_equal(f0[:, 0].view(np.uint32), f1[:, 0].view(np.uint32))
    assert out[(False, "visits")] < out[(True, "visits")], (out[(False, "visits")], out[(True, "visits")])


def test_quad_mesh_matches_oracle(b200_device):
    """Quad meshes (vec4ui index): two BLAS triangles per quad reporting the
    quad's primID; closest hits, IDs and t bit for bit, any-hit exactly, and
    AO frames (epsilon over the quad's 4 vertices) against the oracle."""
    import ospray_gb300 as og
    from test_cpu_oracle import _heightfield_quads
    v, q = _heightfield_quads(n=96)

    def build(s):
        s.add_instance(s.add_quad_mesh(v, q), 0, 0)
        s.commit()
    g, o = both(b200_device, build)
    rng = np.random.default_rng(2)
    n = 100000
    org = np.concatenate([rng.uniform(0, 1, (n, 1)), np.full((n, 1), 0.8), rng.uniform(0, 1, (n, 1))], 1)
    d = np.concatenate([rng.normal(0, 0.4, (n, 1)), -np.ones((n, 1)), rng.normal(0, 0.4, (n, 1))], 1)
    rays = np.concatenate([org, np.zeros((n, 1)), d, np.full((n, 1), np.inf)], 1).astype(np.float32)
    gf, gi = gpu_trace(g, rays)
    of, oi = o.trace(rays)
    assert np.isfinite(of[:, 0]).mean() > 0.5
    assert oi[np.isfinite(of[:, 0]), 0].max() < len(q)
    assert_closest_parity(gf, gi, of, oi, min_agree=0.9999)
    go, _ = gpu_trace(g, rays, occlusion=True)
    oo, _ = o.trace(rays, occlusion=True)
    assert np.mean(go[:, 0] == oo[:, 0]) >= 0.9999
    W = H = 64
    pos, dirn, up = (0.5, 1.2, -0.6), (0.0, -1.2, 1.1), (0.0, 1.0, 0.0)
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_DEPTH | og.FB_ID_PRIMITIVE)
    og.render_ao(g, og.camera_desc(pos, dirn, up), og.ao_params(pixel_filter=og.PF_POINT, ao_samples=2), fb)
    ref = oracle.render_ao(o, oracle.camera(pos, dirn, up), og.PF_POINT, W, H, ao_samples=2)
    assert np.mean(fb.read(og.FB_ID_PRIMITIVE) == ref["primID"]) >= 0.999
    c, r = fb.read(og.FB_COLOR), ref["color"]
    assert np.mean(np.all(np.abs(c - r) <= 1e-4, axis=2)) >= 0.999


def test_boxes_match_oracle(b200_device):
    """Box geometry (12 face triangles per box reporting the box's primID, no
    geometry epsilon): closest hits bit for bit, any-hit exactly, rays
    starting inside boxes hit the exit face, and AO frames agree."""
    import ospray_gb300 as og
    from test_cpu_oracle import _random_boxes
    b = _random_boxes(n=400, seed=9)

    def build(s):
        s.add_instance(s.add_boxes(b), 0, 0)
        s.commit()
    g, o = both(b200_device, build)
    rng = np.random.default_rng(3)
    n = 100000
    org = rng.uniform(-0.2, 1.2, (n, 3))
    inside = rng.integers(0, len(b), 2000)
    org[:2000] = (b[inside, :3] + b[inside, 3:]) / 2
    d = rng.normal(size=(n, 3))
    rays = np.concatenate([org, np.zeros((n, 1)), d, np.full((n, 1), np.inf)], 1).astype(np.float32)
    gf, gi = gpu_trace(g, rays)
    of, oi = o.trace(rays)
    assert np.isfinite(of[:2000, 0]).all()
    assert_closest_parity(gf, gi, of, oi, min_agree=0.9999)
    go, _ = gpu_trace(g, rays, occlusion=True)
    oo, _ = o.trace(rays, occlusion=True)
    assert np.mean(go[:, 0] == oo[:, 0]) >= 0.9999
    W = H = 64
    pos, dirn, up = (0.5, 1.6, -1.2), (0.0, -1.2, 1.4), (0.0, 1.0, 0.0)
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_DEPTH | og.FB_ID_PRIMITIVE)
    og.render_ao(g, og.camera_desc(pos, dirn, up), og.ao_params(pixel_filter=og.PF_POINT, ao_samples=2), fb)
    ref = oracle.render_ao(o, oracle.camera(pos, dirn, up), og.PF_POINT, W, H, ao_samples=2)
    assert np.mean(ref["primID"] != 0xFFFFFFFF) > 0.2
    assert np.mean(fb.read(og.FB_ID_PRIMITIVE) == ref["primID"]) >= 0.999
    c, r = fb.read(og.FB_COLOR), ref["color"]
    assert np.mean(np.all(np.abs(c - r) <= 1e-4, axis=2)) >= 0.999


def _discs_planes(s, rng_seed=4):
    """Ray-facing discs, oriented discs (one instance moved and scaled), an
    unbounded ground plane y = 0 and a tilted plane bounded by a box."""
    rng = np.random.default_rng(rng_seed)
    d = np.concatenate([rng.uniform(-3, 3, (300, 1)), rng.uniform(0.2, 2.5, (300, 1)), rng.uniform(-3, 3, (300, 1)),
                        rng.uniform(0.05, 0.3, (300, 1))], 1).astype(np.float32)
    od = d.copy()
    od[:, 1] += 0.4
    nrm = rng.normal(size=(300, 3)).astype(np.float32)
    k0 = s.add_discs(d)
    k1 = s.add_discs(od, normals=nrm)
    k2 = s.add_planes(np.array([[0, 1, 0, 0]], np.float32))
    k3 = s.add_planes(np.array([[0.3, 0.2, 1.0, 1.5]], np.float32), bounds=np.array([[-2, -1, -3, 2, 3, 3]], np.float32))
    s.add_instance(k0, 0, 0, None, 0)
    s.add_instance(k1, 1, 0, np.array([[1.1, 0, 0, 0.2], [0, 0.9, 0, 0.1], [0, 0, 1.0, -0.3]], np.float32), 1)
    s.add_instance(k2, 2, 0, None, 2)
    s.add_instance(k3, 3, 0, None, 1)
    s.commit()


def test_discs_and_planes_match_oracle(b200_device):
    """Discs facing the ray, oriented discs and planes (unbounded and boxed):
    closest hits (IDs, t bit for bit, Ng), any-hit, and AO frames with the
    discs' radius epsilon and the planes' zero geometry epsilon."""
    import ospray_gb300 as og
    g, o = both(b200_device, _discs_planes)
    rng = np.random.default_rng(5)
    n = 100000
    org = np.concatenate([rng.uniform(-4, 4, (n, 1)), rng.uniform(0.5, 4, (n, 1)), rng.uniform(-4, 4, (n, 1))], 1)
    dirn = rng.normal(size=(n, 3))
    rays = np.concatenate([org, np.zeros((n, 1)), dirn, np.full((n, 1), np.inf)], 1).astype(np.float32)
    gf, gi = gpu_trace(g, rays)
    of, oi = o.trace(rays)
    hit = np.isfinite(of[:, 0])
    for inst in range(4):
        assert np.sum(oi[hit, 2] == inst) > 100, inst
    assert_closest_parity(gf, gi, of, oi, min_agree=0.9999)
    same = np.all(gi == oi, axis=1) & hit
    np.testing.assert_allclose(gf[same, 3:6], of[same, 3:6], rtol=1e-5, atol=1e-6)
    go, _ = gpu_trace(g, rays, occlusion=True)
    oo, _ = o.trace(rays, occlusion=True)
    assert np.mean(go[:, 0] == oo[:, 0]) >= 0.9999
    W = H = 96
    pos, dirc, up = (0.0, 3.0, -6.5), (0.0, -2.0, 6.0), (0.0, 1.0, 0.0)
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_DEPTH | og.FB_ID_PRIMITIVE | og.FB_ID_INSTANCE)
    og.render_ao(g, og.camera_desc(pos, dirc, up), og.ao_params(pixel_filter=og.PF_POINT, ao_samples=2), fb)
    ref = oracle.render_ao(o, oracle.camera(pos, dirc, up), og.PF_POINT, W, H, ao_samples=2)
    assert np.mean(fb.read(og.FB_ID_INSTANCE) == ref["instID"]) >= 0.999
    assert np.mean(fb.read(og.FB_ID_PRIMITIVE) == ref["primID"]) >= 0.999
    c, r = fb.read(og.FB_COLOR), ref["color"]
    assert np.mean(np.all(np.abs(c - r) <= 1e-4, axis=2)) >= 0.999


def test_discs_and_planes_path_traced_match_oracle(b200_device):
    import ospray_gb300 as og
    g, o = both(b200_device, _discs_planes)
    lights = [dict(type="quad", position=(-1.0, 6.0, -1.0), edge1=(2.0, 0.0, 0.0), edge2=(0.0, 0.0, 2.0),
                   intensity=10.0), dict(type="ambient", intensity=0.1)]
    g.set_lights([og.quad_light(L["position"], L["edge1"], L["edge2"], L["intensity"]) if L["type"] == "quad"
                  else og.ambient_light(L["intensity"]) for L in lights])
    mats = [(0.8, 0.3, 0.2, 0.4, 0.0), (0.2, 0.7, 0.3, 0.2, 1.0), (0.7, 0.7, 0.7, 0.9, 0.0)]
    W, H = 128, 96
    pos, dirc, up = (0.0, 3.0, -6.5), (0.0, -2.0, 6.0), (0.0, 1.0, 0.0)
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_ACCUM | og.FB_ID_PRIMITIVE)
    og.render_pt(g, og.camera_desc(pos, dirc, up, aspect=W / H), og.pt_params(spp=4, max_path_length=4),
                 og.materials_array(mats), fb)
    ref = oracle.render_pt(o, oracle.PtWorld(mats, lights), oracle.camera(pos, dirc, up, aspect=W / H),
                           oracle.pt_params(spp=4, max_path_length=4), W, H)
    assert np.mean(fb.read(og.FB_ID_PRIMITIVE) == ref["primID"]) >= 0.999
    gc, rc = fb.read(og.FB_ACCUM)[..., :3], ref["color"][..., :3]
    close = np.all(np.abs(gc - rc) <= 1e-3 * np.maximum(1.0, np.abs(rc)), axis=2)
    assert close.mean() >= 0.995, close.mean()
