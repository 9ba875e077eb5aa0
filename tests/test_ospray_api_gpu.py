"""OSPRay applications on the b200 device, through libospray.so.

* tests/c/osp_app.c (a C99 client of include/ospray, the flow of OSPRay's
  tutorial: mesh + obj material + ambient light, path tracer, sRGB
  framebuffer, accumulation, futures, pick) is built and run;
* the AO workload (height field + spheres) is built with OSPRay API calls
  from Python (shared data, geometric models, group, instance, world, "ao"
  renderer, RGBA32F framebuffer with depth and ID channels) and must match
  the oracle exactly on depth and IDs, like the b200 ABI path does;
* unsupported object types fail with an error code and message.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
import osp_api
from osp_api import lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def osp_device():
    L = lib()
    assert L.ospInit(None, None) == 0, L.ospDeviceGetLastErrorMsg(None)
    yield L
    L.ospShutdown()


def test_c_application_renders(tmp_path):
    exe = str(tmp_path / "osp_app")
    cc = shutil.which("gcc") or shutil.which("cc")
    r = subprocess.run([cc, "-std=c99", os.path.join(osp_api.ROOT, "tests", "c", "osp_app.c"), "-I",
                        os.path.join(osp_api.ROOT, "include"), "-L", osp_api.BUILD, "-lospray",
                        "-Wl,-rpath," + osp_api.BUILD, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    tok = r.stdout.split()
    vals = dict(bounds=[float(v) for v in tok[1:7]], hit=int(tok[8]), prim=int(tok[9]), mean0=float(tok[11]),
                mean10=float(tok[13]), duration=float(tok[15]))
    np.testing.assert_allclose(vals["bounds"], [-1, -1, 0.3, 1, 1, 3], rtol=1e-6)
    assert vals["hit"] == 1 and vals["prim"] in (0, 1)
    assert 20.0 < vals["mean10"] < 255.0 and vals["duration"] > 0.0
    assert os.path.getsize(tmp_path / "accumulatedFrame.ppm") > 320 * 240 * 3


# a side-by-side stereo camera over a sub-image (Camera "imageStart" /
# "imageEnd", PerspectiveCamera "stereoMode" / "interpupillaryDistance")
STEREO = dict(stereo_mode=3, interpupillary_distance=0.05, image_start=(0.1, 0.2), image_end=(0.9, 0.95))


@pytest.mark.parametrize("stereo", [False, True])
def test_ao_through_ospray_api_matches_oracle(osp_device, stereo):
    from ospray_gb300 import scenes
    L = osp_device
    d = scenes.ao_heightfield_scene()
    keep = []
    W = H = 256
    mesh = L.ospNewGeometry(b"mesh")
    osp_api.set_data(mesh, "vertex.position", d["vertex"].astype(np.float32), osp_api.OSP_VEC3F,
                     len(d["vertex"]), keep)
    osp_api.set_data(mesh, "index", d["index"].astype(np.uint32), osp_api.OSP_VEC3UI, len(d["index"]), keep)
    L.ospCommit(mesh)
    sph = L.ospNewGeometry(b"sphere")
    s = np.asarray(d["spheres"], np.float32)
    osp_api.set_data(sph, "sphere.position", s[:, :3].copy(), osp_api.OSP_VEC3F, len(s), keep)
    osp_api.set_data(sph, "sphere.radius", s[:, 3].copy(), osp_api.OSP_FLOAT, len(s), keep)
    L.ospCommit(sph)
    models = []
    for g in (mesh, sph):
        m = L.ospNewGeometricModel(g)
        L.ospCommit(m)
        models.append(m)
        L.ospRelease(g)
    arr = (ctypes.c_void_p * 2)(*models)
    md = L.ospNewSharedData(ctypes.addressof(arr), osp_api.OSP_GEOMETRIC_MODEL, 2, 0, 1, 0, 1, 0, None, None)
    group = L.ospNewGroup()
    osp_api.set_param(group, "geometry", osp_api.OSP_DATA, md)
    L.ospRelease(md)
    for m in models:
        L.ospRelease(m)
    L.ospCommit(group)
    inst = L.ospNewInstance(group)
    L.ospCommit(inst)
    L.ospRelease(group)
    world = L.ospNewWorld()
    L.ospSetObjectAsData(world, b"instance", osp_api.OSP_INSTANCE, inst)
    L.ospRelease(inst)
    L.ospCommit(world)
    b = L.ospGetBounds(world)
    assert b.lower[1] < 0.3 and b.upper[0] > 0.9

    c = d["camera"]
    cam = L.ospNewCamera(b"perspective")
    osp_api.set_param(cam, "position", osp_api.OSP_VEC3F, np.float32(c["position"]))
    osp_api.set_param(cam, "direction", osp_api.OSP_VEC3F, np.float32(c["direction"]))
    osp_api.set_param(cam, "up", osp_api.OSP_VEC3F, np.float32(c["up"]))
    osp_api.set_param(cam, "fovy", osp_api.OSP_FLOAT, np.float32(c["fovy"]))
    osp_api.set_param(cam, "aspect", osp_api.OSP_FLOAT, np.float32(1.0))
    if stereo:
        osp_api.set_param(cam, "stereoMode", osp_api.OSP_UINT, np.uint32(STEREO["stereo_mode"]))
        osp_api.set_param(cam, "interpupillaryDistance", osp_api.OSP_FLOAT,
                          np.float32(STEREO["interpupillary_distance"]))
        osp_api.set_param(cam, "imageStart", osp_api.OSP_VEC2F, np.float32(STEREO["image_start"]))
        osp_api.set_param(cam, "imageEnd", osp_api.OSP_VEC2F, np.float32(STEREO["image_end"]))
    L.ospCommit(cam)
    ren = L.ospNewRenderer(b"ao")
    osp_api.set_param(ren, "pixelFilter", osp_api.OSP_UINT, np.uint32(0))
    osp_api.set_param(ren, "aoSamples", osp_api.OSP_INT, np.int32(1))
    L.ospCommit(ren)
    ch = osp_api.OSP_FB_COLOR | osp_api.OSP_FB_DEPTH | osp_api.OSP_FB_ACCUM | osp_api.OSP_FB_ID_PRIMITIVE | \
        osp_api.OSP_FB_ID_OBJECT | osp_api.OSP_FB_ID_INSTANCE
    fb = L.ospNewFrameBuffer(W, H, osp_api.OSP_FB_RGBA32F, ch)
    fut = L.ospRenderFrame(fb, ren, cam, world)
    L.ospWait(fut, osp_api.OSP_TASK_FINISHED)
    assert L.ospIsReady(fut, osp_api.OSP_TASK_FINISHED) == 1
    L.ospRelease(fut)
    color = osp_api.map_channel(fb, osp_api.OSP_FB_COLOR, (H, W, 4), np.float32)
    depth = osp_api.map_channel(fb, osp_api.OSP_FB_DEPTH, (H, W), np.float32)
    ids = [osp_api.map_channel(fb, ch, (H, W), np.uint32) for ch in
           (osp_api.OSP_FB_ID_PRIMITIVE, osp_api.OSP_FB_ID_OBJECT, osp_api.OSP_FB_ID_INSTANCE)]

    o = oracle.Scene()
    scenes.build_ao_scene(o, d)
    ref = oracle.render_ao(o, oracle.camera(c["position"], c["direction"], c["up"], **(STEREO if stereo else {})),
                           0, W, H)
    assert np.mean(depth.view(np.uint32) == ref["depth"].view(np.uint32)) >= 0.9999
    for got, key in zip(ids, ("primID", "geomID", "instID")):
        assert np.mean(got == ref[key]) >= 0.9999, key
    assert np.mean(np.all(color == ref["color"], axis=2)) >= 0.999
    assert {0, 1} <= set(np.unique(ids[1]).tolist())  # both geometric models seen
    if stereo:
        for h in (fb, ren, cam, world):
            L.ospRelease(h)
        return

    res = osp_api.OSPPickResult()
    L.ospPick(ctypes.byref(res), fb, ren, cam, world, 0.5, 0.5)
    rhit, rpos, rids = oracle.pick(o, oracle.camera(c["position"], c["direction"], c["up"]), 0.5, 0.5)
    assert bool(res.hasHit) == rhit
    if rhit:
        assert res.primID == rids[2] and res.model and res.instance
        np.testing.assert_array_equal(np.float32(list(res.worldPosition)), rpos)
        L.ospRelease(res.model)
        L.ospRelease(res.instance)
    for h in (fb, ren, cam, world):
        L.ospRelease(h)


def test_discs_and_planes_through_ospray_api_match_oracle(osp_device):
    """"sphere" geometry of "type" OSP_DISC / OSP_ORIENTED_DISC (with
    "sphere.normal") and "plane" geometry ("plane.coefficients", "plane.bounds")
    made through libospray.so render the oracle's AO frame."""
    L = osp_device
    keep = []
    W = H = 128
    rng = np.random.default_rng(12)
    c = np.concatenate([rng.uniform(-2, 2, (60, 1)), rng.uniform(0.3, 2, (60, 1)), rng.uniform(-2, 2, (60, 1))], 1)
    r = rng.uniform(0.1, 0.4, 60).astype(np.float32)
    nrm = rng.normal(size=(60, 3)).astype(np.float32)
    geoms = []
    for kind in (51, 52):  # OSP_DISC, OSP_ORIENTED_DISC
        g = L.ospNewGeometry(b"sphere")
        osp_api.set_data(g, "sphere.position", (c + (kind - 51) * 0.3).astype(np.float32), osp_api.OSP_VEC3F, 60, keep)
        osp_api.set_data(g, "sphere.radius", r, osp_api.OSP_FLOAT, 60, keep)
        osp_api.set_param(g, "type", osp_api.OSP_UINT, np.uint32(kind))
        if kind == 52:
            osp_api.set_data(g, "sphere.normal", nrm, osp_api.OSP_VEC3F, 60, keep)
        L.ospCommit(g)
        geoms.append(g)
    pl = L.ospNewGeometry(b"plane")
    coeffs = np.array([[0, 1, 0, 0], [0.3, 0.2, 1.0, 1.5]], np.float32)
    bounds = np.array([[-1e30, -1e30, -1e30, 1e30, 1e30, 1e30], [-2, -1, -3, 2, 3, 3]], np.float32)
    osp_api.set_data(pl, "plane.coefficients", coeffs, 6003, 2, keep)      # OSP_VEC4F
    osp_api.set_data(pl, "plane.bounds", bounds, 10002, 2, keep)           # OSP_BOX3F
    L.ospCommit(pl)
    geoms.append(pl)
    models = []
    for g in geoms:
        m = L.ospNewGeometricModel(g)
        L.ospCommit(m)
        models.append(m)
        L.ospRelease(g)
    arr = (ctypes.c_void_p * 3)(*models)
    md = L.ospNewSharedData(ctypes.addressof(arr), osp_api.OSP_GEOMETRIC_MODEL, 3, 0, 1, 0, 1, 0, None, None)
    group = L.ospNewGroup()
    osp_api.set_param(group, "geometry", osp_api.OSP_DATA, md)
    L.ospRelease(md)
    for m in models:
        L.ospRelease(m)
    L.ospCommit(group)
    inst = L.ospNewInstance(group)
    L.ospCommit(inst)
    L.ospRelease(group)
    world = L.ospNewWorld()
    L.ospSetObjectAsData(world, b"instance", osp_api.OSP_INSTANCE, inst)
    L.ospRelease(inst)
    L.ospCommit(world)
    pos, dirc, up = (0.0, 3.0, -6.5), (0.0, -2.0, 6.0), (0.0, 1.0, 0.0)
    cam = L.ospNewCamera(b"perspective")
    for key, val in (("position", pos), ("direction", dirc), ("up", up)):
        osp_api.set_param(cam, key, osp_api.OSP_VEC3F, np.float32(val))
    osp_api.set_param(cam, "aspect", osp_api.OSP_FLOAT, np.float32(1.0))
    L.ospCommit(cam)
    ren = L.ospNewRenderer(b"ao")
    osp_api.set_param(ren, "pixelFilter", osp_api.OSP_UINT, np.uint32(0))
    osp_api.set_param(ren, "aoSamples", osp_api.OSP_INT, np.int32(1))
    L.ospCommit(ren)
    fb = L.ospNewFrameBuffer(W, H, osp_api.OSP_FB_RGBA32F,
                             osp_api.OSP_FB_COLOR | osp_api.OSP_FB_ID_PRIMITIVE | osp_api.OSP_FB_ID_OBJECT)
    fut = L.ospRenderFrame(fb, ren, cam, world)
    assert fut, L.ospDeviceGetLastErrorMsg(L.ospGetCurrentDevice())
    L.ospWait(fut, osp_api.OSP_TASK_FINISHED)
    L.ospRelease(fut)
    color = osp_api.map_channel(fb, osp_api.OSP_FB_COLOR, (H, W, 4), np.float32)
    geom = osp_api.map_channel(fb, osp_api.OSP_FB_ID_OBJECT, (H, W), np.uint32)
    for h in (fb, ren, cam, world):
        L.ospRelease(h)
    o = oracle.Scene()
    o.add_instance(o.add_discs(np.concatenate([c, r[:, None]], 1)), 0, 0)
    o.add_instance(o.add_discs(np.concatenate([c + 0.3, r[:, None]], 1), normals=nrm), 0, 1)
    o.add_instance(o.add_planes(coeffs, bounds), 0, 2)
    o.commit()
    ref = oracle.render_ao(o, oracle.camera(pos, dirc, up), 0, W, H)
    assert set(np.unique(geom).tolist()) >= {0, 1, 2}
    assert np.mean(geom == ref["geomID"]) >= 0.999
    assert np.mean(np.all(np.abs(color - ref["color"]) <= 1e-4, axis=2)) >= 0.999


def test_unsupported_types_report_errors(osp_device):
    L = osp_device
    dev = L.ospGetCurrentDevice()
    assert L.ospNewLight(b"hdri") is None
    assert L.ospDeviceGetLastErrorCode(dev) == 2
    assert b"hdri" in L.ospDeviceGetLastErrorMsg(dev)
    assert L.ospNewCamera(b"omnidirectional") is None
    L.ospDeviceRelease(dev)


def test_quads_boxes_and_lights_through_ospray_api(osp_device):
    """A mesh with vec4ui quads, a "box" geometry, and "distant" + "sphere"
    lights through libospray.so (ospNewGeometry / ospNewLight), rendered by
    the scivis renderer with shadows: IDs and depth bit-exact and colours
    within 1e-3 of the oracle on the same world."""
    from test_cpu_oracle import _heightfield_quads, _random_boxes
    L = osp_device
    keep = []
    W = H = 128
    v, q = _heightfield_quads(n=40)
    boxes = _random_boxes(n=40, seed=11)
    boxes[:, [1, 4]] = boxes[:, [1, 4]] * 0.3 + 0.05  # boxes standing on the height field
    mesh = L.ospNewGeometry(b"mesh")
    osp_api.set_data(mesh, "vertex.position", v.astype(np.float32), osp_api.OSP_VEC3F, len(v), keep)
    osp_api.set_data(mesh, "index", q.astype(np.uint32), 4503, len(q), keep)  # OSP_VEC4UI
    L.ospCommit(mesh)
    box = L.ospNewGeometry(b"box")
    osp_api.set_data(box, "box", boxes.astype(np.float32), 10002, len(boxes), keep)  # OSP_BOX3F
    L.ospCommit(box)
    models = []
    for g in (mesh, box):
        m = L.ospNewGeometricModel(g)
        L.ospCommit(m)
        models.append(m)
        L.ospRelease(g)
    arr = (ctypes.c_void_p * 2)(*models)
    md = L.ospNewSharedData(ctypes.addressof(arr), osp_api.OSP_GEOMETRIC_MODEL, 2, 0, 1, 0, 1, 0, None, None)
    group = L.ospNewGroup()
    osp_api.set_param(group, "geometry", osp_api.OSP_DATA, md)
    L.ospRelease(md)
    for m in models:
        L.ospRelease(m)
    L.ospCommit(group)
    inst = L.ospNewInstance(group)
    L.ospCommit(inst)
    L.ospRelease(group)
    lights_d = [dict(type="distant", direction=(0.3, -1.0, 0.4), intensity=2.0, color=(1.0, 0.9, 0.8)),
                dict(type="sphere", position=(0.2, 0.8, 0.3), radius=0.05, intensity=0.4)]
    lights = []
    for ld in lights_d:
        lh = L.ospNewLight(ld["type"].encode())
        assert lh, L.ospDeviceGetLastErrorMsg(L.ospGetCurrentDevice())
        osp_api.set_param(lh, "intensity", osp_api.OSP_FLOAT, np.float32(ld["intensity"]))
        if "color" in ld:
            osp_api.set_param(lh, "color", osp_api.OSP_VEC3F, np.float32(ld["color"]))
        if ld["type"] == "distant":
            osp_api.set_param(lh, "direction", osp_api.OSP_VEC3F, np.float32(ld["direction"]))
        else:
            osp_api.set_param(lh, "position", osp_api.OSP_VEC3F, np.float32(ld["position"]))
            osp_api.set_param(lh, "radius", osp_api.OSP_FLOAT, np.float32(ld["radius"]))
        L.ospCommit(lh)
        lights.append(lh)
    la = (ctypes.c_void_p * 2)(*lights)
    ld_data = L.ospNewSharedData(ctypes.addressof(la), osp_api.OSP_LIGHT, 2, 0, 1, 0, 1, 0, None, None)
    world = L.ospNewWorld()
    L.ospSetObjectAsData(world, b"instance", osp_api.OSP_INSTANCE, inst)
    osp_api.set_param(world, "light", osp_api.OSP_DATA, ld_data)
    L.ospRelease(ld_data)
    for lh in lights:
        L.ospRelease(lh)
    L.ospRelease(inst)
    L.ospCommit(world)
    pos, dirn, up = (0.5, 1.1, -0.5), (0.0, -1.0, 1.1), (0.0, 1.0, 0.0)
    cam = L.ospNewCamera(b"perspective")
    osp_api.set_param(cam, "position", osp_api.OSP_VEC3F, np.float32(pos))
    osp_api.set_param(cam, "direction", osp_api.OSP_VEC3F, np.float32(dirn))
    osp_api.set_param(cam, "up", osp_api.OSP_VEC3F, np.float32(up))
    osp_api.set_param(cam, "aspect", osp_api.OSP_FLOAT, np.float32(1.0))
    L.ospCommit(cam)
    ren = L.ospNewRenderer(b"scivis")
    osp_api.set_param(ren, "pixelFilter", osp_api.OSP_UINT, np.uint32(0))
    osp_api.set_param(ren, "shadows", osp_api.OSP_BOOL, np.uint8(1))
    L.ospCommit(ren)
    ch = osp_api.OSP_FB_COLOR | osp_api.OSP_FB_DEPTH | osp_api.OSP_FB_ACCUM | osp_api.OSP_FB_ID_PRIMITIVE | \
        osp_api.OSP_FB_ID_OBJECT
    fb = L.ospNewFrameBuffer(W, H, osp_api.OSP_FB_RGBA32F, ch)
    fut = L.ospRenderFrame(fb, ren, cam, world)
    assert fut, L.ospDeviceGetLastErrorMsg(L.ospGetCurrentDevice())
    L.ospWait(fut, osp_api.OSP_TASK_FINISHED)
    L.ospRelease(fut)
    color = osp_api.map_channel(fb, osp_api.OSP_FB_COLOR, (H, W, 4), np.float32)
    depth = osp_api.map_channel(fb, osp_api.OSP_FB_DEPTH, (H, W), np.float32)
    prim = osp_api.map_channel(fb, osp_api.OSP_FB_ID_PRIMITIVE, (H, W), np.uint32)
    geom = osp_api.map_channel(fb, osp_api.OSP_FB_ID_OBJECT, (H, W), np.uint32)
    o = oracle.Scene()
    o.add_instance(o.add_quad_mesh(v, q), 0, 0)
    o.add_instance(o.add_boxes(boxes), 0, 1)
    o.commit()
    ref = oracle.render_scivis(o, None, oracle.camera(pos, dirn, up), lights_d, [], W, H, spp=1, pixel_filter=0,
                               shadows=True)
    assert {0, 1} <= set(np.unique(geom).tolist())  # quads and boxes both seen
    assert np.mean(prim == ref["primID"]) >= 0.999
    assert np.mean(depth.view(np.uint32) == ref["depth"].view(np.uint32)) >= 0.999
    assert ref["color"][..., :3].mean() > 0.05
    close = np.all(np.abs(color - ref["color"]) <= 1e-3 * np.maximum(1.0, np.abs(ref["color"])) + 1e-5, axis=2)
    assert close.mean() >= 0.995, close.mean()
    for h in (fb, ren, cam, world):
        L.ospRelease(h)


def test_motion_blurred_instance_through_ospray_api_matches_oracle(osp_device):
    """An instance with "motion.transform" keys and "time", rendered by the
    AO renderer under a camera with a rolling "shutter" through libospray.so,
    equals the oracle's frame."""
    from test_motion_gpu import _keys, _sphere
    L = osp_device
    keep = []
    W, H = 96, 72
    sv, si = _sphere()
    g = L.ospNewGeometry(b"mesh")
    osp_api.set_data(g, "vertex.position", sv, osp_api.OSP_VEC3F, len(sv), keep)
    osp_api.set_data(g, "index", si, osp_api.OSP_VEC3UI, len(si), keep)
    L.ospCommit(g)
    m = L.ospNewGeometricModel(g)
    L.ospCommit(m)
    L.ospRelease(g)
    group = L.ospNewGroup()
    L.ospSetObjectAsData(group, b"geometry", osp_api.OSP_GEOMETRIC_MODEL, m)
    L.ospRelease(m)
    L.ospCommit(group)
    inst = L.ospNewInstance(group)
    keys = _keys()  # row-major 3x4 -> affine3f (l.vx, l.vy, l.vz, p)
    aff = np.ascontiguousarray(np.concatenate([keys[:, :, 0], keys[:, :, 1], keys[:, :, 2], keys[:, :, 3]], 1),
                               np.float32)
    osp_api.set_data(inst, "motion.transform", aff, osp_api.OSP_AFFINE3F, len(keys), keep)
    osp_api.set_param(inst, "time", 10000, np.float32([0.1, 0.9]))  # OSP_BOX1F
    L.ospCommit(inst)
    L.ospRelease(group)
    world = L.ospNewWorld()
    L.ospSetObjectAsData(world, b"instance", osp_api.OSP_INSTANCE, inst)
    L.ospRelease(inst)
    L.ospCommit(world)
    pos, dirc, up = (0.0, 2.5, -8.0), (0.0, -1.0, 7.0), (0.0, 1.0, 0.0)
    cam = L.ospNewCamera(b"perspective")
    for key, val in (("position", pos), ("direction", dirc), ("up", up)):
        osp_api.set_param(cam, key, osp_api.OSP_VEC3F, np.float32(val))
    osp_api.set_param(cam, "aspect", osp_api.OSP_FLOAT, np.float32(W / H))
    osp_api.set_param(cam, "shutter", 10000, np.float32([0.0, 1.0]))  # OSP_BOX1F
    osp_api.set_param(cam, "shutterType", osp_api.OSP_UINT, np.uint32(3))  # OSP_SHUTTER_ROLLING_DOWN
    osp_api.set_param(cam, "rollingShutterDuration", osp_api.OSP_FLOAT, np.float32(0.25))
    L.ospCommit(cam)
    ren = L.ospNewRenderer(b"ao")
    osp_api.set_param(ren, "pixelFilter", osp_api.OSP_UINT, np.uint32(0))
    osp_api.set_param(ren, "aoSamples", osp_api.OSP_INT, np.int32(1))
    L.ospCommit(ren)
    fb = L.ospNewFrameBuffer(W, H, osp_api.OSP_FB_RGBA32F, osp_api.OSP_FB_COLOR | osp_api.OSP_FB_ID_PRIMITIVE)
    fut = L.ospRenderFrame(fb, ren, cam, world)
    assert fut, L.ospDeviceGetLastErrorMsg(L.ospGetCurrentDevice())
    L.ospWait(fut, osp_api.OSP_TASK_FINISHED)
    L.ospRelease(fut)
    color = osp_api.map_channel(fb, osp_api.OSP_FB_COLOR, (H, W, 4), np.float32)
    prim = osp_api.map_channel(fb, osp_api.OSP_FB_ID_PRIMITIVE, (H, W), np.uint32)
    for h in (fb, ren, cam, world):
        L.ospRelease(h)
    o = oracle.Scene()
    o.add_instance_motion(o.add_mesh(sv, si), 0, 0, keys, (0.1, 0.9))
    o.commit()
    ref = oracle.render_ao(o, oracle.camera(pos, dirc, up, aspect=W / H, shutter=(0.0, 1.0), shutter_type=3,
                                            rolling_shutter_duration=0.25), 0, W, H)
    assert np.mean(prim != 0xFFFFFFFF) > 0.01  # the moving sphere is in view
    np.testing.assert_array_equal(prim, ref["primID"])
    assert np.mean(np.all(np.abs(color - ref["color"]) <= 1e-4, axis=2)) >= 0.999
