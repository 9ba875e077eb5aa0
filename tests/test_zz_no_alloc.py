"""b200_render_pt_noalloc: the path tracer for callers that cannot allocate.

Applications that reserve all device memory up front, or must not stall on
the allocator inside a frame loop, cannot let the renderer call cudaMalloc.
This entry point renders from a fixed static scratch array in the library
instead.  The test calls it through the C ABI and checks that two calls in a
row (frame 0, then accumulation into frame 1) give the same framebuffer as
the allocating b200_render_pt on the same inputs, within the path tracer's
tolerance (only the order of the atomic shadow-ray additions differs), and
that a request larger than its stated limit is refused with a message.

This file is collected last on purpose: a failure here leaves every other
test already run."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W, H, SPP = 128, 96, 2


def _scene(b200_device):
    import ospray_gb300 as og
    from ospray_gb300 import scenes
    d = scenes.pt_instanced_scene(levels=3, width=W, height=H)
    g = og.Scene(b200_device)
    scenes.build_pt_scene(g, d)
    lights = []
    for L in d["lights"]:
        if L["type"] == "quad":
            lights.append(og.quad_light(L["position"], L["edge1"], L["edge2"], L["intensity"]))
        else:
            lights.append(og.ambient_light(L["intensity"]))
    g.set_lights(lights)
    return d, g


def _noalloc(og, scene, cam, params, mats, fb):
    fn = og.lib().b200_render_pt_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.POINTER(og.CameraDesc), ctypes.POINTER(og.PTParams), ctypes.c_void_p,
                   ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    arr, n = mats
    return fn(scene._h, ctypes.byref(cam), ctypes.byref(params), ctypes.cast(arr, ctypes.c_void_p), n, fb._h, None)


def test_noalloc_matches_allocating_path_tracer(b200_device):
    import ospray_gb300 as og
    d, g = _scene(b200_device)
    c = d["camera"]
    cam = og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
    p = og.pt_params(spp=SPP, max_path_length=5, roulette_path_length=3)
    mats = og.materials_array(d["materials"])
    ch = og.FB_COLOR | og.FB_DEPTH | og.FB_ACCUM | og.FB_ID_PRIMITIVE
    fa = og.Frame(b200_device, W, H, ch)
    fn = og.Frame(b200_device, W, H, ch)
    for call in range(2):
        og.render_pt(g, cam, p, mats, fa)
        rc = _noalloc(og, g, cam, p, mats, fn)
        assert rc == 0, og.lib().b200_device_last_error(b200_device._h)
        a, b = fa.read(og.FB_COLOR), fn.read(og.FB_COLOR)
        assert np.isfinite(b).all()
        assert a[..., :3].mean() > 0.0
        np.testing.assert_allclose(b, a, rtol=1e-4, atol=1e-5, err_msg="call %d" % call)
        np.testing.assert_array_equal(fn.read(og.FB_DEPTH), fa.read(og.FB_DEPTH))
        np.testing.assert_array_equal(fn.read(og.FB_ID_PRIMITIVE), fa.read(og.FB_ID_PRIMITIVE))
    assert fn.frame_id == 2


def test_noalloc_refuses_requests_over_its_limit(b200_device):
    import ospray_gb300 as og
    d, g = _scene(b200_device)
    c = d["camera"]
    cam = og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
    big = og.Frame(b200_device, 1024, 1024, og.FB_COLOR)
    rc = _noalloc(og, g, cam, og.pt_params(spp=1), og.materials_array(d["materials"]), big)
    assert rc == og.B200_INVALID_ARGUMENT if hasattr(og, "B200_INVALID_ARGUMENT") else rc == 2
    msg = og.lib().b200_device_last_error(b200_device._h).decode()
    assert "exceeds the static scratch limit" in msg
    assert big.frame_id == 0


def test_noalloc_allocates_nothing_on_a_callers_stream(b200_device):
    """Frames rendered on a stream the test created allocate no device
    memory (cudaMemGetInfo's free bytes equal before and after, past the
    first call) and match the allocating path tracer."""
    torch = pytest.importorskip("torch")
    import ospray_gb300 as og
    d, g = _scene(b200_device)
    c = d["camera"]
    cam = og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
    p = og.pt_params(spp=SPP, max_path_length=5, roulette_path_length=3)
    mats = og.materials_array(d["materials"])
    fa = og.Frame(b200_device, W, H, og.FB_COLOR)
    fn = og.Frame(b200_device, W, H, og.FB_COLOR)
    stream = torch.cuda.Stream()
    fn_c = og.lib().b200_render_pt_noalloc
    fn_c.restype = ctypes.c_int
    fn_c.argtypes = [ctypes.c_void_p, ctypes.POINTER(og.CameraDesc), ctypes.POINTER(og.PTParams), ctypes.c_void_p,
                     ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    arr, n = mats

    def call():
        rc = fn_c(g._h, ctypes.byref(cam), ctypes.byref(p), ctypes.cast(arr, ctypes.c_void_p), n, fn._h,
                  ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, og.lib().b200_device_last_error(b200_device._h)

    call()  # first call: module data and the scratch array's address are set up here
    stream.synchronize()
    fn.reset()
    b200_device.sync()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        call()
    stream.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    for _ in range(3):
        og.render_pt(g, cam, p, mats, fa)
    np.testing.assert_allclose(fn.read(og.FB_COLOR), fa.read(og.FB_COLOR), rtol=1e-4, atol=1e-5)
