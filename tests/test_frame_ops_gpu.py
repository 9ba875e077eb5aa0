"""Framebuffer post-processing and pick on the GPU against the oracle.

Post-processing: a small path-traced frame (HDR colours: the quad light is
visible) is rendered into framebuffers of each format, with and without the
tonemapper.  The accumulated colour (ACCUM) is read back and run through the
oracle's restatement of ToneMapper_kernel + ColorConversion_kernel; the
mapped COLOR must equal it.  Without the tonemapper and for RGBA8/RGBA32F
the arithmetic has no transcendental, so the bytes/floats are exact; pow()
differs between CUDA and the host libm in the last ulp, so tonemapped floats
agree to 1e-5 relative and converted bytes to 1 unit, on all but a few.

Pick: camera rays at a grid of screen positions over the AO workload; hit
flag, IDs and the float world position must equal the oracle's bit for
bit (same camera ray, same intersection arithmetic, same org + t*dir)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

W, H = 96, 64


@pytest.fixture(scope="module")
def pt_world(b200_device):
    import ospray_gb300 as og
    from ospray_gb300 import scenes
    d = scenes.pt_instanced_scene(levels=3, width=W, height=H)
    g = og.Scene(b200_device)
    scenes.build_pt_scene(g, d)
    g.set_lights([og.quad_light(L["position"], L["edge1"], L["edge2"], L["intensity"]) if L["type"] == "quad"
                  else og.ambient_light(L["intensity"]) for L in d["lights"]])
    return d, g


def _render(b200_device, pt_world, fmt, tm):
    import ospray_gb300 as og
    d, g = pt_world
    c = d["camera"]
    cam = og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_ACCUM, format=fmt)
    if tm is not None:
        fb.set_tonemapper(og.tonemapper(**tm))
    og.render_pt(g, cam, og.pt_params(spp=2, max_path_length=4), og.materials_array(d["materials"]), fb)
    return fb.read(og.FB_ACCUM), fb.read(og.FB_COLOR)


TM = dict(exposure=2.0)
TM_ORACLE = dict(exposure=2.0)


@pytest.mark.parametrize("fmt", [1, 2, 3])
@pytest.mark.parametrize("tonemap", [False, True])
def test_post_process_matches_oracle(b200_device, pt_world, fmt, tonemap):
    accum, color = _render(b200_device, pt_world, fmt, TM if tonemap else None)
    assert accum.max() > 1.0  # HDR input: the light is in view
    ref = oracle.frame_post(accum, fmt, oracle.tonemapper(**TM_ORACLE) if tonemap else None)
    assert color.shape == ref.shape and color.dtype == ref.dtype
    if fmt == 3:
        if tonemap:
            np.testing.assert_allclose(color, ref, rtol=1e-5, atol=1e-6)
            assert color[..., :3].max() <= 1.0
        else:
            np.testing.assert_array_equal(color, ref)
    else:
        diff = np.abs(color.astype(np.int32) - ref.astype(np.int32))
        if fmt == 1 and not tonemap:
            assert diff.max() == 0
        else:
            assert diff.max() <= 1
            assert np.mean(diff > 0) < 0.01


def test_tonemapper_removed_restores_plain_conversion(b200_device, pt_world):
    import ospray_gb300 as og
    d, g = pt_world
    c = d["camera"]
    cam = og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_ACCUM, format=og.FB_RGBA8)
    fb.set_tonemapper(og.tonemapper())
    p = og.pt_params(spp=1, max_path_length=3)
    og.render_pt(g, cam, p, og.materials_array(d["materials"]), fb)
    fb.set_tonemapper(None)
    og.render_pt(g, cam, p, og.materials_array(d["materials"]), fb)
    np.testing.assert_array_equal(fb.read(og.FB_COLOR), oracle.frame_post(fb.read(og.FB_ACCUM), 1))


def test_pick_matches_oracle(b200_device):
    import ospray_gb300 as og
    from ospray_gb300 import scenes
    d = scenes.ao_heightfield_scene()
    g = og.Scene(b200_device)
    scenes.build_ao_scene(g, d)
    o = oracle.Scene()
    scenes.build_ao_scene(o, d)
    c = d["camera"]
    cam = og.camera_desc(c["position"], c["direction"], c["up"])
    ocam = oracle.camera(c["position"], c["direction"], c["up"])
    hits = misses = 0
    for y in np.linspace(0.0, 1.0, 21):
        for x in np.linspace(0.0, 1.0, 21):
            hit, pos, inst, geom, prim = og.pick(g, cam, x, y)
            rhit, rpos, rids = oracle.pick(o, ocam, x, y)
            assert hit == rhit, (x, y)
            assert (inst, geom, prim) == tuple(int(v) for v in rids), (x, y)
            if hit:
                hits += 1
                np.testing.assert_array_equal(np.float32(pos), rpos)
            else:
                misses += 1
                assert (inst, geom, prim) == (0xffffffff,) * 3
    assert hits >= 10 and misses >= 10  # both surfaces and the sky were picked


def test_variance_estimate_matches_oracle(b200_device, pt_world):
    """ospGetVariance: inf until an odd frame has been accumulated, then the
    task-error estimate of the oracle restatement of Variance_kernel."""
    import os
    import sys
    import ospray_gb300 as og
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
    import variance as vref
    d, g = pt_world
    c = d["camera"]
    cam = og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_ACCUM | og.FB_VARIANCE)
    p = og.pt_params(spp=1, max_path_length=4)
    og.render_pt(g, cam, p, og.materials_array(d["materials"]), fb)
    assert fb.variance() == float("inf")
    values = []
    for frame in range(2, 9):
        og.render_pt(g, cam, p, og.materials_array(d["materials"]), fb)
        if frame % 2 == 0:  # an odd frame (0-based) was just accumulated
            err = vref.task_errors(fb.read(og.FB_ACCUM), fb.read(og.FB_VARIANCE))
            for thr in (0.0, float(np.median(err))):
                exp = vref.avg_error(err, thr)
                got = fb.variance(thr)
                assert abs(got - exp) <= 1e-4 * max(1.0, exp), (frame, thr, got, exp)
            values.append(fb.variance(0.0))
    assert values[-1] < values[0]  # the estimate falls as frames accumulate


def _vref():
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
    import variance as vref
    return vref


def test_variance_buffer_accumulates_the_picked_frames(b200_device, pt_world):
    """FrameBuffer::beginFrame: the variance buffer takes one frame of every
    even/odd pair, picked by std::mt19937(43) coin flips (restated by the
    oracle); a frame that is not picked leaves it bit for bit unchanged, and
    the first pick stores that frame's samples exactly (scale 1)."""
    import ospray_gb300 as og
    vref = _vref()
    d, g = pt_world
    c = d["camera"]
    cam = og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_ACCUM | og.FB_VARIANCE)
    p = og.pt_params(spp=1, max_path_length=3)
    picks = vref.variance_frame_picks(8)
    prev_v = np.zeros((H, W, 4), np.float32)
    acc0 = None
    for f in range(8):
        og.render_pt(g, cam, p, og.materials_array(d["materials"]), fb)
        acc, v = fb.read(og.FB_ACCUM), fb.read(og.FB_VARIANCE)
        if f == 0:
            acc0 = acc
            if picks[0]:
                np.testing.assert_array_equal(v, acc)
        changed = not np.array_equal(v, prev_v)
        assert changed == picks[f], (f, picks)
        if f == 1 and picks[1]:  # the frame-1 samples: 2 * acc1 - acc0
            np.testing.assert_allclose(v, 2.0 * acc - acc0, rtol=1e-4, atol=1e-5)
        prev_v = v


@pytest.mark.parametrize("renderer", ["pt", "ao"])
def test_adaptive_accumulation_renders_selected_tasks(b200_device, pt_world, renderer):
    """varianceThreshold (LocalFrameBuffer::getRenderTaskIDs): from frame
    max(2, 16 / spp) on, a frame renders only the 8x8 tasks whose error
    estimate exceeds the threshold.  Against a second framebuffer rendering
    every task of the same frames: the selected tasks get the same new values
    and every other pixel keeps its previous value bit for bit."""
    import ospray_gb300 as og
    vref = _vref()
    d, g = pt_world
    c = d["camera"]
    cam = og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
    mats = og.materials_array(d["materials"])
    spp = 4 if renderer == "pt" else 1
    start = max(2, 16 // spp)  # first adaptive frame
    if renderer == "pt":
        p = og.pt_params(spp=spp, max_path_length=3)

        def render(fb):
            og.render_pt(g, cam, p, mats, fb)
    else:
        p = og.ao_params(spp=spp, ao_samples=2)

        def render(fb):
            og.render_ao(g, cam, p, fb)
    chans = og.FB_COLOR | og.FB_ACCUM | og.FB_VARIANCE | og.FB_DEPTH
    fa, fr = og.Frame(b200_device, W, H, chans), og.Frame(b200_device, W, H, chans)
    for _ in range(start):
        render(fa)
        render(fr)
    acc_before = fa.read(og.FB_ACCUM)
    err = vref.task_errors(acc_before, fa.read(og.FB_VARIANCE))
    thr = float(np.median(err))
    fa.set_variance_threshold(thr)
    render(fa)
    render(fr)
    acc_a, acc_r = fa.read(og.FB_ACCUM), fr.read(og.FB_ACCUM)
    ty, tx = err.shape
    active = vref.selected_tasks(err, thr)
    clear = np.abs(err - thr) > 1e-3 * max(thr, 1e-6)  # tasks not at the threshold's rounding edge
    assert active[clear].sum() > 5 and (~active[clear]).sum() > 5
    checked = 0
    for y in range(ty):
        for x in range(tx):
            if not clear[y, x]:
                continue
            sl = (slice(8 * y, 8 * y + 8), slice(8 * x, 8 * x + 8))
            if active[y, x]:
                np.testing.assert_allclose(acc_a[sl], acc_r[sl], rtol=1e-5, atol=1e-6)
            else:
                np.testing.assert_array_equal(acc_a[sl], acc_before[sl])
            checked += 1
    assert checked > 0.8 * tx * ty


def test_frame_map_returns_the_channel_in_page_locked_memory(b200_device):
    """b200_frame_map copies a channel into the frame's page-locked buffer for
    it (reused by later maps of the channel) with the bytes b200_frame_read
    returns."""
    import ctypes
    import ospray_gb300 as og
    from ospray_gb300 import scenes
    dev = b200_device
    d = scenes.ao_heightfield_scene()
    g = og.Scene(dev)
    scenes.build_ao_scene(g, d)
    c = d["camera"]
    fb = og.Frame(dev, 64, 48, og.FB_COLOR | og.FB_DEPTH, format=og.FB_RGBA8)
    og.render_ao(g, og.camera_desc(c["position"], c["direction"], c["up"], aspect=64 / 48), og.ao_params(), fb)
    ptrs = []
    for ch, shape, dt in ((og.FB_COLOR, (48, 64, 4), np.uint8), (og.FB_DEPTH, (48, 64), np.float32)):
        p = ctypes.c_void_p()
        dev._check(og.lib().b200_frame_map(fb._h, ch, ctypes.byref(p)))
        n = int(np.prod(shape)) * np.dtype(dt).itemsize
        got = np.frombuffer(ctypes.string_at(p.value, n), dt).reshape(shape)
        np.testing.assert_array_equal(got, fb.read(ch))
        ptrs.append(p.value)
    p2 = ctypes.c_void_p()
    dev._check(og.lib().b200_frame_map(fb._h, og.FB_COLOR, ctypes.byref(p2)))
    assert p2.value == ptrs[0] and ptrs[0] != ptrs[1]
