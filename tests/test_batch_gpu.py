"""Batched rendering: many requests in one wavefront (b200_batch_*).

A batch of mixed requests (AO with one and with three AO rays per sample,
path tracing, different scenes, sizes and spp) is rendered with a small wave
size, so waves split requests and hold several of them.  Every framebuffer
must equal what the single-request call renders on the same inputs: AO
bit-identical (the batch forms each pixel from the same samples with the
same operation order), path tracing within the tolerance of the shadow-ray
addition order, depth and IDs exact.  Two frames check accumulation; the
CUDA-graph replay, the plain launches and the one persistent launch agree
(including the mapped, tonemapped colour the persistent kernel converts
itself); the autotuner returns one of its candidates and restarts
accumulation."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pt_world(og, dev, levels, w, h):
    from ospray_gb300 import scenes
    d = scenes.pt_instanced_scene(levels=levels, width=w, height=h)
    g = og.Scene(dev)
    scenes.build_pt_scene(g, d)
    g.set_lights([og.quad_light(L["position"], L["edge1"], L["edge2"], L["intensity"]) if L["type"] == "quad"
                  else og.ambient_light(L["intensity"]) for L in d["lights"]])
    c = d["camera"]
    cam = og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"])
    return d, g, cam


def _ao_world(og, dev, w, h):
    from ospray_gb300 import scenes
    d = scenes.ao_heightfield_scene()
    g = og.Scene(dev)
    scenes.build_ao_scene(g, d)
    c = d["camera"]
    return g, og.camera_desc(c["position"], c["direction"], c["up"], aspect=w / h)


CH = None


def _requests(og, dev):
    ch = og.FB_COLOR | og.FB_DEPTH | og.FB_ACCUM | og.FB_ID_PRIMITIVE | og.FB_ID_OBJECT | og.FB_ID_INSTANCE
    reqs = []
    g, cam = _ao_world(og, dev, 96, 64)
    reqs.append(("ao", g, cam, og.ao_params(spp=2, ao_samples=1, pixel_filter=2, bg=(0.1, 0.2, 0.3, 1.0)), 96, 64))
    d, gp, camp = _pt_world(og, dev, 3, 80, 60)
    reqs.append(("pt", gp, camp, og.pt_params(spp=3, max_path_length=4, roulette_path_length=2),
                 og.materials_array(d["materials"]), 80, 60))
    g2, cam2 = _ao_world(og, dev, 70, 50)
    reqs.append(("ao", g2, cam2, og.ao_params(spp=1, ao_samples=3, pixel_filter=0), 70, 50))
    d2, gp2, camp2 = _pt_world(og, dev, 2, 64, 48)
    reqs.append(("pt", gp2, camp2, og.pt_params(spp=1, max_path_length=2), og.materials_array(d2["materials"]),
                 64, 48))
    return ch, reqs


def _single(og, dev, ch, r):
    fb = og.Frame(dev, r[-2], r[-1], ch)
    return fb


@pytest.mark.parametrize("mode", ["graph", "persistent"])
def test_batch_matches_single_requests(b200_device, mode):
    import ospray_gb300 as og
    dev = b200_device
    ch, reqs = _requests(og, dev)
    batch = og.Batch(dev)
    bfbs, sfbs = [], []
    for r in reqs:
        fb = og.Frame(dev, r[-2], r[-1], ch)
        sf = og.Frame(dev, r[-2], r[-1], ch)
        if r[0] == "ao":
            batch.add_ao(r[1], r[2], r[3], fb)
        else:
            batch.add_pt(r[1], r[2], r[3], r[4], fb)
        bfbs.append(fb)
        sfbs.append(sf)
    t = og.BatchTuning(4096, 3, 1)  # small waves: requests split across waves
    batch.tuning = t
    for frame in range(2):
        batch.render(mode=og.BATCH_GRAPH if mode == "graph" else og.BATCH_PERSISTENT)
        for r, sf in zip(reqs, sfbs):
            if r[0] == "ao":
                og.render_ao(r[1], r[2], r[3], sf)
            else:
                og.render_pt(r[1], r[2], r[3], r[4], sf)
        for i, (r, bf, sf) in enumerate(zip(reqs, bfbs, sfbs)):
            msg = "request %d frame %d" % (i, frame)
            for c in (og.FB_DEPTH, og.FB_ID_PRIMITIVE, og.FB_ID_OBJECT, og.FB_ID_INSTANCE):
                np.testing.assert_array_equal(bf.read(c), sf.read(c), err_msg=msg)
            if r[0] == "ao":
                np.testing.assert_array_equal(bf.read(og.FB_COLOR), sf.read(og.FB_COLOR), err_msg=msg)
            else:
                np.testing.assert_allclose(bf.read(og.FB_COLOR), sf.read(og.FB_COLOR), rtol=1e-4, atol=1e-5,
                                           err_msg=msg)
            assert bf.frame_id == frame + 1
    ms, rays = batch.timings()
    assert rays > sum(r[-2] * r[-1] for r in reqs)
    assert np.all(ms > 0) and np.all(np.diff(ms) >= 0)  # requests complete in order
    info = batch.info()
    assert info["waves"] > 1
    if mode == "persistent":
        assert info["kernels"] == 1


def test_persistent_launch_equals_graph_with_post_processing(b200_device):
    """AO requests with mapped RGBA8 (tonemapped) and sRGBA colour: the one
    persistent launch post-processes each request after the wave that
    completes it; bytes equal to the wavefront-kernel graph's, accumulation
    over three frames, the same ray count."""
    import ospray_gb300 as og
    dev = b200_device
    _, reqs = _requests(og, dev)
    ao = [reqs[0], reqs[2]]
    out, counts = {}, {}
    for mode in (og.BATCH_GRAPH, og.BATCH_PERSISTENT):
        batch = og.Batch(dev)
        fbs = []
        for r, fmt in zip(ao, (og.FB_RGBA8, og.FB_SRGBA)):
            fb = og.Frame(dev, r[-2], r[-1], og.FB_COLOR | og.FB_DEPTH | og.FB_ACCUM, format=fmt)
            if fmt == og.FB_RGBA8:
                fb.set_tonemapper(og.tonemapper(exposure=1.5))
            batch.add_ao(r[1], r[2], r[3], fb)
            fbs.append(fb)
        batch.tuning = og.BatchTuning(2048, 3, 1)
        for _ in range(3):
            batch.render(mode=mode)
        out[mode] = [(fb.read(og.FB_COLOR), fb.read(og.FB_ACCUM), fb.read(og.FB_DEPTH)) for fb in fbs]
        counts[mode] = batch.timings()[1]
        assert all(fb.frame_id == 3 for fb in fbs)
    for a, b in zip(out[og.BATCH_GRAPH], out[og.BATCH_PERSISTENT]):
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)
    assert counts[og.BATCH_GRAPH] == counts[og.BATCH_PERSISTENT]
    assert out[og.BATCH_GRAPH][0][0].dtype == np.uint8 and out[og.BATCH_GRAPH][0][0].max() > 0


def test_bad_batch_mode_is_refused(b200_device):
    import ospray_gb300 as og
    dev = b200_device
    _, reqs = _requests(og, dev)
    batch = og.Batch(dev)
    fb = og.Frame(dev, reqs[0][-2], reqs[0][-1])
    batch.add_ao(reqs[0][1], reqs[0][2], reqs[0][3], fb)
    with pytest.raises(og.B200Error):
        batch.render(mode=7)


def test_graph_replay_equals_plain_launch_and_autotune(b200_device):
    import ospray_gb300 as og
    dev = b200_device
    ch, reqs = _requests(og, dev)
    out = []
    for use_graph in (False, True):
        batch = og.Batch(dev)
        fbs = []
        for r in reqs[:1] + reqs[2:3]:  # the AO requests: bit-exact either way
            fb = og.Frame(dev, r[-2], r[-1], ch)
            batch.add_ao(r[1], r[2], r[3], fb)
            fbs.append(fb)
        batch.render(use_graph=use_graph)
        batch.render(use_graph=use_graph)
        out.append([fb.read(og.FB_COLOR) for fb in fbs])
        if use_graph:
            best = batch.autotune(candidates=4)
            assert best.wavePaths >= 2 and best.traceBlocksPerSM in (2, 3, 4, 5) and best.shadeBlocksPerSM in (1, 2)
            assert all(fb.frame_id == 0 for fb in fbs)
            batch.render()
            np.testing.assert_array_equal(fbs[0].read(og.FB_DEPTH), fbs[0].read(og.FB_DEPTH))
    for a, b in zip(out[0], out[1]):
        np.testing.assert_array_equal(a, b)


def test_persistent_barrier_timeout_is_reported_and_recovers(b200_device):
    """Failure detection of the persistent launch without a GPU fault: with a
    barrier bound far shorter than a stage, a wait runs out, every block
    leaves the kernel and the host reports the frame as failed; with the
    default bound the next frames render as the graph does."""
    import ospray_gb300 as og
    dev = b200_device
    _, reqs = _requests(og, dev)
    ao = [reqs[0], reqs[2]]
    out = {}
    for mode in (og.BATCH_GRAPH, og.BATCH_PERSISTENT):
        batch = og.Batch(dev)
        fbs = []
        for r in ao:
            fb = og.Frame(dev, r[-2], r[-1], og.FB_COLOR | og.FB_DEPTH | og.FB_ACCUM)
            batch.add_ao(r[1], r[2], r[3], fb)
            fbs.append(fb)
        batch.tuning = og.BatchTuning(2048, 3, 1)
        if mode == og.BATCH_PERSISTENT:
            batch.set_barrier_timeout(1000)  # 1 us: shorter than any stage
            batch.render(mode=mode)
            with pytest.raises(og.B200Error, match="timed out"):
                batch.timings()
            batch.set_barrier_timeout(0)
            for fb in fbs:
                fb.reset()
        for _ in range(2):
            batch.render(mode=mode)
        batch.timings()
        out[mode] = [fb.read(og.FB_ACCUM) for fb in fbs]
    for a, b in zip(out[og.BATCH_GRAPH], out[og.BATCH_PERSISTENT]):
        np.testing.assert_array_equal(a, b)
