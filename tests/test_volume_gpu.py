"""SciVis volume parity: b200_render_scivis against the oracle's restatement
of SciVis_renderSample / integrateVolumeIntervalsGradient on a seeded
fractal-noise volume.  Both sides step through the same macrocell intervals
with the same jitter (PCG RandomSampler, bit-exact) and sample positions;
they differ only in float contraction and exp() rounding, so per-pixel
colours agree to 1e-4 relative on nearly every pixel."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def vol_setup(b200_device):
    import ospray_gb300 as og
    from ospray_gb300 import scenes
    d = scenes.volume_scene(n=96, width=160, height=120)
    g = og.Scene(b200_device)
    g.set_volume(d["volume"], d["origin"], d["spacing"], d["color"], d["opacity"], d["value_range"])
    o = oracle.VolumeModel(d["volume"], d["origin"], d["spacing"], d["color"], d["opacity"], d["value_range"])
    return d, g, o


def render_both(vol_setup, b200_device, spp=2, frames=1, pf=2, rate=1.0, bg=(0, 0, 0, 0), **cam_kw):
    import ospray_gb300 as og
    d, g, o = vol_setup
    W, H = d["width"], d["height"]
    c = d["camera"]
    fb = og.Frame(b200_device, W, H, og.FB_COLOR | og.FB_ACCUM)
    cam = og.camera_desc(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"], **cam_kw)
    for _ in range(frames):
        og.render_scivis(g, cam, og.scivis_params(spp=spp, sampling_rate=rate, bg=bg, pixel_filter=pf), fb)
    gpu = fb.read(og.FB_COLOR)
    ocam = oracle.camera(c["position"], c["direction"], c["up"], fovy=c["fovy"], aspect=c["aspect"], **cam_kw)
    ref = oracle.render_scivis_volume(o, ocam, pf, W, H, spp=spp, sampling_rate=rate, bg=bg, frames=frames)
    return gpu, ref


@pytest.mark.parametrize("pf,rate", [(2, 1.0), (0, 0.5), (1, 2.0)])
def test_volume_matches_oracle(vol_setup, b200_device, pf, rate):
    gpu, ref = render_both(vol_setup, b200_device, pf=pf, rate=rate)
    assert ref[..., 3].max() > 0.05  # the volume is visible
    close = np.all(np.abs(gpu - ref) <= 1e-4 * np.maximum(1.0, np.abs(ref)) + 1e-6, axis=2)
    assert close.mean() >= 0.999, close.mean()
    assert abs(gpu.mean() - ref.mean()) < 1e-5


@pytest.mark.parametrize("mode", [3, 4])
def test_stereo_volume_matches_oracle(vol_setup, b200_device, mode):
    """Side-by-side and top / bottom stereo over a sub-image (the stereo
    split and Camera_subRegion ahead of the march)."""
    gpu, ref = render_both(vol_setup, b200_device, stereo_mode=mode, interpupillary_distance=0.2,
                           image_start=(0.1, 0.05), image_end=(0.95, 0.9))
    assert ref[..., 3].max() > 0.05
    close = np.all(np.abs(gpu - ref) <= 1e-4 * np.maximum(1.0, np.abs(ref)) + 1e-6, axis=2)
    assert close.mean() >= 0.999, close.mean()


def test_volume_accumulation_and_background(vol_setup, b200_device):
    gpu, ref = render_both(vol_setup, b200_device, spp=1, frames=3, bg=(0.1, 0.2, 0.3, 1.0))
    close = np.all(np.abs(gpu - ref) <= 1e-4, axis=2)
    assert close.mean() >= 0.999, close.mean()


def test_volume_requires_volume(b200_device):
    import ospray_gb300 as og
    s = og.Scene(b200_device)
    fb = og.Frame(b200_device, 8, 8)
    with pytest.raises(og.B200Error) as e:
        og.render_scivis(s, og.camera_desc((0, 0, -1), (0, 0, 1)), og.scivis_params(), fb)
    assert e.value.code == 3
    with pytest.raises(og.B200Error):
        s.set_volume(np.zeros((1, 4, 4), np.float32), (0, 0, 0), (1, 1, 1), np.ones((2, 3)), np.ones(2))
