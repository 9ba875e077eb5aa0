"""The oracle's stereo cameras and sub-images on the CPU (PerspectiveCamera
camera/PerspectiveCamera.cpp:37-91 and .ispc:28-41, PanoramicCamera
.cpp:45-52 and .ispc:24-45, Camera_subRegion camera/Camera.ih:28-31).

With power-of-two frame sizes every mapped screen position is exact, so:
the left half of a side-by-side frame is the left-eye frame of half the
width (the aspect halved as side by side halves it); the bottom half of a
top / bottom frame is the right-eye frame of half the height (the aspect
doubled); the sub-image [0, 0.5] x [0, 1] at half the width is the left half
of the whole frame.  Compared: the first hits (depth and IDs), which depend
on the camera rays alone."""
import numpy as np
import pytest

import oracle
from test_motion_gpu import CAM, _build

W, H = 128, 64
KEYS = ("depth", "primID", "instID")


def _ao(w, h, kind=0, **kw):
    o = oracle.Scene()
    _build(o, False)
    aspect = kw.pop("aspect", W / H)
    cam = oracle.camera(CAM["position"], CAM["direction"], CAM["up"], fovy=CAM["fovy"], aspect=aspect, kind=kind,
                        **kw)
    return oracle.render_ao(o, cam, 2, w, h, spp=1, ao_samples=1)


def _eq(a, b):
    for k in KEYS:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.parametrize("kind", [0, 2])
def test_side_by_side_left_half_is_the_left_eye(kind):
    sbs = _ao(W, H, kind, stereo_mode=3, interpupillary_distance=0.3)
    left = _ao(W // 2, H, kind, stereo_mode=1, interpupillary_distance=0.3, aspect=W / H * 0.5)
    right = _ao(W // 2, H, kind, stereo_mode=2, interpupillary_distance=0.3, aspect=W / H * 0.5)
    _eq({k: sbs[k][:, :W // 2] for k in KEYS}, left)
    _eq({k: sbs[k][:, W // 2:] for k in KEYS}, right)
    # the eyes see different images
    hit = np.isfinite(left["depth"])
    assert hit.mean() > 0.1 and np.mean(left["depth"][hit] != right["depth"][hit]) > 0.2


@pytest.mark.parametrize("kind", [0, 2])
def test_top_bottom_puts_the_left_eye_at_the_top(kind):
    tb = _ao(W, H, kind, stereo_mode=4, interpupillary_distance=0.3)
    right = _ao(W, H // 2, kind, stereo_mode=2, interpupillary_distance=0.3, aspect=W / H * 2.0)
    left = _ao(W, H // 2, kind, stereo_mode=1, interpupillary_distance=0.3, aspect=W / H * 2.0)
    _eq({k: tb[k][:H // 2] for k in KEYS}, right)
    _eq({k: tb[k][H // 2:] for k in KEYS}, left)


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_sub_image_is_a_crop_of_the_whole_frame(kind):
    whole = _ao(W, H, kind)
    half = _ao(W // 2, H, kind, image_start=(0.0, 0.0), image_end=(0.5, 1.0))
    _eq({k: whole[k][:, :W // 2] for k in KEYS}, half)
    top = _ao(W, H // 2, kind, image_start=(0.0, 0.5), image_end=(1.0, 1.0))
    _eq({k: whole[k][H // 2:] for k in KEYS}, top)
