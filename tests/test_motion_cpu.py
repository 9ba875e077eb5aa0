"""The oracle's motion blur restatement on the CPU: at a key's time the
blended instance transform is that key exactly, so a closed shutter there
renders the static instance bit for bit; between keys the instance moves
(the blurred image differs from every key's); the TLAS bounds of a moving
instance hold every key."""
import numpy as np
import pytest

import oracle
from test_motion_gpu import CAM, LIGHTS, _build, _material_dicts

W, H = 64, 48


def _render(shutter, static_key=None):
    o = oracle.Scene()
    _build(o, True, static_key)
    world = oracle.PtWorld(_material_dicts(), LIGHTS)
    cam = oracle.camera(CAM["position"], CAM["direction"], CAM["up"], fovy=CAM["fovy"], aspect=W / H,
                        shutter=shutter)
    return oracle.render_pt(o, world, cam, oracle.pt_params(spp=1, max_path_length=3), W, H)


@pytest.mark.parametrize("t,key", [(0.0, 0), (0.5, 1), (1.0, 2)])
def test_oracle_closed_shutter_at_a_key_is_the_static_key(t, key):
    a, b = _render((t, t)), _render((t, t), static_key=key)
    for k in ("color", "depth", "primID", "instID"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_oracle_open_shutter_blurs():
    blur = _render((0.0, 1.0))
    keys = [_render((t, t)) for t in (0.0, 0.5, 1.0)]
    # the moving sphere shows in pixels where no single key puts it
    b1 = blur["instID"] == 1
    assert all(np.sum(b1 & (k["instID"] != 1)) > 10 for k in keys)
    assert all(np.abs(blur["color"] - k["color"]).max() > 0.05 for k in keys)
