import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def b200_device():
    import ospray_gb300 as og
    og.lib()  # raises when the CUDA library is missing: no fallback
    dev = og.Device(0)
    yield dev
    dev.release()  # scenes/frames still alive keep the C-side device until they go
