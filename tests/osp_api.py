"""The OSPRay C API through ctypes, for the tests (ospray_gb300.osp)."""
from ospray_gb300.osp import *  # noqa: F401,F403
from ospray_gb300.osp import BUILD, ROOT, lib  # noqa: F401
