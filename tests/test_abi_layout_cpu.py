"""The ctypes mirrors of the b200 C ABI structs have the C compiler's sizes
and field offsets (a mismatch shifts every array element after the first)."""
import ctypes
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    "b200_material": ("Material", ["baseColorMap", "specular", "edgeColor", "specularMetallic"]),
    "b200_pt_params": ("PTParams", ["backplate", "mipMapBias", "maxDepth"]),
    "b200_ao_params": ("AOParams", ["backplate", "maxDepth", "materials", "nmaterials"]),
    "b200_scivis_params": ("ScivisParams", ["backplate", "maxDepth", "mipMapBias"]),
    "b200_scivis_material": ("ScivisMaterial", ["kdMap"]),
    "b200_camera_desc": ("CameraDesc", ["shutter", "shutterType", "rollingShutterDuration", "apertureRadius", "imageStart",
                                        "imageEnd", "stereoMode", "interpupillaryDistance",
                                        "architectural"]),
    "b200_light": ("Light", []),
}


def test_ctypes_structs_match_the_c_abi(tmp_path):
    import ospray_gb300 as og
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "b200.h"', "int main(void) {"]
    for cname, (_, fields) in STRUCTS.items():
        lines.append('  printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f in fields:
            lines.append('  printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = str(tmp_path / "layout")
    r = subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = dict(line.split() for line in subprocess.run([exe], capture_output=True, text=True,
                                                        check=True).stdout.splitlines())
    for cname, (pyname, fields) in STRUCTS.items():
        cls = getattr(og, pyname)
        assert ctypes.sizeof(cls) == int(out[cname]), cname
        for f in fields:
            assert getattr(cls, f).offset == int(out["%s.%s" % (cname, f)]), (cname, f)
