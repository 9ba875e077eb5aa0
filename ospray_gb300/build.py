"""Builds the b200 device library (CUDA, sm_103a) and the scene generator.

    python -m ospray_gb300.build          # or __graft_entry__.build()

Outputs go to ospray_gb300/_build/ (git-ignored): libb200.so (the C ABI of
include/b200.h), libospray.so + libospray_module_b200.so (the OSPRay C API of
include/ospray/ospray.h over it, with the "b200" device module) and
libb200_scenes.so (seeded synthetic scene generators).
Translation units are compiled in parallel; a unit is rebuilt only when it or
a header it may include is newer than its object file.
"""
import json
import os
import shutil
import subprocess
import sys
import time
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.environ.get("B200_BUILD_DIR") or os.path.join(HERE, "_build")
ROOT = os.path.dirname(HERE)
TUNED = os.path.join(HERE, "tuned.json")


def tuned_defines():
    """-D flags of the build parameters chosen by tune_build.py (tuned.json),
    overridden by B200_DEFINES (e.g. "B200_STACK_SMEM=32 B200_TRACE_MINBLOCKS=6")."""
    vals = {}
    if os.path.exists(TUNED):
        with open(TUNED) as f:
            vals.update(json.load(f).get("defines", {}))
    for kv in os.environ.get("B200_DEFINES", "").split():
        k, _, v = kv.partition("=")
        vals[k] = v
    return ["-D%s=%s" % (k, v) for k, v in sorted(vals.items())]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + os.path.join(ROOT, "include"),
]
CUDA_UNITS = ["bvh.cu", "render_ao.cu", "render_pt.cu", "render_volume.cu", "render_scivis.cu", "api.cu", "pt_noalloc.cu", "frame_ops.cu", "batch.cu", "nrc.cu", "texture.cu"]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


OSP = os.path.join(CSRC, "osp")
OSP_MODULE_UNITS = ["objects.cpp", "scene_objects.cpp", "b200_device.cpp"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function"]


def _newest_header():
    t = 0.0
    for d in (CSRC, OSP, os.path.join(ROOT, "include"), os.path.join(ROOT, "include", "ospray")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                t = max(t, os.path.getmtime(os.path.join(d, f)))
    return t


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    hdr = _newest_header()
    if os.path.exists(TUNED):
        hdr = max(hdr, os.path.getmtime(TUNED))
    defines = tuned_defines()
    stamp = os.path.join(OUT, "defines.txt")
    if not os.path.exists(stamp) or open(stamp).read() != " ".join(defines):
        hdr = max(hdr, time.time())  # parameters changed: rebuild every unit
    nv = nvcc()
    jobs = []
    objs = []
    for u in CUDA_UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(OUT, u + ".o")
        objs.append(obj)
        if not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr):
            jobs.append([nv] + NVCC_FLAGS + defines + ["-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and r.stderr:
                print(r.stderr, file=sys.stderr)
    lib = os.path.join(OUT, "libb200.so")
    if jobs or not os.path.exists(lib):
        _run([nv] + ARCH + ["-shared", "-o", lib] + objs)
    with open(stamp, "w") as f:
        f.write(" ".join(defines))
    _build_ospray(hdr)
    scenes = os.path.join(OUT, "libb200_scenes.so")
    src = os.path.join(CSRC, "scenegen.cpp")
    if not os.path.exists(scenes) or os.path.getmtime(scenes) < os.path.getmtime(src):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-o", scenes, src, "-lpthread"])
    return lib


def _stale(out, srcs, hdr):
    if not os.path.exists(out):
        return True
    return os.path.getmtime(out) < max([hdr] + [os.path.getmtime(s) for s in srcs])


def _build_ospray(hdr):
    """libospray.so (API entry points) and libospray_module_b200.so (the device)."""
    api = os.path.join(OUT, "libospray.so")
    mod = os.path.join(OUT, "libospray_module_b200.so")
    api_src = [os.path.join(OSP, "api.cpp")]
    if _stale(api, api_src, hdr):
        _run(["g++"] + CXX_FLAGS + ["-shared", "-Wl,-soname,libospray.so", "-o", api] + api_src + ["-ldl"])
    mod_src = [os.path.join(OSP, u) for u in OSP_MODULE_UNITS]
    if _stale(mod, mod_src + [os.path.join(OUT, "libb200.so"), api], hdr):
        _run(["g++"] + CXX_FLAGS + ["-shared", "-o", mod] + mod_src +
             ["-L" + OUT, "-lb200", "-lospray", "-Wl,-rpath,$ORIGIN"])


if __name__ == "__main__":
    print(build(verbose=True))
