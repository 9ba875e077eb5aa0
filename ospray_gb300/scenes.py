"""Seeded synthetic workloads (the render configurations the module is
measured on), built by the C generators in csrc/scenegen.cpp.

Each function returns plain numpy arrays plus camera/renderer settings, so
the CUDA renderer and the CPU oracle consume identical inputs.
"""
import ctypes

import numpy as np

from . import scenes_lib

_U64, _I, _F, _P, _U32 = ctypes.c_uint64, ctypes.c_int, ctypes.c_float, ctypes.c_void_p, ctypes.c_uint32


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def heightfield(seed, n):
    """n x n vertices over [0,1]^2, 2 (n-1)^2 triangles (see scenegen.cpp)."""
    v = np.empty((n * n, 3), np.float32)
    i = np.empty((2 * (n - 1) * (n - 1), 3), np.uint32)
    f = scenes_lib().b200sg_heightfield
    f.argtypes = [_U64, _I, _P, _P]
    f(seed, n, _p(v), _p(i))
    return v, i


def spheres(seed, count, r0=0.005, r1=0.02):
    s = np.empty((count, 4), np.float32)
    f = scenes_lib().b200sg_spheres
    f.argtypes = [_U64, _I, _F, _F, _P]
    f(seed, count, r0, r1, _p(s))
    return s


def displaced_sphere(levels=6, amp=0.05, freq=8.0, seed=7):
    f = scenes_lib().b200sg_displaced_sphere
    f.argtypes = [_I, _F, _F, _U32, _P, _P, _P]
    nv = ctypes.c_int()
    f(levels, amp, freq, seed, None, None, ctypes.byref(nv))
    v = np.empty((nv.value, 3), np.float32)
    i = np.empty((8 * 4 ** levels, 3), np.uint32)
    f(levels, amp, freq, seed, _p(v), _p(i), ctypes.byref(nv))
    return v, i


def instances(seed, count, s0=0.5, s1=2.0, box=10.0, pmetal=0.2):
    x = np.empty((count, 12), np.float32)
    m = np.empty((count, 5), np.float32)
    f = scenes_lib().b200sg_instances
    f.argtypes = [_U64, _I, _F, _F, _F, _F, _P, _P]
    f(seed, count, s0, s1, box, pmetal, _p(x), _p(m))
    return x, m


def fractal_volume(n, octaves=5, base_freq=4.0, seed=11):
    out = np.empty((n, n, n), np.float32)
    f = scenes_lib().b200sg_fractal_volume
    f.argtypes = [_I, _I, _F, _U32, _P]
    f(n, octaves, base_freq, seed, _p(out))
    return out


def color_ramp(seed, count=256):
    out = np.empty((count, 3), np.float32)
    f = scenes_lib().b200sg_color_ramp
    f.argtypes = [_U64, _I, _P]
    f(seed, count, _p(out))
    return out


def ao_heightfield_scene(seed=0, n=256, nspheres=1000):
    """AO workload: 256x256-vertex height field (130,050 triangles) and 1,000
    spheres from seed 0, one instance holding both models (geomID 0 mesh,
    1 spheres), camera at (0.5, 2, -1.5) looking at (0.5, 0, 0.5), fovy 60."""
    v, i = heightfield(seed, n)
    s = spheres(seed + 1, nspheres)
    cam = dict(position=(0.5, 2.0, -1.5), direction=(0.0, -2.0, 2.0), up=(0.0, 1.0, 0.0), fovy=60.0, aspect=1.0)
    return dict(vertex=v, index=i, spheres=s, camera=cam)


def pt_instanced_scene(seed=1, count=64, levels=6, width=1920, height=1080):
    """Path-tracer workload: `count` instances of one displaced sphere
    (subdivided octahedron, 8*4^levels = 32,768 triangles at levels 6,
    displaced by 0.05 * value noise of frequency 8) with seeded rotation,
    scale U(0.5, 2) and position U([0,10]^3), each with its own principled
    material (baseColor U(0,1)^3, roughness U(0.05,1), metallic 1 with
    p = 0.2), over a 20x20 two-triangle ground at y = -2.2 (grey 0.8,
    roughness 1).  Lights: a 2x2 quad of intensity 20 at y = 14 facing down
    and an ambient light of intensity 0.1 (in that order).  Camera at
    (5, 9, -13) looking at (5, 3, 5), fovy 50."""
    v, i = displaced_sphere(levels)
    xfm, mat = instances(seed, count)
    ground_v = np.array([[-5, -2.2, -5], [15, -2.2, -5], [-5, -2.2, 15], [15, -2.2, 15]], np.float32)
    ground_i = np.array([[0, 2, 1], [1, 2, 3]], np.uint32)
    mats = [tuple(float(x) for x in m) for m in mat] + [(0.8, 0.8, 0.8, 1.0, 0.0)]
    lights = [dict(type="quad", position=(4.0, 14.0, 4.0), edge1=(2.0, 0.0, 0.0), edge2=(0.0, 0.0, 2.0),
                   intensity=20.0),
              dict(type="ambient", intensity=0.1)]
    cam = dict(position=(5.0, 9.0, -13.0), direction=(0.0, -6.0, 18.0), up=(0.0, 1.0, 0.0), fovy=50.0,
               aspect=width / height)
    return dict(vertex=v, index=i, xfm=xfm, materials=mats, ground_vertex=ground_v, ground_index=ground_i,
                lights=lights, camera=cam, width=width, height=height)


def build_pt_scene(scene, data):
    """Adds the path-tracer workload's geometry to a b200 Scene (or the
    oracle): instance k < count holds the sphere mesh with material k; the
    ground is instance `count` with the last material."""
    gm = scene.add_mesh(data["vertex"], data["index"])
    for k, x in enumerate(data["xfm"]):
        scene.add_instance(gm, k, 0, x, k)
    gg = scene.add_mesh(data["ground_vertex"], data["ground_index"])
    n = len(data["xfm"])
    scene.add_instance(gg, n, 0, None, n)
    scene.commit()


def volume_scene(n=512, seed=11, width=1024, height=1024, orbit_deg=30.0):
    """SciVis volume workload: n^3 float32 of 5-octave fractal value noise
    (base frequency 4, lacunarity 2, gain 0.5) normalised to [0,1] over the
    unit cube (spacing 1/(n-1)); transfer function of 256 seeded ramp
    colours and 256 opacities (0 below 0.3, then linear to 0.8 at 1.0);
    camera on an orbit at 2.5 x the cube diagonal, azimuth `orbit_deg`,
    elevation 20 degrees, looking at the centre, fovy 30."""
    vol = fractal_volume(n, 5, 4.0, seed)
    color = color_ramp(seed, 256)
    v = np.linspace(0.0, 1.0, 256, dtype=np.float32)
    opacity = np.where(v < 0.3, 0.0, 0.8 * (v - 0.3) / 0.7).astype(np.float32)
    d = 2.5 * np.sqrt(3.0)
    az, el = np.radians(orbit_deg), np.radians(20.0)
    eye = np.array([0.5 + d * np.cos(el) * np.sin(az), 0.5 + d * np.sin(el), 0.5 - d * np.cos(el) * np.cos(az)])
    cam = dict(position=tuple(eye), direction=tuple(np.array([0.5, 0.5, 0.5]) - eye), up=(0.0, 1.0, 0.0),
               fovy=30.0, aspect=width / height)
    sp = 1.0 / (n - 1)
    return dict(volume=vol, origin=(0.0, 0.0, 0.0), spacing=(sp, sp, sp), color=color, opacity=opacity,
                value_range=(0.0, 1.0), camera=cam, width=width, height=height)


def build_ao_scene(scene, data):
    """Adds the AO workload's geometry to a b200 Scene (or the oracle)."""
    gm = scene.add_mesh(data["vertex"], data["index"])
    gs = scene.add_spheres(data["spheres"])
    scene.add_instance(gm, 0, 0)
    scene.add_instance(gs, 0, 1)
    scene.commit()


BATCH_SIZES = [(256, 256), (512, 512), (768, 768), (1024, 1024), (1280, 720)]


def batch_requests(seed=0, count=64, n_min=182, n_max=708):
    """Batched-serving workload: `count` independent requests from one seeded
    stream.  Each draws a resolution uniformly from 256^2, 512^2, 768^2,
    1024^2, 1280x720, spp uniformly from 1..8, the AO or the path-tracing
    renderer with probability 1/2, and a height field of its own seed with
    n x n vertices, n uniform in [n_min, n_max] (2 (n-1)^2 = 65k .. 1M
    triangles), plus the AO workload's 1,000 spheres at the same seed."""
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(count):
        w, h = BATCH_SIZES[int(rng.integers(0, len(BATCH_SIZES)))]
        reqs.append(dict(width=w, height=h, spp=int(rng.integers(1, 9)),
                         renderer="ao" if rng.random() < 0.5 else "pathtracer",
                         n=int(rng.integers(n_min, n_max + 1)), seed=1000 + k,
                         material=(float(rng.random()), float(rng.random()), float(rng.random()),
                                   float(0.05 + 0.95 * rng.random()), 0.0)))
    return reqs


def build_batch_request_scene(scene, req, lights=True):
    """The height field (geomID 0) and spheres (geomID 1) of a batch request,
    one instance with material 0; path-tracing requests also get a 0.4 x 0.4
    quad light above the field (intensity 20) and an ambient light (0.2)."""
    import ospray_gb300 as og
    v, i = heightfield(req["seed"], req["n"])
    s = spheres(req["seed"] + 1, 1000)
    gm = scene.add_mesh(v, i)
    gs = scene.add_spheres(s)
    scene.add_instance(gm, 0, 0, None, 0)
    scene.add_instance(gs, 0, 1, None, 0)
    if lights and req["renderer"] == "pathtracer":
        scene.set_lights([og.quad_light((0.3, 1.2, 0.3), (0.4, 0.0, 0.0), (0.0, 0.0, 0.4), 20.0),
                          og.ambient_light(0.2)])
    scene.commit()
    return int(len(i))
