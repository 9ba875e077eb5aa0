"""ctypes wrapper of the CPU oracle (oracle/_build/liboracle.so).

Test infrastructure only: the tests and bench.py's CPU-baseline leg use it
as the checker/baseline; nothing in the product imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB = os.path.join(ORACLE_DIR, "_build", "liboracle.so")
_lib = None

P, I, U32, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_float


class OrCamera(ctypes.Structure):
    _fields_ = [("pos", F * 3), ("dir", F * 3), ("up", F * 3), ("fovy", F), ("aspect", F), ("nearClip", F),
                ("type", I), ("height", F), ("shutter", F * 2), ("shutterType", I), ("rollingDuration", F),
                ("apertureRadius", F), ("focusDistance", F), ("architectural", I),
                ("imageStart", F * 2), ("imageEnd", F * 2), ("stereoMode", I), ("interpupillaryDistance", F)]


class OrFrame(ctypes.Structure):
    _fields_ = [("color", P), ("depth", P), ("primID", P), ("geomID", P), ("instID", P)]


class OrToneMapper(ctypes.Structure):
    _fields_ = [("exposure", F), ("contrast", F), ("shoulder", F), ("midIn", F), ("midOut", F), ("hdrMax", F),
                ("acesColor", I)]


def tonemapper(exposure=1.0, contrast=1.6773, shoulder=0.9714, mid_in=0.18, mid_out=0.18, hdr_max=11.0785,
               aces_color=True):
    """ToneMapper parameters with the reference's defaults (fb/frame_ops/ToneMapper.cpp:18-36)."""
    return OrToneMapper(exposure, contrast, shoulder, mid_in, mid_out, hdr_max, int(aces_color))


def frame_post(color, fmt, tm=None):
    """Tonemap (tm or None) + colour conversion of an (h,w,4) float32 image.
    fmt 1 RGBA8 / 2 SRGBA -> (h,w,4) uint8; 3 RGBA32F -> (h,w,4) float32."""
    c = np.ascontiguousarray(color, np.float32)
    n = c.shape[0] * c.shape[1]
    out = np.zeros(c.shape, np.float32 if fmt == 3 else np.uint8)
    lib().or_frame_post(_p(c), n, fmt, ctypes.byref(tm) if tm is not None else None, _p(out))
    return out


def tonemap_coefficients(tm):
    out = np.zeros(5, np.float32)
    lib().or_tonemap_coefficients(ctypes.byref(tm), _p(out))
    return dict(zip(("exposure", "a", "b", "c", "d"), out.tolist()))


def pick(scene, cam, x, y):
    pos = np.zeros(3, np.float32)
    ids = np.zeros(3, np.uint32)
    hit = lib().or_pick(scene.h, ctypes.byref(cam), float(x), float(y), _p(pos), _p(ids))
    return bool(hit), pos, ids


class OrPtParams(ctypes.Structure):
    _fields_ = [("spp", I), ("maxPathLength", I), ("roulettePathLength", I), ("maxScatteringEvents", I),
                ("lightSamples", I), ("limitIndirectLightSamples", I), ("minContribution", F),
                ("maxContribution", F), ("bg", F * 4), ("pixelFilter", I), ("backplate", P), ("mipMapBias", F),
                ("maxDepth", P)]


def pt_params(spp=1, max_path_length=20, roulette_path_length=5, max_scattering_events=20, light_samples=-1,
              limit_indirect=True, min_contribution=0.001, max_contribution=float("inf"), bg=(0, 0, 0, 0),
              pixel_filter=2, backplate=None, mip_map_bias=0.0, max_depth=None):
    """backplate / max_depth: OrTextures or None."""
    p = OrPtParams()
    p.maxDepth = None if max_depth is None else max_depth.h
    p.backplate = None if backplate is None else backplate.h
    p.mipMapBias = float(mip_map_bias)
    p.spp, p.maxPathLength, p.roulettePathLength = spp, max_path_length, roulette_path_length
    p.maxScatteringEvents, p.lightSamples, p.limitIndirectLightSamples = max_scattering_events, light_samples, \
        int(limit_indirect)
    p.minContribution, p.maxContribution = min_contribution, max_contribution
    p.bg[:] = list(bg)
    p.pixelFilter = pixel_filter
    return p


# the reference's material parameter defaults per type (Principled.cpp:37-79,
# OBJ.cpp:28-38, Metal.cpp:27-31 with math/spectrum.h's aluminium, Glass.cpp:27-38,
# ThinGlass.cpp:27-33), in the 31-float order of or_pt_add_material2
MATERIAL_TYPES = {"principled": 0, "obj": 1, "metal": 2, "glass": 3, "thinGlass": 4}
_MAT_FIELDS = [("baseColor", 3), ("roughness", 1), ("metallic", 1), ("opacity", 1), ("ks", 3), ("ns", 1),
               ("tf", 3), ("eta", 3), ("k", 3), ("attenuationColor", 3), ("attenuationDistance", 1),
               ("thickness", 1), ("specular", 1), ("ior", 1), ("diffuse", 1), ("edgeColor", 3),
               ("specularMetallic", 1)]
_MAT_DEFAULTS = {
    0: dict(baseColor=(0.8, 0.8, 0.8)),
    1: dict(baseColor=(0.8, 0.8, 0.8), ns=10.0),
    2: dict(eta=(1.47, 0.984, 0.602), k=(7.64, 6.55, 5.36), roughness=0.1),
    3: dict(eta=(1.5, 1.0, 0.0)),
    4: dict(eta=(1.5, 0.0, 0.0)),
}


def material_floats(m):
    """(type, 31 floats) of a material dict, the reference's defaults filled in."""
    t = MATERIAL_TYPES[m.get("type", "principled")]
    vals = dict(opacity=1.0, attenuationColor=(1.0, 1.0, 1.0), attenuationDistance=1.0, thickness=1.0, ns=10.0,
                specular=1.0, ior=1.0, diffuse=1.0, edgeColor=(1.0, 1.0, 1.0), specularMetallic=1.0)
    vals.update(_MAT_DEFAULTS[t])
    vals.update({k: v for k, v in m.items() if k != "type"})
    out = []
    for name, n in _MAT_FIELDS:
        v = vals.get(name, (0.0,) * n if n > 1 else 0.0)
        out.extend([float(x) for x in v] if n > 1 else [float(v)])
    return t, np.asarray(out, np.float32)


class OrTexture:
    """A CPU texture: data (height, width[, channels]) of an OSPTextureFormat,
    rows from the bottom (the layout b200_texture_create takes)."""

    def __init__(self, data, format, filter=0, wrap=(0, 0), mipmaps=True):
        a = np.ascontiguousarray(data)
        if isinstance(wrap, int):
            wrap = (wrap, wrap)
        self.data = a
        self.h = lib().or_texture_new(a.shape[1], a.shape[0], format, filter, wrap[0], wrap[1], int(bool(mipmaps)),
                                      _p(a))

    @property
    def levels(self):
        return lib().or_texture_levels(self.h)

    def read_level(self, level):
        h, w = max(self.data.shape[0] >> level, 1), max(self.data.shape[1] >> level, 1)
        out = np.empty((h, w) + self.data.shape[2:], dtype=self.data.dtype)
        lib().or_texture_read_level(self.h, level, _p(out), out.nbytes)
        return out

    def sample(self, st, footprint):
        st = np.ascontiguousarray(st, np.float32).reshape(-1, 2)
        fp = np.ascontiguousarray(np.broadcast_to(np.asarray(footprint, np.float32), (len(st),)))
        out = np.zeros((len(st), 4), np.float32)
        lib().or_texture_sample(self.h, len(st), _p(st), _p(fp), _p(out))
        return out

    def __del__(self):
        try:
            lib().or_texture_free(self.h)
        except Exception:
            pass


def set_mesh_attributes(scene, geom, normal=None, color=None, texcoord=None):
    """The oracle scene's per-vertex attributes of triangle mesh `geom`
    (colours (n, 4) or (n, 3): alpha 1)."""
    n = None if normal is None else np.ascontiguousarray(normal, np.float32).reshape(-1, 3)
    c = None
    if color is not None:
        c = np.asarray(color, np.float32)
        if c.shape[-1] == 3:
            c = np.concatenate([c.reshape(-1, 3), np.ones((c.size // 3, 1), np.float32)], axis=1)
        c = np.ascontiguousarray(c, np.float32).reshape(-1, 4)
    t = None if texcoord is None else np.ascontiguousarray(texcoord, np.float32).reshape(-1, 2)
    lib().or_scene_set_mesh_attributes(scene.h, geom, _p(n), _p(c), _p(t))


class PtWorld:
    """Materials and lights of the oracle path tracer.  A material dict's
    "baseColorMap" is an OrTexture (principled map_baseColor / obj map_kd)."""

    def __init__(self, materials, lights):
        self.h = lib().or_pt_new()
        self._keep = []
        for m in materials:
            if isinstance(m, dict):
                tex = m.get("baseColorMap")
                t, f = material_floats({k: v for k, v in m.items() if k != "baseColorMap"})
                idx = lib().or_pt_add_material2(self.h, t, _p(f))
                if tex is not None:
                    lib().or_pt_set_material_map(self.h, idx, tex.h)
                    self._keep.append(tex)
                continue
            bc = np.asarray(m[:3], np.float32)
            lib().or_pt_add_material(self.h, _p(bc), float(m[3]), float(m[4]))
        for L in lights:
            rad = np.asarray(L.get("color", (1, 1, 1)), np.float32) * np.float32(L["intensity"])
            if L["type"] == "quad":
                a = [np.asarray(L[k], np.float32) for k in ("position", "edge1", "edge2")]
                lib().or_pt_add_quad_light(self.h, _p(a[0]), _p(a[1]), _p(a[2]), _p(rad))
            elif L["type"] == "distant":
                d = np.asarray(L["direction"], np.float32)
                lib().or_pt_add_distant_light(self.h, _p(d), float(L.get("angular_diameter", 0.0)), _p(rad))
            elif L["type"] == "sphere":
                pos = np.asarray(L["position"], np.float32)
                lib().or_pt_add_sphere_light(self.h, _p(pos), float(L.get("radius", 0.0)), _p(rad))
            elif L["type"] == "spot":
                pos, d = np.asarray(L["position"], np.float32), np.asarray(L["direction"], np.float32)
                lib().or_pt_add_spot_light(self.h, _p(pos), _p(d), float(L.get("opening_angle", 180.0)),
                                           float(L.get("penumbra_angle", 5.0)), float(L.get("radius", 0.0)),
                                           float(L.get("inner_radius", 0.0)), _p(rad))
            else:
                lib().or_pt_add_ambient_light(self.h, _p(rad))

    def __del__(self):
        try:
            lib().or_pt_free(self.h)
        except Exception:
            pass


def render_pt(scene, world, cam, params, w, h, frames=1, rows=None, nthreads=0):
    """Returns color (h,w,4), depth (h,w), ids (3,h,w); rows=(y0,y1) renders
    only those rows (the others stay zero)."""
    color = np.zeros((h, w, 4), np.float32)
    depth = np.zeros((h, w), np.float32)
    ids = np.zeros((3, h, w), np.uint32)
    y0, y1 = rows if rows else (0, 0)
    lib().or_render_pt(scene.h, world.h, ctypes.byref(cam), ctypes.byref(params), w, h, frames, y0, y1,
                       _p(color), _p(depth), _p(ids), nthreads)
    return dict(color=color, depth=depth, primID=ids[0], geomID=ids[1], instID=ids[2])


def build():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.or_scene_new.restype = P
        L.or_scene_free.argtypes = [P]
        L.or_scene_add_mesh.argtypes = [P, P, I, P, I]
        L.or_scene_add_quad_mesh.argtypes = [P, P, I, P, I]
        L.or_scene_add_boxes.argtypes = [P, P, I]
        L.or_set_aux_output.argtypes = [P, P]
        L.or_set_ao_volume.argtypes = [P, F]
        L.or_scene_add_spheres.argtypes = [P, P, I]
        L.or_scene_add_discs.argtypes = [P, P, I, P]
        L.or_scene_add_planes.argtypes = [P, P, I, P]
        L.or_scene_add_instance.argtypes = [P, I, U32, U32, P, I]
        L.or_scene_add_instance_motion.argtypes = [P, I, U32, U32, P, I, F, F, I]
        L.or_pt_new.restype = P
        L.or_pt_free.argtypes = [P]
        L.or_pt_add_material.argtypes = [P, P, F, F]
        L.or_pt_add_material2.argtypes = [P, I, P]
        L.or_pt_set_material_map.argtypes = [P, I, P]
        L.or_scene_set_mesh_attributes.argtypes = [P, I, P, P, P]
        L.or_texture_new.restype = P
        L.or_texture_new.argtypes = [I, I, I, I, I, I, I, P]
        L.or_texture_free.argtypes = [P]
        L.or_texture_levels.argtypes = [P]
        L.or_texture_read_level.restype = ctypes.c_size_t
        L.or_texture_read_level.argtypes = [P, I, P, ctypes.c_size_t]
        L.or_texture_sample.argtypes = [P, I, P, P, P]
        L.or_pt_add_quad_light.argtypes = [P, P, P, P, P]
        L.or_pt_add_ambient_light.argtypes = [P, P]
        L.or_pt_add_distant_light.argtypes = [P, P, F, P]
        L.or_pt_add_sphere_light.argtypes = [P, P, F, P]
        L.or_pt_add_spot_light.argtypes = [P, P, P, F, F, F, F, P]
        L.or_render_pt.argtypes = [P, P, ctypes.POINTER(OrCamera), ctypes.POINTER(OrPtParams), I, I, I, I, I,
                                   P, P, P, I]
        L.or_ray_count.restype = ctypes.c_uint64
        L.or_ray_count.argtypes = [I]
        L.or_volume_new.restype = P
        L.or_volume_new.argtypes = [P, I, I, I, P, P, P, I, P, I, F, F, F]
        L.or_volume_free.argtypes = [P]
        L.or_volume_set_gradient_shading.argtypes = [P, F]
        L.or_volume_set_transform.argtypes = [P, P]
        L.or_volume_sample_count.restype = ctypes.c_uint64
        L.or_volume_sample_count.argtypes = [I]
        L.or_render_scivis_volume.argtypes = [P, ctypes.POINTER(OrCamera), I, I, I, I, F, P, I, I, I, P, I]
        L.or_render_scivis.argtypes = [P, P, ctypes.POINTER(OrCamera), ctypes.POINTER(OrScivisParams), P, I, P, I,
                                       I, I, I, I, I, P, P, P, I]
        L.or_scene_commit.argtypes = [P]
        L.or_trace.argtypes = [P, P, I, I, P, P, I]
        L.or_camera_rays.argtypes = [ctypes.POINTER(OrCamera), I, I, I, I, I, P]
        L.or_render_ao.argtypes = [P, ctypes.POINTER(OrCamera), I, I, I, I, I, F, F, P, I,
                                   ctypes.POINTER(OrFrame), I, ctypes.POINTER(OrAoExtra)]
        L.or_tables.argtypes = [P, P, P, P]
        L.or_frame_post.argtypes = [P, ctypes.c_longlong, I, ctypes.POINTER(OrToneMapper), P]
        L.or_tonemap_coefficients.argtypes = [ctypes.POINTER(OrToneMapper), P]
        L.or_pick.restype = I
        L.or_pick.argtypes = [P, ctypes.POINTER(OrCamera), F, F, P, P]
        _lib = L
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def camera(position, direction, up=(0, 1, 0), fovy=60.0, aspect=1.0, near_clip=1e-6, kind=0, height=1.0,
           shutter=(0.5, 0.5), shutter_type=0, rolling_shutter_duration=0.0, aperture_radius=0.0,
           focus_distance=1.0, architectural=False, image_start=(0.0, 0.0), image_end=(1.0, 1.0), stereo_mode=0,
           interpupillary_distance=0.0635):
    """kind 0 perspective, 1 orthographic (image `height`), 2 panoramic; shutter, sub-image and stereo as the
    b200 camera."""
    c = OrCamera()
    c.imageStart[:], c.imageEnd[:] = list(map(float, image_start)), list(map(float, image_end))
    c.stereoMode, c.interpupillaryDistance = int(stereo_mode), float(interpupillary_distance)
    c.pos[:], c.dir[:], c.up[:] = list(position), list(direction), list(up)
    c.fovy, c.aspect, c.nearClip = fovy, aspect, near_clip
    c.type, c.height = int(kind), float(height)
    c.shutter[:] = [float(shutter[0]), float(shutter[1])]
    c.shutterType, c.rollingDuration = int(shutter_type), float(rolling_shutter_duration)
    c.apertureRadius, c.focusDistance = float(aperture_radius), float(focus_distance)
    c.architectural = int(bool(architectural))
    return c


class Scene:
    def __init__(self):
        self.h = lib().or_scene_new()
        self._keep = []

    def add_mesh(self, vertex, index):
        v = np.ascontiguousarray(vertex, np.float32)
        i = np.ascontiguousarray(index, np.uint32)
        return lib().or_scene_add_mesh(self.h, _p(v), len(v), _p(i), len(i))

    def add_quad_mesh(self, vertex, index):
        v = np.ascontiguousarray(vertex, np.float32)
        i = np.ascontiguousarray(index, np.uint32).reshape(-1, 4)
        return lib().or_scene_add_quad_mesh(self.h, _p(v), len(v), _p(i), len(i))

    def add_boxes(self, boxes):
        b = np.ascontiguousarray(boxes, np.float32).reshape(-1, 6)
        return lib().or_scene_add_boxes(self.h, _p(b), len(b))

    def add_spheres(self, xyzr):
        s = np.ascontiguousarray(xyzr, np.float32)
        return lib().or_scene_add_spheres(self.h, _p(s), len(s))

    def add_discs(self, xyzr, normals=None):
        s = np.ascontiguousarray(xyzr, np.float32).reshape(-1, 4)
        n = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
        return lib().or_scene_add_discs(self.h, _p(s), len(s), _p(n))

    def add_planes(self, coeffs, bounds=None):
        c = np.ascontiguousarray(coeffs, np.float32).reshape(-1, 4)
        b = None if bounds is None else np.ascontiguousarray(bounds, np.float32).reshape(-1, 6)
        return lib().or_scene_add_planes(self.h, _p(c), len(c), _p(b))

    def add_instance_motion(self, geom, inst_id, geom_id, xfms, time=(0.0, 1.0), material=-1):
        x = np.ascontiguousarray(xfms, dtype=np.float32).reshape(-1, 12)
        lib().or_scene_add_instance_motion(self.h, geom, inst_id, geom_id, _p(x), len(x), float(time[0]),
                                           float(time[1]), material)

    def add_instance(self, geom, inst_id, geom_id, xfm=None, material=-1):
        x = None if xfm is None else np.ascontiguousarray(xfm, np.float32).reshape(12)
        lib().or_scene_add_instance(self.h, geom, inst_id, geom_id, _p(x), material)

    def commit(self):
        lib().or_scene_commit(self.h)

    def trace(self, rays, occlusion=False, nthreads=0):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        f = np.zeros((len(rays), 6), np.float32)
        ids = np.zeros((len(rays), 3), np.uint32)
        lib().or_trace(self.h, _p(rays), len(rays), int(occlusion), _p(f), _p(ids), nthreads)
        return f, ids

    def __del__(self):
        try:
            lib().or_scene_free(self.h)
        except Exception:
            pass


def camera_rays(cam, pixel_filter, w, h, spp=1, frame_id=0):
    out = np.empty((h, w, spp, 8), np.float32)
    lib().or_camera_rays(ctypes.byref(cam), pixel_filter, w, h, spp, frame_id, _p(out))
    return out


class OrAoExtra(ctypes.Structure):
    _fields_ = [("backplate", P), ("maxDepth", P), ("mipMapBias", F), ("materials", P), ("nmaterials", I)]


def _scivis_material_array(materials):
    M = (OrScivisMaterial * max(1, len(materials)))()
    for i, m in enumerate(materials):
        if m is None:
            continue
        M[i].isObj = 1
        M[i].kd[:] = [float(x) for x in m.get("kd", (0.8, 0.8, 0.8))]
        M[i].ks[:] = [float(x) for x in m.get("ks", (0, 0, 0))]
        M[i].ns, M[i].d = float(m.get("ns", 10.0)), float(m.get("d", 1.0))
        M[i].tf[:] = [float(x) for x in m.get("tf", (0, 0, 0))]
        M[i].kdMap = None if m.get("map_kd") is None else m["map_kd"].h
    return M


def render_ao(scene, cam, pixel_filter, w, h, spp=1, ao_samples=1, ao_radius=1e20, ao_intensity=1.0,
              bg=(0, 0, 0, 0), frames=1, nthreads=0, backplate=None, max_depth=None, mip_map_bias=0.0,
              materials=None):
    """materials: obj material dicts (kd, d, map_kd an OrTexture) or None per slot;
    backplate / max_depth: OrTextures."""
    x = OrAoExtra()
    x.backplate = None if backplate is None else backplate.h
    x.maxDepth = None if max_depth is None else max_depth.h
    x.mipMapBias = float(mip_map_bias)
    M = _scivis_material_array(materials or [])
    x.materials = ctypes.cast(M, P) if materials else None
    x.nmaterials = len(materials) if materials else 0
    color = np.zeros((h, w, 4), np.float32)
    depth = np.zeros((h, w), np.float32)
    ids = [np.zeros((h, w), np.uint32) for _ in range(3)]
    fr = OrFrame(color.ctypes.data, depth.ctypes.data, ids[0].ctypes.data, ids[1].ctypes.data, ids[2].ctypes.data)
    bgv = np.asarray(bg, np.float32)
    lib().or_render_ao(scene.h, ctypes.byref(cam), pixel_filter, w, h, spp, ao_samples, ao_radius, ao_intensity,
                       _p(bgv), frames, ctypes.byref(fr), nthreads, ctypes.byref(x))
    return dict(color=color, depth=depth, primID=ids[0], geomID=ids[1], instID=ids[2])


class AOVolume:
    """Within the block, oracle AO renders composite `model` (a
    VolumeModel) in front of each layer at `rate` (the AO renderer's
    volumeSamplingRate)."""

    def __init__(self, model, rate=1.0):
        self.model, self.rate = model, rate

    def __enter__(self):
        lib().or_set_ao_volume(self.model.h, float(self.rate))
        return self

    def __exit__(self, *a):
        lib().or_set_ao_volume(None, 1.0)


class AuxOutput:
    """Within the block, oracle renders also return the accumulated normal
    and albedo channels: `with AuxOutput(w, h) as aux: ...; aux.normal`."""

    def __init__(self, w, h):
        self.normal = np.zeros((h, w, 3), np.float32)
        self.albedo = np.zeros((h, w, 3), np.float32)

    def __enter__(self):
        lib().or_set_aux_output(_p(self.normal), _p(self.albedo))
        return self

    def __exit__(self, *a):
        lib().or_set_aux_output(None, None)


def tables():
    p3, p5, p7 = np.zeros(243, np.uint32), np.zeros(125, np.uint32), np.zeros(343, np.uint32)
    s = np.zeros(128, np.uint32)
    lib().or_tables(_p(p3), _p(p5), _p(p7), _p(s))
    return {"halton_perm3": p3, "halton_perm5": p5, "halton_perm7": p7, "Sobol_revMatrices": s}


class VolumeModel:
    """Oracle structured-regular volume + transfer function."""

    def __init__(self, data, origin, spacing, color, opacity, value_range=(0.0, 1.0), density_scale=1.0):
        d = np.ascontiguousarray(data, np.float32)
        nz, ny, nx = d.shape
        o, sp = np.asarray(origin, np.float32), np.asarray(spacing, np.float32)
        c = np.ascontiguousarray(color, np.float32).reshape(-1, 3)
        op = np.ascontiguousarray(opacity, np.float32).reshape(-1)
        self.h = lib().or_volume_new(_p(d), nx, ny, nz, _p(o), _p(sp), _p(c), len(c), _p(op), len(op),
                                     float(value_range[0]), float(value_range[1]), float(density_scale))

    def set_transform(self, xfm):
        """The volume's instance transform (3x4 row-major) or None."""
        self._xfm = None if xfm is None else np.ascontiguousarray(xfm, np.float32).reshape(12)
        lib().or_volume_set_transform(self.h, _p(self._xfm) if self._xfm is not None else None)

    def set_gradient_shading(self, scale):
        """The volumetric model's gradientShadingScale (default 0: off)."""
        lib().or_volume_set_gradient_shading(self.h, float(scale))

    def __del__(self):
        try:
            lib().or_volume_free(self.h)
        except Exception:
            pass


def render_scivis_volume(model, cam, pixel_filter, w, h, spp=1, sampling_rate=1.0, bg=(0, 0, 0, 0), frames=1,
                         rows=None, nthreads=0):
    color = np.zeros((h, w, 4), np.float32)
    bgv = np.asarray(bg, np.float32)
    y0, y1 = rows if rows else (0, 0)
    lib().or_render_scivis_volume(model.h, ctypes.byref(cam), pixel_filter, w, h, spp, sampling_rate, _p(bgv),
                                  frames, y0, y1, _p(color), nthreads)
    return color


class OrScivisLight(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("visible", ctypes.c_int), ("pos", ctypes.c_float * 3),
                ("e1", ctypes.c_float * 3), ("e2", ctypes.c_float * 3), ("radiance", ctypes.c_float * 3),
                ("dir", ctypes.c_float * 3), ("angularDiameter", ctypes.c_float), ("radius", ctypes.c_float),
                ("openingAngle", ctypes.c_float), ("penumbraAngle", ctypes.c_float), ("innerRadius", ctypes.c_float)]


class OrScivisMaterial(ctypes.Structure):
    _fields_ = [("isObj", ctypes.c_int), ("kd", ctypes.c_float * 3), ("ks", ctypes.c_float * 3),
                ("ns", ctypes.c_float), ("d", ctypes.c_float), ("tf", ctypes.c_float * 3), ("kdMap", P)]


class OrScivisParams(ctypes.Structure):
    _fields_ = [("spp", ctypes.c_int), ("samplingRate", ctypes.c_float), ("bg", ctypes.c_float * 4),
                ("shadows", ctypes.c_int), ("visibleLights", ctypes.c_int), ("aoSamples", ctypes.c_int),
                ("aoRadius", ctypes.c_float), ("minContribution", ctypes.c_float), ("pixelFilter", ctypes.c_int),
                ("backplate", P), ("maxDepth", P), ("mipMapBias", F)]


def render_scivis(scene, volume, cam, lights, materials, w, h, spp=1, pixel_filter=2, sampling_rate=1.0,
                  bg=(0, 0, 0, 0), shadows=False, visible_lights=False, ao_samples=0, ao_radius=1e20,
                  min_contribution=0.001, frames=1, rows=None, nthreads=0, backplate=None, max_depth=None,
                  mip_map_bias=0.0):
    """SciVis over a world with surfaces (and optionally `volume`, a
    VolumeModel); scene None renders the volume alone through the same
    integrator (gradient shading included).  lights: dicts as PtWorld takes them (+ "visible");
    materials: dicts {"kd", "ks", "ns", "d", "tf"} for obj materials or None.
    Returns color (h,w,4), depth (h,w), ids (3,h,w)."""
    L = (OrScivisLight * max(1, len(lights)))()
    for i, l in enumerate(lights):
        rad = np.asarray(l.get("color", (1, 1, 1)), np.float32) * np.float32(l["intensity"])
        L[i].kind = {"quad": 0, "ambient": 1, "distant": 2, "sphere": 3, "spot": 4}[l["type"]]
        L[i].visible = int(l.get("visible", True))
        L[i].radiance[:] = [float(x) for x in rad]
        if l["type"] == "quad":
            L[i].pos[:], L[i].e1[:], L[i].e2[:] = ([float(x) for x in l[k]] for k in ("position", "edge1", "edge2"))
        elif l["type"] == "distant":
            L[i].dir[:] = [float(x) for x in l["direction"]]
            L[i].angularDiameter = float(l.get("angular_diameter", 0.0))
        elif l["type"] == "sphere":
            L[i].pos[:] = [float(x) for x in l["position"]]
            L[i].radius = float(l.get("radius", 0.0))
        elif l["type"] == "spot":
            L[i].pos[:] = [float(x) for x in l["position"]]
            L[i].dir[:] = [float(x) for x in l["direction"]]
            L[i].openingAngle = float(l.get("opening_angle", 180.0))
            L[i].penumbraAngle = float(l.get("penumbra_angle", 5.0))
            L[i].radius = float(l.get("radius", 0.0))
            L[i].innerRadius = float(l.get("inner_radius", 0.0))
    M = _scivis_material_array(materials)
    p = OrScivisParams()
    p.backplate = None if backplate is None else backplate.h
    p.maxDepth = None if max_depth is None else max_depth.h
    p.mipMapBias = float(mip_map_bias)
    p.spp, p.samplingRate = int(spp), float(sampling_rate)
    p.bg[:] = [float(x) for x in bg]
    p.shadows, p.visibleLights, p.aoSamples = int(bool(shadows)), int(bool(visible_lights)), int(ao_samples)
    p.aoRadius, p.minContribution, p.pixelFilter = float(ao_radius), float(min_contribution), int(pixel_filter)
    color = np.zeros((h, w, 4), np.float32)
    depth = np.zeros((h, w), np.float32)
    ids = np.zeros((3, h, w), np.uint32)
    y0, y1 = rows if rows else (0, 0)
    lib().or_render_scivis(scene.h if scene is not None else None, volume.h if volume is not None else None, ctypes.byref(cam), ctypes.byref(p), L,
                           len(lights), M, len(materials), w, h, frames, y0, y1, _p(color), _p(depth), _p(ids),
                           nthreads)
    return dict(color=color, depth=depth, primID=ids[0], geomID=ids[1], instID=ids[2])
