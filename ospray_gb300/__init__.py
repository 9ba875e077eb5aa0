"""ospray_gb300: GB300-native device module for the OSPRay render path.

The compute path is the CUDA library ``_build/libb200.so`` (C ABI in
``include/b200.h``); this package is a thin ctypes layer over it, used by the
tests, the benchmark and Python callers.  There is no CPU fallback: every
call goes to the CUDA library, and importing a renderer without the built
library raises.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.environ.get("B200_BUILD_DIR") or os.path.join(HERE, "_build")

_lib = None
_scenes = None

# OSPFrameBufferFormat
FB_NONE, FB_RGBA8, FB_SRGBA, FB_RGBA32F = 0, 1, 2, 3
# OSPFrameBufferChannel bits
FB_COLOR, FB_DEPTH, FB_ACCUM, FB_VARIANCE = 1, 2, 4, 8
FB_NORMAL, FB_ALBEDO = 16, 32
FB_ID_PRIMITIVE, FB_ID_OBJECT, FB_ID_INSTANCE = 64, 128, 256
# OSPPixelFilterType
PF_POINT, PF_BOX, PF_GAUSS, PF_MITCHELL, PF_BLACKMAN_HARRIS = range(5)

ERRORS = {0: "OSP_NO_ERROR", 1: "OSP_UNKNOWN_ERROR", 2: "OSP_INVALID_ARGUMENT",
          3: "OSP_INVALID_OPERATION", 4: "OSP_OUT_OF_MEMORY", 5: "OSP_UNSUPPORTED_CPU",
          6: "OSP_VERSION_MISMATCH"}


class B200Error(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (ERRORS.get(code, code), msg))
        self.code = code


class CameraDesc(ctypes.Structure):
    _fields_ = [("position", ctypes.c_float * 3), ("direction", ctypes.c_float * 3),
                ("up", ctypes.c_float * 3), ("fovy", ctypes.c_float), ("aspect", ctypes.c_float),
                ("nearClip", ctypes.c_float), ("type", ctypes.c_int), ("height", ctypes.c_float),
                ("shutter", ctypes.c_float * 2), ("shutterType", ctypes.c_int),
                ("rollingShutterDuration", ctypes.c_float), ("apertureRadius", ctypes.c_float),
                ("focusDistance", ctypes.c_float), ("architectural", ctypes.c_int),
                ("imageStart", ctypes.c_float * 2), ("imageEnd", ctypes.c_float * 2), ("stereoMode", ctypes.c_int),
                ("interpupillaryDistance", ctypes.c_float)]


class AOParams(ctypes.Structure):
    _fields_ = [("pixelSamples", ctypes.c_int), ("aoSamples", ctypes.c_int),
                ("aoDistance", ctypes.c_float), ("aoIntensity", ctypes.c_float),
                ("backgroundColor", ctypes.c_float * 4), ("pixelFilter", ctypes.c_int),
                ("collectStats", ctypes.c_int), ("volumeSamplingRate", ctypes.c_float),
                ("backplate", ctypes.c_void_p), ("maxDepth", ctypes.c_void_p), ("mipMapBias", ctypes.c_float),
                ("materials", ctypes.c_void_p), ("nmaterials", ctypes.c_int)]


LIGHT_QUAD, LIGHT_AMBIENT, LIGHT_DISTANT, LIGHT_SPHERE, LIGHT_SPOT = 0, 1, 2, 3, 4


class Light(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int), ("visible", ctypes.c_int), ("position", ctypes.c_float * 3),
                ("edge1", ctypes.c_float * 3), ("edge2", ctypes.c_float * 3), ("color", ctypes.c_float * 3),
                ("intensity", ctypes.c_float), ("direction", ctypes.c_float * 3), ("angularDiameter", ctypes.c_float),
                ("radius", ctypes.c_float), ("openingAngle", ctypes.c_float), ("penumbraAngle", ctypes.c_float),
                ("innerRadius", ctypes.c_float)]


class ToneMapper(ctypes.Structure):
    """b200_tonemapper: the ACES-fit tonemapper frame operation."""
    _fields_ = [("exposure", ctypes.c_float), ("contrast", ctypes.c_float), ("shoulder", ctypes.c_float),
                ("midIn", ctypes.c_float), ("midOut", ctypes.c_float), ("hdrMax", ctypes.c_float),
                ("acesColor", ctypes.c_int)]


class PickResult(ctypes.Structure):
    _fields_ = [("hasHit", ctypes.c_int), ("worldPosition", ctypes.c_float * 3), ("instID", ctypes.c_uint32),
                ("geomID", ctypes.c_uint32), ("primID", ctypes.c_uint32)]


class Material(ctypes.Structure):
    _fields_ = [("baseColor", ctypes.c_float * 3), ("roughness", ctypes.c_float), ("metallic", ctypes.c_float),
                ("type", ctypes.c_int), ("opacity", ctypes.c_float), ("ks", ctypes.c_float * 3),
                ("ns", ctypes.c_float), ("tf", ctypes.c_float * 3), ("eta", ctypes.c_float * 3),
                ("k", ctypes.c_float * 3), ("attenuationColor", ctypes.c_float * 3),
                ("attenuationDistance", ctypes.c_float), ("thickness", ctypes.c_float),
                ("baseColorMap", ctypes.c_void_p), ("specular", ctypes.c_float), ("ior", ctypes.c_float),
                ("diffuse", ctypes.c_float), ("edgeColor", ctypes.c_float * 3), ("specularMetallic", ctypes.c_int)]


MATERIAL_PRINCIPLED, MATERIAL_OBJ, MATERIAL_METAL, MATERIAL_GLASS, MATERIAL_THINGLASS = 0, 1, 2, 3, 4
_MATERIAL_TYPES = {"principled": MATERIAL_PRINCIPLED, "obj": MATERIAL_OBJ, "metal": MATERIAL_METAL,
                   "glass": MATERIAL_GLASS, "thinGlass": MATERIAL_THINGLASS}


def principled(base_color=(0.8, 0.8, 0.8), roughness=0.0, metallic=0.0, opacity=1.0, base_color_map=None,
               specular=1.0, ior=1.0, diffuse=1.0, edge_color=(1.0, 1.0, 1.0), specular_metallic=True):
    """base_color_map: a Texture (map_baseColor)."""
    return dict(type="principled", baseColor=base_color, roughness=roughness, metallic=metallic, opacity=opacity,
                baseColorMap=base_color_map, specular=specular, ior=ior, diffuse=diffuse, edgeColor=edge_color,
                specularMetallic=int(bool(specular_metallic)))


def obj_material(kd=(0.8, 0.8, 0.8), ks=(0.0, 0.0, 0.0), ns=10.0, d=1.0, tf=(0.0, 0.0, 0.0), map_kd=None):
    """map_kd: a Texture."""
    return dict(type="obj", baseColor=kd, ks=ks, ns=ns, opacity=d, tf=tf, baseColorMap=map_kd)


def metal(eta=(1.47, 0.984, 0.602), k=(7.64, 6.55, 5.36), roughness=0.1):
    return dict(type="metal", eta=eta, k=k, roughness=roughness)


def glass(eta_inside=1.5, eta_outside=1.0, attenuation_color=(1.0, 1.0, 1.0), attenuation_distance=1.0):
    return dict(type="glass", eta=(eta_inside, eta_outside, 0.0), attenuationColor=attenuation_color,
                attenuationDistance=attenuation_distance)


def thin_glass(eta=1.5, attenuation_color=(1.0, 1.0, 1.0), attenuation_distance=1.0, thickness=1.0):
    return dict(type="thinGlass", eta=(eta, 0.0, 0.0), attenuationColor=attenuation_color,
                attenuationDistance=attenuation_distance, thickness=thickness)


def material_struct(m):
    """A b200_material from a (r, g, b, roughness, metallic) principled tuple
    or a dict made by principled / obj_material / metal / glass / thin_glass."""
    out = Material()
    if isinstance(m, dict):
        t = _MATERIAL_TYPES[m.get("type", "principled")]
        lib().b200_material_defaults(ctypes.byref(out), t)
        for key, val in m.items():
            if key == "type":
                continue
            if key == "baseColorMap":
                out.baseColorMap = None if val is None else val._h.value
                continue
            if isinstance(val, (tuple, list, np.ndarray)):
                getattr(out, key)[:] = [float(x) for x in val]
            elif key == "specularMetallic":
                out.specularMetallic = int(val)
            else:
                setattr(out, key, float(val))
        return out
    lib().b200_material_defaults(ctypes.byref(out), MATERIAL_PRINCIPLED)
    out.baseColor[:] = [float(m[0]), float(m[1]), float(m[2])]
    out.roughness, out.metallic = float(m[3]), float(m[4])
    return out


class PTParams(ctypes.Structure):
    _fields_ = [("pixelSamples", ctypes.c_int), ("maxPathLength", ctypes.c_int),
                ("roulettePathLength", ctypes.c_int), ("maxScatteringEvents", ctypes.c_int),
                ("lightSamples", ctypes.c_int), ("limitIndirectLightSamples", ctypes.c_int),
                ("minContribution", ctypes.c_float), ("maxContribution", ctypes.c_float),
                ("backgroundColor", ctypes.c_float * 4), ("pixelFilter", ctypes.c_int),
                ("collectStats", ctypes.c_int), ("backplate", ctypes.c_void_p), ("mipMapBias", ctypes.c_float),
                ("maxDepth", ctypes.c_void_p)]


def quad_light(position, edge1, edge2, intensity=1.0, color=(1, 1, 1), visible=True):
    L = Light()
    L.type, L.visible = LIGHT_QUAD, int(visible)
    L.position[:], L.edge1[:], L.edge2[:] = list(position), list(edge1), list(edge2)
    L.color[:], L.intensity = list(color), float(intensity)
    return L


def ambient_light(intensity=1.0, color=(1, 1, 1), visible=True):
    L = Light()
    L.type, L.visible = LIGHT_AMBIENT, int(visible)
    L.color[:], L.intensity = list(color), float(intensity)
    return L


def distant_light(direction, intensity=1.0, color=(1, 1, 1), angular_diameter=0.0, visible=True):
    """direction: the direction the light travels; irradiance = color * intensity."""
    L = Light()
    L.type, L.visible = LIGHT_DISTANT, int(visible)
    L.direction[:] = list(direction)
    L.angularDiameter = float(angular_diameter)
    L.color[:], L.intensity = list(color), float(intensity)
    return L


def sphere_light(position, radius=0.0, intensity=1.0, color=(1, 1, 1), visible=True):
    """Radiative intensity = color * intensity; radius 0 is a point light."""
    L = Light()
    L.type, L.visible = LIGHT_SPHERE, int(visible)
    L.position[:] = list(position)
    L.radius = float(radius)
    L.color[:], L.intensity = list(color), float(intensity)
    return L


def spot_light(position, direction, intensity=1.0, color=(1, 1, 1), opening_angle=180.0, penumbra_angle=5.0,
               radius=0.0, inner_radius=0.0, visible=True):
    """Radiative intensity = color * intensity; radius 0 is a point spot."""
    L = Light()
    L.type, L.visible = LIGHT_SPOT, int(visible)
    L.position[:], L.direction[:] = list(position), list(direction)
    L.openingAngle, L.penumbraAngle = float(opening_angle), float(penumbra_angle)
    L.radius, L.innerRadius = float(radius), float(inner_radius)
    L.color[:], L.intensity = list(color), float(intensity)
    return L


def light_from_dict(L):
    """A b200 light from the dict form the tests and the oracle share."""
    t = L["type"]
    col, vis = L.get("color", (1, 1, 1)), L.get("visible", True)
    if t == "quad":
        return quad_light(L["position"], L["edge1"], L["edge2"], L["intensity"], color=col, visible=vis)
    if t == "distant":
        return distant_light(L["direction"], L["intensity"], col, L.get("angular_diameter", 0.0), vis)
    if t == "sphere":
        return sphere_light(L["position"], L.get("radius", 0.0), L["intensity"], col, vis)
    if t == "spot":
        return spot_light(L["position"], L["direction"], L["intensity"], col, L.get("opening_angle", 180.0),
                          L.get("penumbra_angle", 5.0), L.get("radius", 0.0), L.get("inner_radius", 0.0), vis)
    return ambient_light(L["intensity"], col, visible=vis)


def materials_array(mats):
    """mats: iterable of principled (r, g, b, roughness, metallic) tuples or
    material dicts (principled / obj_material / metal / glass / thin_glass)."""
    arr = (Material * max(1, len(mats)))()
    for i, m in enumerate(mats):
        arr[i] = material_struct(m)
    return arr, len(mats)


def pt_params(spp=1, max_path_length=20, roulette_path_length=5, max_scattering_events=20, light_samples=-1,
              limit_indirect_light_samples=True, min_contribution=0.001, max_contribution=float("inf"),
              bg=(0, 0, 0, 0), pixel_filter=PF_GAUSS, stats=False, backplate=None, mip_map_bias=0.0,
              max_depth=None):
    """backplate / max_depth: Textures (map_backplate, map_maxDepth) or None."""
    p = PTParams()
    p.maxDepth = _tex(max_depth)
    p.pixelSamples, p.maxPathLength, p.roulettePathLength = int(spp), int(max_path_length), int(roulette_path_length)
    p.maxScatteringEvents, p.lightSamples = int(max_scattering_events), int(light_samples)
    p.limitIndirectLightSamples = int(bool(limit_indirect_light_samples))
    p.minContribution, p.maxContribution = float(min_contribution), float(max_contribution)
    p.backgroundColor[:] = list(map(float, bg))
    p.pixelFilter, p.collectStats = int(pixel_filter), int(bool(stats))
    p.backplate = None if backplate is None else backplate._h.value
    p.mipMapBias = float(mip_map_bias)
    return p


class ScivisParams(ctypes.Structure):
    _fields_ = [("pixelSamples", ctypes.c_int), ("volumeSamplingRate", ctypes.c_float),
                ("backgroundColor", ctypes.c_float * 4), ("pixelFilter", ctypes.c_int),
                ("collectStats", ctypes.c_int), ("shadows", ctypes.c_int), ("visibleLights", ctypes.c_int),
                ("aoSamples", ctypes.c_int), ("aoDistance", ctypes.c_float), ("minContribution", ctypes.c_float),
                ("backplate", ctypes.c_void_p), ("maxDepth", ctypes.c_void_p), ("mipMapBias", ctypes.c_float)]


def _tex(t):
    return None if t is None else t._h.value


def scivis_params(spp=1, sampling_rate=1.0, bg=(0, 0, 0, 0), pixel_filter=PF_GAUSS, stats=False, shadows=False,
                  visible_lights=False, ao_samples=0, ao_distance=1e20, min_contribution=0.001, backplate=None,
                  max_depth=None, mip_map_bias=0.0):
    """backplate / max_depth: Textures (map_backplate, map_maxDepth) or None."""
    p = ScivisParams()
    p.backplate, p.maxDepth, p.mipMapBias = _tex(backplate), _tex(max_depth), float(mip_map_bias)
    p.pixelSamples, p.volumeSamplingRate = int(spp), float(sampling_rate)
    p.backgroundColor[:] = list(map(float, bg))
    p.pixelFilter, p.collectStats = int(pixel_filter), int(bool(stats))
    p.shadows, p.visibleLights, p.aoSamples = int(bool(shadows)), int(bool(visible_lights)), int(ao_samples)
    p.aoDistance, p.minContribution = float(ao_distance), float(min_contribution)
    return p


class ScivisMaterial(ctypes.Structure):
    _fields_ = [("isObj", ctypes.c_int), ("kd", ctypes.c_float * 3), ("ks", ctypes.c_float * 3),
                ("ns", ctypes.c_float), ("d", ctypes.c_float), ("tf", ctypes.c_float * 3),
                ("kdMap", ctypes.c_void_p)]


def scivis_materials_array(mats):
    """mats: iterable of dicts {"kd", "ks", "ns", "d", "tf", "map_kd"} for
    "obj" materials (values after OBJ commit; map_kd a Texture), or None for
    any other material.  The AO renderer reads kd, d and map_kd of them."""
    arr = (ScivisMaterial * max(1, len(mats)))()
    for i, m in enumerate(mats):
        if m is None:
            continue
        arr[i].isObj = 1
        arr[i].kd[:] = [float(x) for x in m.get("kd", (0.8, 0.8, 0.8))]
        arr[i].ks[:] = [float(x) for x in m.get("ks", (0, 0, 0))]
        arr[i].ns, arr[i].d = float(m.get("ns", 10.0)), float(m.get("d", 1.0))
        arr[i].tf[:] = [float(x) for x in m.get("tf", (0, 0, 0))]
        arr[i].kdMap = _tex(m.get("map_kd"))
    return arr, len(mats)


def lib_path():
    return os.path.join(BUILD, "libb200.so")


def lib():
    """The loaded CUDA library; raises if it was not built."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            raise RuntimeError("b200 CUDA library missing (%s): run __graft_entry__.build()" % path)
        L = ctypes.CDLL(path)
        P, I, I64, U32, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_uint32, ctypes.c_float
        sig = {
            "b200_device_create": (I, [I, ctypes.POINTER(P)]),
            "b200_device_release": (I, [P]),
            "b200_device_last_error": (ctypes.c_char_p, [P]),
            "b200_device_stream": (P, [P]),
            "b200_device_sync": (I, [P]),
            "b200_kernel_timing": (I, [P, I]),
            "b200_kernel_timing_read": (I, [P, P, P, I, I]),
            "b200_scene_create": (I, [P, ctypes.POINTER(P)]),
            "b200_scene_release": (I, [P]),
            "b200_scene_add_mesh": (I, [P, P, I64, P, I64, ctypes.POINTER(I)]),
            "b200_scene_add_quad_mesh": (I, [P, P, I64, P, I64, ctypes.POINTER(I)]),
            "b200_scene_add_boxes": (I, [P, P, I64, ctypes.POINTER(I)]),
            "b200_scene_add_spheres": (I, [P, P, I64, ctypes.POINTER(I)]),
            "b200_scene_add_discs": (I, [P, P, I64, P, ctypes.POINTER(I)]),
            "b200_scene_add_planes": (I, [P, P, I64, P, ctypes.POINTER(I)]),
            "b200_scene_add_instance": (I, [P, I, U32, U32, P, I]),
            "b200_scene_add_instance_motion": (I, [P, I, U32, U32, P, I, ctypes.c_float, ctypes.c_float, I]),
            "b200_scene_commit": (I, [P]),
            "b200_scene_set_dynamic": (I, [P, I]),
            "b200_scene_bounds": (I, [P, P]),
            "b200_scene_stats": (I, [P, P]),
            "b200_scene_counters": (I, [P, P, I]),
            "b200_trace": (I, [P, P, I64, I, P, P, P]),
            "b200_frame_create": (I, [P, I, I, I, U32, ctypes.POINTER(P)]),
            "b200_frame_channel_bytes": (ctypes.c_size_t, [P, U32]),
            "b200_tonemapper_defaults": (None, [ctypes.POINTER(ToneMapper)]),
            "b200_material_defaults": (None, [ctypes.POINTER(Material), I]),
            "b200_tensor_core_check": (I, [P, P, P, I, P]),
            "b200_frame_set_tonemapper": (I, [P, ctypes.POINTER(ToneMapper)]),
            "b200_pick": (I, [P, ctypes.POINTER(CameraDesc), F, F, ctypes.POINTER(PickResult)]),
            "b200_batch_create": (I, [P, ctypes.POINTER(P)]),
            "b200_batch_release": (I, [P]),
            "b200_batch_add_ao": (I, [P, P, ctypes.POINTER(CameraDesc), ctypes.POINTER(AOParams), P]),
            "b200_batch_add_pt": (I, [P, P, ctypes.POINTER(CameraDesc), ctypes.POINTER(PTParams), P, I, P]),
            "b200_batch_get_tuning": (I, [P, ctypes.POINTER(BatchTuning)]),
            "b200_batch_set_tuning": (I, [P, ctypes.POINTER(BatchTuning)]),
            "b200_batch_autotune": (I, [P, I, ctypes.POINTER(BatchTuning)]),
            "b200_batch_render": (I, [P, I]),
            "b200_batch_set_barrier_timeout": (I, [P, ctypes.c_uint64]),
            "b200_batch_timings": (I, [P, P, I, ctypes.POINTER(ctypes.c_uint64)]),
            "b200_batch_info": (I, [P, P]),
            "b200_nrc_create": (I, [P, ctypes.POINTER(NrcDesc), ctypes.POINTER(P)]),
            "b200_nrc_release": (I, [P]),
            "b200_nrc_infer": (I, [P, P, I64, P, P]),
            "b200_nrc_train": (I, [P, P, I64, P, P]),
            "b200_nrc_gradients": (I, [P, P, I64, P, P, P, P]),
            "b200_nrc_get_params": (I, [P, P, P]),
            "b200_nrc_set_params": (I, [P, P, P]),
            "b200_nrc_grid": (I, [P, P, P, P]),
            "b200_nrc_frame_defaults": (None, [P]),
            "b200_render_pt_nrc": (I, [P, ctypes.POINTER(CameraDesc), ctypes.POINTER(PTParams), P, I, P, P, P, P]),
            "b200_frame_relmse": (I, [P, P, ctypes.POINTER(ctypes.c_double)]),
            "b200_frame_relmse_hits": (I, [P, P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)]),
            "b200_frame_variance": (I, [P, F, ctypes.POINTER(F)]),
            "b200_event_record": (I, [P, ctypes.POINTER(P)]),
            "b200_event_query": (I, [P]),
            "b200_event_wait": (I, [P]),
            "b200_event_elapsed_ms": (F, [P, P]),
            "b200_event_release": (I, [P]),
            "b200_frame_release": (I, [P]),
            "b200_frame_reset": (I, [P]),
            "b200_frame_id": (I, [P]),
            "b200_frame_channel": (P, [P, U32]),
            "b200_frame_read": (I, [P, U32, P, ctypes.c_size_t]),
            "b200_frame_map": (I, [P, U32, ctypes.POINTER(P)]),
            "b200_render_ao": (I, [P, ctypes.POINTER(CameraDesc), ctypes.POINTER(AOParams), P, P]),
            "b200_scene_set_lights": (I, [P, P, I]),
            "b200_scene_set_volume": (I, [P, P, I, I, I, P, P, P, I, P, I, P, F]),
            "b200_frame_set_variance_threshold": (I, [P, F]),
            "b200_scene_set_volume_gradient_shading": (I, [P, F]),
            "b200_scene_set_volume_transform": (I, [P, P]),
            "b200_render_scivis": (I, [P, ctypes.POINTER(CameraDesc), ctypes.POINTER(ScivisParams), P, I, P, P]),
            "b200_render_pt": (I, [P, ctypes.POINTER(CameraDesc), ctypes.POINTER(PTParams), P, I, P, P]),
            "b200_scene_set_mesh_attributes": (I, [P, I, P, P, P]),
            "b200_texture_create": (I, [P, I, I, I, I, I, I, I, P, ctypes.POINTER(P)]),
            "b200_texture_release": (I, [P]),
            "b200_texture_levels": (I, [P]),
            "b200_texture_read_level": (I, [P, I, P, ctypes.c_size_t]),
            "b200_texture_sample": (I, [P, I64, P, P, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def scenes_lib():
    global _scenes
    if _scenes is None:
        path = os.path.join(BUILD, "libb200_scenes.so")
        if not os.path.exists(path):
            raise RuntimeError("scene generator library missing (%s): run __graft_entry__.build()" % path)
        _scenes = ctypes.CDLL(path)
    return _scenes


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


class Device:
    def __init__(self, cuda_device=0):
        self._h = ctypes.c_void_p()
        self._check(lib().b200_device_create(cuda_device, ctypes.byref(self._h)), None)

    def _check(self, code, h="self"):
        if code != 0:
            msg = lib().b200_device_last_error(self._h if h == "self" else None)
            raise B200Error(code, (msg or b"").decode())

    @property
    def stream(self):
        return lib().b200_device_stream(self._h)

    def record_event(self):
        """b200_event on the device stream (an OSPFuture's completion point)."""
        e = ctypes.c_void_p()
        self._check(lib().b200_event_record(self._h, ctypes.byref(e)))
        return e

    @staticmethod
    def event_ms(a, b):
        return lib().b200_event_elapsed_ms(a, b)

    @staticmethod
    def release_event(e):
        lib().b200_event_release(e)

    def sync(self):
        self._check(lib().b200_device_sync(self._h))

    KERNEL_KINDS = ("trace_closest", "trace_shadow", "pt_shade", "ao", "scivis")

    def kernel_timing(self, enable):
        """Starts (True) or stops live event timing of the hot kernels."""
        self._check(lib().b200_kernel_timing(self._h, 1 if enable else 0))

    def kernel_times(self, reset=False):
        """{kind: (device ms, launches)} since timing started or the last reset."""
        n = len(self.KERNEL_KINDS)
        ms = np.zeros(n, np.float64)
        cnt = np.zeros(n, np.int64)
        self._check(lib().b200_kernel_timing_read(self._h, ms.ctypes.data, cnt.ctypes.data, n, 1 if reset else 0))
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(self.KERNEL_KINDS)}

    def release(self):
        if self._h:
            lib().b200_device_release(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


# OSPTextureFormat / OSPTextureFilter / OSPTextureWrapMode values
(TEX_RGBA8, TEX_SRGBA, TEX_RGBA32F, TEX_RGB8, TEX_SRGB, TEX_RGB32F, TEX_R8, TEX_R32F, TEX_L8, TEX_RA8, TEX_LA8,
 TEX_RGBA16, TEX_RGB16, TEX_RA16, TEX_R16, TEX_RA32F) = range(16)
TEX_FILTER_LINEAR, TEX_FILTER_NEAREST = 0, 1
TEX_WRAP_REPEAT, TEX_WRAP_MIRRORED_REPEAT, TEX_WRAP_CLAMP_TO_EDGE = 0, 1, 2
_TEX_CHANNELS = {TEX_RGBA8: 4, TEX_SRGBA: 4, TEX_RGBA32F: 4, TEX_RGB8: 3, TEX_SRGB: 3, TEX_RGB32F: 3, TEX_R8: 1,
                 TEX_R32F: 1, TEX_L8: 1, TEX_RA8: 2, TEX_LA8: 2, TEX_RGBA16: 4, TEX_RGB16: 3, TEX_RA16: 2,
                 TEX_R16: 1, TEX_RA32F: 2}
_TEX_DTYPE = {TEX_RGBA32F: np.float32, TEX_RGB32F: np.float32, TEX_R32F: np.float32, TEX_RA32F: np.float32,
              TEX_RGBA16: np.uint16, TEX_RGB16: np.uint16, TEX_RA16: np.uint16, TEX_R16: np.uint16}


class Texture:
    """A 2D texture (texture2d): data (height, width[, channels]) with rows
    from the bottom, of the dtype its format names (uint8, uint16, float32)."""

    def __init__(self, device, data, format, filter=TEX_FILTER_LINEAR, wrap=(TEX_WRAP_REPEAT, TEX_WRAP_REPEAT),
                 mipmaps=True):
        a = np.ascontiguousarray(data, dtype=_TEX_DTYPE.get(format, np.uint8))
        h, w = a.shape[0], a.shape[1]
        if a.size != h * w * _TEX_CHANNELS[format]:
            raise ValueError("texture data does not match its format")
        if isinstance(wrap, int):
            wrap = (wrap, wrap)
        self.device, self.data, self.format = device, a, format
        self._h = ctypes.c_void_p()
        device._check(lib().b200_texture_create(device._h, w, h, format, filter, wrap[0], wrap[1], int(bool(mipmaps)),
                                                _ptr(a), ctypes.byref(self._h)))

    @property
    def levels(self):
        return lib().b200_texture_levels(self._h)

    def read_level(self, level):
        """The texels of one level (the MIP chain as generated on the device)."""
        h, w = max(self.data.shape[0] >> level, 1), max(self.data.shape[1] >> level, 1)
        out = np.empty((h, w) + self.data.shape[2:], dtype=self.data.dtype)
        self.device._check(lib().b200_texture_read_level(self._h, level, _ptr(out), out.nbytes))
        return out

    def sample(self, st, footprint):
        """Texture2D_get at texture coordinates st (n, 2) with pixel footprints (n,) or a scalar: (n, 4)."""
        st = np.ascontiguousarray(st, dtype=np.float32).reshape(-1, 2)
        fp = np.ascontiguousarray(np.broadcast_to(np.asarray(footprint, np.float32), (len(st),)))
        out = np.zeros((len(st), 4), np.float32)
        self.device._check(lib().b200_texture_sample(self._h, len(st), _ptr(st), _ptr(fp), _ptr(out)))
        return out

    def release(self):
        if self._h:
            lib().b200_texture_release(self._h)
            self._h = ctypes.c_void_p()


class Scene:
    """A committed world: geometries (BLAS each) and instance entries (TLAS)."""

    def __init__(self, device):
        self.device = device
        self._h = ctypes.c_void_p()
        device._check(lib().b200_scene_create(device._h, ctypes.byref(self._h)))
        self._keep = []

    def add_mesh(self, vertex, index):
        v = np.ascontiguousarray(vertex, dtype=np.float32).reshape(-1, 3)
        i = np.ascontiguousarray(index, dtype=np.uint32).reshape(-1, 3)
        g = ctypes.c_int()
        self.device._check(lib().b200_scene_add_mesh(self._h, _ptr(v), len(v), _ptr(i), len(i), ctypes.byref(g)))
        return g.value

    def set_mesh_attributes(self, geom, normal=None, color=None, texcoord=None):
        """Per-vertex normals (n, 3), colours (n, 4 or 3: alpha 1) and texture
        coordinates (n, 2) of triangle mesh `geom`, before the commit."""
        n = None if normal is None else np.ascontiguousarray(normal, dtype=np.float32).reshape(-1, 3)
        c = None
        if color is not None:
            c = np.asarray(color, dtype=np.float32)
            if c.shape[-1] == 3:
                c = np.concatenate([c.reshape(-1, 3), np.ones((c.size // 3, 1), np.float32)], axis=1)
            c = np.ascontiguousarray(c, dtype=np.float32).reshape(-1, 4)
        t = None if texcoord is None else np.ascontiguousarray(texcoord, dtype=np.float32).reshape(-1, 2)
        self.device._check(lib().b200_scene_set_mesh_attributes(self._h, geom, _ptr(n), _ptr(c), _ptr(t)))

    def add_quad_mesh(self, vertex, index):
        """index: (n, 4) uint32 quads (Embree's decomposition into two triangles)."""
        v = np.ascontiguousarray(vertex, dtype=np.float32).reshape(-1, 3)
        i = np.ascontiguousarray(index, dtype=np.uint32).reshape(-1, 4)
        g = ctypes.c_int()
        self.device._check(lib().b200_scene_add_quad_mesh(self._h, _ptr(v), len(v), _ptr(i), len(i), ctypes.byref(g)))
        return g.value

    def add_boxes(self, boxes):
        """boxes: (n, 6) float32 (lower xyz, upper xyz)."""
        b = np.ascontiguousarray(boxes, dtype=np.float32).reshape(-1, 6)
        g = ctypes.c_int()
        self.device._check(lib().b200_scene_add_boxes(self._h, _ptr(b), len(b), ctypes.byref(g)))
        return g.value

    def add_spheres(self, xyzr):
        s = np.ascontiguousarray(xyzr, dtype=np.float32).reshape(-1, 4)
        g = ctypes.c_int()
        self.device._check(lib().b200_scene_add_spheres(self._h, _ptr(s), len(s), ctypes.byref(g)))
        return g.value

    def add_discs(self, xyzr, normals=None):
        """Discs (n, 4): facing the ray (OSP_DISC), or oriented by normals (n, 3) (OSP_ORIENTED_DISC)."""
        s = np.ascontiguousarray(xyzr, dtype=np.float32).reshape(-1, 4)
        n = None if normals is None else np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
        g = ctypes.c_int()
        self.device._check(lib().b200_scene_add_discs(self._h, _ptr(s), len(s), _ptr(n), ctypes.byref(g)))
        return g.value

    def add_planes(self, coeffs, bounds=None):
        """Planes (n, 4) a x + b y + c z = d, optionally bounded by boxes (n, 6) lower, upper."""
        c = np.ascontiguousarray(coeffs, dtype=np.float32).reshape(-1, 4)
        b = None if bounds is None else np.ascontiguousarray(bounds, dtype=np.float32).reshape(-1, 6)
        g = ctypes.c_int()
        self.device._check(lib().b200_scene_add_planes(self._h, _ptr(c), len(c), _ptr(b), ctypes.byref(g)))
        return g.value

    def add_instance(self, geom, inst_id, geom_id, xfm=None, material=-1):
        x = None if xfm is None else np.ascontiguousarray(xfm, dtype=np.float32).reshape(12)
        self.device._check(lib().b200_scene_add_instance(self._h, geom, inst_id, geom_id, _ptr(x), material))

    def add_instance_motion(self, geom, inst_id, geom_id, xfms, time=(0.0, 1.0), material=-1):
        """xfms: (n >= 2, 3, 4) key transforms evenly spaced over `time`."""
        x = np.ascontiguousarray(xfms, dtype=np.float32).reshape(-1, 12)
        self.device._check(lib().b200_scene_add_instance_motion(self._h, geom, inst_id, geom_id, _ptr(x), len(x),
                                                                float(time[0]), float(time[1]), material))

    def set_dynamic(self, dynamic=True):
        """LBVH-only builds for the commits that follow (default: binned-SAH splits)."""
        self.device._check(lib().b200_scene_set_dynamic(self._h, int(bool(dynamic))))

    def commit(self):
        self.device._check(lib().b200_scene_commit(self._h))

    def set_volume(self, data, origin, spacing, color, opacity, value_range=(0.0, 1.0), density_scale=1.0):
        """data: (nz, ny, nx) float32 (x fastest); color (n,3); opacity (m,)."""
        d = np.ascontiguousarray(data, np.float32)
        nz, ny, nx = d.shape
        o, sp = np.asarray(origin, np.float32), np.asarray(spacing, np.float32)
        c = np.ascontiguousarray(color, np.float32).reshape(-1, 3)
        op = np.ascontiguousarray(opacity, np.float32).reshape(-1)
        vr = np.asarray(value_range, np.float32)
        self.device._check(lib().b200_scene_set_volume(self._h, _ptr(d), nx, ny, nz, _ptr(o), _ptr(sp), _ptr(c),
                                                       len(c), _ptr(op), len(op), _ptr(vr), float(density_scale)))

    def set_volume_transform(self, xfm):
        """The volume's instance transform (3x4 row-major) or None."""
        x = None if xfm is None else np.ascontiguousarray(xfm, np.float32).reshape(12)
        self.device._check(lib().b200_scene_set_volume_transform(self._h, _ptr(x) if x is not None else None))

    def set_volume_gradient_shading(self, scale):
        """The volumetric model's gradientShadingScale (0: off)."""
        self.device._check(lib().b200_scene_set_volume_gradient_shading(self._h, float(scale)))

    def set_lights(self, lights):
        arr = (Light * max(1, len(lights)))(*lights)
        self.device._check(lib().b200_scene_set_lights(self._h, ctypes.cast(arr, ctypes.c_void_p), len(lights)))

    def bounds(self):
        b = np.zeros(6, np.float32)
        self.device._check(lib().b200_scene_bounds(self._h, _ptr(b)))
        return b

    def stats(self):
        s = np.zeros(3, np.int64)
        self.device._check(lib().b200_scene_stats(self._h, _ptr(s)))
        return s

    def counters(self, reset=False):
        """[rays, node visits, triangle tests, sphere tests] from stats renders."""
        c = np.zeros(4, np.int64)
        self.device._check(lib().b200_scene_counters(self._h, _ptr(c), int(bool(reset))))
        return c

    def trace(self, rays_ptr, n, hit_f_ptr, hit_id_ptr, occlusion=False, stream=None):
        """Device pointers (e.g. torch tensor data_ptr())."""
        self.device._check(lib().b200_trace(self._h, ctypes.c_void_p(rays_ptr), n, int(bool(occlusion)),
                                            ctypes.c_void_p(hit_f_ptr),
                                            ctypes.c_void_p(hit_id_ptr) if hit_id_ptr else None,
                                            ctypes.c_void_p(stream) if stream else None))

    def release(self):
        if self._h:
            lib().b200_scene_release(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


def tonemapper(**kw):
    """A b200_tonemapper with the reference's defaults, fields overridden by keyword."""
    t = ToneMapper()
    lib().b200_tonemapper_defaults(ctypes.byref(t))
    for k, v in kw.items():
        setattr(t, k, v)
    return t


class Frame:
    def __init__(self, device, width, height, channels=FB_COLOR | FB_DEPTH | FB_ACCUM, format=FB_RGBA32F):
        self.device = device
        self.width, self.height, self.channels, self.format = width, height, channels, format
        self._h = ctypes.c_void_p()
        device._check(lib().b200_frame_create(device._h, width, height, format, channels, ctypes.byref(self._h)))

    def variance(self, threshold=0.0):
        """ospGetVariance: the task error estimate (inf before the first odd frame)."""
        v = ctypes.c_float()
        self.device._check(lib().b200_frame_variance(self._h, float(threshold), ctypes.byref(v)))
        return v.value

    def set_variance_threshold(self, threshold):
        """The renderer's varianceThreshold: later renders of this frame
        render only the 8x8 tasks whose error estimate exceeds it (0: all)."""
        self.device._check(lib().b200_frame_set_variance_threshold(self._h, float(threshold)))

    def set_tonemapper(self, tm):
        """tm: ToneMapper (see tonemapper()) or None to remove it; applies from the next render."""
        self.device._check(lib().b200_frame_set_tonemapper(self._h, ctypes.byref(tm) if tm is not None else None))

    def reset(self):
        self.device._check(lib().b200_frame_reset(self._h))

    @property
    def frame_id(self):
        return lib().b200_frame_id(self._h)

    def channel_ptr(self, ch):
        return lib().b200_frame_channel(self._h, ch)

    def read(self, ch=FB_COLOR):
        n = self.width * self.height
        if ch == FB_COLOR and self.format in (FB_RGBA8, FB_SRGBA):
            out = np.empty((self.height, self.width, 4), np.uint8)
        elif ch in (FB_COLOR, FB_VARIANCE, FB_ACCUM):
            out = np.empty((self.height, self.width, 4), np.float32)
        elif ch in (FB_NORMAL, FB_ALBEDO):
            out = np.empty((self.height, self.width, 3), np.float32)
        elif ch == FB_DEPTH:
            out = np.empty((self.height, self.width), np.float32)
        else:
            out = np.empty((self.height, self.width), np.uint32)
        self.device._check(lib().b200_frame_read(self._h, ch, _ptr(out), out.nbytes))
        assert out.nbytes == lib().b200_frame_channel_bytes(self._h, ch)
        return out

    def release(self):
        if self._h:
            lib().b200_frame_release(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


CAMERA_PERSPECTIVE, CAMERA_ORTHOGRAPHIC, CAMERA_PANORAMIC = 0, 1, 2


def camera_desc(position, direction, up=(0, 1, 0), fovy=60.0, aspect=1.0, near_clip=1e-6, kind=CAMERA_PERSPECTIVE,
                height=1.0, shutter=(0.5, 0.5), shutter_type=0, rolling_shutter_duration=0.0, aperture_radius=0.0,
                focus_distance=1.0, architectural=False, image_start=(0.0, 0.0), image_end=(1.0, 1.0),
                stereo_mode=0, interpupillary_distance=0.0635):
    """kind: CAMERA_PERSPECTIVE (fovy), CAMERA_ORTHOGRAPHIC (image `height`) or CAMERA_PANORAMIC.
    shutter / shutter_type (OSPShutterType) / rolling_shutter_duration: the ray times (motion blur).
    image_start / image_end: the sub-image the frame covers; stereo_mode (OSPStereoMode: 0 none, 1 left,
    2 right, 3 side by side, 4 top / bottom) with interpupillary_distance."""
    c = CameraDesc()
    c.imageStart[:] = [float(image_start[0]), float(image_start[1])]
    c.imageEnd[:] = [float(image_end[0]), float(image_end[1])]
    c.stereoMode, c.interpupillaryDistance = int(stereo_mode), float(interpupillary_distance)
    c.type, c.height = int(kind), float(height)
    c.shutter[:] = [float(shutter[0]), float(shutter[1])]
    c.shutterType, c.rollingShutterDuration = int(shutter_type), float(rolling_shutter_duration)
    c.apertureRadius, c.focusDistance = float(aperture_radius), float(focus_distance)
    c.architectural = int(bool(architectural))
    c.position[:] = list(map(float, position))
    c.direction[:] = list(map(float, direction))
    c.up[:] = list(map(float, up))
    c.fovy, c.aspect, c.nearClip = float(fovy), float(aspect), float(near_clip)
    return c


def ao_params(spp=1, ao_samples=1, ao_distance=1e20, ao_intensity=1.0, bg=(0, 0, 0, 0), pixel_filter=PF_GAUSS,
              stats=False, volume_sampling_rate=1.0, backplate=None, max_depth=None, mip_map_bias=0.0,
              materials=None):
    """materials: (ctypes array, count) from scivis_materials_array() (surface colours), or None."""
    p = AOParams()
    p.backplate, p.maxDepth, p.mipMapBias = _tex(backplate), _tex(max_depth), float(mip_map_bias)
    if materials:
        p._materials = materials  # keeps the array alive with the parameters
        p.materials, p.nmaterials = ctypes.cast(materials[0], ctypes.c_void_p), int(materials[1])
    p.volumeSamplingRate = float(volume_sampling_rate)
    p.collectStats = int(bool(stats))
    p.pixelSamples, p.aoSamples = int(spp), int(ao_samples)
    p.aoDistance, p.aoIntensity = float(ao_distance), float(ao_intensity)
    p.backgroundColor[:] = list(map(float, bg))
    p.pixelFilter = int(pixel_filter)
    return p


def pick(scene, camera, x, y):
    """ospPick: (hit, world position, instID, geomID, primID) at normalised screen (x, y)."""
    r = PickResult()
    scene.device._check(lib().b200_pick(scene._h, ctypes.byref(camera), float(x), float(y), ctypes.byref(r)))
    return bool(r.hasHit), tuple(r.worldPosition), r.instID, r.geomID, r.primID


def render_ao(scene, camera, params, frame, stream=None):
    scene.device._check(lib().b200_render_ao(scene._h, ctypes.byref(camera), ctypes.byref(params), frame._h,
                                             ctypes.c_void_p(stream) if stream else None))


def render_scivis(scene, camera, params, frame, materials=None, stream=None):
    """materials: (ctypes array, count) from scivis_materials_array(), or None."""
    arr, n = materials if materials else (None, 0)
    scene.device._check(lib().b200_render_scivis(scene._h, ctypes.byref(camera), ctypes.byref(params),
                                                 ctypes.cast(arr, ctypes.c_void_p) if arr is not None else None, n,
                                                 frame._h, ctypes.c_void_p(stream) if stream else None))


def render_pt(scene, camera, params, materials, frame, stream=None):
    """materials: (ctypes array, count) from materials_array()."""
    arr, n = materials
    scene.device._check(lib().b200_render_pt(scene._h, ctypes.byref(camera), ctypes.byref(params),
                                             ctypes.cast(arr, ctypes.c_void_p), n, frame._h,
                                             ctypes.c_void_p(stream) if stream else None))


class BatchTuning(ctypes.Structure):
    _fields_ = [("wavePaths", ctypes.c_int64), ("traceBlocksPerSM", ctypes.c_int), ("shadeBlocksPerSM", ctypes.c_int)]


BATCH_KERNELS, BATCH_GRAPH, BATCH_PERSISTENT = 0, 1, 2


class Batch:
    """b200_batch: many render requests served by one wavefront (wavefront
    kernels replayed as a CUDA graph, or one persistent launch)."""

    def __init__(self, device):
        self.device = device
        self._h = ctypes.c_void_p()
        self._keep = []
        self.n = 0
        device._check(lib().b200_batch_create(device._h, ctypes.byref(self._h)))

    def add_ao(self, scene, camera, params, frame):
        self.device._check(lib().b200_batch_add_ao(self._h, scene._h, ctypes.byref(camera), ctypes.byref(params),
                                                   frame._h))
        self._keep += [scene, frame]
        self.n += 1

    def add_pt(self, scene, camera, params, materials, frame):
        arr, n = materials
        self.device._check(lib().b200_batch_add_pt(self._h, scene._h, ctypes.byref(camera), ctypes.byref(params),
                                                   ctypes.cast(arr, ctypes.c_void_p), n, frame._h))
        self._keep += [scene, frame]
        self.n += 1

    @property
    def tuning(self):
        t = BatchTuning()
        self.device._check(lib().b200_batch_get_tuning(self._h, ctypes.byref(t)))
        return t

    @tuning.setter
    def tuning(self, t):
        self.device._check(lib().b200_batch_set_tuning(self._h, ctypes.byref(t)))

    def autotune(self, candidates=0):
        t = BatchTuning()
        self.device._check(lib().b200_batch_autotune(self._h, candidates, ctypes.byref(t)))
        return t

    def render(self, use_graph=True, mode=None):
        """mode: BATCH_KERNELS, BATCH_GRAPH or BATCH_PERSISTENT (default: graph
        if use_graph else kernels)."""
        if mode is None:
            mode = BATCH_GRAPH if use_graph else BATCH_KERNELS
        self.device._check(lib().b200_batch_render(self._h, int(mode)))

    def set_barrier_timeout(self, ns):
        """Bound of the persistent launch's barrier waits in ns (0: default 4 s)."""
        self.device._check(lib().b200_batch_set_barrier_timeout(self._h, int(ns)))

    def timings(self):
        """(per-request completion ms since the render began, rays traced); waits for the device."""
        self.device.sync()
        ms = np.zeros(self.n, np.float64)
        rays = ctypes.c_uint64()
        self.device._check(lib().b200_batch_timings(self._h, _ptr(ms), self.n, ctypes.byref(rays)))
        return ms, rays.value

    def info(self):
        """plan of the last render: dict(waves, kernels, paths, requests)."""
        a = np.zeros(4, np.int64)
        self.device._check(lib().b200_batch_info(self._h, _ptr(a)))
        return dict(zip(("waves", "kernels", "paths", "requests"), (int(x) for x in a)))

    def release(self):
        if self._h:
            lib().b200_batch_release(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class NrcDesc(ctypes.Structure):
    _fields_ = [("boundsLo", ctypes.c_float * 3), ("boundsHi", ctypes.c_float * 3), ("learningRate", ctypes.c_float),
                ("seed", ctypes.c_uint32)]


NRC_NUM_W = 4 * 64 * 64 + 64 * 16
NRC_NUM_T = 16 * (1 << 19) * 2


class RadianceCache:
    """b200_nrc: the neural radiance cache (hash grid + fused BF16 MLP).
    Query / sample arrays are device pointers to n x 16 float records."""

    def __init__(self, device, lo, hi, learning_rate=1e-2, seed=1):
        self.device = device
        d = NrcDesc()
        d.boundsLo[:], d.boundsHi[:] = list(map(float, lo)), list(map(float, hi))
        d.learningRate, d.seed = float(learning_rate), int(seed)
        self._h = ctypes.c_void_p()
        device._check(lib().b200_nrc_create(device._h, ctypes.byref(d), ctypes.byref(self._h)))

    def infer(self, queries_ptr, n, out_ptr, stream=None):
        self.device._check(lib().b200_nrc_infer(self._h, ctypes.c_void_p(queries_ptr), n, ctypes.c_void_p(out_ptr),
                                                ctypes.c_void_p(stream) if stream else None))

    def train(self, samples_ptr, n, loss_ptr=None, stream=None):
        self.device._check(lib().b200_nrc_train(self._h, ctypes.c_void_p(samples_ptr), n,
                                                ctypes.c_void_p(loss_ptr) if loss_ptr else None,
                                                ctypes.c_void_p(stream) if stream else None))

    def gradients(self, samples_ptr, n, wgrad_ptr, tgrad_ptr, loss_ptr=None):
        self.device._check(lib().b200_nrc_gradients(self._h, ctypes.c_void_p(samples_ptr), n,
                                                     ctypes.c_void_p(wgrad_ptr), ctypes.c_void_p(tgrad_ptr),
                                                     ctypes.c_void_p(loss_ptr) if loss_ptr else None, None))

    def get_params(self):
        w = np.empty(NRC_NUM_W, np.float32)
        t = np.empty(NRC_NUM_T, np.float32)
        self.device._check(lib().b200_nrc_get_params(self._h, _ptr(w), _ptr(t)))
        return w, t

    def set_params(self, weights=None, table=None):
        w = None if weights is None else np.ascontiguousarray(weights, np.float32)
        t = None if table is None else np.ascontiguousarray(table, np.float32)
        self.device._check(lib().b200_nrc_set_params(self._h, _ptr(w), _ptr(t)))

    def grid(self):
        a = np.empty(4, np.float32)
        s = np.empty(16, np.float32)
        dn = np.empty(16, np.uint32)
        self.device._check(lib().b200_nrc_grid(self._h, _ptr(a), _ptr(s), _ptr(dn)))
        return dict(lo=a[:3].copy(), inv_extent=float(a[3]), scales=s, dense=dn)

    def release(self):
        if self._h:
            lib().b200_nrc_release(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class NrcFrame(ctypes.Structure):
    _fields_ = [("trainPaths", ctypes.c_int), ("trainSteps", ctypes.c_int), ("trainBatch", ctypes.c_int),
                ("train", ctypes.c_int), ("useCache", ctypes.c_int), ("epochs", ctypes.c_int)]


def render_pt_nrc(scene, camera, params, materials, frame, cache, train=True, train_paths=16384, train_steps=4,
                  train_batch=16384, use_cache=True, epochs=1, stream=None):
    """One path-traced frame ending paths in the radiance cache (and training it)."""
    f = NrcFrame(int(train_paths), int(train_steps), int(train_batch), int(bool(train)), int(bool(use_cache)),
                 int(epochs))
    arr, n = materials
    scene.device._check(lib().b200_render_pt_nrc(scene._h, ctypes.byref(camera), ctypes.byref(params),
                                                 ctypes.cast(arr, ctypes.c_void_p), n, frame._h, cache._h,
                                                 ctypes.byref(f), ctypes.c_void_p(stream) if stream else None))


def relmse(frame, reference):
    """mean over pixels and rgb of (x - r)^2 / (r^2 + 0.01) of the accumulated colours."""
    v = ctypes.c_double()
    frame.device._check(lib().b200_frame_relmse(frame._h, reference._h, ctypes.byref(v)))
    return v.value


def tensor_core_check(device, a, b):
    """D = A B^T (A 128 x 64, B n x 64, BF16 operands) on the tcgen05 tensor cores."""
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    out = np.zeros((128, b.shape[0]), np.float32)
    device._check(lib().b200_tensor_core_check(device._h, _ptr(a), _ptr(b), int(b.shape[0]), _ptr(out)))
    return out


def relmse_hits(frame, reference):
    """relmse over the pixels whose reference depth is finite (first hit is
    geometry); the reference needs FB_DEPTH.  Returns (relmse, pixels)."""
    v, n = ctypes.c_double(), ctypes.c_int64()
    frame.device._check(lib().b200_frame_relmse_hits(frame._h, reference._h, ctypes.byref(v), ctypes.byref(n)))
    return v.value, n.value
