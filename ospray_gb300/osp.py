"""ctypes access to libospray.so (the OSPRay C API of include/ospray/ospray.h):
the same calls an OSPRay application makes, for the tests and for the
benchmark's end-to-end leg (ospRenderFrame + ospWait + ospMapFrameBuffer)."""
import ctypes
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.environ.get("B200_BUILD_DIR") or os.path.join(ROOT, "ospray_gb300", "_build")
P, I, U32, F, U64, I64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_float, ctypes.c_uint64, \
    ctypes.c_int64

# OSPDataType values used here
OSP_OBJECT, OSP_DATA = 0x8000000, 0x8000000 + 100
OSP_GEOMETRIC_MODEL, OSP_INSTANCE, OSP_LIGHT, OSP_MATERIAL = (0x8000000 + 104, 0x8000000 + 108,
                                                             0x8000000 + 109, 0x8000000 + 110)
OSP_INT, OSP_UINT, OSP_FLOAT, OSP_VEC3F, OSP_VEC4F, OSP_VEC3UI = 4000, 4500, 6000, 6002, 6003, 4502
OSP_AFFINE3F, OSP_BOOL = 12003, 250
OSP_TEXTURE = 0x8000000 + 112
OSP_UCHAR, OSP_VEC3UC, OSP_VEC4UC, OSP_VEC2F, OSP_VEC2UI = 2500, 2502, 2503, 6001, 4501
OSP_FB_NONE, OSP_FB_RGBA8, OSP_FB_SRGBA, OSP_FB_RGBA32F = 0, 1, 2, 3
OSP_FB_COLOR, OSP_FB_DEPTH, OSP_FB_ACCUM = 1, 2, 4
OSP_FB_ID_PRIMITIVE, OSP_FB_ID_OBJECT, OSP_FB_ID_INSTANCE = 64, 128, 256
OSP_TASK_FINISHED = 100000


class OSPBounds(ctypes.Structure):
    _fields_ = [("lower", F * 3), ("upper", F * 3)]


class OSPPickResult(ctypes.Structure):
    _fields_ = [("hasHit", I), ("worldPosition", F * 3), ("instance", P), ("model", P), ("primID", U32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(os.path.join(BUILD, "libospray.so"), mode=ctypes.RTLD_GLOBAL)
        sig = {
            "ospInit": (I, [ctypes.POINTER(I), P]),
            "ospShutdown": (None, []),
            "ospNewDevice": (P, [ctypes.c_char_p]),
            "ospDeviceCommit": (None, [P]),
            "ospDeviceRelease": (None, [P]),
            "ospSetCurrentDevice": (None, [P]),
            "ospGetCurrentDevice": (P, []),
            "ospDeviceGetLastErrorMsg": (ctypes.c_char_p, [P]),
            "ospDeviceGetLastErrorCode": (I, [P]),
            "ospLoadModule": (I, [ctypes.c_char_p]),
            "ospNewSharedData": (P, [P, I, U64, I64, U64, I64, U64, I64, P, P]),
            "ospNewData": (P, [I, U64, U64, U64]),
            "ospCopyData": (None, [P, P, U64, U64, U64]),
            "ospNewGeometry": (P, [ctypes.c_char_p]),
            "ospNewMaterial": (P, [ctypes.c_char_p]),
            "ospNewLight": (P, [ctypes.c_char_p]),
            "ospNewCamera": (P, [ctypes.c_char_p]),
            "ospNewRenderer": (P, [ctypes.c_char_p]),
            "ospNewImageOperation": (P, [ctypes.c_char_p]),
            "ospNewTexture": (P, [ctypes.c_char_p]),
            "ospNewGeometricModel": (P, [P]),
            "ospNewGroup": (P, []),
            "ospNewInstance": (P, [P]),
            "ospNewWorld": (P, []),
            "ospGetBounds": (OSPBounds, [P]),
            "ospSetParam": (None, [P, ctypes.c_char_p, I, P]),
            "ospSetObjectAsData": (None, [P, ctypes.c_char_p, I, P]),
            "ospCommit": (None, [P]),
            "ospRelease": (None, [P]),
            "ospNewFrameBuffer": (P, [I, I, I, U32]),
            "ospMapFrameBuffer": (P, [P, I]),
            "ospUnmapFrameBuffer": (None, [P, P]),
            "ospResetAccumulation": (None, [P]),
            "ospRenderFrame": (P, [P, P, P, P]),
            "ospRenderFrameBlocking": (F, [P, P, P, P]),
            "ospWait": (None, [P, I]),
            "ospIsReady": (I, [P, I]),
            "ospGetTaskDuration": (F, [P]),
            "ospPick": (None, [ctypes.POINTER(OSPPickResult), P, P, P, P, F, F]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def set_param(obj, name, typ, value):
    """value: numpy array / scalar of the parameter's bytes, or a handle for object types."""
    if typ >= OSP_OBJECT:
        h = ctypes.c_void_p(value)
        lib().ospSetParam(obj, name.encode(), typ, ctypes.byref(h))
        return
    a = np.ascontiguousarray(value)
    lib().ospSetParam(obj, name.encode(), typ, a.ctypes.data)


def shared_data(arr, typ, count, keep):
    """ospNewSharedData1D over a numpy array (kept alive in `keep`)."""
    a = np.ascontiguousarray(arr)
    keep.append(a)
    return lib().ospNewSharedData(a.ctypes.data, typ, count, 0, 1, 0, 1, 0, None, None)


def set_data(obj, name, arr, typ, count, keep):
    d = shared_data(arr, typ, count, keep)
    lib().ospCommit(d)
    set_param(obj, name, OSP_DATA, d)
    lib().ospRelease(d)


def new_texture(img, fmt, data_type, filter=0, wrap=0, keep=None):
    """A committed "texture2d" over an (h, w[, c]) array with OSPTextureFormat
    `fmt` and OSPDataType `data_type` (its texel type); wrap: one mode or two."""
    L = lib()
    keep = [] if keep is None else keep
    a = np.ascontiguousarray(img)
    keep.append(a)
    d = L.ospNewSharedData(a.ctypes.data, data_type, a.shape[1], 0, a.shape[0], 0, 1, 0, None, None)
    L.ospCommit(d)
    t = L.ospNewTexture(b"texture2d")
    set_param(t, "data", OSP_DATA, d)
    L.ospRelease(d)
    set_param(t, "format", OSP_UINT, np.uint32(fmt))
    set_param(t, "filter", OSP_UINT, np.uint32(filter))
    if isinstance(wrap, (tuple, list)):
        set_param(t, "wrapMode", OSP_VEC2UI, np.asarray(wrap, np.uint32))
    else:
        set_param(t, "wrapMode", OSP_UINT, np.uint32(wrap))
    L.ospCommit(t)
    return t


def map_channel(fb, ch, shape, dtype):
    p = lib().ospMapFrameBuffer(fb, ch)
    assert p, "ospMapFrameBuffer returned null"
    n = int(np.prod(shape)) * np.dtype(dtype).itemsize
    out = np.frombuffer(ctypes.string_at(p, n), dtype=dtype).reshape(shape).copy()
    lib().ospUnmapFrameBuffer(p, fb)
    return out


def _new_model(geom, material):
    L = lib()
    m = L.ospNewGeometricModel(geom)
    set_param(m, "material", OSP_MATERIAL, material)
    L.ospCommit(m)
    return m


def _object_data(handles, typ):
    arr = (ctypes.c_void_p * len(handles))(*handles)
    d = lib().ospNewSharedData(ctypes.addressof(arr), typ, len(handles), 0, 1, 0, 1, 0, None, None)
    lib().ospCommit(d)
    return d


class PathTracerApp:
    """The path-tracer workload of scenes.pt_instanced_scene built the way an
    OSPRay application builds it: a "mesh" geometry per shape, one
    geometric model per instance with its own "principled" material, one
    group + "instance" (with its affine "transform") per sphere and one for
    the ground, "quad" and "ambient" lights on the world, a "pathtracer"
    renderer and a "perspective" camera, an RGBA32F framebuffer with
    accumulation.  frame() is one ospRenderFrame + ospWait +
    ospMapFrameBuffer (colour copied to host memory) + ospUnmapFrameBuffer."""

    def __init__(self, data, spp, max_path_length=5, roulette_path_length=3, width=None, height=None,
                 materials=None):
        """materials: optional (OSPRay material type, {parameter: value}) per
        sphere instance in place of the workload's principled ones."""
        L = lib()
        self.keep = []
        self.W = width or data["width"]
        self.H = height or data["height"]
        mesh = L.ospNewGeometry(b"mesh")
        set_data(mesh, "vertex.position", data["vertex"].astype(np.float32), OSP_VEC3F, len(data["vertex"]),
                 self.keep)
        set_data(mesh, "index", data["index"].astype(np.uint32), OSP_VEC3UI, len(data["index"]), self.keep)
        L.ospCommit(mesh)
        ground = L.ospNewGeometry(b"mesh")
        set_data(ground, "vertex.position", data["ground_vertex"].astype(np.float32), OSP_VEC3F,
                 len(data["ground_vertex"]), self.keep)
        set_data(ground, "index", data["ground_index"].astype(np.uint32), OSP_VEC3UI, len(data["ground_index"]),
                 self.keep)
        L.ospCommit(ground)
        insts = []
        n = len(data["xfm"])
        for k in range(n + 1):
            if materials is not None and k < n:
                typ, params = materials[k]
                mat = L.ospNewMaterial(typ.encode())
                if not mat:
                    raise RuntimeError(L.ospDeviceGetLastErrorMsg(L.ospGetCurrentDevice()))
                for key, val in params.items():
                    if isinstance(val, (tuple, list)):
                        set_param(mat, key, OSP_VEC3F, np.float32(val))
                    else:
                        set_param(mat, key, OSP_FLOAT, np.float32(val))
            else:
                mt = data["materials"][k]
                mat = L.ospNewMaterial(b"principled")
                set_param(mat, "baseColor", OSP_VEC3F, np.float32(mt[:3]))
                set_param(mat, "roughness", OSP_FLOAT, np.float32(mt[3]))
                set_param(mat, "metallic", OSP_FLOAT, np.float32(mt[4]))
            L.ospCommit(mat)
            model = _new_model(mesh if k < n else ground, mat)
            L.ospRelease(mat)
            md = _object_data([model], OSP_GEOMETRIC_MODEL)
            L.ospRelease(model)
            group = L.ospNewGroup()
            set_param(group, "geometry", OSP_DATA, md)
            L.ospRelease(md)
            L.ospCommit(group)
            inst = L.ospNewInstance(group)
            L.ospRelease(group)
            if k < n:
                # OSPRay's affine3f: the 3x3 linear part column by column, then the translation
                x = np.asarray(data["xfm"][k], np.float32).reshape(3, 4)
                set_param(inst, "transform", OSP_AFFINE3F, np.ascontiguousarray(
                    np.concatenate([x[:, 0], x[:, 1], x[:, 2], x[:, 3]]).astype(np.float32)))
            L.ospCommit(inst)
            insts.append(inst)
        L.ospRelease(mesh)
        L.ospRelease(ground)
        lights = []
        for ld in data["lights"]:
            lh = L.ospNewLight(ld["type"].encode())
            set_param(lh, "intensity", OSP_FLOAT, np.float32(ld["intensity"]))
            if ld["type"] == "quad":
                for key in ("position", "edge1", "edge2"):
                    set_param(lh, key, OSP_VEC3F, np.float32(ld[key]))
            L.ospCommit(lh)
            lights.append(lh)
        self.world = L.ospNewWorld()
        idata = _object_data(insts, OSP_INSTANCE)
        set_param(self.world, "instance", OSP_DATA, idata)
        L.ospRelease(idata)
        ldata = _object_data(lights, OSP_LIGHT)
        set_param(self.world, "light", OSP_DATA, ldata)
        L.ospRelease(ldata)
        for h in insts + lights:
            L.ospRelease(h)
        L.ospCommit(self.world)
        c = data["camera"]
        self.cam = L.ospNewCamera(b"perspective")
        set_param(self.cam, "position", OSP_VEC3F, np.float32(c["position"]))
        set_param(self.cam, "direction", OSP_VEC3F, np.float32(c["direction"]))
        set_param(self.cam, "up", OSP_VEC3F, np.float32(c["up"]))
        set_param(self.cam, "fovy", OSP_FLOAT, np.float32(c["fovy"]))
        set_param(self.cam, "aspect", OSP_FLOAT, np.float32(self.W / self.H))
        L.ospCommit(self.cam)
        self.ren = L.ospNewRenderer(b"pathtracer")
        set_param(self.ren, "pixelSamples", OSP_INT, np.int32(spp))
        set_param(self.ren, "maxPathLength", OSP_INT, np.int32(max_path_length))
        set_param(self.ren, "roulettePathLength", OSP_INT, np.int32(roulette_path_length))
        L.ospCommit(self.ren)
        self.fb = L.ospNewFrameBuffer(self.W, self.H, OSP_FB_RGBA32F, OSP_FB_COLOR | OSP_FB_ACCUM)
        self.color = np.empty((self.H, self.W, 4), np.float32)

    def frame(self):
        """One rendered frame read back to host memory; returns (h2d, d2h) bytes."""
        L = lib()
        fut = L.ospRenderFrame(self.fb, self.ren, self.cam, self.world)
        if not fut:
            raise RuntimeError(L.ospDeviceGetLastErrorMsg(L.ospGetCurrentDevice()))
        L.ospWait(fut, OSP_TASK_FINISHED)
        L.ospRelease(fut)
        p = L.ospMapFrameBuffer(self.fb, OSP_FB_COLOR)
        ctypes.memmove(self.color.ctypes.data, p, self.color.nbytes)
        L.ospUnmapFrameBuffer(p, self.fb)
        # per frame the camera and renderer parameters go to the device with the launches
        return 40 + 76, self.color.nbytes

    def reset(self):
        lib().ospResetAccumulation(self.fb)

    def release(self):
        L = lib()
        for h in (self.fb, self.ren, self.cam, self.world):
            L.ospRelease(h)
