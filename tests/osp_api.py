"""ctypes access to libospray.so (the OSPRay C API of include/ospray/ospray.h)
for the tests: the same calls an OSPRay application makes."""
import ctypes
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "ospray_gb300", "_build")
P, I, U32, F, U64, I64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_float, ctypes.c_uint64, \
    ctypes.c_int64

# OSPDataType values used here
OSP_OBJECT, OSP_DATA = 0x8000000, 0x8000000 + 100
OSP_GEOMETRIC_MODEL, OSP_INSTANCE, OSP_LIGHT, OSP_MATERIAL = (0x8000000 + 104, 0x8000000 + 108,
                                                             0x8000000 + 109, 0x8000000 + 110)
OSP_INT, OSP_UINT, OSP_FLOAT, OSP_VEC3F, OSP_VEC4F, OSP_VEC3UI = 4000, 4500, 6000, 6002, 6003, 4502
OSP_AFFINE3F, OSP_BOOL = 12003, 250
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


def map_channel(fb, ch, shape, dtype):
    p = lib().ospMapFrameBuffer(fb, ch)
    assert p, "ospMapFrameBuffer returned null"
    n = int(np.prod(shape)) * np.dtype(dtype).itemsize
    out = np.frombuffer(ctypes.string_at(p, n), dtype=dtype).reshape(shape).copy()
    lib().ospUnmapFrameBuffer(p, fb)
    return out
