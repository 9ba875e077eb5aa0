// libospray.so: the OSPRay C API entry points.
//
// Every entry point forwards to the current device (ospapi::Device) and
// catches what the device throws: the error code and message become the
// device's last error, the error callback is called, and the function
// returns its null/zero default, as ospray/api/API.cpp:28-66 does.  Devices
// come from modules: ospLoadModule(name) dlopens libospray_module_<name>.so
// (first beside this library, then on the loader's search path) and calls
// its ospray_module_init_<name>(major, minor, patch), which registers device
// types by name (ospray/common/OSPCommon.cpp:749-782).  The only device type
// this project provides is "b200"; the API's default device type "cpu"
// resolves to it when no "cpu" device is registered.
#include <dlfcn.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../../include/ospray/ospray_util.h"
#include "device.h"

using ospapi::Device;
using ospapi::Error;

namespace {

std::map<std::string, ospapi::DeviceFactory> &registry() {
  static std::map<std::string, ospapi::DeviceFactory> r;
  return r;
}
std::map<std::string, void *> &loadedModules() {
  static std::map<std::string, void *> m;
  return m;
}

Device *g_current = nullptr;
// errors raised while no device exists (ospInit, ospNewDevice)
OSPError g_noDeviceCode = OSP_NO_ERROR;
std::string g_noDeviceMsg;

void retainDevice(Device *d) {
  if (d) d->refs.fetch_add(1);
}
void releaseDevice(Device *d) {
  if (d && d->refs.fetch_sub(1) == 1) delete d;
}

void handleError(Device *d, OSPError code, const char *msg) {
  if (!d) {
    g_noDeviceCode = code;
    g_noDeviceMsg = msg;
    fprintf(stderr, "OSPRay error: %s\n", msg);
    return;
  }
  d->lastCode = code;
  d->lastMsg = msg;
  if (d->errorCallback)
    d->errorCallback(d->errorUserData, code, msg);
  else
    d->status(OSP_LOG_ERROR, std::string("OSPRay error: ") + msg);
}

Device &current() {
  if (!g_current) throw Error(OSP_INVALID_OPERATION, "OSPRay not yet initialized (no current device)");
  return *g_current;
}

// runs f; on failure records the error on the current device (or the global
// slot) and returns `fallback`
template <class R, class F>
R guard(R fallback, F f) {
  try {
    return f();
  } catch (const Error &e) {
    handleError(g_current, e.code, e.what());
  } catch (const std::bad_alloc &) {
    handleError(g_current, OSP_OUT_OF_MEMORY, "out of host memory");
  } catch (const std::exception &e) {
    handleError(g_current, OSP_UNKNOWN_ERROR, e.what());
  } catch (...) {
    handleError(g_current, OSP_UNKNOWN_ERROR, "unknown error");
  }
  return fallback;
}
template <class F>
void guardVoid(F f) {
  guard(0, [&]() {
    f();
    return 0;
  });
}

std::string libraryDir() {
  Dl_info info;
  if (dladdr(reinterpret_cast<void *>(&ospLoadModule), &info) && info.dli_fname) {
    std::string p(info.dli_fname);
    const size_t s = p.rfind('/');
    if (s != std::string::npos) return p.substr(0, s + 1);
  }
  return "";
}

OSPError loadModule(const std::string &name) {
  if (loadedModules().count(name)) return OSP_NO_ERROR;
  const std::string file = "libospray_module_" + name + ".so";
  void *h = dlopen((libraryDir() + file).c_str(), RTLD_NOW | RTLD_GLOBAL);
  if (!h) h = dlopen(file.c_str(), RTLD_NOW | RTLD_GLOBAL);
  if (!h) throw Error(OSP_INVALID_ARGUMENT, "could not load module '" + name + "': " + dlerror());
  const std::string sym = "ospray_module_init_" + name;
  using InitFn = OSPError (*)(int16_t, int16_t, int16_t);
  InitFn init = reinterpret_cast<InitFn>(dlsym(h, sym.c_str()));
  if (!init) {
    dlclose(h);
    throw Error(OSP_INVALID_ARGUMENT, "module '" + name + "' has no " + sym);
  }
  const OSPError e = init(ospapi::kVersionMajor, ospapi::kVersionMinor, ospapi::kVersionPatch);
  if (e != OSP_NO_ERROR) {
    dlclose(h);
    throw Error(e, "initialisation of module '" + name + "' failed" +
                       (e == OSP_VERSION_MISMATCH ? std::string(" (version mismatch)") : std::string()));
  }
  loadedModules()[name] = h;
  return OSP_NO_ERROR;
}

Device *createDevice(const std::string &type) {
  std::string t = type;
  if (!registry().count(t)) {
    // a device type of the same name as a module is loaded on demand
    try {
      loadModule(t);
    } catch (const Error &) {
      if (t != "cpu" && t != "default") throw;
    }
  }
  if (!registry().count(t) && (t == "cpu" || t == "default")) {
    if (!registry().count("b200")) loadModule("b200");
    t = "b200";
  }
  auto it = registry().find(t);
  if (it == registry().end()) throw Error(OSP_INVALID_ARGUMENT, "unknown device type '" + type + "'");
  return it->second();
}

std::string argValue(const std::string &a) {
  const size_t eq = a.find('=');
  return eq == std::string::npos ? std::string() : a.substr(eq + 1);
}

void removeArg(int &ac, const char **av, int i) {
  for (int k = i; k + 1 < ac; k++) av[k] = av[k + 1];
  ac--;
}

std::vector<std::string> split(const std::string &s, char c) {
  std::vector<std::string> out;
  size_t b = 0;
  while (b <= s.size()) {
    const size_t e = s.find(c, b);
    const std::string part = s.substr(b, e == std::string::npos ? std::string::npos : e - b);
    if (!part.empty()) out.push_back(part);
    if (e == std::string::npos) break;
    b = e + 1;
  }
  return out;
}

void setDeviceInt(Device &d, const char *name, int v) { d.setParam(name, OSP_INT, &v); }
void setDeviceBool(Device &d, const char *name, bool b) {
  const int v = b ? 1 : 0;
  d.setParam(name, OSP_BOOL, &v);
}

}  // namespace

extern "C" {

__attribute__((visibility("default"))) void ospray_register_device_type(const char *name, ospapi::DeviceFactory f) {
  if (name && f) registry()[name] = f;
}

// ---------------------------------------------------------------- devices

OSPError ospInit(int *argc, const char **argv) {
  return guard(OSP_INVALID_OPERATION, [&]() {
    if (g_current) throw Error(OSP_INVALID_OPERATION, "device already exists [ospInit() called twice?]");
    if (const char *m = getenv("OSPRAY_LOAD_MODULES"))
      for (const auto &name : split(m, ',')) loadModule(name);
    Device *dev = nullptr;
    std::vector<std::pair<std::string, std::string>> flags;
    if (argc && argv) {
      for (int i = 1; i < *argc;) {
        const std::string a(argv[i]);
        if (a.rfind("--osp:load-modules", 0) == 0) {
          const auto mods = split(argValue(a), ',');
          if (mods.empty()) throw Error(OSP_INVALID_ARGUMENT, "--osp:load-modules needs <module1>[,<module2>...]");
          for (const auto &name : mods) loadModule(name);
          removeArg(*argc, argv, i);
        } else if (a.rfind("--osp:device=", 0) == 0) {
          if (dev) releaseDevice(dev);
          dev = createDevice(argValue(a));
          removeArg(*argc, argv, i);
        } else if (a == "--osp:debug" || a == "--osp:warn-as-error" || a == "--osp:verbose" || a == "--osp:vv" ||
                   a.rfind("--osp:log-level", 0) == 0 || a.rfind("--osp:num-threads", 0) == 0 ||
                   a.rfind("--osp:set-affinity", 0) == 0 || a.rfind("--osp:log-output", 0) == 0 ||
                   a.rfind("--osp:error-output", 0) == 0) {
          flags.emplace_back(a.substr(0, a.find('=')), argValue(a));
          removeArg(*argc, argv, i);
        } else {
          ++i;
        }
      }
    }
    if (!dev) {
      const char *env = getenv("OSPRAY_DEVICE");
      dev = createDevice(env && *env ? env : "cpu");
    }
    for (const auto &f : flags) {
      if (f.first == "--osp:debug") {
        setDeviceBool(*dev, "debug", true);
        setDeviceInt(*dev, "logLevel", OSP_LOG_DEBUG);
      } else if (f.first == "--osp:warn-as-error") {
        setDeviceBool(*dev, "warnAsError", true);
      } else if (f.first == "--osp:verbose") {
        setDeviceInt(*dev, "logLevel", OSP_LOG_INFO);
      } else if (f.first == "--osp:vv") {
        setDeviceInt(*dev, "logLevel", OSP_LOG_DEBUG);
      } else if (f.first == "--osp:log-level") {
        static const char *names[] = {"", "debug", "info", "warning", "error", "none"};
        int lvl = atoi(f.second.c_str());
        for (int k = 1; k <= 5; k++)
          if (f.second == names[k]) lvl = k;
        if (lvl >= 1 && lvl <= 5) setDeviceInt(*dev, "logLevel", lvl);
      } else if (f.first == "--osp:num-threads") {
        setDeviceInt(*dev, "numThreads", atoi(f.second.c_str()));
      }
    }
    try {
      dev->commit();
    } catch (...) {
      releaseDevice(dev);
      throw;
    }
    g_current = dev;  // the creation reference becomes the current-device reference
    return OSP_NO_ERROR;
  });
}

int64_t ospDeviceGetProperty(OSPDevice d, OSPDeviceProperty p) {
  return guard<int64_t>(0, [&]() -> int64_t {
    if (!d) throw Error(OSP_INVALID_ARGUMENT, "null device");
    return reinterpret_cast<Device *>(d)->property(p);
  });
}

void ospShutdown() {
  guardVoid([&]() {
    Device *d = g_current;
    g_current = nullptr;
    releaseDevice(d);
  });
}

OSPDevice ospNewDevice(const char *type) {
  return guard<OSPDevice>(nullptr, [&]() {
    if (!type) throw Error(OSP_INVALID_ARGUMENT, "null device type");
    return reinterpret_cast<OSPDevice>(createDevice(type));
  });
}

void ospSetCurrentDevice(OSPDevice d) {
  guardVoid([&]() {
    Device *dev = reinterpret_cast<Device *>(d);
    retainDevice(dev);
    releaseDevice(g_current);
    g_current = dev;
  });
}

OSPDevice ospGetCurrentDevice() {
  retainDevice(g_current);
  return reinterpret_cast<OSPDevice>(g_current);
}

void ospDeviceSetParam(OSPDevice d, const char *id, OSPDataType t, const void *mem) {
  guardVoid([&]() {
    if (!d || !id) throw Error(OSP_INVALID_ARGUMENT, "null device or parameter name");
    reinterpret_cast<Device *>(d)->setParam(id, t, mem);
  });
}

void ospDeviceRemoveParam(OSPDevice d, const char *id) {
  guardVoid([&]() {
    if (!d || !id) throw Error(OSP_INVALID_ARGUMENT, "null device or parameter name");
    reinterpret_cast<Device *>(d)->removeParam(id);
  });
}

void ospDeviceSetStatusCallback(OSPDevice d, OSPStatusCallback cb, void *user) {
  if (!d) return;
  Device *dev = reinterpret_cast<Device *>(d);
  dev->statusCallback = cb;
  dev->statusUserData = user;
}

void ospDeviceSetErrorCallback(OSPDevice d, OSPErrorCallback cb, void *user) {
  if (!d) return;
  Device *dev = reinterpret_cast<Device *>(d);
  dev->errorCallback = cb;
  dev->errorUserData = user;
}

OSPError ospDeviceGetLastErrorCode(OSPDevice d) {
  return d ? reinterpret_cast<Device *>(d)->lastCode : g_noDeviceCode;
}

const char *ospDeviceGetLastErrorMsg(OSPDevice d) {
  return d ? reinterpret_cast<Device *>(d)->lastMsg.c_str() : g_noDeviceMsg.c_str();
}

void ospDeviceCommit(OSPDevice d) {
  guardVoid([&]() {
    if (!d) throw Error(OSP_INVALID_ARGUMENT, "null device");
    reinterpret_cast<Device *>(d)->commit();
  });
}

void ospDeviceRelease(OSPDevice d) { releaseDevice(reinterpret_cast<Device *>(d)); }
void ospDeviceRetain(OSPDevice d) { retainDevice(reinterpret_cast<Device *>(d)); }

OSPError ospLoadModule(const char *name) {
  // errors are reported as the return value (and recorded), never thrown
  try {
    if (!name) throw Error(OSP_INVALID_ARGUMENT, "null module name");
    return loadModule(name);
  } catch (const Error &e) {
    handleError(g_current, e.code, e.what());
    return e.code;
  }
}

// ---------------------------------------------------------------- data

OSPData ospNewSharedData(const void *shared, OSPDataType t, uint64_t n1, int64_t s1, uint64_t n2, int64_t s2,
                         uint64_t n3, int64_t s3, OSPDeleterCallback del, const void *user) {
  return guard<OSPData>(nullptr, [&]() { return current().newSharedData(shared, t, n1, s1, n2, s2, n3, s3, del, user); });
}

OSPData ospNewData(OSPDataType t, uint64_t n1, uint64_t n2, uint64_t n3) {
  return guard<OSPData>(nullptr, [&]() { return current().newData(t, n1, n2, n3); });
}

void ospCopyData(const OSPData src, OSPData dst, uint64_t i1, uint64_t i2, uint64_t i3) {
  guardVoid([&]() { current().copyData(src, dst, i1, i2, i3); });
}

// ---------------------------------------------------------------- objects

#define OSP_NEW_TYPED(fn, Handle, kind)                                                                  \
  Handle fn(const char *type) {                                                                          \
    return guard<Handle>(nullptr, [&]() {                                                                \
      if (!type) throw Error(OSP_INVALID_ARGUMENT, "null type string");                                  \
      return reinterpret_cast<Handle>(current().newObject(kind, type));                                  \
    });                                                                                                  \
  }
OSP_NEW_TYPED(ospNewLight, OSPLight, OSP_LIGHT)
OSP_NEW_TYPED(ospNewCamera, OSPCamera, OSP_CAMERA)
OSP_NEW_TYPED(ospNewGeometry, OSPGeometry, OSP_GEOMETRY)
OSP_NEW_TYPED(ospNewVolume, OSPVolume, OSP_VOLUME)
OSP_NEW_TYPED(ospNewMaterial, OSPMaterial, OSP_MATERIAL)
OSP_NEW_TYPED(ospNewTransferFunction, OSPTransferFunction, OSP_TRANSFER_FUNCTION)
OSP_NEW_TYPED(ospNewTexture, OSPTexture, OSP_TEXTURE)
OSP_NEW_TYPED(ospNewImageOperation, OSPImageOperation, OSP_IMAGE_OPERATION)
OSP_NEW_TYPED(ospNewRenderer, OSPRenderer, OSP_RENDERER)
#undef OSP_NEW_TYPED

OSPGeometricModel ospNewGeometricModel(OSPGeometry g) {
  return guard<OSPGeometricModel>(nullptr, [&]() { return current().newGeometricModel(g); });
}
OSPVolumetricModel ospNewVolumetricModel(OSPVolume v) {
  return guard<OSPVolumetricModel>(nullptr, [&]() { return current().newVolumetricModel(v); });
}
OSPGroup ospNewGroup() {
  return guard<OSPGroup>(nullptr, [&]() { return current().newGroup(); });
}
OSPInstance ospNewInstance(OSPGroup g) {
  return guard<OSPInstance>(nullptr, [&]() { return current().newInstance(g); });
}
OSPWorld ospNewWorld() {
  return guard<OSPWorld>(nullptr, [&]() { return current().newWorld(); });
}

OSPBounds ospGetBounds(OSPObject o) {
  OSPBounds empty = {{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
  return guard(empty, [&]() {
    if (!o) throw Error(OSP_INVALID_ARGUMENT, "null object");
    return current().bounds(o);
  });
}

void ospSetParam(OSPObject o, const char *id, OSPDataType t, const void *mem) {
  guardVoid([&]() {
    if (!o || !id) throw Error(OSP_INVALID_ARGUMENT, "null object or parameter name");
    current().setObjectParam(o, id, t, mem);
  });
}

void ospRemoveParam(OSPObject o, const char *id) {
  guardVoid([&]() {
    if (!o || !id) throw Error(OSP_INVALID_ARGUMENT, "null object or parameter name");
    current().removeObjectParam(o, id);
  });
}

void ospCommit(OSPObject o) {
  guardVoid([&]() {
    if (!o) throw Error(OSP_INVALID_ARGUMENT, "null object committed");
    current().commitObject(o);
  });
}

void ospRelease(OSPObject o) {
  if (!o) return;
  guardVoid([&]() { current().release(o); });
}

void ospRetain(OSPObject o) {
  if (!o) return;
  guardVoid([&]() { current().retain(o); });
}

// ---------------------------------------------------------------- framebuffer

OSPFrameBuffer ospNewFrameBuffer(int w, int h, OSPFrameBufferFormat fmt, uint32_t channels) {
  return guard<OSPFrameBuffer>(nullptr, [&]() { return current().newFrameBuffer(w, h, fmt, channels); });
}

const void *ospMapFrameBuffer(OSPFrameBuffer fb, OSPFrameBufferChannel ch) {
  return guard<const void *>(nullptr, [&]() {
    if (!fb) throw Error(OSP_INVALID_ARGUMENT, "null framebuffer");
    return current().mapFrameBuffer(fb, ch);
  });
}

void ospUnmapFrameBuffer(const void *mapped, OSPFrameBuffer fb) {
  guardVoid([&]() {
    if (!fb) throw Error(OSP_INVALID_ARGUMENT, "null framebuffer");
    current().unmapFrameBuffer(mapped, fb);
  });
}

float ospGetVariance(OSPFrameBuffer fb) {
  return guard(INFINITY, [&]() {
    if (!fb) throw Error(OSP_INVALID_ARGUMENT, "null framebuffer");
    return current().variance(fb);
  });
}

void ospResetAccumulation(OSPFrameBuffer fb) {
  guardVoid([&]() {
    if (!fb) throw Error(OSP_INVALID_ARGUMENT, "null framebuffer");
    current().resetAccumulation(fb);
  });
}

// ---------------------------------------------------------------- rendering

OSPFuture ospRenderFrame(OSPFrameBuffer fb, OSPRenderer r, OSPCamera c, OSPWorld w) {
  return guard<OSPFuture>(nullptr, [&]() {
    if (!fb || !r || !c || !w) throw Error(OSP_INVALID_ARGUMENT, "ospRenderFrame: null framebuffer, renderer, camera or world");
    return current().renderFrame(fb, r, c, w);
  });
}

int ospIsReady(OSPFuture f, OSPSyncEvent e) {
  return guard(1, [&]() { return f ? current().isReady(f, e) : 1; });
}

void ospWait(OSPFuture f, OSPSyncEvent e) {
  guardVoid([&]() {
    if (f) current().wait(f, e);
  });
}

void ospCancel(OSPFuture f) {
  guardVoid([&]() {
    if (f) current().cancel(f);
  });
}

float ospGetProgress(OSPFuture f) {
  return guard(1.f, [&]() { return f ? current().progress(f) : 1.f; });
}

float ospGetTaskDuration(OSPFuture f) {
  return guard(0.f, [&]() { return f ? current().taskDuration(f) : 0.f; });
}

void ospPick(OSPPickResult *res, OSPFrameBuffer fb, OSPRenderer r, OSPCamera c, OSPWorld w, float x, float y) {
  guardVoid([&]() {
    if (!res) throw Error(OSP_INVALID_ARGUMENT, "null pick result");
    res->hasHit = 0;
    res->instance = nullptr;
    res->model = nullptr;
    res->primID = 0xffffffffu;
    if (!fb || !r || !c || !w) throw Error(OSP_INVALID_ARGUMENT, "ospPick: null framebuffer, renderer, camera or world");
    current().pick(res, fb, r, c, w, x, y);
  });
}

// ---------------------------------------------------------------- ospray_util.h

OSPData ospNewSharedData1D(const void *d, OSPDataType t, uint64_t n) {
  return ospNewSharedData(d, t, n, 0, 1, 0, 1, 0, nullptr, nullptr);
}
OSPData ospNewAssignedData1D(const void *d, OSPDataType t, uint64_t n, OSPDeleterCallback del, const void *user) {
  return ospNewSharedData(d, t, n, 0, 1, 0, 1, 0, del, user);
}
OSPData ospNewSharedData1DStride(const void *d, OSPDataType t, uint64_t n, int64_t s) {
  return ospNewSharedData(d, t, n, s, 1, 0, 1, 0, nullptr, nullptr);
}
OSPData ospNewSharedData2D(const void *d, OSPDataType t, uint64_t n1, uint64_t n2) {
  return ospNewSharedData(d, t, n1, 0, n2, 0, 1, 0, nullptr, nullptr);
}
OSPData ospNewSharedData2DStride(const void *d, OSPDataType t, uint64_t n1, int64_t s1, uint64_t n2, int64_t s2) {
  return ospNewSharedData(d, t, n1, s1, n2, s2, 1, 0, nullptr, nullptr);
}
OSPData ospNewSharedData3D(const void *d, OSPDataType t, uint64_t n1, uint64_t n2, uint64_t n3) {
  return ospNewSharedData(d, t, n1, 0, n2, 0, n3, 0, nullptr, nullptr);
}
OSPData ospNewData1D(OSPDataType t, uint64_t n) { return ospNewData(t, n, 1, 1); }
OSPData ospNewData2D(OSPDataType t, uint64_t n1, uint64_t n2) { return ospNewData(t, n1, n2, 1); }
void ospCopyData1D(const OSPData s, OSPData d, uint64_t i) { ospCopyData(s, d, i, 0, 0); }
void ospCopyData2D(const OSPData s, OSPData d, uint64_t i1, uint64_t i2) { ospCopyData(s, d, i1, i2, 0); }

void ospSetString(OSPObject o, const char *n, const char *s) { ospSetParam(o, n, OSP_STRING, s); }
void ospSetObject(OSPObject o, const char *n, OSPObject v) { ospSetParam(o, n, OSP_OBJECT, &v); }
void ospSetBool(OSPObject o, const char *n, int x) { ospSetParam(o, n, OSP_BOOL, &x); }
void ospSetFloat(OSPObject o, const char *n, float x) { ospSetParam(o, n, OSP_FLOAT, &x); }
void ospSetInt(OSPObject o, const char *n, int x) { ospSetParam(o, n, OSP_INT, &x); }
void ospSetUInt(OSPObject o, const char *n, unsigned int x) { ospSetParam(o, n, OSP_UINT, &x); }
void ospSetBox1f(OSPObject o, const char *n, float x, float y) {
  const float v[2] = {x, y};
  ospSetParam(o, n, OSP_BOX1F, v);
}
void ospSetLinear2f(OSPObject o, const char *n, float x, float y, float z, float w) {
  const float v[4] = {x, y, z, w};
  ospSetParam(o, n, OSP_LINEAR2F, v);
}
void ospSetVec2f(OSPObject o, const char *n, float x, float y) {
  const float v[2] = {x, y};
  ospSetParam(o, n, OSP_VEC2F, v);
}
void ospSetVec3f(OSPObject o, const char *n, float x, float y, float z) {
  const float v[3] = {x, y, z};
  ospSetParam(o, n, OSP_VEC3F, v);
}
void ospSetVec4f(OSPObject o, const char *n, float x, float y, float z, float w) {
  const float v[4] = {x, y, z, w};
  ospSetParam(o, n, OSP_VEC4F, v);
}
void ospSetVec2i(OSPObject o, const char *n, int x, int y) {
  const int v[2] = {x, y};
  ospSetParam(o, n, OSP_VEC2I, v);
}
void ospSetVec3i(OSPObject o, const char *n, int x, int y, int z) {
  const int v[3] = {x, y, z};
  ospSetParam(o, n, OSP_VEC3I, v);
}
void ospSetVec4i(OSPObject o, const char *n, int x, int y, int z, int w) {
  const int v[4] = {x, y, z, w};
  ospSetParam(o, n, OSP_VEC4I, v);
}

void ospSetObjectAsData(OSPObject target, const char *n, OSPDataType type, OSPObject obj) {
  OSPData d = ospNewSharedData(&obj, type, 1, 0, 1, 0, 1, 0, nullptr, nullptr);
  ospSetParam(target, n, OSP_DATA, &d);
  ospRelease(d);
}

float ospRenderFrameBlocking(OSPFrameBuffer fb, OSPRenderer r, OSPCamera c, OSPWorld w) {
  OSPFuture f = ospRenderFrame(fb, r, c, w);
  ospWait(f, OSP_TASK_FINISHED);
  ospRelease(f);
  return ospGetVariance(fb);
}

}  // extern "C"
