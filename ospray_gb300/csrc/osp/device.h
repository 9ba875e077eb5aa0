// The device interface between libospray.so (the OSPRay C API entry points)
// and a device module such as libospray_module_b200.so.
//
// Mirrors the split of the reference: ospray/api/API.cpp forwards every API
// call to the current api::Device (ospray/api/Device.h), and a module
// registers device types by name from its ospray_module_init_<name>
// (modules/cpu/ModuleInit.cpp:24-54).  Errors are C++ exceptions inside the
// library; the API layer turns them into the device's last error, the error
// callback and a null/zero return (ospray/api/API.cpp:28-66), so nothing
// throws across the C ABI.
#pragma once

#include <atomic>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "../../../include/ospray/ospray.h"

namespace ospapi {

// OSPRay API version implemented by this library
constexpr int kVersionMajor = 3;
constexpr int kVersionMinor = 3;
constexpr int kVersionPatch = 0;

struct Error : std::runtime_error {
  OSPError code;
  Error(OSPError c, const std::string &m) : std::runtime_error(m), code(c) {}
};

class Device {
 public:
  virtual ~Device() = default;

  std::atomic<int> refs{1};
  OSPError lastCode = OSP_NO_ERROR;
  std::string lastMsg;
  OSPErrorCallback errorCallback = nullptr;
  void *errorUserData = nullptr;
  OSPStatusCallback statusCallback = nullptr;
  void *statusUserData = nullptr;
  int logLevel = OSP_LOG_WARNING;
  bool warnAsError = false;

  // status / warning messages (routed to the status callback, or stderr)
  void status(int level, const std::string &msg);

  // ---- device
  virtual void setParam(const char *id, OSPDataType, const void *mem) = 0;
  virtual void removeParam(const char *id) = 0;
  virtual void commit() = 0;
  virtual int64_t property(OSPDeviceProperty) = 0;

  // ---- data
  virtual OSPData newSharedData(const void *shared, OSPDataType, uint64_t n1, int64_t s1, uint64_t n2, int64_t s2,
                                uint64_t n3, int64_t s3, OSPDeleterCallback, const void *userPtr) = 0;
  virtual OSPData newData(OSPDataType, uint64_t n1, uint64_t n2, uint64_t n3) = 0;
  virtual void copyData(OSPData src, OSPData dst, uint64_t i1, uint64_t i2, uint64_t i3) = 0;

  // ---- objects.  `kind` is the handle type (OSP_LIGHT, OSP_CAMERA, ...)
  virtual OSPObject newObject(OSPDataType kind, const char *type) = 0;
  virtual OSPGeometricModel newGeometricModel(OSPGeometry) = 0;
  virtual OSPVolumetricModel newVolumetricModel(OSPVolume) = 0;
  virtual OSPGroup newGroup() = 0;
  virtual OSPInstance newInstance(OSPGroup) = 0;
  virtual OSPWorld newWorld() = 0;
  virtual OSPFrameBuffer newFrameBuffer(int w, int h, OSPFrameBufferFormat, uint32_t channels) = 0;
  virtual OSPBounds bounds(OSPObject) = 0;

  virtual void setObjectParam(OSPObject, const char *id, OSPDataType, const void *mem) = 0;
  virtual void removeObjectParam(OSPObject, const char *id) = 0;
  virtual void commitObject(OSPObject) = 0;
  virtual void release(OSPObject) = 0;
  virtual void retain(OSPObject) = 0;

  // ---- framebuffer
  virtual const void *mapFrameBuffer(OSPFrameBuffer, OSPFrameBufferChannel) = 0;
  virtual void unmapFrameBuffer(const void *mapped, OSPFrameBuffer) = 0;
  virtual float variance(OSPFrameBuffer) = 0;
  virtual void resetAccumulation(OSPFrameBuffer) = 0;

  // ---- rendering
  virtual OSPFuture renderFrame(OSPFrameBuffer, OSPRenderer, OSPCamera, OSPWorld) = 0;
  virtual int isReady(OSPFuture, OSPSyncEvent) = 0;
  virtual void wait(OSPFuture, OSPSyncEvent) = 0;
  virtual void cancel(OSPFuture) = 0;
  virtual float progress(OSPFuture) = 0;
  virtual float taskDuration(OSPFuture) = 0;
  virtual void pick(OSPPickResult *, OSPFrameBuffer, OSPRenderer, OSPCamera, OSPWorld, float x, float y) = 0;
};

inline void Device::status(int level, const std::string &msg) {
  if (level < logLevel) return;
  if (statusCallback)
    statusCallback(statusUserData, msg.c_str());
  else
    fprintf(stderr, "%s\n", msg.c_str());
}

typedef Device *(*DeviceFactory)();

}  // namespace ospapi

// exported by libospray.so: called from a module's ospray_module_init_<name>
extern "C" __attribute__((visibility("default"))) void ospray_register_device_type(const char *name,
                                                                                     ospapi::DeviceFactory f);
