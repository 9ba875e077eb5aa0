// The "b200" OSPRay device: implements the OSPRay API's device interface on
// the b200 C ABI (libb200.so).  Counterpart of the reference's ISPCDevice
// (modules/cpu/ISPCDevice.cpp).
#pragma once

#include "scene_objects.h"

namespace b200osp {

class B200Device : public ospapi::Device {
 public:
  B200Device();
  ~B200Device() override;

  b200_device handle();
  // throws the b200 status as an OSPError with the device's message
  void check(int rc);
  void warn(const std::string &msg);

  void setParam(const char *id, OSPDataType, const void *mem) override;
  void removeParam(const char *id) override;
  void commit() override;
  int64_t property(OSPDeviceProperty) override;

  OSPData newSharedData(const void *shared, OSPDataType, uint64_t n1, int64_t s1, uint64_t n2, int64_t s2,
                        uint64_t n3, int64_t s3, OSPDeleterCallback, const void *userPtr) override;
  OSPData newData(OSPDataType, uint64_t n1, uint64_t n2, uint64_t n3) override;
  void copyData(OSPData src, OSPData dst, uint64_t i1, uint64_t i2, uint64_t i3) override;

  OSPObject newObject(OSPDataType kind, const char *type) override;
  OSPGeometricModel newGeometricModel(OSPGeometry) override;
  OSPVolumetricModel newVolumetricModel(OSPVolume) override;
  OSPGroup newGroup() override;
  OSPInstance newInstance(OSPGroup) override;
  OSPWorld newWorld() override;
  OSPFrameBuffer newFrameBuffer(int w, int h, OSPFrameBufferFormat, uint32_t channels) override;
  OSPBounds bounds(OSPObject) override;

  void setObjectParam(OSPObject, const char *id, OSPDataType, const void *mem) override;
  void removeObjectParam(OSPObject, const char *id) override;
  void commitObject(OSPObject) override;
  void release(OSPObject) override;
  void retain(OSPObject) override;

  const void *mapFrameBuffer(OSPFrameBuffer, OSPFrameBufferChannel) override;
  void unmapFrameBuffer(const void *mapped, OSPFrameBuffer) override;
  float variance(OSPFrameBuffer) override;
  void resetAccumulation(OSPFrameBuffer) override;

  OSPFuture renderFrame(OSPFrameBuffer, OSPRenderer, OSPCamera, OSPWorld) override;
  int isReady(OSPFuture, OSPSyncEvent) override;
  void wait(OSPFuture, OSPSyncEvent) override;
  void cancel(OSPFuture) override;
  float progress(OSPFuture) override;
  float taskDuration(OSPFuture) override;
  void pick(OSPPickResult *, OSPFrameBuffer, OSPRenderer, OSPCamera, OSPWorld, float x, float y) override;

 private:
  Obj params_{OSP_DEVICE, "b200"};
  b200_device dev_ = nullptr;
  int cudaDevice_ = 0;
};

}  // namespace b200osp
