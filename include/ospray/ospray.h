/* The OSPRay 3.x C API, provided by this project's libospray.so.
 *
 * Applications written against OSPRay (ospray/include/ospray/ospray.h) build
 * and link against this library unchanged: the functions, their parameter
 * lists, the handle types and the enumeration values (OSPEnums.h) are the
 * API's.  The device behind it is "b200", the GB300 module
 * (libospray_module_b200.so, entry point ospray_module_init_b200), which
 * renders with CUDA.  Object types the b200 device does not implement are
 * refused at creation with OSP_INVALID_ARGUMENT and a message naming them. */
#pragma once

#include <stdint.h>
#include <sys/types.h>

#include "OSPEnums.h"

#ifndef NULL
#ifdef __cplusplus
#define NULL nullptr
#else
#define NULL 0
#endif
#endif

#if defined(_WIN32) && defined(ospray_EXPORTS)
#define OSPRAY_INTERFACE __declspec(dllexport)
#elif defined(_WIN32)
#define OSPRAY_INTERFACE __declspec(dllimport)
#else
#define OSPRAY_INTERFACE __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
#define OSP_DEFAULT_VAL(a) = a
#else
#define OSP_DEFAULT_VAL(a)
#endif

/* Handles.  In C++ every handle type derives from OSPObject so a geometry
 * handle can be passed where an object handle is expected; in C they are
 * all void pointers. */
#ifdef __cplusplus
namespace osp {
struct Device;
struct ManagedObject {};
struct Camera : ManagedObject {};
struct Data : ManagedObject {};
struct FrameBuffer : ManagedObject {};
struct Future : ManagedObject {};
struct GeometricModel : ManagedObject {};
struct Geometry : ManagedObject {};
struct Group : ManagedObject {};
struct ImageOperation : ManagedObject {};
struct Instance : ManagedObject {};
struct Light : ManagedObject {};
struct Material : ManagedObject {};
struct Renderer : ManagedObject {};
struct Texture : ManagedObject {};
struct TransferFunction : ManagedObject {};
struct Volume : ManagedObject {};
struct VolumetricModel : ManagedObject {};
struct World : ManagedObject {};
}  // namespace osp
typedef osp::Device *OSPDevice;
typedef osp::ManagedObject *OSPObject;
typedef osp::Camera *OSPCamera;
typedef osp::Data *OSPData;
typedef osp::FrameBuffer *OSPFrameBuffer;
typedef osp::Future *OSPFuture;
typedef osp::GeometricModel *OSPGeometricModel;
typedef osp::Geometry *OSPGeometry;
typedef osp::Group *OSPGroup;
typedef osp::ImageOperation *OSPImageOperation;
typedef osp::Instance *OSPInstance;
typedef osp::Light *OSPLight;
typedef osp::Material *OSPMaterial;
typedef osp::Renderer *OSPRenderer;
typedef osp::Texture *OSPTexture;
typedef osp::TransferFunction *OSPTransferFunction;
typedef osp::Volume *OSPVolume;
typedef osp::VolumetricModel *OSPVolumetricModel;
typedef osp::World *OSPWorld;
#else
typedef void *OSPDevice;
typedef void _OSPManagedObject;
typedef _OSPManagedObject *OSPManagedObject, *OSPObject, *OSPCamera, *OSPData, *OSPFrameBuffer, *OSPFuture,
    *OSPGeometricModel, *OSPGeometry, *OSPGroup, *OSPImageOperation, *OSPInstance, *OSPLight, *OSPMaterial,
    *OSPRenderer, *OSPTexture, *OSPTransferFunction, *OSPVolume, *OSPVolumetricModel, *OSPWorld;
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- initialisation and devices */
/* parses --osp:device=<type>, --osp:load-modules=<a,b>, --osp:log-level=,
 * --osp:verbose, --osp:debug (removed from argv) and the OSPRAY_DEVICE /
 * OSPRAY_LOAD_MODULES environment; creates and sets the current device */
OSPRAY_INTERFACE OSPError ospInit(int *argc OSP_DEFAULT_VAL(NULL), const char **argv OSP_DEFAULT_VAL(NULL));
OSPRAY_INTERFACE int64_t ospDeviceGetProperty(OSPDevice, OSPDeviceProperty);
OSPRAY_INTERFACE void ospShutdown();
OSPRAY_INTERFACE OSPDevice ospNewDevice(const char *deviceType OSP_DEFAULT_VAL("cpu"));
OSPRAY_INTERFACE void ospSetCurrentDevice(OSPDevice);
OSPRAY_INTERFACE OSPDevice ospGetCurrentDevice();
OSPRAY_INTERFACE void ospDeviceSetParam(OSPDevice, const char *id, OSPDataType, const void *mem);
OSPRAY_INTERFACE void ospDeviceRemoveParam(OSPDevice, const char *id);

typedef void (*OSPStatusCallback)(void *userData, const char *messageText);
OSPRAY_INTERFACE void ospDeviceSetStatusCallback(OSPDevice, OSPStatusCallback, void *userData);
typedef void (*OSPErrorCallback)(void *userData, OSPError, const char *errorDetails);
OSPRAY_INTERFACE void ospDeviceSetErrorCallback(OSPDevice, OSPErrorCallback, void *userData);
OSPRAY_INTERFACE OSPError ospDeviceGetLastErrorCode(OSPDevice);
OSPRAY_INTERFACE const char *ospDeviceGetLastErrorMsg(OSPDevice);
OSPRAY_INTERFACE void ospDeviceCommit(OSPDevice);
OSPRAY_INTERFACE void ospDeviceRelease(OSPDevice);
OSPRAY_INTERFACE void ospDeviceRetain(OSPDevice);

/* loads libospray_module_<name>.so and calls its ospray_module_init_<name> */
OSPRAY_INTERFACE OSPError ospLoadModule(const char *name);

/* ---- data arrays */
typedef void (*OSPDeleterCallback)(const void *userData, const void *sharedData);
OSPRAY_INTERFACE OSPData ospNewSharedData(const void *sharedData, OSPDataType, uint64_t numItems1,
                                          int64_t byteStride1 OSP_DEFAULT_VAL(0),
                                          uint64_t numItems2 OSP_DEFAULT_VAL(1),
                                          int64_t byteStride2 OSP_DEFAULT_VAL(0),
                                          uint64_t numItems3 OSP_DEFAULT_VAL(1),
                                          int64_t byteStride3 OSP_DEFAULT_VAL(0),
                                          OSPDeleterCallback OSP_DEFAULT_VAL(NULL),
                                          const void *userPtr OSP_DEFAULT_VAL(NULL));
OSPRAY_INTERFACE OSPData ospNewData(OSPDataType, uint64_t numItems1, uint64_t numItems2 OSP_DEFAULT_VAL(1),
                                    uint64_t numItems3 OSP_DEFAULT_VAL(1));
OSPRAY_INTERFACE void ospCopyData(const OSPData source, OSPData destination,
                                  uint64_t destinationIndex1 OSP_DEFAULT_VAL(0),
                                  uint64_t destinationIndex2 OSP_DEFAULT_VAL(0),
                                  uint64_t destinationIndex3 OSP_DEFAULT_VAL(0));

/* ---- scene objects */
OSPRAY_INTERFACE OSPLight ospNewLight(const char *type);
OSPRAY_INTERFACE OSPCamera ospNewCamera(const char *type);
OSPRAY_INTERFACE OSPGeometry ospNewGeometry(const char *type);
OSPRAY_INTERFACE OSPVolume ospNewVolume(const char *type);
OSPRAY_INTERFACE OSPGeometricModel ospNewGeometricModel(OSPGeometry OSP_DEFAULT_VAL(NULL));
OSPRAY_INTERFACE OSPVolumetricModel ospNewVolumetricModel(OSPVolume OSP_DEFAULT_VAL(NULL));
OSPRAY_INTERFACE OSPMaterial ospNewMaterial(const char *materialType);
OSPRAY_INTERFACE OSPTransferFunction ospNewTransferFunction(const char *type);
OSPRAY_INTERFACE OSPTexture ospNewTexture(const char *type);
OSPRAY_INTERFACE OSPGroup ospNewGroup();
OSPRAY_INTERFACE OSPInstance ospNewInstance(OSPGroup OSP_DEFAULT_VAL(NULL));
OSPRAY_INTERFACE OSPWorld ospNewWorld();

typedef struct {
  float lower[3];
  float upper[3];
} OSPBounds;
OSPRAY_INTERFACE OSPBounds ospGetBounds(OSPObject);

/* ---- parameters (staged; take effect at ospCommit) and lifetime */
OSPRAY_INTERFACE void ospSetParam(OSPObject, const char *id, OSPDataType, const void *mem);
OSPRAY_INTERFACE void ospRemoveParam(OSPObject, const char *id);
OSPRAY_INTERFACE void ospCommit(OSPObject);
OSPRAY_INTERFACE void ospRelease(OSPObject);
OSPRAY_INTERFACE void ospRetain(OSPObject);

/* ---- framebuffer */
OSPRAY_INTERFACE OSPFrameBuffer ospNewFrameBuffer(int size_x, int size_y,
                                                  OSPFrameBufferFormat format OSP_DEFAULT_VAL(OSP_FB_SRGBA),
                                                  uint32_t frameBufferChannels OSP_DEFAULT_VAL(OSP_FB_COLOR));
OSPRAY_INTERFACE OSPImageOperation ospNewImageOperation(const char *type);
OSPRAY_INTERFACE const void *ospMapFrameBuffer(OSPFrameBuffer,
                                               OSPFrameBufferChannel OSP_DEFAULT_VAL(OSP_FB_COLOR));
OSPRAY_INTERFACE void ospUnmapFrameBuffer(const void *mapped, OSPFrameBuffer);
OSPRAY_INTERFACE float ospGetVariance(OSPFrameBuffer);
OSPRAY_INTERFACE void ospResetAccumulation(OSPFrameBuffer);

/* ---- rendering */
OSPRAY_INTERFACE OSPRenderer ospNewRenderer(const char *type);
OSPRAY_INTERFACE OSPFuture ospRenderFrame(OSPFrameBuffer, OSPRenderer, OSPCamera, OSPWorld);
OSPRAY_INTERFACE int ospIsReady(OSPFuture, OSPSyncEvent OSP_DEFAULT_VAL(OSP_TASK_FINISHED));
OSPRAY_INTERFACE void ospWait(OSPFuture, OSPSyncEvent OSP_DEFAULT_VAL(OSP_TASK_FINISHED));
OSPRAY_INTERFACE void ospCancel(OSPFuture);
OSPRAY_INTERFACE float ospGetProgress(OSPFuture);
OSPRAY_INTERFACE float ospGetTaskDuration(OSPFuture);

typedef struct {
  int hasHit;
  float worldPosition[3];
  OSPInstance instance;
  OSPGeometricModel model;
  uint32_t primID;
} OSPPickResult;
OSPRAY_INTERFACE void ospPick(OSPPickResult *result, OSPFrameBuffer, OSPRenderer, OSPCamera, OSPWorld,
                              float screenPos_x, float screenPos_y);

#ifdef __cplusplus
}  // extern "C"
#endif
