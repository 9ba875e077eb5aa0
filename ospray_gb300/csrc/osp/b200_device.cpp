// libospray_module_b200.so: the "b200" device and its module entry point.
#include "b200_device.h"

#include <cmath>

namespace b200osp {

namespace {

Obj *asObj(const void *h) { return reinterpret_cast<Obj *>(const_cast<void *>(h)); }

template <class T>
T *asKind(const void *h, OSPDataType kind, const char *what) {
  Obj *o = asObj(h);
  if (!o) throw Error(OSP_INVALID_ARGUMENT, std::string(what) + ": null handle");
  if (o->kind != kind) throw Error(OSP_INVALID_ARGUMENT, std::string(what) + ": handle is a " + kindName(o->kind));
  return static_cast<T *>(o);
}

bool known(OSPDataType kind, const std::string &t) {
  switch (kind) {
    case OSP_GEOMETRY: return t == "mesh" || t == "sphere" || t == "box" || t == "plane";
    case OSP_MATERIAL: return t == "principled" || t == "obj" || t == "metal" || t == "glass" || t == "thinGlass";
    case OSP_LIGHT: return t == "quad" || t == "ambient" || t == "distant" || t == "sphere" || t == "spot";
    case OSP_CAMERA: return t == "perspective" || t == "orthographic" || t == "panoramic";
    case OSP_RENDERER: return t == "ao" || t == "pathtracer" || t == "scivis";
    case OSP_VOLUME: return t == "structuredRegular";
    case OSP_TRANSFER_FUNCTION: return t == "piecewiseLinear";
    case OSP_IMAGE_OPERATION: return t == "tonemapper";
    case OSP_TEXTURE: return t == "texture2d";
    default: return false;
  }
}

std::string msgOf(b200_device d) {
  const char *m = b200_device_last_error(d);
  return m && *m ? std::string(m) : std::string("b200 device error");
}

}  // namespace

B200Device::B200Device() = default;

B200Device::~B200Device() {
  if (dev_) b200_device_release(dev_);
}

b200_device B200Device::handle() {
  if (!dev_) throw Error(OSP_INVALID_OPERATION, "the b200 device is not committed");
  return dev_;
}

void B200Device::check(int rc) {
  if (rc != B200_NO_ERROR) throw Error(OSPError(rc), msgOf(dev_));
}

void B200Device::warn(const std::string &msg) {
  if (warnAsError) throw Error(OSP_INVALID_OPERATION, msg);
  status(OSP_LOG_WARNING, "b200 warning: " + msg);
}

// ---------------------------------------------------------------- device

void B200Device::setParam(const char *id, OSPDataType t, const void *mem) { params_.setParam(id, t, mem); }
void B200Device::removeParam(const char *id) { params_.removeParam(id); }

// ISPCDevice::commit (modules/cpu/ISPCDevice.cpp:207-326) and Device::commit
// (ospray/api/Device.cpp:72-120): log level, warn-as-error; plus the CUDA
// device ordinal this device renders on ("cudaDevice", default 0)
void B200Device::commit() {
  logLevel = params_.getInt("logLevel", logLevel);
  warnAsError = params_.getBool("warnAsError", warnAsError);
  params_.getBool("debug", false);
  params_.getInt("numThreads", 0);
  params_.getBool("setAffinity", false);
  const int cd = params_.getInt("cudaDevice", 0);
  if (dev_ && cd != cudaDevice_) {
    b200_device_release(dev_);
    dev_ = nullptr;
  }
  cudaDevice_ = cd;
  if (!dev_) {
    b200_device d = nullptr;
    const int rc = b200_device_create(cudaDevice_, &d);
    if (rc != B200_NO_ERROR) throw Error(OSPError(rc), "b200 device: " + msgOf(nullptr));
    dev_ = d;
  }
}

int64_t B200Device::property(OSPDeviceProperty p) {
  switch (p) {
    case OSP_DEVICE_VERSION:
      return 10000 * ospapi::kVersionMajor + 100 * ospapi::kVersionMinor + ospapi::kVersionPatch;
    case OSP_DEVICE_VERSION_MAJOR: return ospapi::kVersionMajor;
    case OSP_DEVICE_VERSION_MINOR: return ospapi::kVersionMinor;
    case OSP_DEVICE_VERSION_PATCH: return ospapi::kVersionPatch;
    case OSP_DEVICE_SO_VERSION: return ospapi::kVersionMajor;
  }
  throw Error(OSP_INVALID_ARGUMENT, "unknown device property");
}

// ---------------------------------------------------------------- data

OSPData B200Device::newSharedData(const void *shared, OSPDataType t, uint64_t n1, int64_t s1, uint64_t n2, int64_t s2,
                                  uint64_t n3, int64_t s3, OSPDeleterCallback del, const void *user) {
  return reinterpret_cast<OSPData>(new DataObj(t, shared, n1, s1, n2, s2, n3, s3, del, user));
}

OSPData B200Device::newData(OSPDataType t, uint64_t n1, uint64_t n2, uint64_t n3) {
  return reinterpret_cast<OSPData>(new DataObj(t, n1, n2, n3));
}

void B200Device::copyData(OSPData src, OSPData dst, uint64_t i1, uint64_t i2, uint64_t i3) {
  asKind<DataObj>(dst, OSP_DATA, "ospCopyData destination")
      ->copyFrom(*asKind<DataObj>(src, OSP_DATA, "ospCopyData source"), i1, i2, i3);
}

// ---------------------------------------------------------------- objects

OSPObject B200Device::newObject(OSPDataType kind, const char *type) {
  const std::string t(type);
  if (!known(kind, t))
    throw Error(OSP_INVALID_ARGUMENT, std::string("the b200 device has no ") + kindName(kind) + " type '" + t + "'");
  SceneObj *o = nullptr;
  switch (kind) {
    case OSP_GEOMETRY: o = new GeometryObj(kind, t); break;
    case OSP_MATERIAL: o = new MaterialObj(kind, t); break;
    case OSP_LIGHT: o = new LightObj(kind, t); break;
    case OSP_CAMERA: o = new CameraObj(kind, t); break;
    case OSP_RENDERER: o = new RendererObj(kind, t); break;
    case OSP_VOLUME: o = new VolumeObj(kind, t); break;
    case OSP_TRANSFER_FUNCTION: o = new TransferFunctionObj(kind, t); break;
    case OSP_IMAGE_OPERATION: o = new ImageOpObj(kind, t); break;
    case OSP_TEXTURE: o = new TextureObj(kind, t); break;
    default: break;
  }
  return reinterpret_cast<OSPObject>(static_cast<Obj *>(o));
}

OSPGeometricModel B200Device::newGeometricModel(OSPGeometry g) {
  auto *m = new GeometricModelObj(OSP_GEOMETRIC_MODEL, "geometricModel");
  if (g) {
    Obj *go = asKind<Obj>(g, OSP_GEOMETRY, "ospNewGeometricModel");
    m->setParam("geometry", OSP_GEOMETRY, &go);
  }
  return reinterpret_cast<OSPGeometricModel>(static_cast<Obj *>(m));
}

OSPVolumetricModel B200Device::newVolumetricModel(OSPVolume v) {
  auto *m = new VolumetricModelObj(OSP_VOLUMETRIC_MODEL, "volumetricModel");
  if (v) {
    Obj *vo = asKind<Obj>(v, OSP_VOLUME, "ospNewVolumetricModel");
    m->setParam("volume", OSP_VOLUME, &vo);
  }
  return reinterpret_cast<OSPVolumetricModel>(static_cast<Obj *>(m));
}

OSPGroup B200Device::newGroup() {
  return reinterpret_cast<OSPGroup>(static_cast<Obj *>(new GroupObj(OSP_GROUP, "group")));
}

OSPInstance B200Device::newInstance(OSPGroup g) {
  auto *i = new InstanceObj(OSP_INSTANCE, "instance");
  if (g) {
    Obj *go = asKind<Obj>(g, OSP_GROUP, "ospNewInstance");
    i->setParam("group", OSP_GROUP, &go);
  }
  return reinterpret_cast<OSPInstance>(static_cast<Obj *>(i));
}

OSPWorld B200Device::newWorld() {
  return reinterpret_cast<OSPWorld>(static_cast<Obj *>(new WorldObj(OSP_WORLD, "world")));
}

OSPFrameBuffer B200Device::newFrameBuffer(int w, int h, OSPFrameBufferFormat fmt, uint32_t ch) {
  if (w <= 0 || h <= 0) throw Error(OSP_INVALID_ARGUMENT, "framebuffer size must be positive");
  auto *f = new FrameBufferObj(*this, w, h, fmt, ch);
  return reinterpret_cast<OSPFrameBuffer>(static_cast<Obj *>(f));
}

OSPBounds B200Device::bounds(OSPObject o) {
  OSPBounds b = {{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
  Obj *obj = asObj(o);
  if (obj->kind == OSP_WORLD) {
    WorldObj *w = static_cast<WorldObj *>(obj);
    if (!w->scene) throw Error(OSP_INVALID_OPERATION, "ospGetBounds: world not committed");
    float box[6];
    check(b200_scene_bounds(w->scene, box));
    std::memcpy(b.lower, box, 12);
    std::memcpy(b.upper, box + 3, 12);
  } else if (obj->kind == OSP_GEOMETRY) {
    static_cast<GeometryObj *>(obj)->bounds(b.lower, b.upper);
  } else {
    throw Error(OSP_INVALID_ARGUMENT, std::string("ospGetBounds: not supported for a ") + kindName(obj->kind));
  }
  return b;
}

void B200Device::setObjectParam(OSPObject o, const char *id, OSPDataType t, const void *mem) {
  asObj(o)->setParam(id, t, mem);
}

void B200Device::removeObjectParam(OSPObject o, const char *id) { asObj(o)->removeParam(id); }

void B200Device::commitObject(OSPObject o) {
  Obj *obj = asObj(o);
  if (obj->kind == OSP_DATA) return;  // data arrays are read at their holder's commit
  if (obj->kind == OSP_FUTURE) throw Error(OSP_INVALID_ARGUMENT, "ospCommit on a future");
  obj->resetUsed();
  static_cast<SceneObj *>(obj)->commit(*this);
  obj->committed = true;
  for (const std::string &p : obj->unusedParams())
    status(OSP_LOG_WARNING, std::string("b200 warning: ") + kindName(obj->kind) + " '" + obj->type +
                                "': parameter '" + p + "' is not used by the b200 device");
}

void B200Device::release(OSPObject o) { asObj(o)->release(); }
void B200Device::retain(OSPObject o) { asObj(o)->retain(); }

// ---------------------------------------------------------------- framebuffer

// LocalFrameBuffer::mapBuffer (fb/LocalFB.cpp:487-524): a host copy of the
// channel, valid until ospUnmapFrameBuffer; waits for the frames in flight
const void *B200Device::mapFrameBuffer(OSPFrameBuffer h, OSPFrameBufferChannel ch) {
  FrameBufferObj *f = asKind<FrameBufferObj>(h, OSP_FRAMEBUFFER, "ospMapFrameBuffer");
  if (ch == OSP_FB_COLOR && f->format == OSP_FB_NONE) return nullptr;
  if (!(f->channels & ch) && ch != OSP_FB_COLOR) return nullptr;
  const size_t bytes = b200_frame_channel_bytes(f->fb, uint32_t(ch));
  if (!bytes) return nullptr;
  // the frame's page-locked buffer for the channel, unless it is mapped already
  bool inUse = false;
  for (const auto &m : f->pinnedMapped) inUse = inUse || m.second == uint32_t(ch);
  if (!inUse) {
    const void *p = nullptr;
    check(b200_frame_map(f->fb, uint32_t(ch), &p));
    f->pinnedMapped[p] = uint32_t(ch);
    f->retain();
    return p;
  }
  std::vector<unsigned char> buf(bytes);
  check(b200_frame_read(f->fb, uint32_t(ch), buf.data(), bytes));
  const void *p = buf.data();
  f->mapped[p] = std::move(buf);
  f->retain();
  return p;
}

void B200Device::unmapFrameBuffer(const void *mapped, OSPFrameBuffer h) {
  FrameBufferObj *f = asKind<FrameBufferObj>(h, OSP_FRAMEBUFFER, "ospUnmapFrameBuffer");
  auto pt = f->pinnedMapped.find(mapped);
  if (pt != f->pinnedMapped.end()) {
    f->pinnedMapped.erase(pt);
    f->release();
    return;
  }
  auto it = f->mapped.find(mapped);
  if (it == f->mapped.end()) throw Error(OSP_INVALID_ARGUMENT, "ospUnmapFrameBuffer: pointer was not mapped");
  f->mapped.erase(it);
  f->release();
}

// LocalFrameBuffer::getVariance (fb/LocalFB.cpp:263-272): the task error
// estimate against the last renderer's varianceThreshold; inf without a
// VARIANCE channel or before the first odd frame
float B200Device::variance(OSPFrameBuffer h) {
  FrameBufferObj *f = asKind<FrameBufferObj>(h, OSP_FRAMEBUFFER, "ospGetVariance");
  float v = INFINITY;
  check(b200_frame_variance(f->fb, f->errorThreshold, &v));
  return v;
}

void B200Device::resetAccumulation(OSPFrameBuffer h) {
  check(b200_frame_reset(asKind<FrameBufferObj>(h, OSP_FRAMEBUFFER, "ospResetAccumulation")->fb));
}

// ---------------------------------------------------------------- rendering

// ISPCDevice::renderFrame (modules/cpu/ISPCDevice.cpp:578-595): renders
// asynchronously on the device stream; the future holds the objects the
// frame reads until it is released
OSPFuture B200Device::renderFrame(OSPFrameBuffer hf, OSPRenderer hr, OSPCamera hc, OSPWorld hw) {
  FrameBufferObj *f = asKind<FrameBufferObj>(hf, OSP_FRAMEBUFFER, "ospRenderFrame framebuffer");
  RendererObj *r = asKind<RendererObj>(hr, OSP_RENDERER, "ospRenderFrame renderer");
  CameraObj *c = asKind<CameraObj>(hc, OSP_CAMERA, "ospRenderFrame camera");
  WorldObj *w = asKind<WorldObj>(hw, OSP_WORLD, "ospRenderFrame world");
  if (!r->committed || !c->committed || !w->committed || !w->scene)
    throw Error(OSP_INVALID_OPERATION, "ospRenderFrame: renderer, camera and world must be committed");
  auto *fut = new FutureObj();
  try {
    // LocalTiledLoadBalancer::renderFrame (render/LoadBalancer.cpp:15-30):
    // the renderer's varianceThreshold selects the tasks of this frame
    check(b200_frame_set_variance_threshold(f->fb, r->varianceThreshold));
    check(b200_event_record(dev_, &fut->start));
    // texture handles as of now (a texture committed again since has a new one)
    b200_texture bp = r->backplate ? r->backplate->tex : nullptr, md = r->maxDepth ? r->maxDepth->tex : nullptr;
    if (r->type == "ao") {
      std::vector<b200_scivis_material> mats;
      for (const auto *list : {&w->objectMaterials, &r->materials})
        for (const auto &m : *list) mats.push_back(m->scivis());
      b200_ao_params ao = r->ao;
      ao.backplate = bp;
      ao.maxDepth = md;
      ao.mipMapBias = r->mipMapBias;
      ao.materials = mats.data();
      ao.nmaterials = int(mats.size());
      check(b200_render_ao(w->scene, &c->desc, &ao, f->fb, nullptr));
    } else if (r->type == "pathtracer") {
      if (w->hasVolume) warn("pathtracer: volumes are not rendered by the b200 device");
      std::vector<b200_material> mats;
      // texture handles as of now (a texture committed again since has a new one)
      for (const auto *list : {&w->objectMaterials, &r->materials})
        for (const auto &m : *list) {
          mats.push_back(m->mat);
          mats.back().baseColorMap = m->colorMapHandle();
        }
      b200_pt_params pt = r->pt;
      pt.backplate = bp;
      pt.maxDepth = md;
      check(b200_render_pt(w->scene, &c->desc, &pt, mats.data(), int(mats.size()), f->fb, nullptr));
    } else {
      if (!w->hasGeometry && !w->hasVolume)
        throw Error(OSP_INVALID_OPERATION, "scivis renderer: the world has no geometry and no volume");
      std::vector<b200_scivis_material> mats;
      for (const auto *list : {&w->objectMaterials, &r->materials})
        for (const auto &m : *list) mats.push_back(m->scivis());
      b200_scivis_params sv = r->scivis;
      sv.backplate = bp;
      sv.maxDepth = md;
      sv.mipMapBias = r->mipMapBias;
      check(b200_render_scivis(w->scene, &c->desc, &sv, mats.data(), int(mats.size()), f->fb, nullptr));
    }
    check(b200_event_record(dev_, &fut->end));
  } catch (...) {
    fut->release();
    throw;
  }
  f->errorThreshold = r->varianceThreshold;
  for (Obj *o : {static_cast<Obj *>(f), static_cast<Obj *>(r), static_cast<Obj *>(c), static_cast<Obj *>(w)}) {
    o->retain();
    fut->held.push_back(o);
  }
  return reinterpret_cast<OSPFuture>(static_cast<Obj *>(fut));
}

// all sync events of a frame are reached together when its end event is
int B200Device::isReady(OSPFuture h, OSPSyncEvent) {
  FutureObj *f = asKind<FutureObj>(h, OSP_FUTURE, "ospIsReady");
  const int q = b200_event_query(f->end);
  if (q < 0) throw Error(OSP_UNKNOWN_ERROR, msgOf(dev_));
  return q;
}

void B200Device::wait(OSPFuture h, OSPSyncEvent) {
  check(b200_event_wait(asKind<FutureObj>(h, OSP_FUTURE, "ospWait")->end));
}

// frames are short GPU launches; cancellation is cooperative in the
// reference too (FrameBuffer.cpp:180-186) and here a no-op
void B200Device::cancel(OSPFuture h) { asKind<FutureObj>(h, OSP_FUTURE, "ospCancel"); }

float B200Device::progress(OSPFuture h) { return isReady(h, OSP_TASK_FINISHED) ? 1.f : 0.f; }

float B200Device::taskDuration(OSPFuture h) {
  FutureObj *f = asKind<FutureObj>(h, OSP_FUTURE, "ospGetTaskDuration");
  check(b200_event_wait(f->end));
  return b200_event_elapsed_ms(f->start, f->end) * 1e-3f;
}

// Renderer::pick (render/Renderer.cpp:94-140): the hit's instance and
// geometric model are returned as retained handles
void B200Device::pick(OSPPickResult *res, OSPFrameBuffer, OSPRenderer, OSPCamera hc, OSPWorld hw, float x,
                      float y) {
  CameraObj *c = asKind<CameraObj>(hc, OSP_CAMERA, "ospPick camera");
  WorldObj *w = asKind<WorldObj>(hw, OSP_WORLD, "ospPick world");
  if (!w->scene) throw Error(OSP_INVALID_OPERATION, "ospPick: world not committed");
  b200_pick_result p;
  check(b200_pick(w->scene, &c->desc, x, y, &p));
  if (!p.hasHit || p.instID >= w->instances.size()) return;
  InstanceObj *inst = w->instances[p.instID].get();
  if (p.geomID >= inst->group->models.size()) return;
  GeometricModelObj *model = inst->group->models[p.geomID].get();
  inst->retain();
  model->retain();
  res->hasHit = 1;
  std::memcpy(res->worldPosition, p.worldPosition, 12);
  res->instance = reinterpret_cast<OSPInstance>(static_cast<Obj *>(inst));
  res->model = reinterpret_cast<OSPGeometricModel>(static_cast<Obj *>(model));
  res->primID = p.primID;
}

}  // namespace b200osp

namespace {
ospapi::Device *makeB200Device() { return new b200osp::B200Device(); }
}  // namespace

// Module entry point, called by ospLoadModule("b200") (ospray/common/
// OSPCommon.cpp:749-782): checks the API version like moduleVersionCheck
// and registers the "b200" device type (modules/cpu/ModuleInit.cpp:24-54).
extern "C" __attribute__((visibility("default"))) OSPError ospray_module_init_b200(int16_t major, int16_t minor,
                                                                                    int16_t patch) {
  (void)patch;
  if (major != ospapi::kVersionMajor || minor > ospapi::kVersionMinor) return OSP_VERSION_MISMATCH;
  ospray_register_device_type("b200", &makeB200Device);
  return OSP_NO_ERROR;
}
