// b200_render_pt_noalloc: the path tracer for callers that cannot allocate
// device memory.
//
// Some callers of this module may not call cudaMalloc at render time: a host
// application that reserves all device memory up front and hands the module
// only its own buffers, a real-time loop that must not stall on the
// allocator, or a process whose memory is capped by an external pool.
// b200_render_pt grows a path workspace with cudaMalloc on first use; this
// entry point instead uses a fixed scratch array in the module's own static
// device memory (declared below), so the call itself allocates nothing.
//
// The array's address is a device address.  Host code must not pass the
// symbol itself to a kernel (in host code it names a host-side stand-in);
// it asks the runtime for the device address with cudaGetSymbolAddress once
// per device, with that device current, and passes that pointer.
#include <cstring>
#include <mutex>

#include "../../include/b200.h"
#include "api_internal.h"

namespace b200 {

namespace {

// Scratch for one call: microfacet albedo tables, the material list, then
// the path workspace.  Every GPU that loads the library holds it until the
// process exits.
constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(48) << 20;  // 48 MiB
constexpr int NOALLOC_MAX_MATERIALS = 4096;
static __device__ __align__(256) unsigned char g_ptScratch[NOALLOC_SCRATCH_BYTES];

constexpr size_t alignUp(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t OFF_ALBEDO = 0;
constexpr size_t OFF_MATERIALS = alignUp(sizeof(AlbedoTablesD));
constexpr size_t OFF_WORKSPACE = OFF_MATERIALS + alignUp(sizeof(MaterialD) * NOALLOC_MAX_MATERIALS);
constexpr size_t WORKSPACE_BYTES = NOALLOC_SCRATCH_BYTES - OFF_WORKSPACE;

// host staging for the material list (pageable, so an async copy from it has
// left it when the call returns)
MaterialD g_hostMaterials[NOALLOC_MAX_MATERIALS];

struct DeviceScratch {
  unsigned char *base = nullptr;  // device address of g_ptScratch
  bool tablesReady = false;
};
std::mutex g_setupMutex;
DeviceScratch g_scratch[64];

// set-up, once per device, with that device current: look up the array's
// device address and fill the albedo tables in it
int setupDevice(DeviceObj *dev, std::string &err) {
  std::lock_guard<std::mutex> lock(g_setupMutex);
  if (dev->dev < 0 || dev->dev >= 64) {
    err = "device index out of range for the static scratch";
    return B200_INVALID_ARGUMENT;
  }
  DeviceScratch &s = g_scratch[dev->dev];
  if (!s.base) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_ptScratch);
    if (e != cudaSuccess) {
      err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return B200_UNKNOWN_ERROR;
    }
    s.base = static_cast<unsigned char *>(p);
  }
  if (!s.tablesReady) {
    cudaError_t e = computeAlbedoTables(reinterpret_cast<AlbedoTablesD *>(s.base + OFF_ALBEDO), dev->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(dev->stream);
    if (e != cudaSuccess) {
      err = std::string("albedo tables: ") + cudaGetErrorString(e);
      return B200_UNKNOWN_ERROR;
    }
    s.tablesReady = true;
  }
  return B200_NO_ERROR;
}

}  // namespace

long long ptNoallocMaxPaths() {
  // the largest path count whose workspace fits the scratch
  long long lo = 0, hi = 1ll << 32;
  while (lo < hi) {
    const long long mid = (lo + hi + 1) / 2;
    if (ptWorkspaceBytes(mid) <= WORKSPACE_BYTES)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

}  // namespace b200

using namespace b200;

extern "C" {

// Same inputs, outputs and result as b200_render_pt, without allocating.
// Limits: width * height * pixelSamples <= 190,000 paths (the 48 MiB
// scratch less its tables; e.g. 256 x 256 at 2 spp) and nmaterials <= 4096;
// larger requests fail with B200_INVALID_ARGUMENT and say so.
// The first call on a device sets up the static scratch (see b200.h); make
// it before capturing any stream.  All calls share one scratch array and
// keep its last contents: calls that overlap on the GPU (different streams,
// or different host threads, without ordering) race and must not be issued.
// The caller's material array may be reused as soon as the call returns: the
// materials are converted into a static host staging array and copied from
// there (pageable memory, so the copy has left it when the call returns).
int b200_render_pt_noalloc(b200_scene s, const b200_camera_desc *camera, const b200_pt_params *p,
                           const b200_material *materials, int nmaterials, b200_frame f, void *stream) {
  if (!s || !camera || !p || !f) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  FrameObj *fb = reinterpret_cast<FrameObj *>(f);
  DeviceObj *dev = sc->dev;
  auto fail = [&](int code, const std::string &msg) {
    dev->lastError = msg;
    return code;
  };
  try {
    cudaError_t e = cudaSetDevice(dev->dev);
    if (e != cudaSuccess) return fail(B200_UNKNOWN_ERROR, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    if (!sc->committed) return fail(B200_INVALID_OPERATION, "scene not committed");
    if (sc->hasMotion())  // the per-path ray times would need memory of their own
      return fail(B200_INVALID_ARGUMENT, "scenes with motion-blurred instances are rendered by b200_render_pt");
    if (p->pixelSamples < 1 || p->maxPathLength < 0) return fail(B200_INVALID_ARGUMENT, "bad path tracer parameters");
    if (p->pixelFilter < B200_PF_POINT || p->pixelFilter > B200_PF_BLACKMAN_HARRIS)
      return fail(B200_INVALID_ARGUMENT, "bad pixel filter");
    if (nmaterials < 0 || (nmaterials > 0 && !materials)) return fail(B200_INVALID_ARGUMENT, "bad material array");
    if (nmaterials > NOALLOC_MAX_MATERIALS)
      return fail(B200_INVALID_ARGUMENT, "b200_render_pt_noalloc: more than 4096 materials");
    const long long npaths = (long long)fb->W * fb->H * p->pixelSamples;
    const long long maxPaths = ptNoallocMaxPaths();
    if (npaths > maxPaths)
      return fail(B200_INVALID_ARGUMENT, "b200_render_pt_noalloc: width*height*pixelSamples = " +
                                             std::to_string(npaths) + " exceeds the static scratch limit of " +
                                             std::to_string(maxPaths) + " paths");
    std::string err;
    const int rc = setupDevice(dev, err);
    if (rc != B200_NO_ERROR) return fail(rc, err);
    unsigned char *base = g_scratch[dev->dev].base;
    cudaStream_t st = stream ? (cudaStream_t)stream : dev->stream;
    bool transparent = false;
    if (nmaterials > 0) {
      std::lock_guard<std::mutex> lock(g_setupMutex);
      for (int i = 0; i < nmaterials; i++) {
        g_hostMaterials[i] = toMaterialD(materials[i]);
        transparent = transparent || (g_hostMaterials[i].flags & MATF_TRANSPARENT);
      }
      e = cudaMemcpyAsync(base + OFF_MATERIALS, g_hostMaterials, sizeof(MaterialD) * nmaterials,
                          cudaMemcpyHostToDevice, st);
      if (e != cudaSuccess) return fail(B200_UNKNOWN_ERROR, std::string("upload materials: ") + cudaGetErrorString(e));
    }
    const PtParamsD d = makePtParams(*p, sc, materials, nmaterials, transparent);
    fb->beginFrame(p->pixelSamples, st);
    e = launchRenderPT(dev->tables, sc->view(), makeCamera(*camera), dev->filter(p->pixelFilter), d,
                       reinterpret_cast<const MaterialD *>(base + OFF_MATERIALS), sc->dLights, sc->dLightCdf,
                       reinterpret_cast<const AlbedoTablesD *>(base + OFF_ALBEDO), fb->view(), p->collectStats != 0,
                       base + OFF_WORKSPACE, WORKSPACE_BYTES, st);
    if (e != cudaSuccess) return fail(B200_UNKNOWN_ERROR, std::string("path tracer launch: ") + cudaGetErrorString(e));
    fb->frameID++;
    framePostProcess(fb, st);
    return B200_NO_ERROR;
  } catch (const Error &ex) {
    return fail(ex.code, ex.what());
  } catch (const std::bad_alloc &) {
    return fail(B200_OUT_OF_MEMORY, "host out of memory");
  } catch (const std::exception &ex) {
    return fail(B200_UNKNOWN_ERROR, ex.what());
  }
}

}  // extern "C"
