// Host objects behind the b200 C ABI handles.
#pragma once
#include <stdexcept>
#include <string>
#include <random>
#include <vector>

#include "../../include/b200.h"
#include "bvh.h"
#include "kernels.h"

namespace b200 {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

void check(cudaError_t e, const char *what);

struct FilterLUT {
  float width = 0.f;
  int lutW = 0;
  float *cdf_x = nullptr, *cdf_y = nullptr;
};

// Handles are reference counted like OSPRay objects (ospRetain/ospRelease):
// b200_device_release drops the creator's reference, and every scene and
// framebuffer holds one on its device, so a device outlives its objects.
struct DeviceObj {
  int refs = 1;
  void retain() { __atomic_add_fetch(&refs, 1, __ATOMIC_ACQ_REL); }
  void release() {
    if (__atomic_sub_fetch(&refs, 1, __ATOMIC_ACQ_REL) == 0) delete this;
  }
  int dev;
  cudaStream_t stream = nullptr;
  std::string lastError;
  SamplerTables *tables = nullptr;
  FilterLUT luts[5];
  AlbedoTablesD *albedo = nullptr;  // computed at the first path-traced frame
  unsigned int *work = nullptr;     // pixel work counter of the persistent renderers
  uint32_t *pickBuf = nullptr;      // one pick result (8 words)
  void *ptWs = nullptr;             // path-tracer path/queue workspace
  size_t ptWsBytes = 0;
  float *ptTimes = nullptr;         // per-path ray times (frames with motion-blurred instances)
  size_t ptTimesCap = 0;
  KernelTimer *timer = nullptr;     // live kernel timing (b200_kernel_timing)
  explicit DeviceObj(int cudaDev);
  const AlbedoTablesD *albedoTables();
  ~DeviceObj();
  PixelFilterD filter(int type) const;
};

struct GeomObj {
  int type = GEOM_TRIANGLES;
  int64_t nprims = 0;  // BLAS primitives (a quad mesh: two triangles per quad)
  float *dverts = nullptr;
  uint32_t *dindex = nullptr;  // 3 per BLAS triangle
  uint32_t *dquad = nullptr;   // quad meshes: the 4 indices per quad (postIntersect)
  uint32_t meshKind = MESH_TRIANGLES;
  int64_t nverts = 0;
  float *dnormals = nullptr, *dcolors = nullptr, *dtexcoords = nullptr;  // per-vertex attributes
  bool colorAlpha = false;  // some vertex colour has alpha != 1
  float4 *dsph = nullptr;   // spheres, discs: (centre, radius) per primitive
  float4 *duser = nullptr;  // oriented discs, planes: primStride(type) float4 per primitive
  BLAS blas;
  bool built = false;
};

struct EntryH {
  int geom;
  uint32_t instID, geomID;
  bool identity;
  float xfm[12];
  int material;
  std::vector<float> motion;  // motion blur: >= 2 row-major 3x4 keys (else empty)
  float t0 = 0.f, t1 = 1.f;   // the keys' time range
};

struct SceneObj {
  DeviceObj *dev;
  std::vector<GeomObj> geoms;
  std::vector<EntryH> entries;
  Entry *dEntries = nullptr;
  WideBVH tlas;
  uint32_t *status = nullptr;
  unsigned long long *counters = nullptr;  // traversal statistics (render stats mode)
  bool committed = false;
  bool dynamic = false;  // LBVH-only builds (fast build, lower quality)
  float bounds[6] = {0, 0, 0, 0, 0, 0};
  // path-tracer state: world lights and the renderer's material list
  LightD *dLights = nullptr;
  float *dLightCdf = nullptr;
  int nLights = 0;
  MaterialD *dMaterials = nullptr;
  int nMaterials = 0, capMaterials = 0;
  // SciVis state: the lights in SciVisData order, the summed ambient radiance
  // and the renderer's material list
  LightD *dScivisLights = nullptr;
  int numVisibleOnly = 0;
  V3 aoColor = {0.f, 0.f, 0.f};
  ScivisMatD *dScivisMats = nullptr;
  int capScivisMats = 0;
  std::vector<ScivisMatD> lastScivisMats;  // the device records last uploaded
  // the AO renderer's surface-colour materials (b200_ao_params.materials)
  ScivisMatD *dAoMats = nullptr;
  int capAoMats = 0;
  std::vector<ScivisMatD> lastAoMats;
  // one structured-regular volumetric model (device copies)
  bool hasVolume = false;
  VolumeD vol = {};
  float gradientShadingScale = 0.f;  // kept across b200_scene_set_volume calls
  bool volIdentity = true;           // the volume's instance transform (kept likewise)
  Xfm volRcp = {};
  float *dVolData = nullptr, *dTfOpacity = nullptr;
  float3 *dTfColor = nullptr;
  uint8_t *dCellEmpty = nullptr;
  std::vector<MaterialD> lastMaterials;  // the device records last uploaded
  bool transparentMaterials = false;  // some material of lastMaterials lets shadow rays through
  // set at commit: some mesh has vertex attributes; some vertex colour has alpha < 1
  bool hasAttributes = false, colorAlpha = false;
  float *dMotion = nullptr;  // every motion-blurred entry's keys
  bool hasMotion() const {
    for (const EntryH &e : entries)
      if (!e.motion.empty()) return true;
    return false;
  }
  explicit SceneObj(DeviceObj *d);
  ~SceneObj();
  void commit();
  Scene view() const;
};

struct FrameObj {
  DeviceObj *dev;
  int W, H;
  int format;  // B200_FB_NONE / RGBA8 / SRGBA / RGBA32F
  uint32_t channels;
  int frameID = 0;
  void *mapped = nullptr;  // converted colour (what ospMapFrameBuffer returns)
  std::vector<std::pair<uint32_t, std::pair<void *, size_t>>> hostMaps;  // b200_frame_map: channel -> pinned buffer
  bool toneMapOn = false;
  ToneMapD toneMap = {};
  float4 *color = nullptr, *variance = nullptr;
  float *depth = nullptr;
  float3 *normal = nullptr, *albedo = nullptr;
  float *aux = nullptr;  // NORMAL or ALBEDO: the path tracer's per-pixel sums of a frame (6 floats)
  uint32_t *primID = nullptr, *geomID = nullptr, *instID = nullptr;
  // per 8x8 render task: the variance estimate of the last odd frame
  // (Variance_kernel, fb/frame_ops/Variance.ispc:11-49); valid once computed
  static constexpr int TASK = 8;
  float *taskErr = nullptr;
  bool taskErrValid = false;
  // Adaptive accumulation (the renderer's varianceThreshold,
  // render/Renderer.cpp:44; LocalFrameBuffer::getRenderTaskIDs
  // fb/LocalFB.cpp:238-260): once frameID >= max(2, 16 / spp), only the
  // tasks whose error exceeds the threshold are rendered.
  float errorThreshold = 0.f;
  uint8_t *taskActive = nullptr;  // per task, written on the device each frame
  bool adaptive = false;          // this frame renders the selected tasks only
  // FrameBuffer::beginFrame (fb/FrameBuffer.cpp:121-136): of each even/odd
  // frame pair one, picked by a coin flip of std::mt19937 seeded 43, goes into
  // the variance buffer
  std::mt19937 mtGen{43u};
  bool pickOdd = false, accumVariance = false;
  // called by every render entry point before its launch, for the frame
  // frameID about to be rendered with spp samples per pixel
  void beginFrame(int spp, cudaStream_t st);
  int tasksX() const { return (W + TASK - 1) / TASK; }
  int tasksY() const { return (H + TASK - 1) / TASK; }
  FrameObj(DeviceObj *d, int w, int h, int format, uint32_t ch);
  ~FrameObj();
  FrameD view() const;
  void *channel(uint32_t c) const;
  size_t channelBytes(uint32_t c) const;
};

CameraD makeCamera(const b200_camera_desc &c);
PtParamsD makePtParams(const b200_pt_params &p, const SceneObj *sc, const b200_material *materials, int nmaterials,
                       bool transparentMaterials);
// b200_material -> device record (throws Error on an unknown type)
MaterialD toMaterialD(const b200_material &m);
bool anyTransparent(const b200_material *materials, int n);
// the device descriptor of a texture (null for null)
const TextureD *textureDevice(b200_texture t);
bool textureHasAlpha(b200_texture t);
bool anyNonPrincipled(const b200_material *materials, int n);
void uploadMaterials(SceneObj *sc, const b200_material *materials, int nmaterials);
// b200_scivis_material -> device records (SciVis surfaces, AO surface colours)
std::vector<ScivisMatD> toScivisMats(const b200_scivis_material *materials, int n);
void ensurePtWorkspace(DeviceObj *dev, size_t need);
AOParamsD makeAOParams(const b200_ao_params &p);
ToneMapD makeToneMap(const b200_tonemapper &u);
// tonemap (if set) + conversion of the accumulated colour into fb->mapped,
// enqueued after every render (LocalFrameBuffer::postProcess)
void framePostProcess(FrameObj *fb, cudaStream_t st, bool variance = true);

}  // namespace b200
