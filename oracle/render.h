// Oracle (test infrastructure only): camera, pixel filter, screen samples,
// differential geometry and framebuffer accumulation shared by the CPU
// renderers.
//   camera:  modules/cpu/camera/PerspectiveCamera.cpp:30-117, .ispc:16-64,
//            modules/cpu/camera/Camera.cpp:38-52
//   filter:  modules/cpu/pf/PixelFilter.cpp:28-55, LUTPixelFilter.ispc:60-144,
//            PixelFilter.ih:20-30, math/Distribution1D.ispc, Distribution2D.ispc
//   pixel:   modules/cpu/render/RendererRenderTaskFn.inl:5-88, ScreenSample.ih
//   dg:      modules/cpu/common/World.ih:389-465, Instance.ih:44-107,
//            geometry/GeometricModel.ih:47-76, Mesh.ispc:30-33,178+,
//            Spheres.ispc:24-42, common/DifferentialGeometry.ih:46-58
//   fb:      modules/cpu/fb/LocalFB.ispc:14-78, FrameBuffer.ih:21-22
#pragma once
#include <atomic>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

#include "samplers.h"
#include "scene.h"
#include "texture.h"

namespace orc {

// type 0 perspective (dir_00, du_size, dv_up as PerspectiveCamera), 1
// orthographic (org = lower-left corner, dir_00 = the view direction), 2
// panoramic (org, frame vx, vy, vz in du_size, dv_up, dir_00)
struct Camera {
  V3 org, dir_00, du_size, dv_up;
  float nearClip;
  int type = 0;
  // the shutter after Camera::commit (camera/Camera.cpp:44-52,100-119):
  // mode 0 global, 1 rolling along screen x, 2 along screen y
  float shutterLo = 0.5f, shutterHi = 0.5f, rollingDuration = 0.f;
  int shutterMode = 0;
  bool needTime = false;
  // perspective depth of field (PerspectiveCamera::commit): lens radius over
  // the image plane (0: pinhole), aspect, image-plane height
  float scaledAperture = 0.f, aspect = 1.f, imgPlaneY = 1.f;
  // the sub-image (Camera::commit camera/Camera.cpp:42-43,108-109) and
  // stereo: split 0 none, 1 side by side, 2 top / bottom; monoEye the fixed
  // eye of a panoramic left / right camera; ipdOffset half the
  // interpupillary distance (perspective: along the film's x axis;
  // panoramic: x); coneScale |imageEnd.y - imageStart.y|, x2 top / bottom
  V2 subLo = {0.f, 0.f}, subHi = {1.f, 1.f};
  int split = 0;
  float monoEye = 0.f;
  V3 ipdOffset = {0.f, 0.f, 0.f};
  float coneScale = 1.f;
};

// imageStart / imageEnd (all zero: the whole image) with the cone scale of
// the stereo mode
void setSubImage(Camera &c, const float lo[2], const float hi[2], int stereoMode);

// The stereo split and Camera_subRegion (PerspectiveCamera.ispc:28-41,
// PanoramicCamera.ispc:24-45, Camera.ih:28-31): maps `screen` of a sample of
// the pixel centred at `center` in place and returns its eye (-1 left, +1
// right, 0 mono)
inline float cameraScreen(const Camera &c, V2 &screen, V2 center) {
  float eye = c.monoEye;
  if (c.split) {
    float &s = c.split == 1 ? screen.x : screen.y;
    s = s * 2.f;
    if ((c.split == 1 ? center.x : center.y) < 0.5f) {
      eye = -1.f;
    } else {
      eye = 1.f;
      s = s - 1.f;
    }
  }
  screen.x = (1.f - screen.x) * c.subLo.x + screen.x * c.subHi.x;
  screen.y = (1.f - screen.y) * c.subLo.y + screen.y * c.subHi.y;
  return eye;
}

// Camera::commit's shutter from the "shutter", "shutterType" and
// "rollingShutterDuration" parameters
void setShutter(Camera &c, float lower, float upper, int type, float duration);

// Camera_shutterTime (camera/Camera.ih:33-42); rkcommon lerp(f, a, b) = (1 - f) a + f b
inline float shutterTime(const Camera &c, V2 screen, float time) {
  if (c.shutterMode == 0) return (1.f - time) * c.shutterLo + time * c.shutterHi;
  const float t = time * c.rollingDuration;
  const float pos = c.shutterMode == 1 ? screen.x : screen.y;
  const float v = t + ((1.f - pos) * c.shutterLo + pos * c.shutterHi);
  return std::fmin(std::fmax(v, 0.f), 1.f);
}

// PerspectiveCamera::commit (camera/PerspectiveCamera.cpp:30-117),
// OrthographicCamera::commit (camera/OrthographicCamera.cpp:25-50) and
// PanoramicCamera::commit (camera/PanoramicCamera.cpp:30-47), without stereo,
// aperture or motion blur
Camera makeCamera(V3 pos, V3 dir, V3 up, float fovy, float aspect, float nearClip, int type = 0,
                  float height = 1.f, float apertureRadius = 0.f, float focusDistance = 1.f,
                  bool architectural = false, int stereoMode = 0, float interpupillaryDistance = 0.0635f);

// lens: the lens sample (PerspectiveCamera.ispc:44-52: uniformSampleDisk);
// screen: the mapped position (cameraScreen), eye its eye
inline Ray cameraRay(const Camera &c, V2 screen, V2 lens = {0.f, 0.f}, float eye = 0.f) {
  if (c.type == 1)  // OrthographicCamera_initRay (camera/OrthographicCamera.ispc:11-49)
    return {c.org + screen.x * c.du_size + screen.y * c.dv_up, c.nearClip, c.dir_00, INFINITY};
  if (c.type == 2) {  // PanoramicCamera_initRay (camera/PanoramicCamera.ispc:12-90), mono
    const float phi = 6.28318530717958647692f * screen.x, theta = 3.14159265358979323846f * screen.y;
    const float st = std::sin(theta), ct = std::cos(theta);
    const V3 l = {std::cos(phi) * st, std::sin(phi) * st, ct};
    const V3 d = c.du_size * -l.y + c.dv_up * -l.z + c.dir_00 * l.x;
    const V3 org = eye != 0.f ? c.org + (eye * c.ipdOffset.x) * cross(d, c.dv_up) : c.org;
    return {org, c.nearClip, d, INFINITY};
  }
  V3 d = c.dir_00 + screen.x * c.du_size + screen.y * c.dv_up;
  V3 org = eye < 0.f ? c.org - c.ipdOffset : eye > 0.f ? c.org + c.ipdOffset : c.org;
  if (c.scaledAperture > 0.f) {
    const float r = std::sqrt(lens.x) * c.scaledAperture, phi = 6.28318530717958647692f * lens.y;
    const V3 lp = (r * std::cos(phi)) * c.du_size + ((r * std::sin(phi)) * c.aspect) * c.dv_up;
    org = org + lp;
    d = d - lp;
  }
  return {org, c.nearClip, normalize(d), INFINITY};
}

// The camera ray's cone at `screen`, in units of the frame height (x: width,
// y: dwdt): perspective 0 wide, widening by the image plane height x
// rsqrt(|unnormalised direction|^2) (PerspectiveCamera.ispc:58-63);
// orthographic as wide as the image height, parallel
// (OrthographicCamera.ispc:52-53); panoramic pi sin(theta)
// (PanoramicCamera.ispc:86-90); all times 1 / height (PathTracer.ispc:186-187)
// (scaled by coneScale; screen: the mapped position)
inline V2 cameraCone(const Camera &c, V2 screen, float rcpH) {
  if (c.type == 1) return {length(c.dv_up) * c.coneScale * rcpH, 0.f};
  if (c.type == 2)
    return {0.f, 3.14159265358979323846f * std::sin(3.14159265358979323846f * screen.y) * c.coneScale * rcpH};
  const V3 d = c.dir_00 + screen.x * c.du_size + screen.y * c.dv_up;
  return {0.f, c.imgPlaneY * c.coneScale * (1.f / std::sqrt(dot(d, d))) * rcpH};
}

enum PixelFilterType { PF_POINT = 0, PF_BOX = 1, PF_GAUSS = 2, PF_MITCHELL = 3, PF_BLACKMAN_HARRIS = 4 };

struct PixelFilter {
  int type = PF_GAUSS;
  float width = 3.f;
  int lutW = 15;
  std::vector<float> cdf_x, cdf_y;
  void init(int t);
  V2 sample(V2 s) const;
};

struct DG {
  V3 P, Ng, Ns;
  V3 dPds;  // DG_TANGENTS: a mesh's first edge (Mesh.ispc:172-175), else (1, 0, 0); world space
  float epsilon;
  uint32_t primID, geomID, instID;
  // with attrs: DG_COLOR (1 without vertex colours), DG_TEXCOORD (the hit's
  // u, v without texture coordinates) and the second tangent dPdt
  V4 color = {1.f, 1.f, 1.f, 1.f};
  V2 st = {0.f, 0.f};
  V3 dPdt = {0.f, 1.f, 0.f};
};

// postIntersect with DG_NG | DG_NS | DG_NORMALIZE | DG_FACEFORWARD; attrs
// adds the triangle mesh's vertex normals, colours and texture coordinates
// (TriangleMesh_postIntersect geometry/Mesh.ispc:178-276, QuadMesh's default
// tangents :171-174, World.ih:397-407 defaults)
DG postIntersect(const Scene &s, const Ray &ray, const Hit &hit, bool attrs = false);

// World.ih:458-464: the ray cone's width projected onto the surface, in
// texture space, times the renderer's mipBiasFactor
inline float pixelFootprint(float coneWidth, V3 rayDir, const DG &dg, float mipBiasFactor) {
  const float texArea = length(cross(dg.dPds, dg.dPdt));
  return coneWidth / -dot(rayDir, dg.Ng) * (1.f / std::sqrt(texArea)) * mipBiasFactor;
}

struct FrameBuffer {
  int W = 0, H = 0;
  int frameID = 0;
  std::vector<float> color;  // RGBA
  std::vector<float> depth;
  std::vector<uint32_t> primID, geomID, instID;
  std::vector<float> normal, albedo;  // 3 per pixel
  void resize(int w, int h) {
    W = w;
    H = h;
    color.assign(size_t(W) * H * 4, 0.f);
    normal.assign(size_t(W) * H * 3, 0.f);
    albedo.assign(size_t(W) * H * 3, 0.f);
    depth.assign(size_t(W) * H, INFINITY);
    primID.assign(size_t(W) * H, INVALID_ID);
    geomID.assign(size_t(W) * H, INVALID_ID);
    instID.assign(size_t(W) * H, INVALID_ID);
    frameID = 0;
  }
};

struct ScreenSample {
  V3 rgb = v3(0.f);
  float alpha = 0.f;
  float z = INFINITY;
  uint32_t primID = INVALID_ID, geomID = INVALID_ID, instID = INVALID_ID;
  V3 normal = v3(0.f), albedo = v3(0.f);  // auxiliary channels (ScreenSample.ih)
};

inline void accumulateScreen(ScreenSample &acc, const ScreenSample &s) {
  acc.rgb = acc.rgb + s.rgb;
  acc.alpha += s.alpha;
  acc.normal = acc.normal + s.normal;
  acc.albedo = acc.albedo + s.albedo;
  if (std::fabs(s.z) < std::fabs(acc.z)) {
    acc.z = s.z;
    acc.primID = s.primID;
    acc.geomID = s.geomID;
    acc.instID = s.instID;
  }
}

// LocalFB_accumulateSample: lerp accumulation, ID buffers from the closest |z|
void fbAccumulate(FrameBuffer &fb, int x, int y, const ScreenSample &s);

// where the renderers copy the accumulated normal / albedo channels after a
// call (null: not wanted); set by or_set_aux_output
extern float *g_auxNormal, *g_auxAlbedo;

// the AO renderer's volume (or_set_ao_volume): integrateVolumeIntervals of
// render/ao/volumes.ispc composited in front of each layer (null: none)
struct AOVolume {
  const void *vm = nullptr;
  float samplingRate = 1.f;
  bool (*overlaps)(const void *vm, const Ray &r) = nullptr;
  V4 (*integrate)(const void *vm, const Ray &r, float jitter, float samplingRate) = nullptr;
};
extern AOVolume g_aoVolume;

// rkcommon rcp(AffineSpace3f) (capi.cpp)
A3 rcpAffine(const A3 &a);
void copyAux(const FrameBuffer &fb);

template <class F>
void parallelRows(int H, int nthreads, F f) {
  if (nthreads <= 0) nthreads = int(std::thread::hardware_concurrency());
  if (nthreads <= 0) nthreads = 1;
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; t++)
    th.emplace_back([=]() {
      for (int y = t; y < H; y += nthreads) f(y);
    });
  for (auto &x : th) x.join();
}

constexpr float ulpEpsilon = 0x1.0fp-21f;

// rays traced by the renderers since the last reset (CPU-baseline Mrays/s)
extern std::atomic<uint64_t> g_rayCount;

// an obj material as getSurfaceColor reads it (render/ao/surfaces.ispc:17-42)
struct AOMaterial {
  int isObj;
  V3 kd;
  float d;
  const Texture *kdMap;
};
struct AOParams {
  int spp, aoSamples;
  float aoRadius, aoIntensity;
  V4 bgColor;
  const Texture *backplate = nullptr, *maxDepth = nullptr;  // map_backplate, map_maxDepth
  float mipBiasFactor = 1.f;
  std::vector<AOMaterial> mats;  // by the instances' material slot; empty: white, opaque
};
// (with materials, attributes, maps, backplate and maxDepth as the AO renderer
// reads them: AORenderer_renderSample, getSurfaceColor, RendererRenderTaskFn.inl)
void renderAO(const Scene &s, const Camera &cam, const PixelFilter &pf, const AOParams &p, FrameBuffer &fb,
              int nthreads);

}  // namespace orc
