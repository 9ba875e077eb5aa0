// Oracle (test infrastructure only): framebuffer post-processing and pick.
//
// Scalar restatement of
//   ToneMapper::commit          modules/cpu/fb/frame_ops/ToneMapper.cpp:16-51
//   ToneMapper_kernel           modules/cpu/fb/frame_ops/ToneMapper.ispc:12-41
//   ColorConversion_kernel      modules/cpu/fb/frame_ops/ColorConversion.ispc:11-36
//   LocalFrameBuffer::postProcess  modules/cpu/fb/LocalFB.cpp:459-477 (order)
//   Renderer_pick               modules/cpu/render/Renderer.ispc:43-95
// The unorm / sRGB conversions are rkcommon 1.14.2 helpers (math/vec.ih,
// not vendored): cvt_uint32 = round-to-nearest-even(255 * clamp(v, 0, 1)),
// linear_to_srgba8 = sRGB curve on rgb (alpha linear, >= 0), 255 * min(., 1),
// truncated.  Restated from their published behaviour.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "render.h"

using namespace orc;

namespace {

struct OrToneMapper {
  float exposure, contrast, shoulder, midIn, midOut, hdrMax;
  int acesColor;
};

struct ToneCoef {
  float exposure, a, b, c, d;
  bool aces;
};

// ToneMapper.cpp:18-50, same operation order
ToneCoef solve(const OrToneMapper &u) {
  ToneCoef t;
  t.exposure = u.exposure;
  t.a = std::max(u.contrast, 0.0001f);
  t.d = std::min(std::max(u.shoulder, 0.0001f), 1.f);
  const float m = std::min(std::max(u.midIn, 0.0001f), 1.f);
  const float n = std::min(std::max(u.midOut, 0.0001f), 1.f);
  const float w = std::max(u.hdrMax, 1.f);
  const float a = t.a, d = t.d;
  t.b = -((powf(m, -a * d) *
           (-powf(m, a) + (n * (powf(m, a * d) * n * powf(w, a) - powf(m, a) * powf(w, a * d))) /
                              (powf(m, a * d) * n - n * powf(w, a * d)))) /
          n);
  t.c = std::max((powf(m, a * d) * n * powf(w, a) - powf(m, a) * powf(w, a * d)) /
                     (powf(m, a * d) * n - n * powf(w, a * d)),
                 0.f);
  t.aces = u.acesColor != 0;
  return t;
}

// LinearSpace3f columns (vx, vy, vz); M * v = vx v.x + vy v.y + vz v.z
const float kAcesIn[3][3] = {{0.5972782409f, 0.0760130499f, 0.0284085382f},
                             {0.3545713181f, 0.9083220973f, 0.1338243154f},
                             {0.0482176639f, 0.0156579968f, 0.8375684636f}};
const float kAcesOut[3][3] = {{1.6047539945f, -0.1020831870f, -0.0032670420f},
                              {-0.5310794927f, 1.1081322801f, -0.0727552477f},
                              {-0.0736720338f, -0.0060518756f, 1.0760219533f}};

void mat3(const float M[3][3], float v[3]) {
  float r[3];
  for (int k = 0; k < 3; k++) r[k] = M[0][k] * v[0] + M[1][k] * v[1] + M[2][k] * v[2];
  std::memcpy(v, r, sizeof(r));
}

// min/max with IEEE fmin/fmax semantics (a NaN operand yields the other),
// as the CUDA side's fminf/fmaxf
float clamp01(float v) { return std::fmin(std::fmax(v, 0.f), 1.f); }

void toneMap(const ToneCoef &t, float c[4]) {
  float x[3] = {c[0] * t.exposure, c[1] * t.exposure, c[2] * t.exposure};
  if (t.aces) mat3(kAcesIn, x);
  for (float &v : x) v = powf(v, t.a) / (powf(v, t.a * t.d) * t.b + t.c);
  if (t.aces) mat3(kAcesOut, x);
  for (int k = 0; k < 3; k++) c[k] = clamp01(x[k]);
}

uint32_t unorm8(float v) { return uint32_t(std::nearbyint(255.f * clamp01(v))); }

float toSrgb(float f) {
  const float c = std::fmax(f, 0.f);
  return c <= 0.0031308f ? 12.92f * c : powf(c, 1.f / 2.4f) * 1.055f - 0.055f;
}

uint32_t srgb8(float v) { return uint32_t(255.f * std::fmin(v, 1.f)); }

}  // namespace

extern "C" {

// color: n RGBA32F pixels (the accumulated colour).  tm: null = no
// tonemapper.  format: 1 RGBA8, 2 SRGBA (out = n uint32), 3 RGBA32F (out =
// n x 4 float).
void or_frame_post(const float *color, long long n, int format, const OrToneMapper *tm, void *out) {
  ToneCoef t = {};
  if (tm) t = solve(*tm);
  for (long long i = 0; i < n; i++) {
    float c[4];
    std::memcpy(c, color + 4 * i, sizeof(c));
    if (tm) toneMap(t, c);
    if (format == 1) {
      static_cast<uint32_t *>(out)[i] = unorm8(c[0]) | unorm8(c[1]) << 8 | unorm8(c[2]) << 16 | unorm8(c[3]) << 24;
    } else if (format == 2) {
      static_cast<uint32_t *>(out)[i] =
          srgb8(toSrgb(c[0])) | srgb8(toSrgb(c[1])) << 8 | srgb8(toSrgb(c[2])) << 16 | srgb8(std::fmax(c[3], 0.f)) << 24;
    } else if (format == 3) {
      float *o = static_cast<float *>(out) + 4 * i;
      for (int k = 0; k < 4; k++) o[k] = std::fmax(c[k], 0.f);
      o[3] = std::fmin(o[3], 1.f);
    }
  }
}

// tonemapper coefficients (exposure, a, b, c, d) after ToneMapper::commit
void or_tonemap_coefficients(const OrToneMapper *tm, float *out5) {
  const ToneCoef t = solve(*tm);
  out5[0] = t.exposure;
  out5[1] = t.a;
  out5[2] = t.b;
  out5[3] = t.c;
  out5[4] = t.d;
}

// Renderer_pick: camera ray at screen (sx, sy), closest hit, position
// org + dir * t.  out: [hit, x, y, z] as floats-in-words, ids[3].
struct OrCameraP {
  float pos[3], dir[3], up[3];
  float fovy, aspect, nearClip;
  int type;  // 0 perspective, 1 orthographic, 2 panoramic
  float height;  // orthographic image height
};

int or_pick(void *sp, const OrCameraP *c, float sx, float sy, float *pos3, uint32_t *ids3) {
  const Scene &s = *static_cast<Scene *>(sp);
  const Camera cam = makeCamera({c->pos[0], c->pos[1], c->pos[2]}, {c->dir[0], c->dir[1], c->dir[2]},
                                {c->up[0], c->up[1], c->up[2]}, c->fovy, c->aspect, c->nearClip, c->type, c->height);
  const Ray ray = cameraRay(cam, {sx, sy});
  Hit h;
  if (!s.intersect(ray, h)) {
    pos3[0] = pos3[1] = pos3[2] = 0.f;
    ids3[0] = ids3[1] = ids3[2] = INVALID_ID;
    return 0;
  }
  const V3 p = ray.org + ray.dir * h.t;
  pos3[0] = p.x;
  pos3[1] = p.y;
  pos3[2] = p.z;
  ids3[0] = h.instID;
  ids3[1] = h.geomID;
  ids3[2] = h.primID;
  return 1;
}

}  // extern "C"
