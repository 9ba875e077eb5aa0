// Per-pixel framebuffer post-processing (tonemapper + colour conversion),
// shared by the post-process kernel and the persistent batch kernel.
#pragma once
#include <cstdint>

#include "../../include/b200.h"

namespace b200 {

// Tonemapper coefficients after ToneMapper::commit's clamping and solve.
struct ToneMapD {
  float exposure, a, b, c, d;
  int aces;
};

namespace {

__device__ __forceinline__ float clamp01(float v) { return fminf(fmaxf(v, 0.f), 1.f); }

// ToneMapper_kernel (fb/frame_ops/ToneMapper.ispc:12-41): exposure, optional
// ACES input matrix, the curve x^a / (x^(a d) b + c), optional ACES output
// matrix, clamp to [0,1]; alpha passes through.  The matrices are stored by
// column (LinearSpace3f vx, vy, vz) and applied as vx*x + vy*y + vz*z.
__constant__ float c_acesIn[9] = {0.5972782409f, 0.0760130499f, 0.0284085382f,  //
                                  0.3545713181f, 0.9083220973f, 0.1338243154f,  //
                                  0.0482176639f, 0.0156579968f, 0.8375684636f};
__constant__ float c_acesOut[9] = {1.6047539945f,  -0.1020831870f, -0.0032670420f,  //
                                   -0.5310794927f, 1.1081322801f,  -0.0727552477f,  //
                                   -0.0736720338f, -0.0060518756f, 1.0760219533f};

__device__ __forceinline__ float3 mat3(const float *m, float3 v) {
  float3 r;
  r.x = __fadd_rn(__fadd_rn(__fmul_rn(m[0], v.x), __fmul_rn(m[3], v.y)), __fmul_rn(m[6], v.z));
  r.y = __fadd_rn(__fadd_rn(__fmul_rn(m[1], v.x), __fmul_rn(m[4], v.y)), __fmul_rn(m[7], v.z));
  r.z = __fadd_rn(__fadd_rn(__fmul_rn(m[2], v.x), __fmul_rn(m[5], v.y)), __fmul_rn(m[8], v.z));
  return r;
}

__device__ __forceinline__ float curve(float x, const ToneMapD &t, float ad) {
  return __fdiv_rn(powf(x, t.a), __fadd_rn(__fmul_rn(powf(x, ad), t.b), t.c));
}

__device__ __forceinline__ float4 toneMap(float4 col, const ToneMapD &t) {
  float3 x = make_float3(__fmul_rn(col.x, t.exposure), __fmul_rn(col.y, t.exposure), __fmul_rn(col.z, t.exposure));
  if (t.aces) x = mat3(c_acesIn, x);
  const float ad = __fmul_rn(t.a, t.d);
  x = make_float3(curve(x.x, t, ad), curve(x.y, t, ad), curve(x.z, t, ad));
  if (t.aces) x = mat3(c_acesOut, x);
  return make_float4(clamp01(x.x), clamp01(x.y), clamp01(x.z), col.w);
}

// rkcommon 1.14.2 (math/vec.ih) conversions used by ColorConversion_kernel:
// cvt_uint32 rounds 255*clamp(v,0,1) to nearest (ties to even, as ISPC's
// round), linear_to_srgba8 converts rgb to sRGB, keeps alpha linear (>= 0),
// scales by 255 after min(.,1) and truncates.
__device__ __forceinline__ uint32_t unorm8(float v) { return __float2uint_rn(__fmul_rn(255.f, clamp01(v))); }

__device__ __forceinline__ float toSrgb(float f) {
  const float c = fmaxf(f, 0.f);
  return c <= 0.0031308f ? __fmul_rn(12.92f, c) : __fsub_rn(__fmul_rn(powf(c, 1.f / 2.4f), 1.055f), 0.055f);
}

__device__ __forceinline__ uint32_t srgb8(float v) { return uint32_t(__fmul_rn(255.f, fminf(v, 1.f))); }

// pixel i of the accumulated colour, tonemapped when asked, converted to the
// mapped buffer's format
__device__ __forceinline__ void postPixel(const float4 *__restrict__ color, long long i, int format, int tonemap,
                                          const ToneMapD &tm, void *__restrict__ out) {
  float4 v = color[i];
  if (tonemap) v = toneMap(v, tm);
  if (format == B200_FB_RGBA8) {
    static_cast<uint32_t *>(out)[i] = unorm8(v.x) | unorm8(v.y) << 8 | unorm8(v.z) << 16 | unorm8(v.w) << 24;
  } else if (format == B200_FB_SRGBA) {
    static_cast<uint32_t *>(out)[i] = srgb8(toSrgb(v.x)) | srgb8(toSrgb(v.y)) << 8 | srgb8(toSrgb(v.z)) << 16 |
                                      srgb8(fmaxf(v.w, 0.f)) << 24;
  } else {
    const float4 c = make_float4(fmaxf(v.x, 0.f), fmaxf(v.y, 0.f), fmaxf(v.z, 0.f), fmaxf(v.w, 0.f));
    static_cast<float4 *>(out)[i] = make_float4(c.x, c.y, c.z, fminf(c.w, 1.f));
  }
}

}  // namespace
}  // namespace b200
