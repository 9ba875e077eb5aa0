// 2D textures on the device, following the reference's Texture2D:
//   texel formats        texture/Texture2DFormats.ispc (getTexel_* / setTexel_*)
//   wrap modes, filters  texture/Texture2D.ispc:13-128 (wrap_coord,
//                        nearest_coords, bilinear_coords, bilerp)
//   MIP level selection  texture/Texture2D.ispc:130-164 (calcLambda, Texture2D_get)
//   MIP generation       texture/MipMapGeneration.ispc (texture.cu)
//   clamp2edge           texture/Texture2D.ih:20-24 (backplate lookups)
// Formats: the 8- and 16-bit integer and 32-bit float ones; the half-float
// formats are refused at creation.
#pragma once
#include "common.cuh"

namespace b200 {

// OSPTextureFormat values (ospray/include/ospray/OSPEnums.h)
enum : int {
  TEX_RGBA8 = 0,
  TEX_SRGBA = 1,
  TEX_RGBA32F = 2,
  TEX_RGB8 = 3,
  TEX_SRGB = 4,
  TEX_RGB32F = 5,
  TEX_R8 = 6,
  TEX_R32F = 7,
  TEX_L8 = 8,
  TEX_RA8 = 9,
  TEX_LA8 = 10,
  TEX_RGBA16 = 11,
  TEX_RGB16 = 12,
  TEX_RA16 = 13,
  TEX_R16 = 14,
  TEX_RA32F = 15
};
enum : int { TEX_FILTER_LINEAR = 0, TEX_FILTER_NEAREST = 1 };
enum : int { TEX_WRAP_REPEAT = 0, TEX_WRAP_MIRRORED_REPEAT = 1, TEX_WRAP_CLAMP_TO_EDGE = 2 };

constexpr int TEX_MAX_LEVELS = 24;

// a texture as the kernels read it (lives in device memory)
struct TextureD {
  const unsigned char *level[TEX_MAX_LEVELS];  // level 0 = the image; MIP levels after it
  int w, h, maxLevel, format, filter, wrapS, wrapT, hasAlpha;
};

B200_HD int texelBytes(int fmt) {
  switch (fmt) {
    case TEX_RGBA8:
    case TEX_SRGBA: return 4;
    case TEX_RGBA32F: return 16;
    case TEX_RGB8:
    case TEX_SRGB: return 3;
    case TEX_RGB32F: return 12;
    case TEX_R8:
    case TEX_L8: return 1;
    case TEX_R32F: return 4;
    case TEX_RA8:
    case TEX_LA8: return 2;
    case TEX_RGBA16: return 8;
    case TEX_RGB16: return 6;
    case TEX_RA16: return 4;
    case TEX_R16: return 2;
    case TEX_RA32F: return 8;
    default: return 0;
  }
}

// sRGB transfer curve (IEC 61966-2-1), as rkcommon's srgb_to_linear
B200_D float srgbToLinear(float c) {
  return c <= 0.04045f ? c * (1.f / 12.92f) : powf((c + 0.055f) * (1.f / 1.055f), 2.4f);
}

B200_D float4 getTexel(int fmt, const unsigned char *d, uint32_t i) {
  constexpr float B = 1.f / 255.f, S = 1.f / 65535.f;
  switch (fmt) {
    case TEX_RGBA8:
    case TEX_SRGBA: {
      const uint32_t c = __ldg(reinterpret_cast<const uint32_t *>(d) + i);
      float4 v = make_float4(float(c & 0xffu) * B, float((c >> 8) & 0xffu) * B, float((c >> 16) & 0xffu) * B,
                             float(c >> 24) * B);
      if (fmt == TEX_SRGBA) v = make_float4(srgbToLinear(v.x), srgbToLinear(v.y), srgbToLinear(v.z), v.w);
      return v;
    }
    case TEX_RGBA32F: return __ldg(reinterpret_cast<const float4 *>(d) + i);
    case TEX_RGB8:
    case TEX_SRGB: {
      const unsigned char *t = d + 3 * size_t(i);
      float4 v = make_float4(float(__ldg(t)) * B, float(__ldg(t + 1)) * B, float(__ldg(t + 2)) * B, 1.f);
      if (fmt == TEX_SRGB) v = make_float4(srgbToLinear(v.x), srgbToLinear(v.y), srgbToLinear(v.z), 1.f);
      return v;
    }
    case TEX_RGB32F: {
      const float *t = reinterpret_cast<const float *>(d) + 3 * size_t(i);
      return make_float4(__ldg(t), __ldg(t + 1), __ldg(t + 2), 1.f);
    }
    case TEX_R8: return make_float4(float(__ldg(d + i)) * B, 0.f, 0.f, 1.f);
    case TEX_L8: {
      const float l = srgbToLinear(float(__ldg(d + i)) * B);
      return make_float4(l, l, l, 1.f);
    }
    case TEX_R32F: return make_float4(__ldg(reinterpret_cast<const float *>(d) + i), 0.f, 0.f, 1.f);
    case TEX_RA8: {
      const uint32_t t = __ldg(reinterpret_cast<const uint16_t *>(d) + i);
      return make_float4(float(t & 0xffu) * B, 0.f, 0.f, float(t >> 8) * B);
    }
    case TEX_LA8: {
      const uint32_t t = __ldg(reinterpret_cast<const uint16_t *>(d) + i);
      const float l = srgbToLinear(float(t & 0xffu) * B);
      return make_float4(l, l, l, float(t >> 8) * B);
    }
    case TEX_RGBA16: {
      const uint2 c = __ldg(reinterpret_cast<const uint2 *>(d) + i);
      return make_float4(float(c.x & 0xffffu) * S, float(c.x >> 16) * S, float(c.y & 0xffffu) * S,
                         float(c.y >> 16) * S);
    }
    case TEX_RGB16: {
      const uint16_t *t = reinterpret_cast<const uint16_t *>(d) + 3 * size_t(i);
      return make_float4(float(__ldg(t)) * S, float(__ldg(t + 1)) * S, float(__ldg(t + 2)) * S, 1.f);
    }
    case TEX_RA16: {
      const uint32_t t = __ldg(reinterpret_cast<const uint32_t *>(d) + i);
      return make_float4(float(t & 0xffffu) * S, 0.f, 0.f, float(t >> 16) * S);
    }
    case TEX_R16: return make_float4(float(__ldg(reinterpret_cast<const uint16_t *>(d) + i)) * S, 0.f, 0.f, 1.f);
    case TEX_RA32F: {
      const float2 v = __ldg(reinterpret_cast<const float2 *>(d) + i);
      return make_float4(v.x, 0.f, 0.f, v.y);
    }
    default: return make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

B200_D float fracf(float x) { return x - floorf(x); }

B200_D float wrapCoord(int mode, float halfTexel, float p) {
  float tc = 0.f;
  if (mode == TEX_WRAP_REPEAT) {
    tc = fracf(p - halfTexel) + halfTexel;
    tc = fmaxf(tc, 0.f);  // filters inf / NaN
  } else if (mode == TEX_WRAP_MIRRORED_REPEAT) {
    tc = 2.f * fracf(p * 0.5f);
    if (tc >= 1.f) tc = 2.f - tc;
    tc = fminf(fmaxf(tc, halfTexel), 1.f - halfTexel);
  } else {
    tc = fminf(fmaxf(p, halfTexel), 1.f - halfTexel);
  }
  return tc;
}

B200_D float4 lerp4(float f, float4 a, float4 b) {
  return make_float4((1.f - f) * a.x + f * b.x, (1.f - f) * a.y + f * b.y, (1.f - f) * a.z + f * b.z,
                     (1.f - f) * a.w + f * b.w);
}

B200_D float4 texNearest(const TextureD &t, float s, float u, int level) {
  const int w = max(t.w >> level, 1), h = max(t.h >> level, 1);
  const float x = wrapCoord(t.wrapS, 0.f, s), y = wrapCoord(t.wrapT, 0.f, u);
  const int ix = min(int(x * float(w)), w - 1), iy = min(int(y * float(h)), h - 1);
  return getTexel(t.format, t.level[level], uint32_t(iy * w + ix));
}

B200_D float4 texBilinear(const TextureD &t, float s, float u, int level) {
  const int w = max(t.w >> level, 1), h = max(t.h >> level, 1);
  const float fw = float(w), fh = float(h);
  const float hx = (1.f / fw) * 0.5f, hy = (1.f / fh) * 0.5f;
  float x = wrapCoord(t.wrapS, hx, s), y = wrapCoord(t.wrapT, hy, u);
  x = (x - hx) * fw;
  y = (y - hy) * fh;
  const float fx = fracf(x), fy = fracf(y);
  const int x0 = min(int(x), w - 1), y0 = min(int(y), h - 1);
  int x1 = x0 + 1, y1 = y0 + 1;
  if (x1 >= w) x1 = 0;  // border cases as REPEAT
  if (y1 >= h) y1 = 0;
  const unsigned char *d = t.level[level];
  const float4 c00 = getTexel(t.format, d, uint32_t(y0 * w + x0)), c01 = getTexel(t.format, d, uint32_t(y0 * w + x1));
  const float4 c10 = getTexel(t.format, d, uint32_t(y1 * w + x0)), c11 = getTexel(t.format, d, uint32_t(y1 * w + x1));
  return lerp4(fy, lerp4(fx, c00, c01), lerp4(fx, c10, c11));
}

// Texture2D_get: MIP level from the pixel footprint (0: level 0)
B200_D float4 texGet(const TextureD &t, float s, float u, float footprint) {
  int level = 0;
  float frac = 0.f;
  const bool nearest = t.filter == TEX_FILTER_NEAREST;
  if (t.maxLevel) {
    float t0 = footprint * float(max(t.w, t.h));
    if (!nearest) t0 *= 0.5f;
    const float lambda = fmaxf(0.f, logf(t0) / logf(2.f));
    level = min(int(lambda), t.maxLevel - 1);
    frac = fminf(lambda - float(level), 1.f);
  }
  const float4 a = nearest ? texNearest(t, s, u, level) : texBilinear(t, s, u, level);
  if (frac == 0.f) return a;
  const float4 b = nearest ? texNearest(t, s, u, level + 1) : texBilinear(t, s, u, level + 1);
  return lerp4(frac, a, b);
}

// Renderer_getMaxDepth (render/Renderer.ispc:30-40): max(0, red) of the
// renderer's maxDepth texture at a screen position; no texture: no limit.
// (The renderer-level lookups are out of line so the texel decoding does not
// count against the register budget of the kernels that call them.)
static __device__ __noinline__ float texMaxDepth(const TextureD *t, float sx, float sy) {
  return t ? fmaxf(0.f, texGet(*t, sx, sy, 0.f).x) : INFINITY;
}

// clamp2edge + a level-0 lookup (the renderer's backplate at a screen position)
static __device__ __noinline__ float4 texGetScreen(const TextureD &t, float sx, float sy) {
  const float hx = (1.f / float(t.w)) * 0.5f, hy = (1.f / float(t.h)) * 0.5f;
  return texGet(t, fminf(fmaxf(sx, hx), 1.f - hx), fminf(fmaxf(sy, hy), 1.f - hy), 0.f);
}

}  // namespace b200
