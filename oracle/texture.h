// Oracle (test infrastructure only): 2D textures on the CPU, restated from
//   texel formats      texture/Texture2DFormats.ispc (getTexel_* / setTexel_*)
//   wrap, filters      texture/Texture2D.ispc:13-128 (wrap_coord,
//                      nearest_coords, bilinear_coords, bilerp)
//   level selection    texture/Texture2D.ispc:130-164 (calcLambda, Texture2D_get)
//   MIP generation     texture/MipMapGeneration.ispc, level sizes
//                      texture/Texture2D.cpp:97-135
//   clamp2edge         texture/Texture2D.ih:20-24
// The colour conversions come from rkcommon 1.14.2 (not vendored with the
// reference; cmake/ospray_options.cmake:15 pins it): cvt_uint32 / cvt_uint16
// round 255 (65535) x clamp(v, 0, 1) to the nearest integer,
// linear_to_srgba8 applies the sRGB transfer curve (IEC 61966-2-1) to rgb,
// keeps alpha, takes min(., 1) x 255 and truncates; srgb_to_linear is the
// inverse curve.
#pragma once
#include <cstdint>
#include <vector>

#include "vecmath.h"

namespace orc {

struct Texture {
  int w = 0, h = 0, format = 0, filter = 0, wrapS = 0, wrapT = 0;
  bool hasAlpha = false;
  std::vector<std::vector<uint8_t>> levels;  // level 0 = the image
  int maxLevel() const { return int(levels.size()) - 1; }
  V4 texel(int level, uint32_t i) const;
  // Texture2D_get at texture coordinates st with the hit's pixel footprint
  V4 get(V2 st, float footprint) const;
  // clamp2edge + Texture2D_get at footprint 0 (the renderer's backplate)
  V4 getScreen(V2 p) const;
};

int texelBytes(int format);
// data: w x h texels of `format`; mipmaps: generate the MIP chain
Texture *makeTexture(int w, int h, int format, int filter, int wrapS, int wrapT, bool mipmaps, const void *data);

}  // namespace orc
