// Oracle (test infrastructure only): CPU 2D textures; citations in texture.h.
#include "texture.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace orc {

namespace {

enum {
  RGBA8 = 0, SRGBA, RGBA32F, RGB8, SRGB, RGB32F, R8, R32F, L8, RA8, LA8, RGBA16, RGB16, RA16, R16, RA32F
};
enum { WRAP_REPEAT = 0, WRAP_MIRRORED_REPEAT = 1 };

float srgbToLinear(float c) { return c <= 0.04045f ? c * (1.f / 12.92f) : std::pow((c + 0.055f) * (1.f / 1.055f), 2.4f); }
float linearToSrgb(float f) {
  const float c = std::fmax(f, 0.f);
  return c <= 0.0031308f ? 12.92f * c : std::pow(c, 1.f / 2.4f) * 1.055f - 0.055f;
}
uint32_t cvt8(float v) { return uint32_t(std::nearbyint(255.f * clampf(v, 0.f, 1.f))); }
uint32_t cvt16(float v) { return uint32_t(std::nearbyint(65535.f * clampf(v, 0.f, 1.f))); }
uint32_t srgbByte(float v) { return uint32_t(255.f * std::fmin(v, 1.f)); }

template <class T>
T load(const uint8_t *d, size_t i) {
  T v;
  std::memcpy(&v, d + i * sizeof(T), sizeof(T));
  return v;
}
template <class T>
void store(uint8_t *d, size_t i, T v) {
  std::memcpy(d + i * sizeof(T), &v, sizeof(T));
}

V4 getTexel(int f, const uint8_t *d, uint32_t i) {
  const float B = 1.f / 255.f, S = 1.f / 65535.f;
  switch (f) {
    case RGBA8:
    case SRGBA: {
      const uint32_t c = load<uint32_t>(d, i);
      V4 v = {float(c & 0xffu) * B, float((c >> 8) & 0xffu) * B, float((c >> 16) & 0xffu) * B, float(c >> 24) * B};
      if (f == SRGBA) v = {srgbToLinear(v.x), srgbToLinear(v.y), srgbToLinear(v.z), v.w};
      return v;
    }
    case RGBA32F: return load<V4>(d, i);
    case RGB8:
    case SRGB: {
      const uint8_t *t = d + 3 * size_t(i);
      V4 v = {float(t[0]) * B, float(t[1]) * B, float(t[2]) * B, 1.f};
      if (f == SRGB) v = {srgbToLinear(v.x), srgbToLinear(v.y), srgbToLinear(v.z), 1.f};
      return v;
    }
    case RGB32F: {
      const V3 c = load<V3>(d, i);
      return {c.x, c.y, c.z, 1.f};
    }
    case R8: return {float(d[i]) * B, 0.f, 0.f, 1.f};
    case L8: {
      const float l = srgbToLinear(float(d[i]) * B);
      return {l, l, l, 1.f};
    }
    case R32F: return {load<float>(d, i), 0.f, 0.f, 1.f};
    case RA8: {
      const uint32_t t = load<uint16_t>(d, i);
      return {float(t & 0xffu) * B, 0.f, 0.f, float(t >> 8) * B};
    }
    case LA8: {
      const uint32_t t = load<uint16_t>(d, i);
      const float l = srgbToLinear(float(t & 0xffu) * B);
      return {l, l, l, float(t >> 8) * B};
    }
    case RGBA16: {
      const uint16_t *t = reinterpret_cast<const uint16_t *>(d) + 4 * size_t(i);
      return {float(t[0]) * S, float(t[1]) * S, float(t[2]) * S, float(t[3]) * S};
    }
    case RGB16: {
      const uint16_t *t = reinterpret_cast<const uint16_t *>(d) + 3 * size_t(i);
      return {float(t[0]) * S, float(t[1]) * S, float(t[2]) * S, 1.f};
    }
    case RA16: {
      const uint32_t t = load<uint32_t>(d, i);
      return {float(t & 0xffffu) * S, 0.f, 0.f, float(t >> 16) * S};
    }
    case R16: return {float(load<uint16_t>(d, i)) * S, 0.f, 0.f, 1.f};
    case RA32F: {
      const V2 v = load<V2>(d, i);
      return {v.x, 0.f, 0.f, v.y};
    }
    default: return {0.f, 0.f, 0.f, 0.f};
  }
}

void setTexel(int f, uint8_t *d, uint32_t i, V4 v) {
  switch (f) {
    case RGBA8: store<uint32_t>(d, i, cvt8(v.x) | cvt8(v.y) << 8 | cvt8(v.z) << 16 | cvt8(v.w) << 24); break;
    case SRGBA:
      store<uint32_t>(d, i, srgbByte(linearToSrgb(v.x)) | srgbByte(linearToSrgb(v.y)) << 8 |
                                srgbByte(linearToSrgb(v.z)) << 16 | srgbByte(std::fmax(v.w, 0.f)) << 24);
      break;
    case RGBA32F: store<V4>(d, i, v); break;
    case RGB8:
      for (int k = 0; k < 3; k++) d[3 * size_t(i) + k] = uint8_t(cvt8(k == 0 ? v.x : (k == 1 ? v.y : v.z)));
      break;
    case SRGB:
      for (int k = 0; k < 3; k++)
        d[3 * size_t(i) + k] = uint8_t(cvt8(linearToSrgb(k == 0 ? v.x : (k == 1 ? v.y : v.z))));
      break;
    case RGB32F: store<V3>(d, i, {v.x, v.y, v.z}); break;
    case R8: d[i] = uint8_t(cvt8(v.x)); break;
    case L8: d[i] = uint8_t(cvt8(linearToSrgb(v.x))); break;
    case R32F: store<float>(d, i, v.x); break;
    case RA8: store<uint16_t>(d, i, uint16_t(cvt8(v.x) | cvt8(v.w) << 8)); break;
    case LA8: store<uint16_t>(d, i, uint16_t(cvt8(linearToSrgb(v.x)) | cvt8(v.w) << 8)); break;
    case RGBA16: {
      uint16_t *t = reinterpret_cast<uint16_t *>(d) + 4 * size_t(i);
      t[0] = uint16_t(cvt16(v.x));
      t[1] = uint16_t(cvt16(v.y));
      t[2] = uint16_t(cvt16(v.z));
      t[3] = uint16_t(cvt16(v.w));
      break;
    }
    case RGB16: {
      uint16_t *t = reinterpret_cast<uint16_t *>(d) + 3 * size_t(i);
      t[0] = uint16_t(cvt16(v.x));
      t[1] = uint16_t(cvt16(v.y));
      t[2] = uint16_t(cvt16(v.z));
      break;
    }
    case RA16: store<uint32_t>(d, i, cvt16(v.x) | cvt16(v.w) << 16); break;
    case R16: store<uint16_t>(d, i, uint16_t(cvt16(v.x))); break;
    case RA32F: store<V2>(d, i, {v.x, v.w}); break;
    default: break;
  }
}

V4 add(V4 a, V4 b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
V4 scale(float s, V4 a) { return {s * a.x, s * a.y, s * a.z, s * a.w}; }
V4 lerp4(float f, V4 a, V4 b) {
  return {(1.f - f) * a.x + f * b.x, (1.f - f) * a.y + f * b.y, (1.f - f) * a.z + f * b.z, (1.f - f) * a.w + f * b.w};
}
float fracf(float x) { return x - std::floor(x); }

// MipMap_generateRows / MipMap_generateRow
void mipRows(int f, const uint8_t *src, int sw, int sh, uint8_t *dst, int dw, int dh) {
  for (int y = 0; y < dh; y++) {
    float rx = 1.f / float(sw), ry = 1.f / float(sh);
    float hx = float(dw) * rx, hy = float(dh) * ry;
    const int srcy = 2 * y * sw;
    int ox = 2, oy = srcy + 2 * sw;
    if ((sw & 1) == 0) {
      hx = 0.5f;
      rx = 0.f;
      ox = 0;
    }
    if ((sh & 1) == 0) {
      hy = 0.5f;
      ry = 0.f;
      oy = srcy;
    }
    const float wy0 = hy - float(y) * ry, wy2 = ry + float(y) * ry;
    for (int x = 0; x < dw; x++) {
      const float tx = float(x) * rx;
      const int sx = 2 * x;
      auto row = [&](int base) {
        return add(add(scale(hx - tx, getTexel(f, src, uint32_t(base + sx))),
                       scale(hx, getTexel(f, src, uint32_t(base + sx + 1)))),
                   scale(rx + tx, getTexel(f, src, uint32_t(base + sx + ox))));
      };
      const V4 v0 = row(srcy), v1 = row(srcy + sw), v2 = row(oy);
      setTexel(f, dst, uint32_t(y * dw + x), add(add(scale(wy0, v0), scale(hy, v1)), scale(wy2, v2)));
    }
  }
}
void mipRow(int f, const uint8_t *src, int ss, uint8_t *dst, int ds) {
  float r = 1.f / float(ss), h = float(ds) * r;
  int o2 = 2;
  if ((ss & 1) == 0) {
    h = 0.5f;
    r = 0.f;
    o2 = 0;
  }
  for (int x = 0; x < ds; x++) {
    const float tx = float(x) * r;
    const int sx = 2 * x;
    const V4 v = add(add(scale(h - tx, getTexel(f, src, uint32_t(sx))), scale(h, getTexel(f, src, uint32_t(sx + 1)))),
                     scale(r + tx, getTexel(f, src, uint32_t(sx + o2))));
    setTexel(f, dst, uint32_t(x), v);
  }
}

float wrapCoord(int mode, float half, float p) {
  float tc;
  if (mode == WRAP_REPEAT) {
    tc = fracf(p - half) + half;
    tc = std::fmax(tc, 0.f);
  } else if (mode == WRAP_MIRRORED_REPEAT) {
    tc = 2.f * fracf(p * 0.5f);
    if (tc >= 1.f) tc = 2.f - tc;
    tc = clampf(tc, half, 1.f - half);
  } else {
    tc = clampf(p, half, 1.f - half);
  }
  return tc;
}

}  // namespace

int texelBytes(int f) {
  static const int b[16] = {4, 4, 16, 3, 3, 12, 1, 4, 1, 2, 2, 8, 6, 4, 2, 8};
  return f >= 0 && f < 16 ? b[f] : 0;
}

V4 Texture::texel(int level, uint32_t i) const { return getTexel(format, levels[size_t(level)].data(), i); }

V4 Texture::get(V2 st, float footprint) const {
  int level = 0;
  float frac = 0.f;
  const bool nearest = (filter & 1) != 0;
  if (maxLevel()) {
    float t0 = footprint * float(std::max(w, h));
    if (!nearest) t0 *= 0.5f;
    const float lambda = std::fmax(0.f, std::log(t0) / std::log(2.f));
    level = std::min(int(lambda), maxLevel() - 1);
    frac = std::fmin(lambda - float(level), 1.f);
  }
  auto at = [&](int l) -> V4 {
    const int lw = std::max(w >> l, 1), lh = std::max(h >> l, 1);
    if (nearest) {
      const float x = wrapCoord(wrapS, 0.f, st.x), y = wrapCoord(wrapT, 0.f, st.y);
      const int ix = std::min(int(x * float(lw)), lw - 1), iy = std::min(int(y * float(lh)), lh - 1);
      return texel(l, uint32_t(iy * lw + ix));
    }
    const float hx = (1.f / float(lw)) * 0.5f, hy = (1.f / float(lh)) * 0.5f;
    float x = wrapCoord(wrapS, hx, st.x), y = wrapCoord(wrapT, hy, st.y);
    x = (x - hx) * float(lw);
    y = (y - hy) * float(lh);
    const float fx = fracf(x), fy = fracf(y);
    const int x0 = std::min(int(x), lw - 1), y0 = std::min(int(y), lh - 1);
    int x1 = x0 + 1, y1 = y0 + 1;
    if (x1 >= lw) x1 = 0;
    if (y1 >= lh) y1 = 0;
    const V4 c00 = texel(l, uint32_t(y0 * lw + x0)), c01 = texel(l, uint32_t(y0 * lw + x1));
    const V4 c10 = texel(l, uint32_t(y1 * lw + x0)), c11 = texel(l, uint32_t(y1 * lw + x1));
    return lerp4(fy, lerp4(fx, c00, c01), lerp4(fx, c10, c11));
  };
  const V4 a = at(level);
  if (frac == 0.f) return a;
  return lerp4(frac, a, at(level + 1));
}

V4 Texture::getScreen(V2 p) const {
  const float hx = (1.f / float(w)) * 0.5f, hy = (1.f / float(h)) * 0.5f;
  return get({clampf(p.x, hx, 1.f - hx), clampf(p.y, hy, 1.f - hy)}, 0.f);
}

Texture *makeTexture(int w, int h, int format, int filter, int wrapS, int wrapT, bool mipmaps, const void *data) {
  Texture *t = new Texture();
  t->w = w;
  t->h = h;
  t->format = format;
  t->filter = filter;
  t->wrapS = wrapS;
  t->wrapT = wrapT;
  t->hasAlpha = format == RGBA8 || format == SRGBA || format == RA8 || format == LA8 || format == RGBA32F ||
                format == RGBA16 || format == RA16 || format == RA32F;
  const int bpt = texelBytes(format);
  t->levels.emplace_back(static_cast<const uint8_t *>(data),
                         static_cast<const uint8_t *>(data) + size_t(w) * h * bpt);
  int sw = w, sh = h;
  while (mipmaps && !(sw == 1 && sh == 1)) {
    const int dw = std::max(sw / 2, 1), dh = std::max(sh / 2, 1);
    std::vector<uint8_t> dst(size_t(dw) * dh * bpt);
    const uint8_t *src = t->levels.back().data();
    if (sw > 1 && sh > 1)
      mipRows(format, src, sw, sh, dst.data(), dw, dh);
    else
      mipRow(format, src, std::max(sw, sh), dst.data(), std::max(dw, dh));
    t->levels.push_back(std::move(dst));
    sw = dw;
    sh = dh;
  }
  return t;
}

}  // namespace orc
