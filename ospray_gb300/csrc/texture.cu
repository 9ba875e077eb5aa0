// 2D texture objects: upload, the MIP chain generated on the device, and the
// b200_texture_* C ABI (Texture2D::commit, texture/Texture2D.cpp:42-146;
// MipMap_generate, texture/MipMapGeneration.ispc).
#include <algorithm>
#include <cstring>
#include <string>

#include "../../include/b200.h"
#include "api_internal.h"
#include "texture.cuh"

namespace b200 {

namespace {

// rkcommon conversions of Texture2D_setTexel (texture/Texture2DFormats.ispc):
// cvt_uint32 / cvt_uint16 round 255 (65535) * clamp(v, 0, 1) to nearest;
// linear_to_srgba8 applies the sRGB curve to rgb, keeps alpha linear, scales
// by 255 after min(., 1) and truncates
__device__ uint32_t cvt8(float v) { return __float2uint_rn(__fmul_rn(255.f, fminf(fmaxf(v, 0.f), 1.f))); }
__device__ uint32_t cvt16(float v) { return __float2uint_rn(__fmul_rn(65535.f, fminf(fmaxf(v, 0.f), 1.f))); }
__device__ float linToSrgb(float f) {
  const float c = fmaxf(f, 0.f);
  return c <= 0.0031308f ? __fmul_rn(12.92f, c) : __fsub_rn(__fmul_rn(powf(c, 1.f / 2.4f), 1.055f), 0.055f);
}
__device__ uint32_t srgbByte(float v) { return uint32_t(__fmul_rn(255.f, fminf(v, 1.f))); }

__device__ void setTexel(int fmt, unsigned char *d, uint32_t i, float4 v) {
  switch (fmt) {
    case TEX_RGBA8:
      reinterpret_cast<uint32_t *>(d)[i] = cvt8(v.x) | cvt8(v.y) << 8 | cvt8(v.z) << 16 | cvt8(v.w) << 24;
      break;
    case TEX_SRGBA:
      reinterpret_cast<uint32_t *>(d)[i] = srgbByte(linToSrgb(v.x)) | srgbByte(linToSrgb(v.y)) << 8 |
                                           srgbByte(linToSrgb(v.z)) << 16 | srgbByte(fmaxf(v.w, 0.f)) << 24;
      break;
    case TEX_RGBA32F: reinterpret_cast<float4 *>(d)[i] = v; break;
    case TEX_RGB8:
      d[3 * size_t(i)] = uint8_t(cvt8(v.x));
      d[3 * size_t(i) + 1] = uint8_t(cvt8(v.y));
      d[3 * size_t(i) + 2] = uint8_t(cvt8(v.z));
      break;
    case TEX_SRGB:  // linear_to_srgba, then cvt_uint32 per channel
      d[3 * size_t(i)] = uint8_t(cvt8(linToSrgb(v.x)));
      d[3 * size_t(i) + 1] = uint8_t(cvt8(linToSrgb(v.y)));
      d[3 * size_t(i) + 2] = uint8_t(cvt8(linToSrgb(v.z)));
      break;
    case TEX_RGB32F: {
      float *t = reinterpret_cast<float *>(d) + 3 * size_t(i);
      t[0] = v.x;
      t[1] = v.y;
      t[2] = v.z;
      break;
    }
    case TEX_R8: d[i] = uint8_t(cvt8(v.x)); break;
    case TEX_L8: d[i] = uint8_t(cvt8(linToSrgb(v.x))); break;
    case TEX_R32F: reinterpret_cast<float *>(d)[i] = v.x; break;
    case TEX_RA8: reinterpret_cast<uint16_t *>(d)[i] = uint16_t(cvt8(v.x) | cvt8(v.w) << 8); break;
    case TEX_LA8: reinterpret_cast<uint16_t *>(d)[i] = uint16_t(cvt8(linToSrgb(v.x)) | cvt8(v.w) << 8); break;
    case TEX_RGBA16:
      reinterpret_cast<uint32_t *>(d)[2 * size_t(i)] = cvt16(v.x) | cvt16(v.y) << 16;
      reinterpret_cast<uint32_t *>(d)[2 * size_t(i) + 1] = cvt16(v.z) | cvt16(v.w) << 16;
      break;
    case TEX_RGB16: {
      uint16_t *t = reinterpret_cast<uint16_t *>(d) + 3 * size_t(i);
      t[0] = uint16_t(cvt16(v.x));
      t[1] = uint16_t(cvt16(v.y));
      t[2] = uint16_t(cvt16(v.z));
      break;
    }
    case TEX_RA16: reinterpret_cast<uint32_t *>(d)[i] = cvt16(v.x) | cvt16(v.w) << 16; break;
    case TEX_R16: reinterpret_cast<uint16_t *>(d)[i] = uint16_t(cvt16(v.x)); break;
    case TEX_RA32F: reinterpret_cast<float2 *>(d)[i] = make_float2(v.x, v.w); break;
    default: break;
  }
}

// (every product and sum rounded on its own: no fused multiply-adds)
__device__ float4 add4(float4 a, float4 b) {
  return make_float4(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z), __fadd_rn(a.w, b.w));
}
__device__ float4 scale4(float s, float4 a) {
  return make_float4(__fmul_rn(s, a.x), __fmul_rn(s, a.y), __fmul_rn(s, a.z), __fmul_rn(s, a.w));
}

// MipMap_generateRows: a dst texel averages a 2x2 (3-tap along an odd axis)
// source block with the weights of a box filter of the source's footprint
__global__ void k_mip_rows(const unsigned char *src, int sw, int sh, unsigned char *dst, int dw, int dh, int fmt) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= dw || y >= dh) return;
  float rx = __fdiv_rn(1.f, float(sw)), ry = __fdiv_rn(1.f, float(sh));
  float hx = __fmul_rn(float(dw), rx), hy = __fmul_rn(float(dh), ry);
  const int srcy = 2 * y * sw;
  int ofsx = 2, ofsy = srcy + 2 * sw;
  if ((sw & 1) == 0) {
    hx = 0.5f;
    rx = 0.f;
    ofsx = 0;
  }
  if ((sh & 1) == 0) {
    hy = 0.5f;
    ry = 0.f;
    ofsy = srcy;
  }
  const float wy0 = __fsub_rn(hy, __fmul_rn(float(y), ry)), wy2 = __fadd_rn(ry, __fmul_rn(float(y), ry));
  const float tx = __fmul_rn(float(x), rx);
  const int sx = 2 * x;
  auto row = [&](int base) {
    return add4(add4(scale4(__fsub_rn(hx, tx), getTexel(fmt, src, uint32_t(base + sx))),
                     scale4(hx, getTexel(fmt, src, uint32_t(base + sx + 1)))),
                scale4(__fadd_rn(rx, tx), getTexel(fmt, src, uint32_t(base + sx + ofsx))));
  };
  const float4 v0 = row(srcy), v1 = row(srcy + sw), v2 = row(ofsy);
  setTexel(fmt, dst, uint32_t(y * dw + x), add4(add4(scale4(wy0, v0), scale4(hy, v1)), scale4(wy2, v2)));
}

// MipMap_generateRow: the one-dimensional case
__global__ void k_mip_row(const unsigned char *src, int ssize, unsigned char *dst, int dsize, int fmt) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= dsize) return;
  float r = __fdiv_rn(1.f, float(ssize)), h = __fmul_rn(float(dsize), r);
  int ofs2 = 2;
  if ((ssize & 1) == 0) {
    h = 0.5f;
    r = 0.f;
    ofs2 = 0;
  }
  const float tx = __fmul_rn(float(x), r);
  const int sx = 2 * x;
  const float4 v = add4(add4(scale4(__fsub_rn(h, tx), getTexel(fmt, src, uint32_t(sx))),
                             scale4(h, getTexel(fmt, src, uint32_t(sx + 1)))),
                        scale4(__fadd_rn(r, tx), getTexel(fmt, src, uint32_t(sx + ofs2))));
  setTexel(fmt, dst, uint32_t(x), v);
}

bool formatSupported(int f) { return f >= TEX_RGBA8 && f <= TEX_RA32F; }

// Texture2D_get at n texture coordinates with per-lookup footprints
__global__ void k_tex_sample(const TextureD *t, int n, const float2 *st, const float *fp, float4 *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float2 c = st[i];
  out[i] = texGet(*t, c.x, c.y, fp[i]);
}

}  // namespace

struct TextureObj {
  DeviceObj *dev;
  TextureD desc = {};
  unsigned char *data = nullptr;  // all levels
  TextureD *dDesc = nullptr;      // the descriptor on the device
  TextureObj(DeviceObj *d, int w, int h, int fmt, int filter, int wrapS, int wrapT, const void *host, bool mips)
      : dev(d) {
    dev->retain();
    const int bpt = texelBytes(fmt);
    // level sizes: halving (at least 1) down to 1 x 1, as Texture2D::commit
    std::vector<size_t> off;
    std::vector<int> lw, lh;
    size_t total = 0;
    int cw = w, ch = h;
    for (int l = 0; l < TEX_MAX_LEVELS; l++) {
      off.push_back(total);
      lw.push_back(cw);
      lh.push_back(ch);
      total += ((size_t(cw) * ch * bpt + 15) & ~size_t(15));
      if ((cw == 1 && ch == 1) || !mips) break;
      cw = std::max(cw / 2, 1);
      ch = std::max(ch / 2, 1);
    }
    const int levels = int(off.size());
    cudaStream_t st = dev->stream;
    check(cudaMalloc(&data, total), "texture allocation");
    check(cudaMemcpyAsync(data, host, size_t(w) * h * bpt, cudaMemcpyHostToDevice, st), "texture upload");
    for (int l = 1; l < levels; l++) {
      const int sw = lw[l - 1], sh = lh[l - 1], dw = lw[l], dh = lh[l];
      if (sw > 1 && sh > 1) {
        const dim3 grid(unsigned((dw + 127) / 128), unsigned(dh));
        k_mip_rows<<<grid, 128, 0, st>>>(data + off[l - 1], sw, sh, data + off[l], dw, dh, fmt);
      } else {
        const int ss = std::max(sw, sh), ds = std::max(dw, dh);
        k_mip_row<<<unsigned((ds + 127) / 128), 128, 0, st>>>(data + off[l - 1], ss, data + off[l], ds, fmt);
      }
      check(cudaGetLastError(), "MIP map generation");
    }
    for (int l = 0; l < levels; l++) desc.level[l] = data + off[l];
    desc.w = w;
    desc.h = h;
    desc.maxLevel = levels - 1;
    desc.format = fmt;
    desc.filter = filter;
    desc.wrapS = wrapS;
    desc.wrapT = wrapT;
    desc.hasAlpha = fmt == TEX_RGBA8 || fmt == TEX_SRGBA || fmt == TEX_RA8 || fmt == TEX_LA8 ||
                    fmt == TEX_RGBA32F || fmt == TEX_RGBA16 || fmt == TEX_RA16 || fmt == TEX_RA32F;
    check(cudaMalloc(&dDesc, sizeof(TextureD)), "texture descriptor");
    check(cudaMemcpyAsync(dDesc, &desc, sizeof(TextureD), cudaMemcpyHostToDevice, st), "texture descriptor");
    check(cudaStreamSynchronize(st), "texture upload");
  }
  ~TextureObj() {
    cudaSetDevice(dev->dev);
    cudaStreamSynchronize(dev->stream);
    if (data) cudaFree(data);
    if (dDesc) cudaFree(dDesc);
    dev->release();
  }
};

const TextureD *textureDevice(b200_texture t) {
  return t ? reinterpret_cast<TextureObj *>(t)->dDesc : nullptr;
}
bool textureHasAlpha(b200_texture t) { return t && reinterpret_cast<TextureObj *>(t)->desc.hasAlpha; }

}  // namespace b200

using namespace b200;

extern "C" {

int b200_texture_create(b200_device d, int width, int height, int format, int filter, int wrapS, int wrapT,
                        int mipmaps, const void *data, b200_texture *out) {
  if (!d || !data || !out) return B200_INVALID_ARGUMENT;
  DeviceObj *dev = reinterpret_cast<DeviceObj *>(d);
  try {
    check(cudaSetDevice(dev->dev), "cudaSetDevice");
    if (width < 1 || height < 1) throw Error(B200_INVALID_ARGUMENT, "texture: width and height must be >= 1");
    if (!formatSupported(format))
      throw Error(B200_INVALID_ARGUMENT,
                  "texture: format " + std::to_string(format) + " is not supported (half-float formats are not)");
    if (filter != TEX_FILTER_LINEAR && filter != TEX_FILTER_NEAREST)
      throw Error(B200_INVALID_ARGUMENT, "texture: bad filter");
    for (int w : {wrapS, wrapT})
      if (w < TEX_WRAP_REPEAT || w > TEX_WRAP_CLAMP_TO_EDGE) throw Error(B200_INVALID_ARGUMENT, "texture: bad wrap mode");
    if (int64_t(width) * height > int64_t(0xffffffffu)) throw Error(B200_INVALID_ARGUMENT, "texture: too large");
    *out = reinterpret_cast<b200_texture>(new TextureObj(dev, width, height, format, filter, wrapS, wrapT, data,
                                                         mipmaps != 0));
    return B200_NO_ERROR;
  } catch (const Error &e) {
    dev->lastError = e.what();
    return e.code;
  } catch (const std::exception &e) {
    dev->lastError = e.what();
    return B200_UNKNOWN_ERROR;
  }
}

int b200_texture_release(b200_texture t) {
  if (!t) return B200_INVALID_ARGUMENT;
  delete reinterpret_cast<TextureObj *>(t);
  return B200_NO_ERROR;
}

int b200_texture_levels(b200_texture t) { return t ? reinterpret_cast<TextureObj *>(t)->desc.maxLevel + 1 : 0; }

int b200_texture_sample(b200_texture t, int64_t n, const float *st, const float *footprint, float *out) {
  if (!t || n < 0 || (n > 0 && (!st || !footprint || !out))) return B200_INVALID_ARGUMENT;
  if (n == 0) return B200_NO_ERROR;
  if (n > (int64_t(1) << 31) - 1) return B200_INVALID_ARGUMENT;
  TextureObj *o = reinterpret_cast<TextureObj *>(t);
  cudaStream_t s = o->dev->stream;
  void *buf = nullptr;
  const size_t outOff = (size_t(n) * 12 + 15) & ~size_t(15);  // st (8 B each), footprints (4 B), then 16-aligned results
  const size_t bytes = outOff + size_t(n) * 16;
  if (cudaSetDevice(o->dev->dev) != cudaSuccess || cudaMallocAsync(&buf, bytes, s) != cudaSuccess)
    return B200_OUT_OF_MEMORY;
  float2 *dst = static_cast<float2 *>(buf);
  float *dfp = reinterpret_cast<float *>(dst + n);
  float4 *dout = reinterpret_cast<float4 *>(static_cast<char *>(buf) + outOff);
  bool ok = cudaMemcpyAsync(dst, st, size_t(n) * 8, cudaMemcpyHostToDevice, s) == cudaSuccess &&
            cudaMemcpyAsync(dfp, footprint, size_t(n) * 4, cudaMemcpyHostToDevice, s) == cudaSuccess;
  if (ok) {
    k_tex_sample<<<unsigned((n + 255) / 256), 256, 0, s>>>(o->dDesc, int(n), dst, dfp, dout);
    ok = cudaGetLastError() == cudaSuccess &&
         cudaMemcpyAsync(out, dout, size_t(n) * 16, cudaMemcpyDeviceToHost, s) == cudaSuccess;
  }
  cudaFreeAsync(buf, s);
  ok = cudaStreamSynchronize(s) == cudaSuccess && ok;
  return ok ? B200_NO_ERROR : B200_UNKNOWN_ERROR;
}

int b200_texture_read_level(b200_texture t, int level, void *dst, size_t bytes) {
  if (!t || !dst) return B200_INVALID_ARGUMENT;
  TextureObj *o = reinterpret_cast<TextureObj *>(t);
  if (level < 0 || level > o->desc.maxLevel) return B200_INVALID_ARGUMENT;
  const size_t need = size_t(std::max(o->desc.w >> level, 1)) * size_t(std::max(o->desc.h >> level, 1)) *
                      size_t(texelBytes(o->desc.format));
  if (bytes < need) return B200_INVALID_ARGUMENT;
  if (cudaSetDevice(o->dev->dev) != cudaSuccess ||
      cudaMemcpyAsync(dst, o->desc.level[level], need, cudaMemcpyDeviceToHost, o->dev->stream) != cudaSuccess ||
      cudaStreamSynchronize(o->dev->stream) != cudaSuccess)
    return B200_UNKNOWN_ERROR;
  return B200_NO_ERROR;
}

}  // extern "C"
