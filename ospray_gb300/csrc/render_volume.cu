// SciVis volume rendering of a structured-regular volume through a
// piecewise-linear transfer function.
//   SciVis_renderSample              render/scivis/SciVis.ispc:24-222
//   integrateVolumeIntervalsGradient render/scivis/volumes.ispc:302-439
//   LinearTransferFunction_get       volume/transferFunction/LinearTransferFunction.ispc:11-43
// The reference samples and iterates the volume through Open VKL 2.0.1
// (not vendored).  Here: vertex-centred trilinear sampling (NaN outside the
// grid); intervals are the maximal runs of non-empty 16^3-voxel macrocells
// along the ray, found by a 3D DDA over a macrocell grid whose cells are
// empty when the transfer function's maximum opacity over the cell's value
// range is 0; nominalDeltaT = the smallest grid spacing.
#include "kernels.h"

namespace b200 {

namespace {

constexpr int CELL = 16;

// separable brick addressing: offset of coordinate i along x, j along y, k along z
B200_D uint32_t brickX(int i) { return uint32_t(i >> 3) * 512u + uint32_t(i & 7); }
B200_D size_t brickY(const VolumeD &v, int j) { return size_t(j >> 3) * size_t(v.bx) * 512u + size_t(j & 7) * 8u; }
B200_D size_t brickZ(const VolumeD &v, int k) {
  return size_t(k >> 3) * size_t(v.bx) * size_t(v.by) * 512u + size_t(k & 7) * 64u;
}

B200_D float vload(const VolumeD &v, int i, int j, int k) {
  return __ldg(v.data + brickX(i) + brickY(v, j) + brickZ(v, k));
}

// The 8 taps of a vertex-centred trilinear sample and its fractions, fetched
// ahead of their use so a ray keeps the next sample's loads in flight while it
// composites the current one.
struct Taps {
  float c[8];  // (x, y, z) = (0,0,0) (1,0,0) (0,1,0) (1,1,0) (0,0,1) (1,0,1) (0,1,1) (1,1,1)
  float fx, fy, fz;
  bool inside;
};

B200_D void fetchTaps(const VolumeD &v, V3 p, Taps &s) {
  const float u = (p.x - v.origin.x) / v.spacing.x, w1 = (p.y - v.origin.y) / v.spacing.y,
              w2 = (p.z - v.origin.z) / v.spacing.z;
  s.inside = u >= 0.f && w1 >= 0.f && w2 >= 0.f && u <= float(v.nx - 1) && w1 <= float(v.ny - 1) &&
             w2 <= float(v.nz - 1);
  // outside the grid the (clamped) taps are fetched but not used
  const int i = min(max(int(u), 0), v.nx - 2), j = min(max(int(w1), 0), v.ny - 2), k = min(max(int(w2), 0), v.nz - 2);
  s.fx = u - float(i);
  s.fy = w1 - float(j);
  s.fz = w2 - float(k);
  const uint32_t x0 = brickX(i), x1 = brickX(i + 1);
  const size_t y0 = brickY(v, j), y1 = brickY(v, j + 1), z0 = brickZ(v, k), z1 = brickZ(v, k + 1);
  const float *d = v.data;
  const size_t r00 = y0 + z0, r10 = y1 + z0, r01 = y0 + z1, r11 = y1 + z1;
  s.c[0] = __ldg(d + r00 + x0);
  s.c[1] = __ldg(d + r00 + x1);
  s.c[2] = __ldg(d + r10 + x0);
  s.c[3] = __ldg(d + r10 + x1);
  s.c[4] = __ldg(d + r01 + x0);
  s.c[5] = __ldg(d + r01 + x1);
  s.c[6] = __ldg(d + r11 + x0);
  s.c[7] = __ldg(d + r11 + x1);
}

// the trilinear value (NaN outside the grid)
B200_D float tapsValue(const Taps &s) {
  if (!s.inside) return NAN;
  const float c00 = lerpF(s.fx, s.c[0], s.c[1]);
  const float c10 = lerpF(s.fx, s.c[2], s.c[3]);
  const float c01 = lerpF(s.fx, s.c[4], s.c[5]);
  const float c11 = lerpF(s.fx, s.c[6], s.c[7]);
  return lerpF(s.fz, lerpF(s.fy, c00, c10), lerpF(s.fy, c01, c11));
}

B200_D float4 tfGet(const VolumeD &v, float value) {
  value = (value - v.vlo) * (1.f / (v.vhi - v.vlo));
  value = fminf(fmaxf(value, 0.f), 0x1.fffffep-1f);
  const int maxC = v.ncolor - 1;
  const float fc = value * float(maxC);
  const int ic = int(fc);
  const int ic1 = min(maxC, ic + 1);
  const float tc = fc - floorf(fc);
  const float3 a = v.tfColor[ic], b = v.tfColor[ic1];
  const int maxO = v.nopacity - 1;
  const float fo = value * float(maxO);
  const int io = int(fo);
  const float to = fo - floorf(fo);
  const float op = lerpF(to, __ldg(v.tfOpacity + io), __ldg(v.tfOpacity + min(maxO, io + 1)));
  return make_float4(lerpF(tc, a.x, b.x), lerpF(tc, a.y, b.y), lerpF(tc, a.z, b.z), op);
}

// maximal runs of non-empty macrocells along the ray
struct IntervalIter {
  float tEnd, t;
  int c[3], step[3];
  float tMax[3], tDelta[3];
  bool done;
  B200_D void init(const VolumeD &v, V3 org, V3 dir, float t0, float t1) {
    done = false;
    const float o[3] = {(org.x - v.origin.x) / v.spacing.x, (org.y - v.origin.y) / v.spacing.y,
                        (org.z - v.origin.z) / v.spacing.z};
    const float d[3] = {dir.x / v.spacing.x, dir.y / v.spacing.y, dir.z / v.spacing.z};
    const float hi[3] = {float(v.nx - 1), float(v.ny - 1), float(v.nz - 1)};
    const int ncell[3] = {v.cx, v.cy, v.cz};
    float ta = t0, tb = t1;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const float r = 1.f / d[k];
      float n = (0.f - o[k]) * r, f = (hi[k] - o[k]) * r;
      if (n > f) {
        const float tmp = n;
        n = f;
        f = tmp;
      }
      ta = n > ta ? n : ta;
      tb = f < tb ? f : tb;
    }
    if (!(ta < tb)) {
      done = true;
      return;
    }
    t = ta;
    tEnd = tb;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const float p = o[k] + t * d[k];
      int ci = int(floorf(p / CELL));
      ci = min(max(ci, 0), ncell[k] - 1);
      c[k] = ci;
      if (d[k] > 0.f) {
        step[k] = 1;
        tMax[k] = (float((ci + 1) * CELL) - o[k]) / d[k];
        tDelta[k] = float(CELL) / d[k];
      } else if (d[k] < 0.f) {
        step[k] = -1;
        tMax[k] = (float(ci * CELL) - o[k]) / d[k];
        tDelta[k] = -float(CELL) / d[k];
      } else {
        step[k] = 0;
        tMax[k] = INFINITY;
        tDelta[k] = INFINITY;
      }
    }
  }
  B200_D bool empty(const VolumeD &v) const {
    return __ldg(v.cellEmpty + (size_t(c[2]) * v.cy + c[1]) * v.cx + c[0]) != 0;
  }
  B200_D bool advance(const VolumeD &v) {
    int k = 0;
    if (tMax[1] < tMax[k]) k = 1;
    if (tMax[2] < tMax[k]) k = 2;
    const float tk = k == 0 ? tMax[0] : (k == 1 ? tMax[1] : tMax[2]);
    t = tk;
    if (!(t < tEnd)) return false;
    const int ncell = k == 0 ? v.cx : (k == 1 ? v.cy : v.cz);
#pragma unroll
    for (int a = 0; a < 3; a++)
      if (a == k) {
        c[a] += step[a];
        tMax[a] += tDelta[a];
      }
    const int ck = k == 0 ? c[0] : (k == 1 ? c[1] : c[2]);
    return ck >= 0 && ck < ncell;
  }
  B200_D bool next(const VolumeD &v, float &lo, float &hi) {
    if (done) return false;
    for (int g = 0; g < (1 << 20); g++) {
      if (!empty(v)) break;
      if (!advance(v)) {
        done = true;
        return false;
      }
    }
    lo = t;
    for (int g = 0; g < (1 << 20); g++) {
      if (!advance(v)) {
        done = true;
        break;
      }
      if (empty(v)) break;
    }
    hi = done ? tEnd : fminf(t, tEnd);
    return true;
  }
};

// Sample positions along the ray: the interval iteration and step rule of
// integrateVolumeIntervalsGradient; next() yields each sample's distance and
// its compositing step dt (distance since the previous sample minus the empty
// space skipped in between).
struct SampleWalk {
  IntervalIter it;
  float step, distance, iuDistance, iuLength, ilo, ihi;
  B200_D void init(const VolumeD &v, const Ray &ray, float jitter, float samplingRate) {
    it.init(v, ray.org, ray.dir, ray.tnear, ray.tfar);
    step = fminf(v.spacing.x, fminf(v.spacing.y, v.spacing.z)) / samplingRate;
    distance = INFINITY;
    iuDistance = jitter;
    iuLength = 0.f;
    ilo = 0.f;
    ihi = INFINITY;
  }
  B200_D bool next(const VolumeD &v, float &newDistance, float &dt) {
    float emptySpace = 0.f;
    while (iuDistance > iuLength) {
      const float prevUpper = ihi;
      if (!it.next(v, ilo, ihi)) return false;
      emptySpace += fmaxf(ilo - prevUpper, 0.f);
      iuDistance -= iuLength;
      iuLength = (ihi - ilo) / step;
      distance = distance == INFINITY ? ilo : distance;
    }
    newDistance = ilo + iuDistance * step;
    dt = newDistance - distance - emptySpace;
    iuDistance += 1.f;
    distance = newDistance;
    return true;
  }
};

// Front-to-back compositing (SciVis ray march with the transfer function,
// alpha = exp(-a * dt * densityScale)) until the transmittance falls to
// minContribution.
B200_D float4 integrate(const VolumeD &v, const Ray &ray, float jitter, float samplingRate, float minContribution,
                        uint32_t &samples) {
  SampleWalk w;
  w.init(v, ray, jitter, samplingRate);
  V3 color = splat(0.f);
  float T = 1.f;
  float d, dt;
  for (int g = 0; g < (1 << 24) && T > minContribution && w.next(v, d, dt); g++) {
    Taps tp;
    fetchTaps(v, ray.org + d * ray.dir, tp);
    const float val = tapsValue(tp);
    samples++;
    if (!isnan(val)) {
      float4 c = tfGet(v, val);
      c.w = expf(-c.w * dt * v.densityScale);
      const float k = T * (1.f - c.w);
      color = color + k * mk(c.x, c.y, c.z);
      T *= c.w;
    }
  }
  return make_float4(color.x, color.y, color.z, T);
}

#ifndef B200_VOL_MINBLOCKS
#define B200_VOL_MINBLOCKS 8  // 64 registers: 67.6 vs 66.4 (6 blocks) G samples/s on 512^3, 1024^2 x 4 spp
#endif
template <bool STATS>
__global__ void __launch_bounds__(128, B200_VOL_MINBLOCKS) k_render_scivis_volume(const SamplerTables *T, Scene sc, VolumeD vol,
                                                              CameraD cam, PixelFilterD pf, ScivisParamsD p,
                                                              FrameD fb) {
  const int x = blockIdx.x * 16 + (threadIdx.x & 15);
  const int y = blockIdx.y * 8 + (threadIdx.x >> 4);
  uint32_t samples = 0, rays = 0;
  if (x < fb.W && y < fb.H) {
    const float rcpW = fdiv(1.f, float(fb.W)), rcpH = fdiv(1.f, float(fb.H));
    const uint32_t start = uint32_t(fb.frameID * p.spp + 1);
    PixelOut acc = {0.f, 0.f, 0.f, 0.f, INFINITY, INVALID_ID, INVALID_ID, INVALID_ID};
    for (int s = 0; s < p.spp; s++) {
      const uint32_t sid = start + s;
      const Ray ray = primaryRay(T, cam, pf, x, y, rcpW, rcpH, sid);
      PCG rs;
      rs.init(uint32_t(x + fb.W * y), sid);
      const float jitter = rs.getFloat();
      rays++;
      const float4 vc = integrate(vol, ray, jitter, p.samplingRate, 0.001f, samples);
      float Tr = vc.w;
      const float r = vc.x + Tr * p.bg[0], g = vc.y + Tr * p.bg[1], b = vc.z + Tr * p.bg[2];
      Tr = Tr * (1.f - p.bg[3]);
      acc.r += r;
      acc.g += g;
      acc.b += b;
      acc.a += 1.f - (0.212671f * Tr + 0.715160f * Tr + 0.072169f * Tr);
    }
    const float rspp = 1.f / float(p.spp);
    acc.r *= rspp;
    acc.g *= rspp;
    acc.b *= rspp;
    acc.a *= rspp;
    fbAccumulate(fb, x, y, acc);
  }
  if (STATS) {
    TraceStats ts = {rays, samples, 0, 0};
    flushStats(sc, ts);
  }
}

// per macrocell: empty when the transfer function is transparent over its value range
__global__ void k_macrocells(VolumeD v, uint8_t *empty) {
  const int ci = blockIdx.x * blockDim.x + threadIdx.x;
  if (ci >= v.cx * v.cy * v.cz) return;
  const int a = ci % v.cx, b = (ci / v.cx) % v.cy, c = ci / (v.cx * v.cy);
  float lo = INFINITY, hi = -INFINITY;
  for (int k = c * CELL; k <= min(v.nz - 1, (c + 1) * CELL); k++)
    for (int j = b * CELL; j <= min(v.ny - 1, (b + 1) * CELL); j++)
      for (int i = a * CELL; i <= min(v.nx - 1, (a + 1) * CELL); i++) {
        const float x = vload(v, i, j, k);
        lo = fminf(lo, x);
        hi = fmaxf(hi, x);
      }
  const int maxO = v.nopacity - 1;
  const float ta = fminf(fmaxf((lo - v.vlo) / (v.vhi - v.vlo), 0.f), 1.f) * maxO;
  const float tb = fminf(fmaxf((hi - v.vlo) / (v.vhi - v.vlo), 0.f), 1.f) * maxO;
  float m = 0.f;
  for (int i = int(floorf(ta)); i <= min(maxO, int(ceilf(tb))); i++) m = fmaxf(m, v.tfOpacity[i]);
  empty[ci] = m <= 0.f ? 1 : 0;
}

// one thread per voxel of the bricked layout (padding voxels get 0)
__global__ void k_brick(VolumeD v, const float *linear, float *bricked, long long total) {
  const long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (o >= total) return;
  const long long b = o >> 9;
  const int w = int(o & 511);
  const long long bxy = (long long)v.bx * v.by;
  const int I = int(b % v.bx), J = int((b / v.bx) % v.by), K = int(b / bxy);
  const int i = I * 8 + (w & 7), j = J * 8 + ((w >> 3) & 7), k = K * 8 + (w >> 6);
  bricked[o] = (i < v.nx && j < v.ny && k < v.nz) ? linear[(size_t(k) * v.ny + j) * v.nx + i] : 0.f;
}

}  // namespace

size_t brickedVolumeBytes(int nx, int ny, int nz) {
  const size_t bx = (nx + 7) / 8, by = (ny + 7) / 8, bz = (nz + 7) / 8;
  return bx * by * bz * 512 * sizeof(float);
}

cudaError_t brickVolume(const VolumeD &v, const float *linear, float *bricked, cudaStream_t st) {
  const long long total = (long long)v.bx * v.by * v.bz * 512;
  k_brick<<<unsigned((total + 255) / 256), 256, 0, st>>>(v, linear, bricked, total);
  return cudaGetLastError();
}

cudaError_t buildMacrocells(VolumeD &v, uint8_t *empty, cudaStream_t st) {
  const int n = v.cx * v.cy * v.cz;
  k_macrocells<<<(n + 127) / 128, 128, 0, st>>>(v, empty);
  return cudaGetLastError();
}

cudaError_t launchRenderScivisVolume(const SamplerTables *T, const Scene &sc, const VolumeD &vol, const CameraD &cam,
                                     const PixelFilterD &pf, const ScivisParamsD &p, const FrameD &fb, bool stats,
                                     cudaStream_t st, KernelTimer *kt) {
  dim3 grid((fb.W + 15) / 16, (fb.H + 7) / 8);
  KernelScope ks(kt, KK_SCIVIS, st);
  if (stats)
    k_render_scivis_volume<true><<<grid, 128, 0, st>>>(T, sc, vol, cam, pf, p, fb);
  else
    k_render_scivis_volume<false><<<grid, 128, 0, st>>>(T, sc, vol, cam, pf, p, fb);
  return cudaGetLastError();
}

}  // namespace b200
