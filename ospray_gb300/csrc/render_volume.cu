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
#include "volume.cuh"

namespace b200 {

namespace {

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
  if (x < fb.W && y < fb.H && pixelActive(fb, x, y)) {
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
