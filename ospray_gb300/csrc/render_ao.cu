// Ray-query entry kernel (rtcIntersect/rtcOccluded over a ray array) and the
// AO renderer.
//   AORenderer_renderSample    modules/cpu/render/ao/AORenderer.ispc:23-149
//   AORenderer_computeShading  modules/cpu/render/ao/surfaces.ispc:44-74
//   computeAO                  modules/cpu/render/util.ispc:12-54
#include "kernels.h"
#include "render_common.cuh"
#include "volume.cuh"

namespace b200 {


namespace {

__global__ void k_trace(Scene sc, const float4 *rays, long long n, int occlusion, float *outF, uint32_t *outI) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 a = rays[2 * i], b = rays[2 * i + 1];
  Ray r;
  r.org = mk(a.x, a.y, a.z);
  r.tnear = a.w;
  r.dir = mk(b.x, b.y, b.z);
  r.tfar = b.w;
  HitRec h;
  if (occlusion) {
    outF[6 * i] = traceScene<true>(sc, r, h) ? 1.f : 0.f;
    return;
  }
  const bool hit = traceScene<false>(sc, r, h);
  float *F = outF + 6 * i;
  uint32_t *I = outI + 3 * i;
  if (!hit) {
    F[0] = INFINITY;
    F[1] = F[2] = F[3] = F[4] = F[5] = 0.f;
    I[0] = I[1] = I[2] = INVALID_ID;
    return;
  }
  F[0] = h.t;
  F[1] = h.u;
  F[2] = h.v;
  F[3] = h.Ng.x;
  F[4] = h.Ng.y;
  F[5] = h.Ng.z;
  I[0] = h.primID;
  I[1] = h.geomID;
  I[2] = h.instID;
}

template <bool STATS>
B200_D float computeAO(const SamplerTables *T, const Scene &sc, const DG &dg, int sampleCnt, float aoRadius, int px, int py,
                       uint32_t sid, TraceStats *ts) {
  const uint32_t accumID = sid * uint32_t(sampleCnt);
  const AOBasis B = aoBasis(dg, px, py);
  int hits = 0;
  for (int i = 0; i < sampleCnt; i++) {
    const V3 dir = aoDirection(T, B, dg.Ns, accumID + i);
    if (dot(dir, dg.Ns) < 0.01f) {
      hits++;
      continue;
    }
    Ray r;
    r.org = dg.P;
    r.tnear = dg.epsilon;
    r.dir = dir;
    r.tfar = aoRadius;
    HitRec h;
    if (traceScene<true, STATS>(sc, r, h, ts)) hits++;
  }
  return 1.f - float(hits) / float(sampleCnt);
}

// Resident blocks per SM the single-frame AO kernel is compiled for.  3 (a
// bound of 170 registers; uncapped the kernel takes 171, one too many for a
// third block) measured best on the 512^2 AO workload: 1,417 Mrays/s at 3
// blocks against 1,290 at 2 and 1,313 / 1,268 / 1,240 when capped for
// 4 / 5 / 6 blocks (those caps spill the traversal and shading state).
#ifndef B200_AO_MINBLOCKS
#define B200_AO_MINBLOCKS 3
#endif
// getSurfaceColor (render/ao/surfaces.ispc:17-42): an obj material's kd x
// map_kd rgb (d x map alpha) times the vertex colour; white and opaque
// without an obj material
B200_D float4 aoSurfaceColor(const AOParamsD &p, uint32_t mi, const DGAttr &at, float fp) {
  V3 c = splat(1.f);
  float op = 1.f;
  if (mi < uint32_t(p.nmats) && p.mats[mi].isObj) {
    const ScivisMatD &m = p.mats[mi];
    c = mk(m.kd[0], m.kd[1], m.kd[2]);
    if (m.kdMap) {
      const float4 t = texGet(*m.kdMap, at.s, at.t, fp);
      c = c * mk(t.x, t.y, t.z);
      op *= t.w;
    }
    op *= m.d;
  }
  return make_float4(c.x * at.color.x, c.y * at.color.y, c.z * at.color.z, op * at.color.w);
}

// VOL: the scene's volume is composited in front of each layer
// (integrateVolumeIntervals, render/ao/volumes.ispc:251-352).
// SURF: surface colours and opacities (materials, vertex attributes, maps
// with ray-cone footprints; AORenderer_computeShading surfaces.ispc:44-77);
// without it every surface is white and opaque.
// The renderer's map_maxDepth limits the camera ray and map_backplate
// replaces the background colour, both at the pixel centre.
template <bool STATS, bool VOL, bool SURF>
__global__ void __launch_bounds__(128, B200_AO_MINBLOCKS) k_render_ao(const SamplerTables *T, Scene sc, CameraD cam, PixelFilterD pf, AOParamsD p, FrameD fb, VolumeD vol) {
  const int x = blockIdx.x * 16 + (threadIdx.x & 15);
  const int y = blockIdx.y * 8 + (threadIdx.x >> 4);
  TraceStats ts = {0, 0, 0, 0};
  if (x >= fb.W || y >= fb.H || !pixelActive(fb, x, y)) {
    if (STATS) flushStats(sc, ts);
    return;
  }
  const float rcpW = fdiv(1.f, float(fb.W)), rcpH = fdiv(1.f, float(fb.H));
  const uint32_t start = uint32_t(fb.frameID * p.spp + 1);
  float ar = 0.f, ag = 0.f, ab = 0.f, aa = 0.f;
  PixelOut acc = {0, 0, 0, 0, INFINITY, INVALID_ID, INVALID_ID, INVALID_ID};
  for (int s = 0; s < p.spp; s++) {
    const uint32_t sid = start + s;
    float2 scr;
    Ray ray = primaryRay(T, cam, pf, x, y, rcpW, rcpH, sid, &scr);
    sc.time = shutterTime(cam, scr.x, scr.y, 0.5f);  // RendererRenderTaskFn.inl:64: time sample 0.5
    if (p.maxDepth)
      ray.tfar = fminf(ray.tfar, texMaxDepth(p.maxDepth, fmul(fadd(float(x), 0.5f), rcpW),
                                             fmul(fadd(float(y), 0.5f), rcpH)));
    const float2 cone = SURF ? cameraCone(cam, scr.x, scr.y, rcpH) : make_float2(0.f, 0.f);
    float coneW = cone.x;
    const float tfar0 = ray.tfar;
    float o[4] = {0.f, 0.f, 0.f, 0.f};
    bool first = true;
    float z = INFINITY;
    uint32_t prim = INVALID_ID, geom = INVALID_ID, inst = INVALID_ID;
    V3 sn = splat(0.f), sal = splat(0.f);
    PCG rs;
    if (VOL) rs.init(uint32_t(x + fb.W * y), sid);
    for (int layer = 0; layer < 64 && o[3] < 0.99f; layer++) {
      HitRec h;
      const bool hit = traceScene<false, STATS>(sc, ray, h, &ts);
      if (VOL) {
        Ray vr = ray;
        vr.tfar = hit ? h.t : ray.tfar;
        if (volumeOverlaps(vol, vr)) {
          const float jitter = rs.getFloat();
          const float4 vc = volumeIntegrateAO<true>(vol, vr, jitter, p.volumeSamplingRate);
          const float f = fsub(1.f, o[3]);
          o[0] = fadd(o[0], fmul(f, vc.x));
          o[1] = fadd(o[1], fmul(f, vc.y));
          o[2] = fadd(o[2], fmul(f, vc.z));
          o[3] = fadd(o[3], fmul(f, vc.w));
        }
      }
      float bl[4];
      if (hit) {
        DGAttr at;
        const DG dg = SURF ? postIntersect<true>(sc, ray, h, &at) : postIntersect(sc, ray, h);
        float4 sc4 = make_float4(1.f, 1.f, 1.f, 1.f);
        if (SURF) {
          coneW += cone.y * h.t;  // World.ih postIntersect: t from the ray's origin
          const uint32_t mi = sc.entries[h.entry].materialID;
          const float fp = mi < uint32_t(p.nmats) && p.mats[mi].isObj && p.mats[mi].kdMap
                               ? pixelFootprint(coneW, ray.dir, dg, at, p.mipBiasFactor)
                               : 0.f;
          sc4 = aoSurfaceColor(p, mi, at, fp);
        }
        float intensity = fabsf(dot(dg.Ns, ray.dir));
        if (SURF) intensity = fmul(intensity, sc4.w);
        if (p.aoSamples > 0 && p.aoIntensity > 0.01f) {
          const float ao = computeAO<STATS>(T, sc, dg, p.aoSamples, p.aoRadius, x, y, sid, &ts);
          intensity = fmul(intensity, fadd(fsub(1.f, p.aoIntensity), fmul(ao, p.aoIntensity)));
        }
        if (SURF) {
          bl[0] = fmul(sc4.x, intensity);
          bl[1] = fmul(sc4.y, intensity);
          bl[2] = fmul(sc4.z, intensity);
          bl[3] = sc4.w;
        } else {
          bl[0] = bl[1] = bl[2] = intensity;
          bl[3] = 1.f;
        }
        if (first) {
          z = h.t;
          prim = h.primID;
          geom = h.geomID;
          inst = h.instID;
          sn = dg.Ns;
          sal = mk(sc4.x, sc4.y, sc4.z);  // AORenderer_computeShading: albedo = surface colour
        }
        ray.tnear = fadd(h.t, dg.epsilon);
        ray.tfar = tfar0;
      } else {
        const float4 bg = p.backplate ? texGetScreen(*p.backplate, fmul(fadd(float(x), 0.5f), rcpW),
                                                     fmul(fadd(float(y), 0.5f), rcpH))
                                      : make_float4(p.bg[0], p.bg[1], p.bg[2], p.bg[3]);
        bl[0] = bg.x;
        bl[1] = bg.y;
        bl[2] = bg.z;
        bl[3] = bg.w;
        if (first) {
          z = ray.tfar;
          sn = ray.dir;
          sal = mk(bg.x, bg.y, bg.z);
        }
      }
      const float f = fsub(1.f, o[3]);
      for (int k = 0; k < 4; k++) o[k] = fadd(o[k], fmul(f, bl[k]));
      first = false;
      if (!hit) break;
    }
    ar = fadd(ar, o[0]);
    ag = fadd(ag, o[1]);
    ab = fadd(ab, o[2]);
    aa = fadd(aa, o[3]);
    acc.n = add(acc.n, sn);
    acc.al = add(acc.al, sal);
    if (fabsf(z) < fabsf(acc.z)) {
      acc.z = z;
      acc.primID = prim;
      acc.geomID = geom;
      acc.instID = inst;
    }
  }
  const float rspp = fdiv(1.f, float(p.spp));
  acc.r = fmul(ar, rspp);
  acc.g = fmul(ag, rspp);
  acc.b = fmul(ab, rspp);
  acc.a = fmul(aa, rspp);
  acc.n = mul(acc.n, rspp);
  acc.al = mul(acc.al, rspp);
  fbAccumulate(fb, x, y, acc);
  if (STATS) flushStats(sc, ts);
}

}  // namespace

cudaError_t launchTrace(const Scene &sc, const float4 *rays, long long n, int occlusion, float *outF, uint32_t *outI,
                        cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int bs = 128;
  k_trace<<<unsigned((n + bs - 1) / bs), TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(sc, rays, n, occlusion, outF, outI);
  return cudaGetLastError();
}

// Renderer_pick (render/Renderer.ispc:43-95): the camera ray at the screen
// position with the lens centre, no depth limit, closest hit; the position is
// org + dir * t.  One warp is launched so the warp-cooperative traversal has
// its usual shape; lane 0 carries the ray.
__global__ void k_pick(Scene sc, CameraD cam, float sx, float sy, uint32_t *out) {
  const bool active = threadIdx.x == 0;
  float mx = sx, my = sy;  // the pick position stands for the pixel centre of a stereo split
  const float eye = cameraScreen(cam, mx, my, sx, sy);
  Ray r = cameraRay(cam, mx, my, make_float2(0.f, 0.f), eye);
  HitRec h;
  bool hit = false;
  if (active) hit = traceScene<false>(sc, r, h);
  if (!active) return;
  out[0] = hit ? 1u : 0u;
  if (hit) {
    const V3 p = add(r.org, mul(r.dir, h.t));
    out[1] = __float_as_uint(p.x);
    out[2] = __float_as_uint(p.y);
    out[3] = __float_as_uint(p.z);
    out[4] = h.instID;
    out[5] = h.geomID;
    out[6] = h.primID;
  } else {
    out[1] = out[2] = out[3] = 0u;
    out[4] = out[5] = out[6] = INVALID_ID;
  }
}

cudaError_t launchPick(const Scene &sc, const CameraD &cam, float sx, float sy, uint32_t *out, cudaStream_t st) {
  k_pick<<<1, 32, TRACE_SMEM_BYTES, st>>>(sc, cam, sx, sy, out);
  return cudaGetLastError();
}

cudaError_t launchRenderAO(const SamplerTables *T, const Scene &sc, const CameraD &cam, const PixelFilterD &pf, const AOParamsD &p,
                           const FrameD &fb, bool stats, cudaStream_t st, KernelTimer *kt, const VolumeD *vol,
                           bool surf) {
  dim3 grid((fb.W + 15) / 16, (fb.H + 7) / 8);
  KernelScope ks(kt, KK_AO, st);
  const VolumeD v = vol ? *vol : VolumeD{};
  decltype(&k_render_ao<false, false, false>) k;
  if (surf)
    k = stats ? (vol ? k_render_ao<true, true, true> : k_render_ao<true, false, true>)
              : (vol ? k_render_ao<false, true, true> : k_render_ao<false, false, true>);
  else
    k = stats ? (vol ? k_render_ao<true, true, false> : k_render_ao<true, false, false>)
              : (vol ? k_render_ao<false, true, false> : k_render_ao<false, false, false>);
  k<<<grid, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(T, sc, cam, pf, p, fb, v);
  return cudaGetLastError();
}

}  // namespace b200
