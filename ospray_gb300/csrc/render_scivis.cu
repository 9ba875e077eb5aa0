// SciVis renderer over worlds with surfaces (and optionally the volume in
// front of them), following
//   SciVis_renderSample        render/scivis/SciVis.ispc:24-222
//   SciVis_computeAO           render/scivis/SciVis.ispc:224-281
//   directIllumination, SciVis_computeShading, evaluateLights
//                              render/scivis/surfaces.ispc:17-128
//   evalMaterial               render/scivis/surfaces.ih:44-84
//   lightAlpha                 render/scivis/lightAlpha.ispc:19-122
//   integrateVolumeIntervals   render/ao/volumes.ispc:32-240 (shadow/AO rays)
//   integrateVolumeIntervalsGradient render/scivis/volumes.ispc:302-439
//                              (gradient shading of volume samples)
//   ray cones, map_maxDepth    render/RendererRenderTaskFn.inl:40-72
//   background, backplate      render/Renderer.ispc:19-40
// One thread per pixel.  ATTR (a mesh has vertex attributes or a material a
// map_kd): dg.color is the interpolated vertex colour and obj map_kd is
// looked up with the ray cone's footprint; otherwise dg.color is
// (1, 1, 1, 1).  A gradient-shaded volume sample passes its transfer-function
// RGBA.  Volume-only worlds without gradient shading use
// k_render_scivis_volume.
#include "kernels.h"
#include "lights.cuh"
#include "volume.cuh"

namespace b200 {

namespace {

struct SvBSDF {
  V3 diffuse, specular;
  float shininess;
  V3 transmission;
  float opacity;
  V3 albedo;  // diffuse + specular before the BRDF normalisation
};

// material slot of a surface hit; ~0u (no material) for volume samples
B200_D uint32_t svMaterialSlot(const Scene &sc, uint32_t entry) { return sc.entries[entry].materialID; }

// at (with footprint fp) addresses the obj map_kd; null: no lookup
B200_D SvBSDF svEvalMaterial(const ScivisSurfD &S, uint32_t mi, float4 color, const DGAttr *at = nullptr,
                             float fp = 0.f) {
  SvBSDF r;
  r.diffuse = mk(color.x, color.y, color.z);
  r.specular = splat(0.f);
  r.shininess = 10.f;
  r.transmission = splat(1.f - color.w);
  r.opacity = color.w;
  if (mi < uint32_t(S.nmats)) {
    const ScivisMatD m = S.mats[mi];
    if (m.isObj) {
      float d = m.d * color.w;
      r.diffuse = r.diffuse * mk(m.kd[0], m.kd[1], m.kd[2]);
      if (at && m.kdMap) {
        const float4 t = texGet(*m.kdMap, at->s, at->t, fp);
        r.diffuse = r.diffuse * mk(t.x, t.y, t.z);
        d *= t.w;
      }
      r.diffuse = r.diffuse * d;
      r.specular = d * mk(m.ks[0], m.ks[1], m.ks[2]);
      r.shininess = m.ns;
      r.transmission = mk(m.tf[0], m.tf[1], m.tf[2]) * d + splat(1.f - d);
      r.opacity = d;
    }
  }
  r.albedo = r.diffuse + r.specular;
  r.shininess *= 4.f;
  r.diffuse = r.diffuse * 0.318309886f;  // 1/pi
  r.specular = r.specular * ((r.shininess + 2.f) * 0.0795774715f *  // 1/(4 pi)
                             (1.f / (2.f - expf(r.shininess * -0.346573590f))));  // ln(2)/2
  return r;
}

// Transmission of a shadow or AO ray through translucent surfaces and the
// volume; any-hit when every material is opaque and there is no volume.
// cone: the shadow cone (width at the origin, dwdt), restarted from the
// origin's width after every surface (lightAlpha.ispc:30,105).
template <bool STATS, bool ATTR>
B200_D V3 svLightAlpha(const Scene &sc, const VolumeD &vol, const ScivisSurfD &S, float samplingRate, Ray ray,
                       PCG &rs, V3 weight, float quality, TraceStats *ts, float2 cone, float mipBias) {
  if (S.opaqueShadows) {
    HitRec h;
    return traceScene<true, STATS>(sc, ray, h, ts) ? splat(0.f) : splat(1.f);
  }
  V3 alpha = splat(1.f);
  const float orgTMax = ray.tfar;
  for (int g = 0; g < 1024; g++) {
    HitRec h;
    const bool hit = S.hasSurfaces && traceScene<false, STATS>(sc, ray, h, ts);
    if (S.hasVolume) {
      Ray vr = ray;
      vr.tfar = hit ? h.t : ray.tfar;
      if (volumeOverlaps(vol, vr)) {
        const float jitter = rs.getFloat();
        alpha = alpha * (1.f - volumeAlpha(vol, vr, jitter, samplingRate * quality));
      }
    }
    if (!hit) break;
    DGAttr at;
    const DG dg = ATTR ? postIntersect<true>(sc, ray, h, &at) : postIntersect(sc, ray, h);
    const uint32_t mi = svMaterialSlot(sc, dg.entry);
    if (ATTR) {
      const float fp = mi < uint32_t(S.nmats) && S.mats[mi].kdMap
                           ? pixelFootprint(cone.x + cone.y * h.t, ray.dir, dg, at, mipBias)
                           : 0.f;
      alpha = alpha * svEvalMaterial(S, mi, at.color, &at, fp).transmission;
    } else {
      alpha = alpha * svEvalMaterial(S, mi, make_float4(1.f, 1.f, 1.f, 1.f)).transmission;
    }
    ray.tnear = h.t + dg.epsilon;
    ray.tfar = orgTMax;
    if (luminance(alpha * weight) < S.minContribution) {
      alpha = splat(0.f);
      break;
    }
  }
  return alpha;
}

template <bool STATS, bool ATTR>
B200_D V3 svComputeAO(const SamplerTables *T, const Scene &sc, const VolumeD &vol, const ScivisSurfD &S,
                      float samplingRate, const DG &dg, int px, int py, uint32_t sampleZ, PCG &rs, TraceStats *ts,
                      float coneWidth, float mipBias) {
  const uint32_t accumID = sampleZ * uint32_t(S.aoSamples);
  const AOBasis B = aoBasis(dg, px, py);
  V3 hits = splat(0.f);
  for (int i = 0; i < S.aoSamples; i++) {
    const V3 dir = aoDirection(T, B, dg.Ns, accumID + uint32_t(i));
    if (dot(dir, dg.Ns) < 0.01f) {
      hits = hits + splat(1.f);
      continue;
    }
    Ray r;
    r.org = dg.P;
    r.tnear = dg.epsilon;
    r.dir = dir;
    r.tfar = S.aoRadius;
    hits = hits + (splat(1.f) - svLightAlpha<STATS, ATTR>(sc, vol, S, samplingRate, r, rs, splat(1.f), 0.1f, ts,
                                                          make_float2(coneWidth, 0.f), mipBias));
  }
  return splat(1.f) - hits * (1.f / float(S.aoSamples));
}

struct SvShading {
  V3 color, transmission;
  float opacity;
  V3 albedo;
};

// SciVis_computeShading (render/scivis/surfaces.ispc:90-128) with
// directIllumination: Blinn-Phong over the non-ambient lights (area lights
// sampled at their centre), hard shadows through lightAlpha, AO tinted by the
// ambient lights x pi.
// at / fp: the hit's attributes and footprint (map_kd); coneWidth: the ray
// cone's width at the hit (the shadow and AO cones start with it)
template <bool STATS, bool ATTR>
B200_D SvShading svComputeShading(const SamplerTables *T, const Scene &sc, const VolumeD &vol, const ScivisSurfD &S,
                                  float samplingRate, const DG &dg, uint32_t mi, float4 dgColor, V3 inDir, int x,
                                  int y, uint32_t sid, PCG &rs, TraceStats *ts, const DGAttr *at, float fp,
                                  float coneWidth, float mipBias) {
  const SvBSDF bsdf = svEvalMaterial(S, mi, dgColor, at, fp);
  V3 color = splat(0.f);
  for (int i = S.numVisibleOnly; i < S.nlights; i++) {
    const LightSampleD ls = sampleLight(S.lights[i], dg.P, dg.Ng, dg.Ns, 0.f, 0.f);
    if (maxc(ls.weight) > 0.f) {
      const float cosNL = fdot(ls.dir, dg.Ns);
      if (cosNL < 0.f) continue;
      const V3 H = fnormalize(ls.dir - inDir);
      const float cosNH = fdot(H, dg.Ns);
      const V3 specular = bsdf.specular * powf(cosNH, bsdf.shininess);
      const V3 diffuse = bsdf.diffuse * cosNL;
      const V3 contrib = (diffuse + specular) * ls.weight;
      if (S.shadows) {
        if (luminance(contrib) > S.minContribution) {
          V3 P = dg.P;
          if (fdot(dg.Ng, ls.dir) < 0.f) P = P - (2.f * dg.epsilon) * dg.Ng;
          Ray sr;
          sr.org = P;
          sr.tnear = 0.f;
          sr.dir = ls.dir;
          sr.tfar = ls.dist;
          const V3 la = svLightAlpha<STATS, ATTR>(sc, vol, S, samplingRate, sr, rs, contrib, 0.25f, ts,
                                                  make_float2(coneWidth, -coneWidth * (1.f / ls.dist)), mipBias);
          color = color + la * contrib;
        }
      } else {
        color = color + contrib;
      }
    }
  }
  const V3 aoColorPi = S.aoColor * 3.14159265358979323846f;
  V3 ao = splat(1.f);
  if (S.aoSamples > 0 && luminance(aoColorPi) > S.minContribution)
    ao = svComputeAO<STATS, ATTR>(T, sc, vol, S, samplingRate, dg, x, y, sid, rs, ts, coneWidth, mipBias);
  color = color + bsdf.diffuse * ao * aoColorPi;
  SvShading r;
  r.color = color;
  r.transmission = bsdf.transmission;
  r.opacity = bsdf.opacity;
  r.albedo = bsdf.albedo;
  return r;
}

// integrateVolumeIntervalsGradient (render/scivis/volumes.ispc:302-439) with
// gradient shading: a sample of non-zero opacity whose gradient does not
// vanish is shaded like a surface without material (colour = its transfer
// function RGBA, Ns = Ng = -normalize(gradient), epsilon = dt / 2) and
// blended into the sample by gradientShadingScale before the Beer-law
// opacity.  The shading's shadow and AO rays draw from the ray's sampler.
template <bool STATS, bool ATTR>
B200_D float4 integrateShaded(const SamplerTables *T, const Scene &sc, const VolumeD &vol, const ScivisSurfD &S,
                              float samplingRate, const Ray &wray, float jitter, int x, int y, uint32_t sid, PCG &rs,
                              uint32_t &samples, TraceStats *ts, float mipBias) {
  const Ray ray = toVolume(vol, wray);  // sampling in volume space, shading in world space
  SampleWalk w;
  w.init(vol, ray, jitter, samplingRate);
  V3 color = splat(0.f);
  float Tr = 1.f;
  float d, dt;
  for (int g = 0; g < (1 << 24) && Tr > S.minContribution && w.next(vol, d, dt); g++) {
    const V3 pos = ray.org + d * ray.dir;
    const float val = sampleAt(vol, pos);
    samples++;
    if (!isnan(val)) {
      float4 c = tfGet(vol, val);
      if (c.w > 0.f) {
        const V3 grad = volumeGradient(vol, pos, val);
        if (dot(grad, grad) > 1e-6f) {
          DG dg;
          dg.P = wray.org + d * wray.dir;
          const V3 ng = mk(-grad.x, -grad.y, -grad.z);
          dg.Ns = dg.Ng = fnormalize(vol.identity ? ng : xfmVectorT(vol.rcp, ng));
          dg.epsilon = dt / 2.f;
          dg.entry = ~0u;
          // (no cone width for volume samples, volumes.ispc:408-416)
          const SvShading sh = svComputeShading<STATS, ATTR>(T, sc, vol, S, samplingRate, dg, ~0u, c, wray.dir, x, y,
                                                             sid, rs, ts, nullptr, 0.f, 0.f, mipBias);
          const float a = 1.f - luminance(sh.transmission), f = vol.gradientShadingScale;
          c = make_float4(lerpF(f, c.x, sh.color.x), lerpF(f, c.y, sh.color.y), lerpF(f, c.z, sh.color.z),
                          lerpF(f, c.w, a));
        }
      }
      c.w = expf(-c.w * dt * vol.densityScale);
      const float k = Tr * (1.f - c.w);
      color = color + k * mk(c.x, c.y, c.z);
      Tr *= c.w;
    }
  }
  return make_float4(color.x, color.y, color.z, Tr);
}

// SHADED: the volume is gradient shaded (an instantiation of its own, so the
// common path keeps its registers)
template <bool STATS, bool SHADED, bool ATTR>
__global__ void __launch_bounds__(128) k_render_scivis_surfaces(const SamplerTables *T, Scene sc, VolumeD vol,
                                                                CameraD cam, PixelFilterD pf, ScivisParamsD p,
                                                                ScivisSurfD S, FrameD fb) {
  const int x = blockIdx.x * 16 + (threadIdx.x & 15);
  const int y = blockIdx.y * 8 + (threadIdx.x >> 4);
  TraceStats ts = {0, 0, 0, 0};
  if (x < fb.W && y < fb.H && pixelActive(fb, x, y)) {
    const float rcpW = fdiv(1.f, float(fb.W)), rcpH = fdiv(1.f, float(fb.H));
    const uint32_t start = uint32_t(fb.frameID * p.spp + 1);
    PixelOut acc = {0.f, 0.f, 0.f, 0.f, INFINITY, INVALID_ID, INVALID_ID, INVALID_ID};
    for (int s = 0; s < p.spp; s++) {
      const uint32_t sid = start + uint32_t(s);
      float2 scr;
      Ray ray = primaryRay(T, cam, pf, x, y, rcpW, rcpH, sid, &scr);
      sc.time = shutterTime(cam, scr.x, scr.y, 0.5f);  // RendererRenderTaskFn.inl:64: time sample 0.5
      const float cx = fmul(fadd(float(x), 0.5f), rcpW), cy = fmul(fadd(float(y), 0.5f), rcpH);
      if (p.maxDepth) ray.tfar = fminf(ray.tfar, texMaxDepth(p.maxDepth, cx, cy));
      const float2 cone = ATTR ? cameraCone(cam, scr.x, scr.y, rcpH) : make_float2(0.f, 0.f);
      float coneW = cone.x;
      PCG rs;
      rs.init(uint32_t(x + fb.W * y), sid);
      bool firstHit = true, allTrans = true;
      const float originalTFar = ray.tfar;
      V3 outColor = splat(0.f), outT = splat(1.f);
      float z = INFINITY;
      uint32_t prim = INVALID_ID, geom = INVALID_ID, inst = INVALID_ID;
      V3 sn = splat(0.f), sal = splat(0.f);
      uint32_t vsamples = 0;
      for (int g = 0; g < 1024; g++) {
        HitRec h;
        const bool hit = S.hasSurfaces && traceScene<false, STATS>(sc, ray, h, &ts);
        const float rayT = hit ? h.t : ray.tfar;
        if (S.hasVolume) {
          Ray vr = ray;
          vr.tfar = rayT;
          if (volumeOverlaps(vol, vr)) {
            const float jitter = rs.getFloat();
            const float4 vc = SHADED
                                  ? integrateShaded<STATS, ATTR>(T, sc, vol, S, p.samplingRate, vr, jitter, x, y, sid,
                                                                 rs, vsamples, &ts, p.mipBiasFactor)
                                  : integrate(vol, vr, jitter, p.samplingRate, S.minContribution, vsamples);
            outColor = outColor + outT * mk(vc.x, vc.y, vc.z);
            outT = outT * vc.w;
          }
        }
        if (S.visibleLights) {
          V3 lc = splat(0.f);
          for (int i = 0; i < S.nlights; i++) {
            const LightD &L = S.lights[i];
            if (!L.visible) continue;
            float lpdf;
            lc = lc + evalLight(L, ray.org, splat(0.f), ray.dir, ray.tnear, rayT, lpdf);
          }
          outColor = outColor + outT * lc;
        }
        if (firstHit || allTrans) z = rayT;
        if (!hit) {
          const float4 bg = p.backplate ? texGetScreen(*p.backplate, cx, cy)
                                        : make_float4(p.bg[0], p.bg[1], p.bg[2], p.bg[3]);
          outColor = outColor + outT * mk(bg.x, bg.y, bg.z);
          outT = outT * (1.f - bg.w);
          break;
        }
        DGAttr at;
        const DG dg = ATTR ? postIntersect<true>(sc, ray, h, &at) : postIntersect(sc, ray, h);
        const uint32_t mi = svMaterialSlot(sc, dg.entry);
        float fp = 0.f;
        if (ATTR) {
          coneW += cone.y * h.t;  // World.ih postIntersect: t from the ray's origin
          if (mi < uint32_t(S.nmats) && S.mats[mi].kdMap) fp = pixelFootprint(coneW, ray.dir, dg, at, p.mipBiasFactor);
        }
        const SvShading sh = svComputeShading<STATS, ATTR>(
            T, sc, vol, S, p.samplingRate, dg, mi, ATTR ? at.color : make_float4(1.f, 1.f, 1.f, 1.f), ray.dir, x, y,
            sid, rs, &ts, ATTR ? &at : nullptr, fp, coneW, p.mipBiasFactor);
        if (firstHit || allTrans) {
          sn = dg.Ns;
          sal = sh.albedo;
          prim = h.primID;
          geom = h.geomID;
          inst = h.instID;
          firstHit = false;
        }
        allTrans = allTrans && sh.opacity < S.minContribution;
        outColor = outColor + outT * sh.color;
        outT = outT * sh.transmission;
        if (luminance(outT) < S.minContribution) {
          outT = splat(0.f);
          break;
        }
        ray.tnear = h.t + dg.epsilon;
        ray.tfar = originalTFar;
      }
      acc.r += outColor.x;
      acc.g += outColor.y;
      acc.b += outColor.z;
      acc.a += 1.f - luminance(outT);
      acc.n = acc.n + sn;
      acc.al = acc.al + sal;
      if (fabsf(z) < fabsf(acc.z)) {
        acc.z = z;
        acc.primID = prim;
        acc.geomID = geom;
        acc.instID = inst;
      }
    }
    const float rspp = 1.f / float(p.spp);
    acc.r *= rspp;
    acc.g *= rspp;
    acc.b *= rspp;
    acc.a *= rspp;
    acc.n = acc.n * rspp;
    acc.al = acc.al * rspp;
    fbAccumulate(fb, x, y, acc);
  }
  if (STATS) flushStats(sc, ts);
}

}  // namespace

cudaError_t launchRenderScivisSurfaces(const SamplerTables *T, const Scene &sc, const VolumeD &vol, const CameraD &cam,
                                       const PixelFilterD &pf, const ScivisParamsD &p, const ScivisSurfD &S,
                                       const FrameD &fb, bool stats, cudaStream_t st, KernelTimer *kt) {
  dim3 grid((fb.W + 15) / 16, (fb.H + 7) / 8);
  KernelScope ks(kt, KK_SCIVIS, st);
  const bool shaded = S.hasVolume && vol.gradientShadingScale > 0.f;
  decltype(&k_render_scivis_surfaces<false, false, false>) k;
  if (S.attrs)
    k = stats ? (shaded ? k_render_scivis_surfaces<true, true, true> : k_render_scivis_surfaces<true, false, true>)
              : (shaded ? k_render_scivis_surfaces<false, true, true> : k_render_scivis_surfaces<false, false, true>);
  else
    k = stats ? (shaded ? k_render_scivis_surfaces<true, true, false> : k_render_scivis_surfaces<true, false, false>)
              : (shaded ? k_render_scivis_surfaces<false, true, false> : k_render_scivis_surfaces<false, false, false>);
  k<<<grid, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(T, sc, vol, cam, pf, p, S, fb);
  return cudaGetLastError();
}

}  // namespace b200
