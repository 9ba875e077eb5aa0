// Structured-regular volume sampling, transfer function, macrocell interval
// iteration and the two ray-march integrators (SciVis colour, and opacity for
// shadow and AO rays), shared by the SciVis kernels.
//   integrateVolumeIntervalsGradient render/scivis/volumes.ispc:302-439
//   integrateVolumeIntervals         render/ao/volumes.ispc:32-240
//   LinearTransferFunction_get       volume/transferFunction/LinearTransferFunction.ispc:11-43
// Sampling and intervals follow this project's definitions of the Open VKL
// 2.0.1 behaviour (vertex-centred trilinear sampling, NaN outside the grid;
// intervals = maximal runs of non-empty 16^3-voxel macrocells; nominalDeltaT
// = the smallest grid spacing).
#pragma once
#include "kernels.h"
#include "pt_bsdf.cuh"

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

// transformRay(tRay, instance->rcp_xfm) (render/scivis/volumes.ispc:311-313):
// the ray in the volume's space, same t
B200_D Ray toVolume(const VolumeD &v, const Ray &r) {
  if (v.identity) return r;
  Ray t = r;
  t.org = xfmPoint(v.rcp, r.org);
  t.dir = xfmVector(v.rcp, r.dir);
  return t;
}

B200_D float sampleAt(const VolumeD &v, V3 p) {
  Taps t;
  fetchTaps(v, p, t);
  return tapsValue(t);
}

// Volume_getGradient (volume/Volume.ih:26-56) over Open VKL's gradient,
// restated as finite differences of the trilinear sample at one grid
// spacing: forward, or backward where the forward point leaves the grid; a
// NaN component becomes 1, as Volume_getGradient does.
B200_D V3 volumeGradient(const VolumeD &v, V3 p, float s0) {
  float g[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const float h = a == 0 ? v.spacing.x : (a == 1 ? v.spacing.y : v.spacing.z);
    V3 q = p;
    if (a == 0) q.x = __fadd_rn(q.x, h); else if (a == 1) q.y = __fadd_rn(q.y, h); else q.z = __fadd_rn(q.z, h);
    const float f = sampleAt(v, q);
    if (!isnan(f)) {
      g[a] = __fdiv_rn(__fsub_rn(f, s0), h);
    } else {
      V3 r = p;
      if (a == 0) r.x = __fsub_rn(r.x, h); else if (a == 1) r.y = __fsub_rn(r.y, h); else r.z = __fsub_rn(r.z, h);
      g[a] = __fdiv_rn(__fsub_rn(s0, sampleAt(v, r)), h);
    }
    if (isnan(g[a])) g[a] = 1.f;
  }
  return mk(g[0], g[1], g[2]);
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
B200_D float4 integrate(const VolumeD &v, const Ray &wray, float jitter, float samplingRate, float minContribution,
                        uint32_t &samples) {
  const Ray ray = toVolume(v, wray);
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

// Does [ray.tnear, ray.tfar] overlap the volume's grid box (the test that
// starts the interval iteration)?
B200_D bool volumeOverlaps(const VolumeD &v, const Ray &wray) {
  const Ray ray = toVolume(v, wray);
  IntervalIter it;
  it.init(v, ray.org, ray.dir, ray.tnear, ray.tfar);
  return !it.done;
}

// integrateVolumeIntervals (render/ao/volumes.ispc:251-352): colour and
// opacity accumulated front to back until 0.99, alpha += (1 - alpha) *
// (1 - exp(-a dt density)), colour += (1 - alpha) * op * rgb (COLOR); NaN
// samples are skipped inside the sample search.  Shadow and AO rays of the
// SciVis renderer use the opacity; the AO renderer composites both.
template <bool COLOR>
B200_D float4 volumeIntegrateAO(const VolumeD &v, const Ray &wray, float jitter, float samplingRate) {
  const Ray ray = toVolume(v, wray);
  IntervalIter it;
  it.init(v, ray.org, ray.dir, ray.tnear, ray.tfar);
  const float nominalDeltaT = fminf(v.spacing.x, fminf(v.spacing.y, v.spacing.z));
  float alpha = 0.f, distance = INFINITY, iuDistance = jitter, iuLength = 0.f, step = 0.f;
  float ilo = 0.f, ihi = INFINITY;
  V3 color = splat(0.f);
  for (int g = 0; g < (1 << 24) && alpha < 0.99f; g++) {
    float dt = 0.f, val = NAN;
    for (int h = 0; h < (1 << 24) && isnan(val); h++) {
      float emptySpace = 0.f;
      while (iuDistance > iuLength) {
        const float prevUpper = ihi;
        if (!it.next(v, ilo, ihi)) return make_float4(color.x, color.y, color.z, alpha);
        emptySpace += fmaxf(ilo - prevUpper, 0.f);
        iuDistance -= iuLength;
        step = nominalDeltaT / samplingRate;
        iuLength = (ihi - ilo) / step;
        distance = distance == INFINITY ? ilo : distance;
      }
      const float newDistance = ilo + iuDistance * step;
      Taps tp;
      fetchTaps(v, ray.org + newDistance * ray.dir, tp);
      val = tapsValue(tp);
      iuDistance += 1.f;
      dt = newDistance - distance - emptySpace;
      distance = newDistance;
    }
    const float4 c = tfGet(v, val);
    const float op = 1.f - expf(-c.w * dt * v.densityScale);
    if (COLOR) color = color + ((1.f - alpha) * op) * mk(c.x, c.y, c.z);
    alpha = alpha + (1.f - alpha) * op;
  }
  return make_float4(color.x, color.y, color.z, alpha);
}

B200_D float volumeAlpha(const VolumeD &v, const Ray &ray, float jitter, float samplingRate) {
  return volumeIntegrateAO<false>(v, ray, jitter, samplingRate).w;
}

}  // namespace
}  // namespace b200
