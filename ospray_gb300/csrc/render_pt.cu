// Path tracer: one thread per pixel runs the reference's samplePath for each
// of the pixel's samples and accumulates into the framebuffer.
//   PathTracer_renderPixel  render/pathtracer/PathTracer.ispc:75-216
//   samplePath              render/pathtracer/PathSampler.ispc:109-415
//   nextEventEstimation     render/pathtracer/NextEventEstimation.ispc:25-160
//   evaluateVirtualLights   render/pathtracer/VirtualLight.ispc:38-107
//   transparentShadow       render/pathtracer/TransparentShadow.ispc:18-85
//     (all materials here are opaque, so a shadow ray is an any-hit query)
//   misHeuristic            render/pathtracer/PathTracerUtil.ih:30-46
#include "kernels.h"
#include "pt_bsdf.cuh"

namespace b200 {

namespace {

// ---------------------------------------------------------------- lights
struct SphQuad {
  V3 e0, e1, z;
  float S, k, n0z, n2z, x0, x1, y0, y1, z0;
};

B200_D SphQuad sphQuad(V3 q0, V3 e0, V3 e1, V3 n, V3 P) {
  const float e0l = sqrtf(fdot(e0, e0)), e1l = sqrtf(fdot(e1, e1));
  SphQuad q;
  q.e0 = e0 * (1.f / e0l);
  q.e1 = e1 * (1.f / e1l);
  const V3 d = q0 - P;
  q.z0 = fdot(d, n);
  q.z = q.z0 > 0.f ? -n : n;
  q.z0 = -fabsf(q.z0);
  q.x0 = fdot(d, q.e0);
  q.y0 = fdot(d, q.e1);
  q.x1 = q.x0 + e0l;
  q.y1 = q.y0 + e1l;
  const V3 v00 = mk(q.x0, q.y0, q.z0), v01 = mk(q.x0, q.y1, q.z0), v10 = mk(q.x1, q.y0, q.z0),
           v11 = mk(q.x1, q.y1, q.z0);
  const V3 n0 = fnormalize(fcross(v00, v10)), n1 = fnormalize(fcross(v10, v11));
  const V3 n2 = fnormalize(fcross(v11, v01)), n3 = fnormalize(fcross(v01, v00));
  q.n0z = n0.z;
  q.n2z = n2.z;
  const float g0 = acosf(fminf(fmaxf(-fdot(n0, n1), -1.f), 1.f));
  const float g1 = acosf(fminf(fmaxf(-fdot(n1, n2), -1.f), 1.f));
  const float g2 = acosf(fminf(fmaxf(-fdot(n2, n3), -1.f), 1.f));
  const float g3 = acosf(fminf(fmaxf(-fdot(n3, n0), -1.f), 1.f));
  q.k = 2.f * PI_F - g2 - g3;
  q.S = fmaxf(0.f, g0 + g1 - q.k);
  return q;
}

B200_D V3 sampleSphQuad(const SphQuad &q, float sx, float sy) {
  const float au = sx * q.S + q.k;
  float sinau, cosau;
  sincosf(au, &sinau, &cosau);
  const float fu = (cosau * q.n0z - q.n2z) / sinau;
  const float sg = float(0.f < fu) - float(fu < 0.f);
  const float cu = fminf(fmaxf(1.f / sqrtf(fu * fu + sqrf(q.n0z)) * sg, -1.f), 1.f);
  const float x0 = -(cu * q.z0) / sqrtf(1.f - cu * cu);
  const float xu = fminf(fmaxf(x0, q.x0), q.x1);
  const float ds2 = sqrf(xu) + sqrf(q.z0);
  const float ds = sqrtf(ds2);
  const float h0 = q.y0 / sqrtf(ds2 + sqrf(q.y0));
  const float h1 = q.y1 / sqrtf(ds2 + sqrf(q.y1));
  const float hv = sy * (h1 - h0) + h0;
  const float hv2 = sqrf(hv);
  const float yv = hv2 < 1.f - 1e-4f ? (hv * ds) / sqrtf(1.f - hv2) : q.y1;
  return xu * q.e0 + yv * q.e1 + q.z0 * q.z;
}

B200_D float solveQuadratic(float A, float B, float C) {
  if (A == 0.f) return -C / B;
  float rad = B * B - 4.f * A * C;
  if (rad < 0.f) return 0.f;
  rad = sqrtf(rad);
  float root;
  if (B >= 0.f) {
    root = (-B - rad) / (2.f * A);
    if (root < 0.f || root > 1.f) root = 2.f * C / (-B - rad);
  } else {
    root = 2.f * C / (-B + rad);
    if (root < 0.f || root > 1.f) root = (-B + rad) / (2.f * A);
  }
  return root;
}

// Hart et al. 2020 bilinear warp toward the cosine-weighted corners
B200_D V3 cosineWeightedRNG(V3 q0, V3 e0, V3 e1, V3 P, V3 Ng, float sx, float sy) {
  const V3 wp0 = q0, wp1 = q0 + e0, wp2 = q0 + e1, wp3 = wp1 + e1;
  const float p0 = fmaxf(0.f, fdot(fnormalize(wp0 - P), Ng)), p1 = fmaxf(0.f, fdot(fnormalize(wp1 - P), Ng));
  const float p2 = fmaxf(0.f, fdot(fnormalize(wp2 - P), Ng)), p3 = fmaxf(0.f, fdot(fnormalize(wp3 - P), Ng));
  if (p0 + p2 == 0.f) return mk(sx, sy, 1.f);
  const float tot = p0 + p2 + p1 + p3;
  const float W00 = p0, W01 = p2, W10 = p1, W11 = p3;
  float u, v;
  {
    const float A = W10 + W11 - W01 - W00, B = 2.f * (W01 + W00);
    u = (A + B == 0.f) ? sx : solveQuadratic(A, B, -(W00 + W01 + W10 + W11) * sx);
  }
  {
    const float A = (1.f - u) * W01 + u * W11 - (1.f - u) * W00 - u * W10;
    const float B = 2.f * (1.f - u) * W00 + 2.f * u * W10;
    v = (A + B == 0.f) ? sy : solveQuadratic(A, B, -((1.f - u) * W01 + u * W11 + (1.f - u) * W00 + u * W10) * sy);
  }
  const float pdf = 4.f * ((1.f - u) * (1.f - v) * p0 + u * (1.f - v) * p1 + u * v * p3 + (1.f - u) * v * p2) / tot;
  return mk(u, v, pdf);
}

struct LightSampleD {
  V3 weight, dir;
  float dist, pdf;
};

B200_D LightSampleD sampleLight(const LightD &L, V3 P, V3 Ng, V3 Ns, float sx, float sy) {
  LightSampleD r;
  if (L.type == LIGHT_QUAD) {
    if (sx == 0.f && sy == 0.f) {
      const V3 p = L.position + L.edge1 * 0.5f + L.edge2 * 0.5f;
      const V3 d = p - P;
      const float dist = sqrtf(fdot(d, d));
      r.dir = d * (1.f / dist);
      r.dist = dist;
      const float cosd = fdot(L.nnormal, r.dir);
      r.pdf = L.ppdf * sqrf(dist) / fabsf(cosd);
      r.weight = L.radiance * (cosd > 0.f ? 1.f / r.pdf : 0.f);
      return r;
    }
    const SphQuad q = sphQuad(L.position, L.edge1, L.edge2, -L.nnormal, P);
    const V3 cw = cosineWeightedRNG(L.position, L.edge1, L.edge2, P, Ng, sx, sy);
    const V3 d = sampleSphQuad(q, cw.x, cw.y);
    const float dist = sqrtf(fdot(d, d));
    r.dir = d * (1.f / dist);
    r.dist = dist;
    const float cosd = fdot(L.nnormal, r.dir);
    r.pdf = q.S == 0.f ? 0.f : cw.z / q.S;
    r.weight = (cosd > 0.f && r.pdf != 0.f) ? L.radiance * (1.f / r.pdf) : splat(0.f);
    return r;
  }
  // ambient: cosine hemisphere about Ns
  V3 dx, dy;
  frame(Ns, dx, dy);
  float sp, cp;
  sincosf(2.f * PI_F * sx, &sp, &cp);
  const float cosT = sqrtf(sy), sinT = sqrtf(1.f - sy);
  r.dir = dx * (cp * sinT) + dy * (sp * sinT) + Ns * cosT;
  r.pdf = cosT / PI_F;
  r.dist = INFINITY;
  r.weight = L.radiance * (1.f / r.pdf);
  return r;
}

B200_D V3 evalLight(const LightD &L, V3 P, V3 Ns, V3 dir, float minDist, float maxDist, float &pdf) {
  pdf = 0.f;
  if (L.type == LIGHT_QUAD) {
    const float cosd = fdot(L.nnormal, dir);
    if (cosd <= 0.f) return splat(0.f);
    const V3 c = L.position - P;
    const V3 r = fcross(c, dir);
    const float rcosd = 1.f / cosd;
    const float u = fdot(r, L.edge1) * rcosd, v = -fdot(r, L.edge2) * rcosd;
    if (fminf(u, v) < 0.f || fmaxf(u, v) * L.ppdf > 1.f) return splat(0.f);
    const float dist = fdot(L.nnormal, c) * rcosd;
    if (dist <= minDist || dist > maxDist) return splat(0.f);
    const SphQuad q = sphQuad(L.position, L.edge1, L.edge2, -L.nnormal, P);
    if (q.S > 0.f) {
      pdf = 1.f / q.S;
      return L.radiance;
    }
    return splat(0.f);
  }
  pdf = fmaxf(fdot(Ns, dir), 0.f) / PI_F;
  return INFINITY <= maxDist ? L.radiance : splat(0.f);
}

B200_D float misH(float p1, float p2) {
  const float p = sqrf(p1) / (sqrf(p1) + sqrf(p2));
  return p1 > 1e17f ? 1.f : p;
}
B200_D float maxc(V3 v) { return fmaxf(fmaxf(v.x, v.y), v.z); }
B200_D float luminance(V3 c) { return 0.212671f * c.x + 0.715160f * c.y + 0.072169f * c.z; }

struct PtCtx {
  const SamplerTables *T;
  Scene sc;
  PtParamsD p;
  const MaterialD *mats;
  const LightD *lights;
  const float *lightCdf;
  const AlbedoTablesD *AT;
};

struct PathResult {
  V3 rgb;
  float alpha, z;
  uint32_t primID, geomID, instID;
};

// Per-thread shadow-ray requests of one NEE step, parked in shared memory
// (slot k of thread t at [k][t]) so they do not occupy registers while the
// thread traces them one by one through the common trace call.
constexpr int MAX_SHADOW = 4;
struct ShadowSlots {
  float4 a[MAX_SHADOW][TRACE_BLOCK];  // org.xyz, dist
  float4 b[MAX_SHADOW][TRACE_BLOCK];  // dir.xyz, contribution.x
  float2 c[MAX_SHADOW][TRACE_BLOCK];  // contribution.yz
};

enum Phase : int { PH_NEW_SAMPLE = 0, PH_EXTEND = 1, PH_SHADOW = 2, PH_DONE = 3 };

// Persistent threads: each thread takes a pixel from the work counter, runs
// its spp samples and accumulates it, then takes the next pixel.  Every loop
// iteration traces exactly one ray per thread -- an extension ray (closest
// hit) or a pending shadow ray (any hit) -- through the same call, so the
// threads of a warp traverse together; shading runs between traces.
template <bool STATS>
__global__ void __launch_bounds__(TRACE_BLOCK) k_render_pt(PtCtx c, CameraD cam, PixelFilterD pf, FrameD fb,
                                                           unsigned int *work) {
  __shared__ ShadowSlots slots;
  TraceStats ts = {0, 0, 0, 0};
  const int npix = fb.W * fb.H;
  const float rcpW = fdiv(1.f, float(fb.W)), rcpH = fdiv(1.f, float(fb.H));
  const int nl = c.p.numLights;
  // pixel state
  int pix = int(atomicAdd(work, 1u));
  int x = 0, y = 0, s = 0;
  uint32_t seed = 0;
  PixelOut acc;
  // sample state
  LDSampler ld;
  V3 throughput = splat(1.f), contribution = splat(0.f), lastP = splat(0.f), lastNs = splat(0.f);
  float alpha = 1.f, z = INFINITY, lastPdf = INFINITY;
  uint32_t prim = INVALID_ID, geom = INVALID_ID, inst = INVALID_ID;
  int depth = 0, lastNLS = 0;
  bool straightPath = true, firstBounceLight = true;
  Ray ray;
  // pending NEE step and continuation
  int nShadow = 0, shadowIdx = 0;
  V3 neeL = splat(0.f);
  bool hasNext = false;
  V3 nextDir = splat(0.f);
  float nextPdf = 0.f;
  int phase = pix < npix ? PH_NEW_SAMPLE : PH_DONE;
  if (phase == PH_NEW_SAMPLE) {
    x = pix % fb.W;
    y = pix / fb.W;
    seed = 0x49c5f37eu ^ uint32_t(fb.W * y + x);
    acc = {0.f, 0.f, 0.f, 0.f, INFINITY, INVALID_ID, INVALID_ID, INVALID_ID};
  }
  // warp-uniform loop: the vote is the reconvergence point of every
  // iteration; lanes without work left idle (and trace nothing) until the
  // whole warp is done
  for (int guard = 0; guard < (1 << 30); guard++) {
    if (!__any_sync(0xffffffffu, phase != PH_DONE)) break;
    if (phase == PH_NEW_SAMPLE) {
      if (s == c.p.spp) {
        const float rspp = 1.f / float(c.p.spp);
        acc.r *= rspp;
        acc.g *= rspp;
        acc.b *= rspp;
        acc.a *= rspp;
        fbAccumulate(fb, x, y, acc);
        pix = int(atomicAdd(work, 1u));
        if (pix >= npix) phase = PH_DONE;
        x = pix % fb.W;
        y = pix / fb.W;
        seed = 0x49c5f37eu ^ uint32_t(fb.W * y + x);
        acc = {0.f, 0.f, 0.f, 0.f, INFINITY, INVALID_ID, INVALID_ID, INVALID_ID};
        s = 0;
      }
    }
    if (phase == PH_NEW_SAMPLE) {
      const uint32_t sampleID = uint32_t(fb.frameID) * uint32_t(c.p.spp) + uint32_t(s);
      ld.init(c.T, seed, sampleID, sampleID * uint32_t(c.p.nFirst), 16, 16);
      uint32_t ss234[3];
      const float2 ps = ld.getNext5Samples(ss234);
      const float2 pfs = filterSample(pf, ps.x, ps.y);
      const float cx = fmul(fadd(float(x), 0.5f), rcpW), cy = fmul(fadd(float(y), 0.5f), rcpH);
      ray = cameraRay(cam, fadd(cx, fmul(pfs.x, rcpW)), fadd(cy, fmul(pfs.y, rcpH)));
      throughput = splat(1.f);
      contribution = splat(0.f);
      alpha = 1.f;
      z = INFINITY;
      prim = geom = inst = INVALID_ID;
      depth = 0;
      straightPath = firstBounceLight = true;
      lastP = ray.org;
      lastNs = ray.dir;
      lastPdf = INFINITY;
      lastNLS = 0;
      phase = PH_EXTEND;
    }
    // ---- the one trace of this iteration
    Ray tr = ray;
    const bool shadow = phase == PH_SHADOW;
    if (shadow) {
      const float4 a = slots.a[shadowIdx][threadIdx.x], b = slots.b[shadowIdx][threadIdx.x];
      tr.org = mk(a.x, a.y, a.z);
      tr.tnear = 0.f;
      tr.dir = mk(b.x, b.y, b.z);
      tr.tfar = a.w;
    }
    HitRec h;
    const bool active = phase != PH_DONE;
    const bool hit = traceRay<STATS>(c.sc, tr, h, shadow, active, &ts);
    if (!active) continue;
    bool endSample = false;
    if (shadow) {
      if (!hit) {
        const float4 b = slots.b[shadowIdx][threadIdx.x];
        const float2 cc = slots.c[shadowIdx][threadIdx.x];
        neeL = neeL + mk(b.w, cc.x, cc.y);
      }
      if (++shadowIdx < nShadow) continue;
      contribution = contribution + neeL;
      // continue the path (or end it) now that the NEE step is complete
      if (!hasNext) {
        endSample = true;
      } else {
        ray.org = lastP;
        ray.tnear = 0.f;
        ray.dir = nextDir;
        ray.tfar = INFINITY;
        lastPdf = nextPdf;
        depth++;
        if (maxc(throughput) > c.p.minContribution)
          phase = PH_EXTEND;
        else
          endSample = true;
      }
    } else {
      // ---- extension ray result: the body of samplePath's loop
      const float t = hit ? h.t : ray.tfar;
      const V3 wo = -ray.dir;
      if (depth == 0) z = t;
      if (!hit && straightPath) {
        alpha -= luminance(throughput) * (1.f - c.p.bg[3]);
        contribution = contribution + throughput * mk(c.p.bg[0], c.p.bg[1], c.p.bg[2]);
      }
      if (nl > 0) {  // evaluateVirtualLights
        const V3 d0 = lastP - ray.org;
        const float lo = sqrtf(fdot(d0, d0));
        float hiD = INFINITY;
        if (hit) {
          const V3 d1 = lastP - (ray.org + t * ray.dir);
          hiD = sqrtf(fdot(d1, d1));
        }
        const float selPdf = float(lastNLS) / float(nl);
        for (int i = 0; i < nl; i++) {
          const LightD &L = c.lights[i];
          if (straightPath && !L.visible) continue;
          float lpdf;
          const V3 rad = evalLight(L, lastP, lastNs, ray.dir, lo, hiD, lpdf);
          if (maxc(rad) > 0.f) {
            const float w = selPdf != 0.f ? misH(lastPdf, selPdf * lpdf) : 1.f;
            contribution = contribution + throughput * rad * w;
          }
        }
      }
      if (!hit || depth >= c.p.maxPathLength) {
        endSample = true;
      } else {
        const DG dg = postIntersect(c.sc, ray, h);
        if (depth == 0) {
          prim = h.primID;
          geom = h.geomID;
          inst = h.instID;
        }
        const Entry &e = c.sc.entries[h.entry];
        if (depth >= c.p.maxScatteringEvents || e.materialID >= uint32_t(c.p.numMaterials)) {
          endSample = true;
        } else {
          // shading frame from the instance tangent (makeShadingFrame)
          V3 U = e.identity ? mk(1.f, 0.f, 0.f) : mk(e.xfm.m[0], e.xfm.m[4], e.xfm.m[8]);
          U = fnormalize(U);
          const V3 Vv = fcross(dg.Ns, U);
          V3 fxv, fyv;
          if (fdot(Vv, Vv) > 0.f) {
            fyv = fnormalize(Vv);
            fxv = fcross(fyv, dg.Ns);
          } else {
            frame(dg.Ns, fxv, fyv);
          }
          Principled bsdf;
          bsdf.init(c.mats[e.materialID], fxv, fyv, dg.Ns, c.AT);
          if (bsdf.impSum == 0.f) {
            endSample = true;
          } else {
            ld.nextGroup();
            // next event estimation: light samples now, shadow rays next
            const int numLS = firstBounceLight ? c.p.nFirst : c.p.nIndirect;
            nShadow = 0;
            neeL = splat(0.f);
            for (int i = 0; i < numLS; i++) {
              float ss;
              const float2 sl = ld.get3LightSamples(uint32_t(i), numLS > 1, ss);
              int first = 0, len = nl;
              while (len > 0) {
                const int half = len >> 1, mid = first + half;
                if (ss < __ldg(c.lightCdf + mid)) {
                  len = half;
                } else {
                  first = mid + 1;
                  len -= half + 1;
                }
              }
              first = min(first, nl - 1);
              const float prob = __ldg(c.lightCdf + first) - (first == 0 ? 0.f : __ldg(c.lightCdf + first - 1));
              const float selProb = prob * float(numLS);
              LightSampleD ls = sampleLight(c.lights[first], dg.P, dg.Ng, dg.Ns, sl.x, sl.y);
              ls.weight = ls.weight * (1.f / selProb);
              ls.pdf *= selProb;
              if (maxc(ls.weight) <= 0.f || ls.pdf <= 0.f) continue;
              const BsdfEval fe = bsdf.eval(wo, ls.dir, c.AT);
              if (maxc(fe.value) <= 0.f) continue;
              V3 org = dg.P;
              if (fdot(dg.Ng, ls.dir) < 0.f) org = org - (2.f * dg.epsilon) * dg.Ng;
              const V3 cval = throughput * fe.value * ls.weight * misH(ls.pdf, fe.pdf);
              if (nShadow < MAX_SHADOW) {
                slots.a[nShadow][threadIdx.x] = make_float4(org.x, org.y, org.z, ls.dist);
                slots.b[nShadow][threadIdx.x] = make_float4(ls.dir.x, ls.dir.y, ls.dir.z, cval.x);
                slots.c[nShadow][threadIdx.x] = make_float2(cval.y, cval.z);
                nShadow++;
              } else {
                // more light samples than slots: trace this one in place
                Ray sr;
                sr.org = org;
                sr.tnear = 0.f;
                sr.dir = ls.dir;
                sr.tfar = ls.dist;
                HitRec sh;
                if (!traceRay<STATS>(c.sc, sr, sh, true, true, &ts)) neeL = neeL + cval;
              }
            }
            firstBounceLight = false;
            lastNLS = numLS;
            // continuation: BSDF sample and Russian roulette
            float ss;
            uint32_t uu3;
            const float2 sb = ld.getNext4Samples(ss, uu3);
            BsdfSample fs = bsdf.sample(wo, sb.x, sb.y, ss, c.AT);
            if (fdot(fs.wi, dg.Ng) < 0.f) fs.weight = splat(0.f);  // reflection lobes only
            hasNext = !(maxc(fs.weight) <= 0.f || fs.pdf <= 0.f);
            if (hasNext) {
              throughput = throughput * fs.weight;
              if (depth >= c.p.roulettePathLength) {
                const float rr = ld.finalizeDim3(uu3);
                const float contProb = fminf(maxc(throughput), 0.95f);
                if (rr > contProb)
                  hasNext = false;
                else
                  throughput = throughput * (1.f / contProb);
              }
            }
            if (hasNext) {
              if (!(ray.dir.x == fs.wi.x && ray.dir.y == fs.wi.y && ray.dir.z == fs.wi.z)) straightPath = false;
              nextDir = fs.wi;
              nextPdf = fs.pdf;
              lastP = dg.P;
              lastNs = dg.Ns;
            }
            if (nShadow > 0) {
              shadowIdx = 0;
              phase = PH_SHADOW;
            } else {
              contribution = contribution + neeL;
              if (!hasNext) {
                endSample = true;
              } else {
                ray.org = lastP;
                ray.tnear = 0.f;
                ray.dir = nextDir;
                ray.tfar = INFINITY;
                lastPdf = nextPdf;
                depth++;
                if (!(maxc(throughput) > c.p.minContribution)) endSample = true;
              }
            }
          }
        }
      }
    }
    if (endSample) {
      V3 rgb = contribution;
      float a = alpha;
      if (isnan(rgb.x) || isnan(rgb.y) || isnan(rgb.z)) {
        rgb = splat(0.f);
        a = 1.f;
      }
      acc.r += fminf(rgb.x, c.p.maxContribution);
      acc.g += fminf(rgb.y, c.p.maxContribution);
      acc.b += fminf(rgb.z, c.p.maxContribution);
      acc.a += a;
      if (fabsf(z) < fabsf(acc.z)) {
        acc.z = z;
        acc.primID = prim;
        acc.geomID = geom;
        acc.instID = inst;
      }
      s++;
      phase = PH_NEW_SAMPLE;
    }
  }
  if (STATS) flushStats(c.sc, ts);
}

// ---------------------------------------------------------------- albedo tables
// MicrofacetAlbedo_integrate / MicrofacetDielectricReflectionAlbedo_integrate:
// 32x32 stratified visible-normal samples per entry.
B200_D float albedoIntegrate(float cosO, float roughness, bool dielectric, float eta) {
  const float a = fmaxf(sqrf(roughness), 0.001f);
  cosO = fmaxf(cosO, 1e-6f);
  const V3 wo = mk(sqrtf(fmaxf(0.f, 1.f - cosO * cosO)), 0.f, cosO);
  float sum = 0.f;
  for (int i = 0; i < 32; i++)
    for (int j = 0; j < 32; j++) {
      const float sx = fminf((i + 0.5f) / 32.f, 1.f - 1e-6f), sy = fminf((j + 0.5f) / 32.f, 1.f - 1e-6f);
      float whPdf;
      const V3 wh = ggxSampleVisible(a, wo, whPdf, sx, sy);
      const float cosOH = fdot(wo, wh);
      const V3 wi = reflectV(wo, wh, cosOH);
      if (wi.z <= 0.f) continue;
      const float w = ggxG2(a, wo, wi, cosOH, fdot(wi, wh)) * rcpSafe(ggxG1(a, wo, cosOH));
      sum += dielectric ? fresnelDiel(cosOH, eta) * w : w;
    }
  return fminf(sum / 1024.f, 1.f);
}

__global__ void k_albedo_dir(AlbedoTablesD *T) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 32 * 32) {
    T->dir[i] = albedoIntegrate(float(i % 32) / 31.f, float(i / 32) / 31.f, false, 1.f);
  } else if (i < 32 * 32 + 16 * 16 * 16) {
    const int k = i - 32 * 32;
    const float t = float((k / 16) % 16) / 15.f;
    const float eta = (1.f - t) * (1.f / 3.f) + t * 1.f;
    T->reflDir[k] = albedoIntegrate(float(k % 16) / 15.f, float(k / 256) / 15.f, true, eta);
  }
}

// MicrofacetAlbedoTable_integrateAvg over each table row
__global__ void k_albedo_avg(AlbedoTablesD *T) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const float *row;
  int n;
  float *out;
  if (r < 32) {
    row = T->dir + r * 32;
    n = 32;
    out = T->avg + r;
  } else if (r < 32 + 256) {
    row = T->reflDir + (r - 32) * 16;
    n = 16;
    out = T->reflAvg + (r - 32);
  } else {
    return;
  }
  float sum = 0.f;
  for (int i = 0; i < 1025; i++) {
    const float c = float(i) / 1024.f;
    sum += interp1(c * (n - 1), row, n) * c * ((i == 0 || i == 1024) ? 0.5f : 1.f);
  }
  *out = fminf(2.f * (sum / 1024.f), 1.f);
}

}  // namespace

cudaError_t computeAlbedoTables(AlbedoTablesD *T, cudaStream_t st) {
  k_albedo_dir<<<(32 * 32 + 4096 + 127) / 128, 128, 0, st>>>(T);
  k_albedo_avg<<<(32 + 256 + 127) / 128, 128, 0, st>>>(T);
  return cudaGetLastError();
}

cudaError_t launchRenderPT(const SamplerTables *T, const Scene &sc, const CameraD &cam, const PixelFilterD &pf,
                           const PtParamsD &p, const MaterialD *mats, const LightD *lights, const float *lightCdf,
                           const AlbedoTablesD *AT, const FrameD &fb, bool stats, unsigned int *work,
                           cudaStream_t st) {
  PtCtx c = {T, sc, p, mats, lights, lightCdf, AT};
  // persistent grid: as many blocks as fit on the device at once
  static int blocksPerSM[2] = {0, 0}, numSMs = 0;
  if (!numSMs) {
    int dev;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&numSMs, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocksPerSM[0], k_render_pt<false>, TRACE_BLOCK,
                                                  TRACE_SMEM_BYTES);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocksPerSM[1], k_render_pt<true>, TRACE_BLOCK, TRACE_SMEM_BYTES);
  }
  const int npix = fb.W * fb.H;
  const int maxBlocks = (npix + TRACE_BLOCK - 1) / TRACE_BLOCK;
  const int blocks = std::max(1, std::min(maxBlocks, numSMs * std::max(1, blocksPerSM[stats ? 1 : 0])));
  cudaError_t err = cudaMemsetAsync(work, 0, sizeof(unsigned int), st);
  if (err != cudaSuccess) return err;
  if (stats)
    k_render_pt<true><<<blocks, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(c, cam, pf, fb, work);
  else
    k_render_pt<false><<<blocks, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(c, cam, pf, fb, work);
  return cudaGetLastError();
}

}  // namespace b200
