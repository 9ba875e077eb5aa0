// Light sampling and evaluation shared by the path tracer and the SciVis
// renderer:
//   QuadLight_sample / QuadLight_eval   lights/QuadLight.ispc:43-215
//     (spherical-quad solid-angle sampling, lights/SphericalQuadSampling.ih)
//   AmbientLight_sample / _eval         lights/AmbientLight.ispc:17-57
//   DirectionalLight_sample / _eval     lights/DirectionalLight.ispc:14-90
//   PointLight_sample / _eval           lights/PointLight.ispc:32-158 (sphere
//                                       lights; no intensity distribution)
//   SpotLight_sample / _eval            lights/SpotLight.ispc:26-170 (no
//                                       intensity distribution)
#pragma once
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

// uniformSampleCone (math/sampling.ih:92-97) about axis n
B200_D V3 sampleCone(V3 n, float cosAngle, float sx, float sy) {
  V3 dx, dy;
  frame(n, dx, dy);
  const float cosT = 1.f - sy * (1.f - cosAngle);
  const float sinT = sqrtf(fmaxf(0.f, 1.f - cosT * cosT));
  float sp, cp;
  sincosf(2.f * PI_F * sx, &sp, &cp);
  return dx * (cp * sinT) + dy * (sp * sinT) + n * cosT;
}

// Distant, spot and sphere lights sit outside the kernels' inlined code (a
// call when a scene has them): inlined, their code slowed the quad-lit path
// tracer by about 5 % (878 -> 828 Mrays/s on the 1080p workload, same box;
// 872 with them out of line).
__noinline__ __device__ LightSampleD sampleOtherLight(const LightD &L, V3 P, float sx, float sy) {
  LightSampleD r;
  if (L.type == LIGHT_DISTANT) {
    r.dir = L.dir;
    r.dist = INFINITY;
    r.pdf = L.conePdf;
    if (L.cosAngle < 0.99999988f) r.dir = sampleCone(L.dir, L.cosAngle, sx, sy);
    r.weight = L.radiance;  // irradiance: pdf / pdf cancel
    return r;
  }
  if (L.type == LIGHT_SPOT) {
    r.dir = L.position - P;
    if (L.radius > 0.f) {  // uniformSampleRing (math/sampling.ih:114-122) in the (c0, c90) frame
      const float rr = sqrtf((1.f - sx) * (L.innerRadius * L.innerRadius) + sx * (L.radius * L.radius));
      float sp, cp;
      sincosf(2.f * PI_F * sy, &sp, &cp);
      r.dir = L.edge1 * (rr * cp) + L.edge2 * (rr * sp) + r.dir;
    }
    const float dist2 = fdot(r.dir, r.dir);
    const float invdist = 1.f / sqrtf(dist2);
    r.dir = r.dir * invdist;
    r.dist = dist2 * invdist;
    const float cosAngle = -fdot(L.dir, r.dir);
    float w = fminf(fmaxf((cosAngle - L.cosAngle) * L.conePdf, 0.f), 1.f);
    if (L.radius > 0.f) {
      r.pdf = L.ppdf * (dist2 / fabsf(cosAngle));
      w = w / r.pdf;
      r.weight = L.radiance * w;
    } else {
      r.pdf = INFINITY;
      w *= fabsf(cosAngle);
      r.weight = L.intensity * ((invdist * invdist) * w);
    }
    return r;
  }
  if (L.type == LIGHT_SPHERE) {
    const V3 d = L.position - P;
    const float dist2 = fdot(d, d);
    const float invdist = 1.f / sqrtf(dist2);
    r.dir = d * invdist;
    r.dist = dist2 * invdist;
    r.pdf = INFINITY;
    const float sinTheta = L.radius * invdist;
    if (L.radius > 0.f && sinTheta > 0.005f) {
      if (sinTheta < 1.f) {
        const float cosTheta = sqrtf(1.f - sinTheta * sinTheta);
        V3 dx, dy;
        frame(r.dir, dx, dy);
        const float c = 1.f - sy * (1.f - cosTheta);
        const float sn = sqrtf(fmaxf(0.f, 1.f - c * c));
        float sp, cp;
        sincosf(2.f * PI_F * sx, &sp, &cp);
        r.dir = dx * (cp * sn) + dy * (sp * sn) + r.dir * c;
        r.pdf = 1.f / (2.f * PI_F * (1.f - cosTheta));
        r.dist = c * r.dist - sqrtf(fmaxf(0.f, L.radius * L.radius - (1.f - c * c) * dist2));
        r.weight = L.radiance * (1.f / r.pdf);
      } else {
        r.weight = splat(0.f);  // inside the sphere: it emits only outwards
      }
    } else {
      r.weight = L.intensity * (invdist * invdist);
    }
    return r;
  }
  r.weight = splat(0.f);
  r.dir = splat(0.f);
  r.dist = 0.f;
  r.pdf = 0.f;
  return r;
}

__noinline__ __device__ V3 evalOtherLight(const LightD &L, V3 P, V3 dir, float minDist, float maxDist, float &pdf) {
  pdf = 0.f;
  if (L.type == LIGHT_DISTANT) {
    if (INFINITY <= maxDist && L.cosAngle < 0.99999988f && fdot(L.dir, dir) > L.cosAngle) {
      pdf = L.conePdf;
      return L.radiance * L.conePdf;
    }
    return splat(0.f);
  }
  if (L.type == LIGHT_SPOT) {
    if (L.radius > 0.f) {  // the emitting ring
      const float cosAngle = -fdot(L.dir, dir);
      if (cosAngle > L.cosAngle) {
        const V3 vp = P - L.position;
        const float t = fdot(vp, L.dir) * (1.f / cosAngle);
        if (t > minDist && t <= maxDist) {
          const V3 vd = vp + dir * t;
          const float d2 = fdot(vd, vd);
          if (d2 < L.radius * L.radius && d2 > L.innerRadius * L.innerRadius) {
            pdf = L.ppdf * (t * t / fabsf(cosAngle));
            return L.radiance * fminf(fmaxf((cosAngle - L.cosAngle) * L.conePdf, 0.f), 1.f);
          }
        }
      }
    }
    return splat(0.f);
  }
  if (L.type == LIGHT_SPHERE) {
    const V3 A = L.position - P;
    const float sinTheta2 = L.radius * L.radius / fdot(A, A);
    if (L.radius > 0.f && sqrtf(sinTheta2) > 0.005f) {
      // intersectSphere (common/Intersect.ih:28-78): the entry distance
      const float rd2 = 1.f / fdot(dir, dir);
      const float projCO = fdot(A, dir) * rd2;
      const V3 perp = A - dir * projCO;
      const float l2 = fdot(perp, perp);
      if (l2 <= L.radius * L.radius) {
        const float t = projCO - sqrtf((L.radius * L.radius - l2) * rd2);
        if (t > minDist && t < maxDist) {
          pdf = 1.f / (2.f * PI_F * (1.f - sqrtf(1.f - sinTheta2)));
          return L.radiance;
        }
      }
    }
    return splat(0.f);
  }
  return splat(0.f);
}

B200_D LightSampleD sampleLight(const LightD &L, V3 P, V3 Ng, V3 Ns, float sx, float sy) {
  LightSampleD r;
  if (L.type >= LIGHT_DISTANT) return sampleOtherLight(L, P, sx, sy);
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
  if (L.type >= LIGHT_DISTANT) return evalOtherLight(L, P, dir, minDist, maxDist, pdf);
  pdf = fmaxf(fdot(Ns, dir), 0.f) / PI_F;
  return INFINITY <= maxDist ? L.radiance : splat(0.f);
}

B200_D float misH(float p1, float p2) {
  const float p = sqrf(p1) / (sqrf(p1) + sqrf(p2));
  return p1 > 1e17f ? 1.f : p;
}
B200_D float luminance(V3 c) { return luminanceV(c); }

}  // namespace
}  // namespace b200
