// Device principled BSDF (plastic + conductor lobes), GGX, Fresnel,
// microfacet albedo tables and the quad / ambient lights for the path tracer.
//   render/materials/Principled.ispc:81-429, PrincipledShared.h:130-163
//   render/bsdfs/MultiBSDF.ih, OrenNayar.ih:13-63, MicrofacetDielectricLayer.ih,
//   MicrofacetConductor.ih:17-146, GGXDistribution.ih:17-144,
//   MicrofacetDistribution.ih:17-22, Fresnel.ih:19-83,226-288, Optics.ih,
//   MicrofacetAlbedo.ih, MicrofacetAlbedoTables.{ih,ispc}, math/interpolation.ih
//   lights/QuadLight.ispc:43-215, lights/SphericalQuadSampling.ih,
//   lights/AmbientLight.ispc:17-57
#pragma once
#include "render_common.cuh"

namespace b200 {

constexpr float PI_F = 3.14159265358979323846f;
constexpr float MAT_EPS = 1e-6f;

struct MaterialD {
  float r, g, b, roughness, metallic;
};

// GGX albedo tables: dir 32x32 (cosThetaO fastest, roughness), avg 32;
// dielectric reflection: dir 16^3 (cos, eta in [1/3,1], roughness), avg 16^2
struct AlbedoTablesD {
  float dir[32 * 32];
  float avg[32];
  float reflDir[16 * 16 * 16];
  float reflAvg[16 * 16];
};

B200_D float sqrf(float x) { return x * x; }
B200_D float clamp01f(float x) { return fminf(fmaxf(x, 0.f), 1.f); }
B200_D float rcpSafe(float x) { return 1.f / (fabsf(x) < 1e-8f ? copysignf(1e-8f, x) : x); }
B200_D float lerpF(float f, float a, float b) { return (1.f - f) * a + f * b; }

B200_D float interp1(float x, const float *f, int n) {
  const float xc = fminf(fmaxf(x, 0.f), float(n - 1));
  const float s = xc - floorf(xc);
  const int x0 = min(int(xc), n - 1), x1 = min(x0 + 1, n - 1);
  return lerpF(s, __ldg(f + x0), __ldg(f + x1));
}
B200_D float interp2(float px, float py, const float *f, int n) {
  const float xc = fminf(fmaxf(px, 0.f), float(n - 1)), yc = fminf(fmaxf(py, 0.f), float(n - 1));
  const float sx = xc - floorf(xc), sy = yc - floorf(yc);
  const int x0 = min(int(xc), n - 1), x1 = min(x0 + 1, n - 1);
  const int y0 = min(int(yc), n - 1), y1 = min(y0 + 1, n - 1);
  const float f0 = lerpF(sx, __ldg(f + x0 + y0 * n), __ldg(f + x1 + y0 * n));
  const float f1 = lerpF(sx, __ldg(f + x0 + y1 * n), __ldg(f + x1 + y1 * n));
  return lerpF(sy, f0, f1);
}
B200_D float interp3(float px, float py, float pz, const float *f, int n) {
  const float zc = fminf(fmaxf(pz, 0.f), float(n - 1));
  const float sz = zc - floorf(zc);
  const int z0 = min(int(zc), n - 1), z1 = min(z0 + 1, n - 1);
  return lerpF(sz, interp2(px, py, f + z0 * n * n, n), interp2(px, py, f + z1 * n * n, n));
}
B200_D float tabEval(const AlbedoTablesD *T, float cosO, float r) { return interp2(cosO * 31.f, r * 31.f, T->dir, 32); }
B200_D float tabAvg(const AlbedoTablesD *T, float r) { return interp1(r * 31.f, T->avg, 32); }
B200_D float etaParam(float eta) { return (eta - 1.f / 3.f) / (1.f - 1.f / 3.f); }
B200_D float tabRefl(const AlbedoTablesD *T, float cosO, float eta, float r) {
  return interp3(cosO * 15.f, etaParam(eta) * 15.f, r * 15.f, T->reflDir, 16);
}
B200_D float tabReflAvg(const AlbedoTablesD *T, float eta, float r) {
  return interp2(etaParam(eta) * 15.f, r * 15.f, T->reflAvg, 16);
}

// ---- GGX, isotropic
B200_D float ggxD(float a, V3 wh) {
  const float c2 = sqrf(wh.z);
  const float e = (sqrf(wh.x / a) + sqrf(wh.y / a)) / c2;
  return 1.f / (PI_F * a * a * sqrf(c2 * (1.f + e)));
}
B200_D float ggxLambda(float a, V3 w) {
  const float inv = (sqrf(w.x * a) + sqrf(w.y * a)) / sqrf(w.z);
  return 0.5f * (-1.f + sqrtf(1.f + inv));
}
B200_D float ggxG1(float a, V3 wo, float cosOH) { return wo.z * cosOH <= 0.f ? 0.f : 1.f / (1.f + ggxLambda(a, wo)); }
B200_D float ggxG2(float a, V3 wo, V3 wi, float cosOH, float cosIH) {
  if (wo.z * cosOH <= 0.f || wi.z * cosIH <= 0.f) return 0.f;
  return 1.f / (1.f + ggxLambda(a, wo) + ggxLambda(a, wi));
}
B200_D float ggxEvalVisible(float a, V3 wh, V3 wo, float cosOH, float &pdf) {
  const float D = ggxD(a, wh);
  pdf = ggxG1(a, wo, cosOH) * fabsf(cosOH) * D / fabsf(wo.z);
  return D;
}
B200_D V3 ggxSampleVisible(float a, V3 wo, float &pdf, float sx, float sy) {
  const V3 V = fnormalize(mk(a * wo.x, a * wo.y, wo.z));
  const V3 T1 = V.z < 0.9999f ? fnormalize(fcross(V, mk(0.f, 0.f, 1.f))) : mk(1.f, 0.f, 0.f);
  const V3 T2 = fcross(T1, V);
  const float h = 1.f / (1.f + V.z);
  const float r = sqrtf(sx);
  const float phi = sy < h ? sy / h * PI_F : PI_F + (sy - h) / (1.f - h) * PI_F;
  float sp, cp;
  sincosf(phi, &sp, &cp);
  const float P1 = r * cp, P2 = r * sp * (sy < h ? 1.f : V.z);
  V3 wh = P1 * T1 + P2 * T2 + sqrtf(fmaxf(0.f, 1.f - P1 * P1 - P2 * P2)) * V;
  wh = fnormalize(mk(a * wh.x, a * wh.y, fmaxf(0.f, wh.z)));
  const float c = fdot(wo, wh);
  pdf = ggxG1(a, wo, c) * fabsf(c) * ggxD(a, wh) / fabsf(wo.z);
  return wh;
}

B200_D V3 reflectV(V3 I, V3 N, float cosI) { return (2.f * cosI) * N - I; }
B200_D float fresnelDiel(float cosI, float eta) {
  const float c2 = 1.f - sqrf(eta) * (1.f - sqrf(cosI));
  if (c2 < 0.f) return 1.f;
  const float cosT = sqrtf(c2);
  const float Rper = (eta * cosI - cosT) / (eta * cosI + cosT);
  const float Rpar = (cosI - eta * cosT) / (cosI + eta * cosT);
  return 0.5f * (sqrf(Rpar) + sqrf(Rper));
}
B200_D float fresnelDielAvg(float eta) {
  if (eta < 1.f) eta = 1.f / eta;
  return (eta - 1.f) / (4.08567f + 1.00071f * eta);
}
B200_D float fresnelCond(float cosI, float eta, float k) {
  const float tmp = sqrf(eta) + sqrf(k);
  const float Rpar = (tmp * sqrf(cosI) - 2.f * eta * cosI + 1.f) / (tmp * sqrf(cosI) + 2.f * eta * cosI + 1.f);
  const float Rper = (tmp - 2.f * eta * cosI + sqrf(cosI)) / (tmp + 2.f * eta * cosI + sqrf(cosI));
  return 0.5f * (Rpar + Rper);
}

struct BsdfEval {
  V3 value;
  float pdf;
};
struct BsdfSample {
  V3 wi, weight;
  float pdf;
};

// Principled with its opacity-1, coat/sheen-free structure: a MultiBSDF of
// a microfacet conductor (child 0) and a dielectric layer over Oren-Nayar
// (child 2, "plastic").  ior = 1 (the default) gives eta = 1.
struct Principled {
  V3 fx, fy, N;  // shading frame
  float rough, alpha;
  float wC, wP, impSum;
  V3 ceta, ck, cFms;
  float cEavg;
  V3 diffuse;
  float eta, lEavg, lFms, lRavg, lAlbedoMax;
  V3 albedo;  // MultiBSDF albedo: sum of the lobes' albedos x weights (the shading AOV)

  B200_D V3 toLocal(V3 v) const { return mk(fdot(v, fx), fdot(v, fy), fdot(v, N)); }
  B200_D V3 toGlobal(V3 v) const { return fx * v.x + fy * v.y + N * v.z; }

  B200_D void init(const MaterialD &m, V3 U, V3 V, V3 Nn, const AlbedoTablesD *T) {
    fx = U;
    fy = V;
    N = Nn;
    const V3 base = mk(clamp01f(m.r), clamp01f(m.g), clamp01f(m.b));
    const float metallic = clamp01f(m.metallic);
    rough = clamp01f(m.roughness);
    alpha = fmaxf(sqrf(rough), 0.001f);
    wC = wP = impSum = 0.f;
    albedo = splat(0.f);
    const float dielectric = 1.f - metallic;
    if (dielectric > MAT_EPS) {
      const float e = 1.f;  // outside ior 1 / ior 1, clamped to [1/3, 3]
      diffuse = base;
      eta = e;
      lEavg = tabAvg(T, rough);
      const float Favg = fresnelDielAvg(e);
      lFms = Favg * (1.f - lEavg) / (1.f - Favg * lEavg);
      lRavg = tabReflAvg(T, eta, rough) + lFms * (1.f - lEavg);
      const float la = 1.f - Favg;  // (1 - weight) + transmittance^thickness (1 - Favg), weight 1
      lAlbedoMax = fmaxf(fmaxf(base.x * la, base.y * la), base.z * la);
      wP = dielectric;
      impSum += dielectric;
      albedo = base * (la * wP);
    }
    const float conductor = metallic;
    if (conductor > MAT_EPS) {
      const float rr[3] = {fminf(base.x, 0.99f), fminf(base.y, 0.99f), fminf(base.z, 0.99f)};
      float ne[3], nk[3], fa[3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const float R = rr[c];
        const float nmin = (1.f - R) / (1.f + R);
        // edge tint 1: n = n_min
        const float n = nmin;
        const float k2 = (sqrf(n + 1.f) * R - sqrf(n - 1.f)) / (1.f - R);
        ne[c] = n;
        nk[c] = sqrtf(fmaxf(k2, 0.f));
        const float R2 = R * R, R3 = R2 * R;
        fa[c] = 0.087237f + 0.0230685f - 0.0864902f + 0.0774594f + 0.782654f * R - 0.136432f * R2 +
                0.278708f * R3 + 0.19744f * R + 0.0360605f * R - 0.2586f * R2;
      }
      ceta = mk(ne[0], ne[1], ne[2]);
      ck = mk(nk[0], nk[1], nk[2]);
      cEavg = tabAvg(T, rough);
      cFms = mk(sqrf(fa[0]) * cEavg / (1.f - fa[0] * (1.f - cEavg)), sqrf(fa[1]) * cEavg / (1.f - fa[1] * (1.f - cEavg)),
                sqrf(fa[2]) * cEavg / (1.f - fa[2] * (1.f - cEavg)));
      wC = conductor;
      impSum += conductor;
      albedo = albedo + mk(fa[0], fa[1], fa[2]) * (cEavg * conductor);
    }
  }

  B200_D BsdfEval evalConductor(V3 wo, V3 wi, const AlbedoTablesD *T) const {
    const float cosO = fdot(wo, N), cosI = fdot(wi, N);
    if (cosO <= 0.f || cosI <= 0.f) return {splat(0.f), 0.f};
    const V3 wh = fnormalize(wi + wo);
    const float cosOH = fdot(wo, wh), cosIH = fdot(wi, wh);
    const V3 wo0 = toLocal(wo), wi0 = toLocal(wi), wh0 = toLocal(wh);
    const V3 F = mk(fresnelCond(cosOH, ceta.x, ck.x), fresnelCond(cosOH, ceta.y, ck.y), fresnelCond(cosOH, ceta.z, ck.z));
    float whPdf;
    const float D = ggxEvalVisible(alpha, wh0, wo0, cosOH, whPdf);
    const float G = ggxG2(alpha, wo0, wi0, cosOH, cosIH);
    const float Eo = tabEval(T, cosO, rough), Ei = tabEval(T, cosI, rough);
    const V3 fms = cFms * ((1.f - Eo) * (1.f - Ei) / (PI_F * (1.f - cEavg)) * cosI);
    return {F * (D * G / (4.f * cosO)) + fms, whPdf / (4.f * fabsf(cosOH))};
  }

  B200_D BsdfSample sampleConductor(V3 wo, float sx, float sy, const AlbedoTablesD *T) const {
    BsdfSample r = {splat(0.f), splat(0.f), 0.f};
    const float cosO = fdot(wo, N);
    if (cosO <= 0.f) return r;
    const V3 wo0 = toLocal(wo);
    float whPdf;
    const V3 wh = toGlobal(ggxSampleVisible(alpha, wo0, whPdf, sx, sy));
    const V3 wi = reflectV(wo, wh, fdot(wo, wh));
    const float cosI = fdot(wi, N);
    if (cosI <= 0.f) return r;
    const float cosOH = fdot(wo, wh), cosIH = fdot(wi, wh);
    const V3 wi0 = toLocal(wi);
    const V3 F = mk(fresnelCond(cosOH, ceta.x, ck.x), fresnelCond(cosOH, ceta.y, ck.y), fresnelCond(cosOH, ceta.z, ck.z));
    const float G = ggxG2(alpha, wo0, wi0, cosOH, cosIH);
    const float Eo = tabEval(T, cosO, rough), Ei = tabEval(T, cosI, rough);
    const V3 fms = cFms * ((1.f - Eo) * (1.f - Ei) / (PI_F * (1.f - cEavg)) * cosI);
    r.wi = wi;
    r.pdf = whPdf / (4.f * fabsf(cosOH));
    r.weight = F * (G * rcpSafe(ggxG1(alpha, wo0, cosOH))) + fms * (1.f / r.pdf);
    return r;
  }

  B200_D BsdfEval evalOrenNayar(V3 wo, V3 wi) const {
    const float cosO = fmaxf(fdot(wo, N), 0.f), cosI = fmaxf(fdot(wi, N), 0.f);
    const float s = fdot(wo, wi) - cosO * cosI;
    const float sInvt = s > 0.f ? s * rcpSafe(fmaxf(cosO, cosI)) : s;
    return {diffuse * (cosI * (1.f + rough * sInvt) / (PI_F + (PI_F / 2.f - 2.f / 3.f) * rough)), cosI / PI_F};
  }

  B200_D BsdfEval evalPlastic(V3 wo, V3 wi, const AlbedoTablesD *T) const {
    const float cosO = fdot(wo, N);
    if (cosO <= 0.f) return {splat(0.f), 0.f};
    const float cosI = fdot(wi, N);
    BsdfEval sub = evalOrenNayar(wo, wi);
    const float Eo = tabEval(T, cosO, rough), Ei = tabEval(T, fabsf(cosI), rough);
    const float Ro = tabRefl(T, cosO, eta, rough) + lFms * (1.f - Eo);
    const float Ri = tabRefl(T, fabsf(cosI), eta, rough) + lFms * (1.f - Ei);
    sub.value = sub.value * ((1.f - Ro) * (1.f - Ri) / (1.f - lRavg));
    const float coatPick = Ro / ((1.f - Ro) * lAlbedoMax + Ro);
    const float subPick = 1.f - coatPick;
    if (cosI > 0.f) {
      const V3 wh = fnormalize(wo + wi);
      const float cosOH = fdot(wo, wh), cosIH = fdot(wi, wh);
      const float F = fresnelDiel(cosOH, eta);
      float whPdf;
      const float D = ggxEvalVisible(alpha, toLocal(wh), toLocal(wo), cosOH, whPdf);
      const float G = ggxG2(alpha, toLocal(wo), toLocal(wi), cosOH, cosIH);
      const float fms = lFms * ((1.f - Eo) * (1.f - Ei) / (PI_F * (1.f - lEavg)) * cosI);
      sub.pdf = coatPick * (whPdf / (4.f * cosOH)) + subPick * sub.pdf;
      sub.value = splat(F * D * G / (4.f * cosO) + fms) + sub.value;
    } else {
      sub.pdf *= subPick;
    }
    return sub;
  }

  B200_D BsdfSample samplePlastic(V3 wo, float sx, float sy, float ss, const AlbedoTablesD *T) const {
    BsdfSample r = {splat(0.f), splat(0.f), 0.f};
    const float cosO = fdot(wo, N);
    if (cosO <= 0.f) return r;
    const V3 wo0 = toLocal(wo);
    const float Eo = tabEval(T, cosO, rough);
    const float Ro = tabRefl(T, cosO, eta, rough) + lFms * (1.f - Eo);
    const float coatPick = Ro / ((1.f - Ro) * lAlbedoMax + Ro);
    const float subPick = 1.f - coatPick;
    V3 wh;
    BsdfEval sub;
    if (ss < coatPick) {
      float whPdf;
      wh = toGlobal(ggxSampleVisible(alpha, wo0, whPdf, sx, sy));
      r.wi = reflectV(wo, wh, fdot(wo, wh));
      sub = evalOrenNayar(wo, r.wi);
    } else {
      float sp, cp;
      sincosf(2.f * PI_F * sx, &sp, &cp);
      const float cosT = sqrtf(sy), sinT = sqrtf(1.f - sy);
      r.wi = toGlobal(mk(cp * sinT, sp * sinT, cosT));
      const BsdfEval e = evalOrenNayar(wo, r.wi);
      r.pdf = e.pdf;
      r.weight = e.value * (1.f / e.pdf);
      if (fmaxf(fmaxf(r.weight.x, r.weight.y), r.weight.z) <= 0.f) return r;
      sub.pdf = r.pdf;
      sub.value = r.weight * r.pdf;
      wh = fnormalize(wo + r.wi);
    }
    const float cosI = fdot(r.wi, N), cosOH = fdot(wo, wh);
    const float Ei = tabEval(T, fabsf(cosI), rough);
    const float Ri = tabRefl(T, fabsf(cosI), eta, rough) + lFms * (1.f - Ei);
    sub.value = sub.value * ((1.f - Ro) * (1.f - Ri) / (1.f - lRavg));
    if (cosI <= 0.f) {
      r.pdf = subPick * sub.pdf;
      r.weight = sub.value * (1.f / r.pdf);
    } else {
      const float F = fresnelDiel(cosOH, eta);
      float whPdf;
      const float D = ggxEvalVisible(alpha, toLocal(wh), wo0, cosOH, whPdf);
      const float G = ggxG2(alpha, wo0, toLocal(r.wi), cosOH, fdot(r.wi, wh));
      const float fms = lFms * ((1.f - Eo) * (1.f - Ei) / (PI_F * (1.f - lEavg)) * cosI);
      r.pdf = coatPick * (whPdf / (4.f * cosOH)) + subPick * sub.pdf;
      r.weight = (splat(F * D * G / (4.f * cosO) + fms) + sub.value) * (1.f / r.pdf);
    }
    return r;
  }

  B200_D BsdfEval eval(V3 wo, V3 wi, const AlbedoTablesD *T) const {
    BsdfEval r = {splat(0.f), 0.f};
    if (wC > 0.f) {
      const BsdfEval c = evalConductor(wo, wi, T);
      r.value = r.value + c.value * wC;
      r.pdf += c.pdf * wC;
    }
    if (wP > 0.f) {
      const BsdfEval c = evalPlastic(wo, wi, T);
      r.value = r.value + c.value * wP;
      r.pdf += c.pdf * wP;
    }
    r.pdf *= 1.f / impSum;
    return r;
  }

  B200_D BsdfSample sample(V3 wo, float sx, float sy, float ss, const AlbedoTablesD *T) const {
    BsdfSample r = {splat(0.f), splat(0.f), 0.f};
    if (impSum == 0.f) return r;
    const float x = ss * impSum;
    int choice;
    if (x < wC) {
      choice = 0;
      r = sampleConductor(wo, sx, sy, T);
      r.weight = r.weight * wC;
    } else if (x < wC + wP) {
      choice = 2;
      r = samplePlastic(wo, sx, sy, (x + wP - (wC + wP)) / wP, T);
      r.weight = r.weight * wP;
    } else {
      return r;
    }
    if ((r.weight.x == 0.f && r.weight.y == 0.f && r.weight.z == 0.f) || r.pdf == 0.f)
      return {splat(0.f), splat(0.f), 0.f};
    V3 value = r.weight * r.pdf;
    float pdf = r.pdf * (choice == 0 ? wC : wP);
    if (choice != 0 && wC > 0.f) {
      const BsdfEval c = evalConductor(wo, r.wi, T);
      value = value + c.value * wC;
      pdf += c.pdf * wC;
    }
    if (choice != 2 && wP > 0.f) {
      const BsdfEval c = evalPlastic(wo, r.wi, T);
      value = value + c.value * wP;
      pdf += c.pdf * wP;
    }
    r.pdf = pdf * (1.f / impSum);
    r.weight = value * (1.f / r.pdf);
    return r;
  }
};

}  // namespace b200
