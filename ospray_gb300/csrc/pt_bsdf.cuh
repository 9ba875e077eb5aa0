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
#include "texture.cuh"

namespace b200 {

constexpr float PI_F = 3.14159265358979323846f;
constexpr float MAT_EPS = 1e-6f;

// Material types of the path tracer (render/materials/*.ispc) and the
// device record the shading kernels read, prepared on the host from
// b200_material (parameters normalised as each type's commit does).
enum : uint32_t { MAT_PRINCIPLED = 0, MAT_OBJ = 1, MAT_METAL = 2, MAT_GLASS = 3, MAT_THINGLASS = 4 };
constexpr uint32_t MATF_TRANSPARENT = 1u;  // getTransparency can be non-zero (shadow rays continue through it)
constexpr uint32_t MATF_MAP_ALPHA = 2u;    // the colour map has alpha (it scales opacity / d)

struct __align__(16) MaterialD {
  float r, g, b, roughness;  // principled baseColor, roughness; obj kd (scaled); metal roughness
  float metallic, opacity;   // principled metallic, opacity; obj d
  uint32_t kind, flags;      // MAT_*, MATF_*
  float ks[3], ns;           // obj ks (scaled), ns
  float tf[3], eta;          // obj tf (scaled); thin glass: 1 / eta
  float ceta[3], pad0;       // metal: eta per channel; principled: pad0 = specularMetallic
  float ck[3], pad1;         // metal: k per channel
  float att[3], iorIn;       // glass: inside medium attenuation (log(colour) / distance) and ior; thin glass: attenuation
  float attOut[3], iorOut;   // glass: outside medium
  const TextureD *map;       // principled map_baseColor / obj map_kd (null: none)
  uint32_t pad2, pad3;
};
static_assert(sizeof(MaterialD) == 144, "MaterialD layout");

// scattering types (render/pathtracer/Scattering.ih:8-47)
constexpr uint32_t ST_SPEC_R = 1u, ST_GLOSSY_R = 2u, ST_DIFFUSE_R = 4u, ST_SPEC_T = 8u, ST_GLOSSY_T = 16u,
                   ST_DIFFUSE_T = 32u;
constexpr uint32_t ST_REFLECTION = ST_SPEC_R | ST_GLOSSY_R | ST_DIFFUSE_R;
constexpr uint32_t ST_TRANSMISSION = ST_SPEC_T | ST_GLOSSY_T | ST_DIFFUSE_T;
constexpr uint32_t ST_SPECULAR = ST_SPEC_R | ST_SPEC_T;
constexpr uint32_t ST_SMOOTH = ST_GLOSSY_R | ST_DIFFUSE_R | ST_GLOSSY_T | ST_DIFFUSE_T;

// GGX albedo tables: dir 32x32 (cosThetaO fastest, roughness), avg 32;
// dielectric reflection: dir 16^3 (cos, eta in [1/3,1], roughness), avg 16^2
struct AlbedoTablesD {
  float dir[32 * 32];
  float avg[32];
  float reflDir[16 * 16 * 16];
  float reflAvg[16 * 16];
};

B200_D float sqrf(float x) { return x * x; }
B200_D float maxc(V3 v) { return fmaxf(fmaxf(v.x, v.y), v.z); }
B200_D float luminanceV(V3 c) { return 0.212671f * c.x + 0.715160f * c.y + 0.072169f * c.z; }
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
  uint32_t type;  // ST_* of the sampled lobe
};

// fresnelDielectricEx (bsdfs/Fresnel.ih:38-47): the Fresnel reflectance and
// the cosine of the refracted direction (0 under total internal reflection)
B200_D float fresnelDielEx(float cosI, float &cosT, float eta) {
  const float c2 = 1.f - sqrf(eta) * (1.f - sqrf(cosI));
  if (c2 < 0.f) {
    cosT = 0.f;
    return 1.f;
  }
  cosT = sqrtf(c2);
  const float Rper = (eta * cosI - cosT) / (eta * cosI + cosT);
  const float Rpar = (cosI - eta * cosT) / (cosI + eta * cosT);
  return 0.5f * (sqrf(Rpar) + sqrf(Rper));
}

// The principled base stack without transmission, coat or sheen
// (Principled.ispc:110-331): a MultiBSDF of a conductor (child 0) and a
// "plastic" dielectric layer over a diffuse substrate (child 2).
//   plastic: weight dielectric, importance dielectric x max(diffuse,
//     specular); the layer has weight `specular` (a pass-through layer for
//     specular 0) and eta = outside ior / ior (inverted inside), clamped to
//     [1/3, 3]; roughness 0: Lambert under a smooth DielectricLayer
//     (bsdfs/DielectricLayer.ih), else Oren-Nayar under a
//     MicrofacetDielectricLayer (bsdfs/MicrofacetDielectricLayer.ih);
//   conductor: weight = importance = metallic (x specular when
//     specularMetallic), FresnelConductorArtistic from baseColor and
//     edgeColor; roughness 0: the smooth Conductor (bsdfs/Conductor.ih), else
//     MicrofacetConductor.
// Material record fields: ns = specular, eta = ior, tf[0] = diffuse,
// ks = edgeColor, pad0 = specularMetallic (0 / 1).
// FULL = false: the parameters at their defaults (specular, ior, diffuse,
// edgeColor 1, specularMetallic) and no smooth conductor (the frame's
// materials are checked on the host, principledNeedsFull); the principled-only
// shading kernel takes this smaller form.
template <bool FULL>
struct PrincipledT {
  V3 fx, fy, N;  // shading frame
  float rough, alpha;
  float wC, wP, iP, impSum;
  V3 ceta, ck, cFms;
  float cEavg;
  V3 diffuse;
  float eta, lEavg, lFms, lRavg, lAlbedoMax, lWeight, lFavg;
  bool smoothBase, hasLayer, smooth;  // roughness 0; a coating layer (specular > 0); diffuse / glossy lobes
  V3 albedo;  // MultiBSDF albedo: sum of the lobes' albedos x weights (the shading AOV)

  B200_D V3 toLocal(V3 v) const { return mk(fdot(v, fx), fdot(v, fy), fdot(v, N)); }
  B200_D V3 toGlobal(V3 v) const { return fx * v.x + fy * v.y + N * v.z; }

  // fromOutside: the path travels in the material's outside medium (vacuum)
  B200_D void init(const MaterialD &m, V3 U, V3 V, V3 Nn, const AlbedoTablesD *T, bool fromOutside = true) {
    fx = U;
    fy = V;
    N = Nn;
    const V3 base = mk(clamp01f(m.r), clamp01f(m.g), clamp01f(m.b));
    const float metallic = clamp01f(m.metallic);
    const float specular = FULL ? clamp01f(m.ns) : 1.f, diffuseW = FULL ? clamp01f(m.tf[0]) : 1.f;
    rough = clamp01f(m.roughness);
    alpha = fmaxf(sqrf(rough), 0.001f);
    smoothBase = FULL && m.roughness < MAT_EPS;
    wC = wP = iP = impSum = 0.f;
    albedo = splat(0.f);
    smooth = false;
    hasLayer = false;
    const float dielectric = 1.f - metallic;
    if (dielectric > MAT_EPS) {
      float ior = FULL ? m.eta : 1.f;
      if (ior < 1.f) ior = 1.f / ior;
      float e = fromOutside ? 1.f * (1.f / ior) : ior * (1.f / 1.f);
      e = fminf(fmaxf(e, 1.f / 3.f), 3.f);
      diffuse = base * diffuseW;
      hasLayer = !FULL || specular > MAT_EPS;
      lWeight = specular;
      eta = e <= 1.f ? e : 1.f / e;
      V3 la = diffuse;  // pass-through: the substrate's albedo
      if (FULL && hasLayer && smoothBase) {
        lFavg = fresnelDielAvg(e) * specular;
        la = diffuse * ((1.f - specular) + 1.f * (1.f - lFavg));
      } else if (hasLayer) {
        lEavg = tabAvg(T, rough);
        const float Favg = fresnelDielAvg(e);
        lFms = Favg * (1.f - lEavg) / (1.f - Favg * lEavg);
        lRavg = (tabReflAvg(T, eta, rough) + lFms * (1.f - lEavg)) * specular;
        la = diffuse * ((1.f - specular) + 1.f * (1.f - Favg));
      }
      lAlbedoMax = fmaxf(fmaxf(la.x, la.y), la.z);
      wP = dielectric;
      iP = dielectric * fmaxf(diffuseW, specular);
      impSum += iP;
      albedo = la * wP;
      smooth = true;  // the diffuse substrate
    }
    const float conductor = metallic * (!FULL || m.pad0 != 0.f ? specular : 1.f);
    if (conductor > MAT_EPS) {
      const float rr[3] = {fminf(base.x, 0.99f), fminf(base.y, 0.99f), fminf(base.z, 0.99f)};
      const float gg[3] = {FULL ? clamp01f(m.ks[0]) : 1.f, FULL ? clamp01f(m.ks[1]) : 1.f,
                           FULL ? clamp01f(m.ks[2]) : 1.f};
      float ne[3], nk[3], fa[3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        // FresnelConductorArtistic (Fresnel.ih): n between n_min and n_max by the edge colour
        const float R = rr[c], G = gg[c];
        const float nmin = (1.f - R) / (1.f + R);
        const float nmax = (1.f + sqrtf(R)) / (1.f - sqrtf(R));
        const float n = G * nmin + (1.f - G) * nmax;
        const float k2 = (sqrf(n + 1.f) * R - sqrf(n - 1.f)) / (1.f - R);
        ne[c] = n;
        nk[c] = sqrtf(fmaxf(k2, 0.f));
        const float R2 = R * R, R3 = R2 * R, G2 = G * G, G3 = G2 * G;
        fa[c] = 0.087237f + 0.0230685f * G - 0.0864902f * G2 + 0.0774594f * G3 + 0.782654f * R - 0.136432f * R2 +
                0.278708f * R3 + 0.19744f * G * R + 0.0360605f * G2 * R - 0.2586f * G * R2;
      }
      ceta = mk(ne[0], ne[1], ne[2]);
      ck = mk(nk[0], nk[1], nk[2]);
      wC = conductor;
      impSum += conductor;
      if (FULL && smoothBase) {
        albedo = albedo + mk(fa[0], fa[1], fa[2]) * conductor;
      } else {
        cEavg = tabAvg(T, rough);
        cFms = mk(sqrf(fa[0]) * cEavg / (1.f - fa[0] * (1.f - cEavg)),
                  sqrf(fa[1]) * cEavg / (1.f - fa[1] * (1.f - cEavg)),
                  sqrf(fa[2]) * cEavg / (1.f - fa[2] * (1.f - cEavg)));
        albedo = albedo + mk(fa[0], fa[1], fa[2]) * (cEavg * conductor);
        smooth = true;
      }
    }
  }

  B200_D BsdfEval evalConductor(V3 wo, V3 wi, const AlbedoTablesD *T) const {
    if (FULL && smoothBase) return {splat(0.f), 0.f};  // Dirac
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
    BsdfSample r = {splat(0.f), splat(0.f), 0.f, 0u};
    if (FULL && smoothBase) {  // Conductor_sample: the mirror direction, weight = Fresnel
      const float c = fdot(wo, N);
      r.wi = reflectV(wo, N, c);
      r.pdf = INFINITY;
      r.type = ST_SPEC_R;
      r.weight = mk(fresnelCond(c, ceta.x, ck.x), fresnelCond(c, ceta.y, ck.y), fresnelCond(c, ceta.z, ck.z));
      return r;
    }
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
    r.type = ST_GLOSSY_R;
    return r;
  }

  // the substrate: Oren-Nayar (Lambert at roughness 0)
  B200_D BsdfEval evalOrenNayar(V3 wo, V3 wi) const {
    const float cosO = fmaxf(fdot(wo, N), 0.f), cosI = fmaxf(fdot(wi, N), 0.f);
    const float s = fdot(wo, wi) - cosO * cosI;
    const float sInvt = s > 0.f ? s * rcpSafe(fmaxf(cosO, cosI)) : s;
    return {diffuse * (cosI * (1.f + rough * sInvt) / (PI_F + (PI_F / 2.f - 2.f / 3.f) * rough)), cosI / PI_F};
  }
  B200_D BsdfSample sampleDiffuse(V3 wo, float sx, float sy) const {
    BsdfSample r;
    float sp, cp;
    sincosf(2.f * PI_F * sx, &sp, &cp);
    const float cosT = sqrtf(sy), sinT = sqrtf(1.f - sy);
    r.wi = toGlobal(mk(cp * sinT, sp * sinT, cosT));
    r.type = ST_DIFFUSE_R;
    const BsdfEval e = evalOrenNayar(wo, r.wi);
    r.pdf = e.pdf;
    r.weight = e.value * (1.f / e.pdf);
    return r;
  }

  B200_D BsdfEval evalPlastic(V3 wo, V3 wi, const AlbedoTablesD *T) const {
    if (FULL && !hasLayer) return evalOrenNayar(wo, wi);  // PassthroughLayer
    const float cosO = fdot(wo, N);
    if (cosO <= 0.f) return {splat(0.f), 0.f};
    const float cosI = fdot(wi, N);
    BsdfEval sub = evalOrenNayar(wo, wi);
    if (FULL && smoothBase) {  // DIELECTRICLAYER_EVAL over a diffuse substrate
      float cosO1, cosI1;
      const float F = fresnelDielEx(cosO, cosO1, eta);
      const float Fo = F * lWeight, Fi = fresnelDielEx(fabsf(cosI), cosI1, eta) * lWeight;
      sub.value = sub.value * ((1.f - Fo) * (1.f - Fi) * (1.f / (1.f - lFavg)));
      const float coatPick = Fo / ((1.f - F) * lAlbedoMax + Fo);
      sub.pdf *= 1.f - coatPick;
      return sub;
    }
    const float Eo = tabEval(T, cosO, rough), Ei = tabEval(T, fabsf(cosI), rough);
    const float Ro = (tabRefl(T, cosO, eta, rough) + lFms * (1.f - Eo)) * lWeight;
    const float Ri = (tabRefl(T, fabsf(cosI), eta, rough) + lFms * (1.f - Ei)) * lWeight;
    sub.value = sub.value * ((1.f - Ro) * (1.f - Ri) / (1.f - lRavg));
    const float coatPick = lWeight * Ro / ((1.f - Ro) * lAlbedoMax + lWeight * Ro);
    const float subPick = 1.f - coatPick;
    if (cosI > 0.f) {
      const V3 wh = fnormalize(wo + wi);
      const float cosOH = fdot(wo, wh), cosIH = fdot(wi, wh);
      const float F = fresnelDiel(cosOH, eta) * lWeight;
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
    BsdfSample r = {splat(0.f), splat(0.f), 0.f, 0u};
    if (FULL && !hasLayer) return sampleDiffuse(wo, sx, sy);  // PassthroughLayer
    const float cosO = fdot(wo, N);
    if (cosO <= 0.f) return r;
    if (FULL && smoothBase) {  // DIELECTRICLAYER_SAMPLE over a diffuse substrate
      float cosO1;
      const float F = fresnelDielEx(cosO, cosO1, eta);
      const float Fo = F * lWeight;
      const float coatPick = Fo / ((1.f - F) * lAlbedoMax + Fo);
      if (ss < coatPick) {
        r.type = ST_SPEC_R;
        r.wi = reflectV(wo, N, cosO);
        r.pdf = INFINITY;
        r.weight = splat(Fo / coatPick);
        return r;
      }
      r = sampleDiffuse(wo, sx, sy);
      if (maxc(r.weight) <= 0.f) return r;
      float cosI1;
      const float Fi = fresnelDielEx(fabsf(fdot(r.wi, N)), cosI1, eta) * lWeight;
      const float Tr = (1.f - Fo) * (1.f - Fi) * (1.f / (1.f - lFavg));
      r.weight = r.weight * (Tr * (1.f / (1.f - coatPick)));
      r.pdf *= 1.f - coatPick;
      return r;
    }
    const V3 wo0 = toLocal(wo);
    const float Eo = tabEval(T, cosO, rough);
    // (the reference's sample weighs only the multiple-scattering term here)
    const float Ro = tabRefl(T, cosO, eta, rough) + lFms * (1.f - Eo) * lWeight;
    const float coatPick = lWeight * Ro / ((1.f - Ro) * lAlbedoMax + lWeight * Ro);
    const float subPick = 1.f - coatPick;
    V3 wh;
    BsdfEval sub;
    if (ss < coatPick) {
      float whPdf;
      wh = toGlobal(ggxSampleVisible(alpha, wo0, whPdf, sx, sy));
      r.wi = reflectV(wo, wh, fdot(wo, wh));
      r.type = ST_GLOSSY_R;
      sub = evalOrenNayar(wo, r.wi);
    } else {
      r = sampleDiffuse(wo, sx, sy);
      if (maxc(r.weight) <= 0.f) return r;
      sub.pdf = r.pdf;
      sub.value = r.weight * r.pdf;
      wh = fnormalize(wo + r.wi);
    }
    const float cosI = fdot(r.wi, N), cosOH = fdot(wo, wh);
    const float Ei = tabEval(T, fabsf(cosI), rough);
    const float Ri = (tabRefl(T, fabsf(cosI), eta, rough) + lFms * (1.f - Ei)) * lWeight;
    sub.value = sub.value * ((1.f - Ro) * (1.f - Ri) / (1.f - lRavg));
    if (cosI <= 0.f) {
      r.pdf = subPick * sub.pdf;
      r.weight = sub.value * (1.f / r.pdf);
    } else {
      const float F = fresnelDiel(cosOH, eta) * lWeight;
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
    if (iP > 0.f) {
      const BsdfEval c = evalPlastic(wo, wi, T);
      r.value = r.value + c.value * wP;
      r.pdf += c.pdf * iP;
    }
    r.pdf *= 1.f / impSum;
    return r;
  }

  B200_D BsdfSample sample(V3 wo, float sx, float sy, float ss, const AlbedoTablesD *T) const {
    BsdfSample r = {splat(0.f), splat(0.f), 0.f, 0u};
    if (impSum == 0.f) return r;
    const float x = ss * impSum;
    int choice;
    if (x < wC) {
      choice = 0;
      r = sampleConductor(wo, sx, sy, T);
      r.weight = r.weight * wC;
    } else if (x < wC + iP) {
      choice = 2;
      r = samplePlastic(wo, sx, sy, (x + iP - (wC + iP)) / iP, T);
      r.weight = r.weight * wP;
    } else {
      return r;
    }
    if ((r.weight.x == 0.f && r.weight.y == 0.f && r.weight.z == 0.f) || r.pdf == 0.f)
      return {splat(0.f), splat(0.f), 0.f, 0u};
    if (FULL && (r.type & ST_SPECULAR)) {  // a Dirac lobe: no other child adds (MultiBSDF_sample)
      r.weight = r.weight * (impSum * (1.f / (choice == 0 ? wC : iP)));
      return r;
    }
    V3 value = r.weight * r.pdf;
    float pdf = r.pdf * (choice == 0 ? wC : iP);
    if (choice != 0 && wC > 0.f) {
      const BsdfEval c = evalConductor(wo, r.wi, T);
      value = value + c.value * wC;
      pdf += c.pdf * wC;
    }
    if (choice != 2 && iP > 0.f) {
      const BsdfEval c = evalPlastic(wo, r.wi, T);
      value = value + c.value * wP;
      pdf += c.pdf * iP;
    }
    r.pdf = pdf * (1.f / impSum);
    r.weight = value * (1.f / r.pdf);
    return r;
  }
};

// ---------------------------------------------------------------- surface BSDFs by material type
// Each type has init / eval / sample with MultiBSDF semantics
// (render/bsdfs/MultiBSDF.ih): eval sums the evaluable children's values
// (x weight) and their pdfs x importance / importance sum; sample picks a
// child by importance, and unless it is specular adds the other children's
// eval.  `smooth` = the BSDF has a diffuse or glossy lobe (isSmooth,
// render/pathtracer/PathTracerUtil.ih:13-28): such vertices do next-event
// estimation.

B200_D V3 expV(V3 a) { return mk(expf(a.x), expf(a.y), expf(a.z)); }

// Principled_BSDF root (render/materials/Principled.ispc:81-429): child 0 the
// cut-out Transmission (weight 1, importance 1 - opacity), child 1 the base
// stack (weight = importance = opacity), built only when opacity > EPS.
// CUT = false: every material of the frame is opaque (1 - opacity <= EPS), so
// the root has the stack child only and the cut-out state drops out.
template <bool CUT>
struct PrincipledBsdfT {
  PrincipledT<CUT> st;
  float op, tr, impSum;
  bool hasStack, hasCut, smooth;
  B200_D V3 N() const { return st.N; }
  B200_D V3 albedoV() const {
    V3 a = hasStack ? st.albedo * op : splat(0.f);
    if (CUT && hasCut) a = a + splat(tr);
    return a;
  }
  B200_D void init(const MaterialD &m, V3 U, V3 V, V3 Nn, const AlbedoTablesD *T) {
    init(m, U, V, Nn, T, clamp01f(m.opacity));
  }
  // opacity: the material's opacity times its colour map's alpha (clamped);
  // the stack exists for the material's own opacity > EPS, the cut-out child
  // for its own opacity < 1 - EPS or a colour map with alpha
  // fromOutside: the path travels in vacuum, the principled material's outside medium
  B200_D void init(const MaterialD &m, V3 U, V3 V, V3 Nn, const AlbedoTablesD *T, float opacity,
                   bool fromOutside = true) {
    op = opacity;
    tr = CUT ? 1.f - op : 0.f;
    hasStack = !CUT || m.opacity > MAT_EPS;
    hasCut = CUT && (1.f - m.opacity > MAT_EPS || (m.flags & MATF_MAP_ALPHA) != 0);
    if (hasStack) {
      st.init(m, U, V, Nn, T, fromOutside);
    } else {
      st.fx = U;
      st.fy = V;
      st.N = Nn;
      st.impSum = 0.f;
      st.albedo = splat(0.f);
    }
    smooth = hasStack && st.smooth;
    impSum = (hasCut ? tr : 0.f) + (hasStack ? op : 0.f);
  }
  B200_D BsdfEval eval(V3 wo, V3 wi, const AlbedoTablesD *T) const {
    BsdfEval r = {splat(0.f), 0.f};
    if (hasStack && op > 0.f) {
      const BsdfEval e = st.eval(wo, wi, T);
      r.value = e.value * op;
      r.pdf = e.pdf * op;
    }
    r.pdf *= 1.f / impSum;
    return r;
  }
  B200_D BsdfSample sample(V3 wo, float sx, float sy, float ss, const AlbedoTablesD *T) const {
    BsdfSample r = {splat(0.f), splat(0.f), 0.f, 0u};
    if (impSum == 0.f) return r;
    const float x = ss * impSum;
    float prefix = 0.f;
    if (CUT && hasCut && x < (prefix += tr)) {
      // Transmission_sample: straight through, a Dirac lobe
      r.wi = -wo;
      r.pdf = INFINITY;
      r.type = ST_SPEC_T;
      r.weight = splat(tr) * (impSum * (1.f / tr));
      return r;
    }
    if (!hasStack) return r;
    prefix += op;
    r = st.sample(wo, sx, sy, (x + op - prefix) * (1.f / op), T);
    r.weight = r.weight * op;
    if ((r.weight.x == 0.f && r.weight.y == 0.f && r.weight.z == 0.f) || r.pdf == 0.f)
      return {splat(0.f), splat(0.f), 0.f, 0u};
    if (r.type & ST_SPECULAR) {
      r.weight = r.weight * (impSum * (1.f / op));
      return r;
    }
    const V3 value = r.weight * r.pdf;
    r.pdf = r.pdf * op * (1.f / impSum);
    r.weight = value * (1.f / r.pdf);
    return r;
  }
};
using PrincipledBsdf = PrincipledBsdfT<true>;

// OBJ_BSDF (render/materials/OBJ.ispc:29-126): Lambert (child 0), specular
// Transmission (child 1), Blinn "Specular" (child 2, bsdfs/Specular.ih),
// each with weight 1 and importance = luminance of its albedo.
struct ObjBsdf {
  V3 fx, fy, Nn;
  V3 Kd, Tt, ksN, specW;
  float ns, iL, iT, iS, impSum;
  bool smooth;
  V3 albedo;
  B200_D V3 albedoV() const { return albedo; }
  B200_D V3 N() const { return Nn; }
  B200_D V3 toGlobal(V3 v) const { return fx * v.x + fy * v.y + Nn * v.z; }
  B200_D void init(const MaterialD &m, V3 U, V3 V, V3 N) {
    fx = U;
    fy = V;
    Nn = N;
    const float d = m.opacity;
    Kd = mk(m.r, m.g, m.b) * d;
    Tt = mk(m.tf[0], m.tf[1], m.tf[2]) * d + splat(1.f - d);
    const V3 Ks = mk(m.ks[0], m.ks[1], m.ks[2]) * d;
    iL = iT = iS = impSum = 0.f;
    albedo = splat(0.f);
    if (maxc(Kd) > 0.f) {
      iL = luminanceV(Kd);
      impSum += iL;
      albedo = albedo + Kd;
    }
    if (maxc(Tt) > 0.f) {
      iT = luminanceV(Tt);
      impSum += iT;
      albedo = albedo + Tt;
    }
    // Specular_Constructor: Phong exponent to Blinn, energy normalisation
    ns = m.ns * 4.f;
    const float tmp = (ns + 2.f) * (1.f / (2.f - expf(ns * -0.34657359027997264f)));
    ksN = Ks * ((1.f / (4.f * PI_F)) * tmp);
    specW = Ks * (2.f * tmp * (1.f / (ns + 1.f)));
    if (maxc(Ks) > 0.f) {
      iS = luminanceV(Ks);
      impSum += iS;
      albedo = albedo + Ks;
    }
    smooth = iL > 0.f || iS > 0.f;
  }
  B200_D BsdfEval evalLambert(V3 wi) const {
    const float c = fmaxf(fdot(wi, Nn), 0.f);
    return {Kd * ((1.f / PI_F) * c), c * (1.f / PI_F)};
  }
  B200_D BsdfEval evalSpecular(V3 wo, V3 wi) const {
    const float cosO = fdot(wo, Nn), cosI = fdot(wi, Nn);
    if (cosO <= 0.f || cosI <= 0.f) return {splat(0.f), 0.f};
    const V3 wh = fnormalize(wo + wi);
    const float cosH = fdot(wh, Nn);
    const float pdf = (ns + 1.f) * (1.f / (2.f * PI_F)) * powf(cosH, ns) * (1.f / (4.f * fdot(wo, wh)));
    return {ksN * powf(cosH, ns), pdf};
  }
  B200_D BsdfEval eval(V3 wo, V3 wi, const AlbedoTablesD *) const { return evalSkip(wo, wi, -1); }
  // the children's eval except child `skip` (-1: all, pdf normalised)
  B200_D BsdfEval evalSkip(V3 wo, V3 wi, int skip) const {
    BsdfEval r = {splat(0.f), 0.f};
    if (iL > 0.f && skip != 0) {
      const BsdfEval c = evalLambert(wi);
      r.value = r.value + c.value;
      r.pdf += c.pdf * iL;
    }
    if (iS > 0.f && skip != 2) {
      const BsdfEval c = evalSpecular(wo, wi);
      r.value = r.value + c.value;
      r.pdf += c.pdf * iS;
    }
    if (skip < 0) r.pdf *= 1.f / impSum;
    return r;
  }
  B200_D BsdfSample sample(V3 wo, float sx, float sy, float ss, const AlbedoTablesD *) const {
    BsdfSample r = {splat(0.f), splat(0.f), 0.f, 0u};
    if (impSum == 0.f) return r;
    const float x = ss * impSum;
    float prefix = 0.f, imp = 0.f;
    int choice;
    if (x < (prefix += iL)) {
      choice = 0;
      imp = iL;
      float sp, cp;
      sincosf(2.f * PI_F * sx, &sp, &cp);
      const float cosT = sqrtf(sy), sinT = sqrtf(1.f - sy);
      const V3 l = mk(cp * sinT, sp * sinT, cosT);
      r.wi = toGlobal(l);
      r.pdf = l.z * (1.f / PI_F);
      r.type = ST_DIFFUSE_R;
      r.weight = Kd;
    } else if (x < (prefix += iT)) {
      choice = 1;
      imp = iT;
      r.wi = -wo;
      r.pdf = INFINITY;
      r.type = ST_SPEC_T;
      r.weight = Tt;
    } else if (x < (prefix += iS)) {
      choice = 2;
      imp = iS;
      // powerCosineSampleHemisphere(ns, s) about N, reflected about the half vector
      const float phi = 2.f * PI_F * sx;
      const float cosT = powf(sy, 1.f / (ns + 1.f));
      float sp, cp;
      sincosf(phi, &sp, &cp);
      const float sinT = sqrtf(fmaxf(0.f, 1.f - cosT * cosT));
      const V3 whl = mk(cp * sinT, sp * sinT, cosT);
      const V3 wh = toGlobal(whl);
      const float cosOH = fdot(wo, wh);
      r.wi = reflectV(wo, wh, cosOH);
      if (fdot(r.wi, Nn) <= 0.f) return {splat(0.f), splat(0.f), 0.f, 0u};
      r.pdf = (ns + 1.f) * (1.f / (2.f * PI_F)) * powf(whl.z, ns) * (1.f / (4.f * cosOH));
      r.type = ST_GLOSSY_R;
      r.weight = specW * cosOH;
    } else {
      return r;
    }
    if ((r.weight.x == 0.f && r.weight.y == 0.f && r.weight.z == 0.f) || r.pdf == 0.f)
      return {splat(0.f), splat(0.f), 0.f, 0u};
    if (r.type & ST_SPECULAR) {
      r.weight = r.weight * (impSum * (1.f / imp));
      return r;
    }
    V3 value = r.weight * r.pdf;
    float pdf = r.pdf * imp;
    const BsdfEval o = evalSkip(wo, r.wi, choice);
    value = value + o.value;
    pdf += o.pdf;
    r.pdf = pdf * (1.f / impSum);
    r.weight = value * (1.f / r.pdf);
    return r;
  }
};

// Metal (render/materials/Metal.ispc:16-48): RGB conductor Fresnel (eta, k)
// in the frame about Ns; roughness 0 the specular Conductor
// (bsdfs/Conductor.ih), else MicrofacetConductor with no energy
// compensation (the RGB Fresnel's average is 0, so fmsScale and the albedo
// are 0).
struct MetalBsdf {
  V3 fx, fy, Nn, ceta, ck;
  float rough, alpha;
  bool specular, smooth;
  V3 albedo;
  B200_D V3 albedoV() const { return albedo; }
  B200_D V3 N() const { return Nn; }
  B200_D V3 toLocal(V3 v) const { return mk(fdot(v, fx), fdot(v, fy), fdot(v, Nn)); }
  B200_D V3 toGlobal(V3 v) const { return fx * v.x + fy * v.y + Nn * v.z; }
  B200_D V3 fresnel(float c) const {
    return mk(fresnelCond(c, ceta.x, ck.x), fresnelCond(c, ceta.y, ck.y), fresnelCond(c, ceta.z, ck.z));
  }
  B200_D void init(const MaterialD &m, V3 Ns) {
    Nn = Ns;
    frame(Ns, fx, fy);
    ceta = mk(m.ceta[0], m.ceta[1], m.ceta[2]);
    ck = mk(m.ck[0], m.ck[1], m.ck[2]);
    rough = m.roughness;
    alpha = fmaxf(sqrf(rough), 0.001f);
    specular = rough == 0.f;
    smooth = !specular;
    albedo = splat(0.f);
  }
  B200_D BsdfEval eval(V3 wo, V3 wi, const AlbedoTablesD *) const {
    if (specular) return {splat(0.f), 0.f};
    const float cosO = fdot(wo, Nn), cosI = fdot(wi, Nn);
    if (cosO <= 0.f || cosI <= 0.f) return {splat(0.f), 0.f};
    const V3 wh = fnormalize(wi + wo);
    const float cosOH = fdot(wo, wh), cosIH = fdot(wi, wh);
    const V3 wo0 = toLocal(wo), wi0 = toLocal(wi), wh0 = toLocal(wh);
    float whPdf;
    const float D = ggxEvalVisible(alpha, wh0, wo0, cosOH, whPdf);
    const float G = ggxG2(alpha, wo0, wi0, cosOH, cosIH);
    return {fresnel(cosOH) * (D * G * (1.f / (4.f * cosO))), whPdf * (1.f / (4.f * fabsf(cosOH)))};
  }
  B200_D BsdfSample sample(V3 wo, float sx, float sy, float, const AlbedoTablesD *) const {
    BsdfSample r = {splat(0.f), splat(0.f), 0.f, 0u};
    if (specular) {
      const float c = fdot(wo, Nn);
      r.wi = reflectV(wo, Nn, c);
      r.pdf = INFINITY;
      r.type = ST_SPEC_R;
      r.weight = fresnel(c);
      return r;
    }
    const float cosO = fdot(wo, Nn);
    if (cosO <= 0.f) return r;
    const V3 wo0 = toLocal(wo);
    float whPdf;
    const V3 wh = toGlobal(ggxSampleVisible(alpha, wo0, whPdf, sx, sy));
    const V3 wi = reflectV(wo, wh, fdot(wo, wh));
    const float cosI = fdot(wi, Nn);
    if (cosI <= 0.f) return r;
    const float cosOH = fdot(wo, wh), cosIH = fdot(wi, wh);
    const float G = ggxG2(alpha, wo0, toLocal(wi), cosOH, cosIH);
    r.wi = wi;
    r.type = ST_GLOSSY_R;
    r.pdf = whPdf * (1.f / (4.f * fabsf(cosOH)));
    r.weight = fresnel(cosOH) * (G * rcpSafe(ggxG1(alpha, wo0, cosOH)));
    return r;
  }
};

// Glass (render/materials/Glass.ispc:16-60) as RobustDielectric
// (bsdfs/RobustDielectric.ih): eta = ior outside / ior inside when the path
// comes from the outside medium, else the inverse; Dirac reflection or
// refraction picked by the Fresnel reflectance, with the robust normal flips
// and grazing nudges.
struct GlassBsdf {
  V3 Ns, Ng;
  float eta;  // as RobustDielectric stores it: the inverse of the refraction ratio it applies
  bool smooth;
  V3 albedo;
  B200_D V3 albedoV() const { return albedo; }
  B200_D V3 N() const { return Ns; }
  B200_D void init(float eta_, V3 ns, V3 ng) {
    eta = eta_;
    Ns = ns;
    Ng = ng;
    smooth = false;
    albedo = splat(1.f);
  }
  B200_D BsdfEval eval(V3, V3, const AlbedoTablesD *) const { return {splat(0.f), 0.f}; }
  B200_D BsdfSample sample(V3 wo, float, float, float ss, const AlbedoTablesD *) const {
    BsdfSample r;
    r.pdf = INFINITY;
    r.weight = splat(1.f);
    const V3 inc = -wo;
    V3 sn = Ns, gn = Ng;
    const float e = 1.f / eta;
    const float geps = 1e-6f;
    const bool canReflect = e < 1.f - geps || e > 1.f + geps;
    if (fdot(inc, sn) > 0.f) sn = -sn;
    if (fdot(inc, gn) > 0.f) gn = -gn;
    // ReflectionDirection
    const V3 par = sn * fdot(inc, sn);
    const V3 dirR = (inc - par) - par;
    // RefractionDirection
    V3 dirT;
    float FR;
    bool mustReflect = false;
    {
      const float cos1 = fdot(inc, sn);
      const float c1 = fabsf(cos1);
      const bool headOn = 1.f - 1e-6f < c1 && c1 < 1.f - 1e-6f;  // never true, as in the reference
      if (headOn) {
        FR = sqrf((e - 1.f) / (e + 1.f));
        dirT = inc;
      } else {
        const V3 dpar = sn * cos1;
        const V3 dperp = inc - dpar;
        const V3 b = fnormalize(dperp);
        const float sin1 = fdot(dperp, b);
        const float sin2 = sin1 / e;
        if (sin2 > 1.f) {
          dirT = splat(0.f);
          FR = 1.f;
          mustReflect = true;
        } else {
          const float cos2 = sqrtf(clamp01f(1.f - sin2 * sin2));
          const V3 N2 = fnormalize(dpar);
          dirT = N2 * cos2 + b * sin2;
          const float q1 = (e * c1 - cos2) / (e * c1 + cos2);
          const float q2 = (c1 - e * cos2) / (c1 + e * cos2);
          FR = 0.5f * (q1 * q1 + q2 * q2);
        }
      }
      FR = clamp01f(FR);
    }
    if ((ss < FR && canReflect) || mustReflect) {
      r.wi = dirR;
      r.type = ST_SPEC_R;
      const float gc = fdot(r.wi, gn);
      if (gc >= 0.f) {
        if (gc < geps) r.wi = fnormalize(r.wi + gn * geps);
      } else {
        r.wi = r.wi - gn * (2.f * gc);
      }
    } else {
      r.wi = dirT;
      r.type = ST_SPEC_T;
      const float gc = fdot(r.wi, gn);
      if (gc <= 0.f) {
        if (gc > -geps) r.wi = fnormalize(r.wi - gn * geps);
      } else {
        r.type = ST_SPEC_R;
      }
    }
    return r;
  }
};

// ThinGlass (render/materials/ThinGlass.ispc:16-70) as RobustThinDielectric
// (bsdfs/RobustThinDielectric.ih): a slab whose inner reflections are summed
// in closed form; reflection or straight transmission picked by luminance.

B200_D void thinSlab(float cosO, float eta, V3 att, V3 &R, V3 &T) {
  float cosT;
  const float Fo = fresnelDielEx(cosO, cosT, eta);
  const float Ft = fresnelDiel(cosT, 1.f / eta);
  const V3 A = expV(att * (1.f / cosT));
  const V3 FA = A * Ft;
  const V3 FA2 = FA * FA;
  const V3 inv = mk(1.f / (1.f - FA2.x), 1.f / (1.f - FA2.y), 1.f / (1.f - FA2.z));
  R = splat(Fo) + (A * A) * ((1.f - Fo) * (1.f - Ft) * Ft) * inv;
  T = A * ((1.f - Fo) * (1.f - Ft)) * (splat(1.f) + FA2 * inv);
}
struct ThinGlassBsdf {
  V3 Nn, att;
  float eta;
  bool smooth;
  V3 albedo;
  B200_D V3 albedoV() const { return albedo; }
  B200_D V3 N() const { return Nn; }
  B200_D void init(const MaterialD &m, V3 Ns) {
    Nn = Ns;
    eta = m.eta;
    att = mk(m.att[0], m.att[1], m.att[2]);
    smooth = false;
    albedo = expV(att);
  }
  B200_D BsdfEval eval(V3, V3, const AlbedoTablesD *) const { return {splat(0.f), 0.f}; }
  B200_D BsdfSample sample(V3 wo, float, float, float ss, const AlbedoTablesD *) const {
    BsdfSample r;
    const float cosO = fmaxf(fdot(wo, Nn), 0.f);
    V3 R, T;
    thinSlab(cosO, eta, att, R, T);
    const float pR = luminanceV(R), pT = luminanceV(T);
    const float p = fminf(fmaxf(pR * (1.f / (pR + pT)), 0.25f), 0.75f);
    if (ss <= p) {
      r.wi = reflectV(wo, Nn, cosO);
      r.type = ST_SPEC_R;
      r.weight = R * (1.f / p);
    } else {
      r.wi = -wo;
      r.type = ST_SPEC_T;
      r.weight = T * (1.f / (1.f - p));
    }
    r.pdf = INFINITY;
    return r;
  }
};

// A medium: ior and attenuation (render/materials/Medium.ih).  Paths carry
// the id of the medium they travel in: MEDIUM_VACUUM, or material m's inside
// (2m) or outside (2m + 1) medium (glass); media compare by value.
constexpr uint32_t MEDIUM_VACUUM = 0xffffffffu;
struct MediumD {
  float ior;
  V3 att;
};
B200_D MediumD mediumOf(const MaterialD *mats, uint32_t id) {
  if (id == MEDIUM_VACUUM) return {1.f, splat(0.f)};
  const MaterialD &m = mats[id >> 1];
  if (id & 1u) return {m.iorOut, mk(m.attOut[0], m.attOut[1], m.attOut[2])};
  return {m.iorIn, mk(m.att[0], m.att[1], m.att[2])};
}
B200_D bool sameMedium(const MediumD &a, const MediumD &b) {
  return a.ior == b.ior && a.att.x == b.att.x && a.att.y == b.att.y && a.att.z == b.att.z;
}
// Glass_selectNextMedium / the eta of Glass_getBSDF: from the outside medium
// into the inside one, otherwise back out
B200_D bool glassFromOutside(const MaterialD *mats, uint32_t mat, uint32_t cur) {
  return sameMedium(mediumOf(mats, cur), mediumOf(mats, 2u * mat + 1u));
}

// The colour map's texel at a hit (Texture2D_get with the hit's texture
// coordinates and pixel footprint), 1 without a map.
B200_D float4 colorMapTexel(const MaterialD &m, const DGAttr &at, float footprint) {
  return m.map ? texGet(*m.map, at.s, at.t, footprint) : make_float4(1.f, 1.f, 1.f, 1.f);
}

// A material's parameters at a hit with its colour map and the vertex colour
// applied (Principled.ispc:110-135: baseColor x map.rgb x colour.rgb,
// clamped, opacity x map alpha; OBJ.ispc:52-66: d x colour alpha x map alpha,
// kd x map.rgb x colour.rgb).  `opacity` gets principled's effective opacity
// (the material's own stays in the record); obj's d goes into the record.
B200_D MaterialD shadedMaterial(const MaterialD &m, const DGAttr &at, float footprint, float &opacity) {
  MaterialD r = m;
  opacity = clamp01f(m.opacity);
  if (m.kind == MAT_PRINCIPLED) {
    const float4 tx = colorMapTexel(m, at, footprint);
    r.r = clamp01f(m.r * tx.x * at.color.x);
    r.g = clamp01f(m.g * tx.y * at.color.y);
    r.b = clamp01f(m.b * tx.z * at.color.z);
    if (m.flags & MATF_MAP_ALPHA) opacity *= tx.w;
  } else if (m.kind == MAT_OBJ) {
    const float4 tx = colorMapTexel(m, at, footprint);
    r.opacity = m.opacity * at.color.w * tx.w;
    r.r = m.r * tx.x * at.color.x;
    r.g = m.g * tx.y * at.color.y;
    r.b = m.b * tx.z * at.color.z;
  }
  return r;
}

// Material_getTransparency of the hit material for a shadow ray
// (TransparentShadow.ispc:18-85): principled 1 - opacity (Principled.ispc:
// 432-580, the opaque base passes nothing), obj tf d + 1 - d (OBJ.ispc:
// 93-110), glass 1 - Fresnel, thin glass the slab's transmission, metal 0;
// opacity and d with the colour map's alpha and the vertex colour's alpha.
B200_D V3 materialTransparency(const MaterialD *mats, uint32_t mi, V3 rayDir, V3 Ns, uint32_t medium,
                               const DGAttr &at, float footprint) {
  const MaterialD &m = mats[mi];
  switch (m.kind) {
    case MAT_PRINCIPLED: {
      float op = clamp01f(m.opacity);
      if (m.flags & MATF_MAP_ALPHA) op *= colorMapTexel(m, at, footprint).w;
      const float tr = 1.f - op;
      if (tr <= MAT_EPS) return splat(0.f);
      return splat(tr);
    }
    case MAT_OBJ: {
      float d = m.opacity * at.color.w;
      if (m.flags & MATF_MAP_ALPHA) d *= colorMapTexel(m, at, footprint).w;
      return mk(m.tf[0], m.tf[1], m.tf[2]) * d + splat(1.f - d);
    }
    case MAT_GLASS: {
      const bool out = glassFromOutside(mats, mi, medium);
      const float eta = out ? m.iorOut * (1.f / m.iorIn) : m.iorIn * (1.f / m.iorOut);
      const float cosO = fmaxf(-fdot(rayDir, Ns), 0.f);
      return splat(1.f - fresnelDiel(cosO, eta));
    }
    case MAT_THINGLASS: {
      V3 R, T;
      thinSlab(fmaxf(-fdot(rayDir, Ns), 0.f), m.eta, mk(m.att[0], m.att[1], m.att[2]), R, T);
      return T;
    }
    default:
      return splat(0.f);
  }
}

}  // namespace b200
