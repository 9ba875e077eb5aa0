// Oracle (test infrastructure only): principled BSDF (plastic and conductor
// sub-paths), GGX microfacet distribution, Fresnel terms, microfacet albedo
// tables, and the quad / ambient lights, restated from
//   render/materials/Principled.ispc:81-429 (getBSDF), PrincipledShared.h:130-163
//   render/bsdfs/MultiBSDF.ih, OrenNayar.ih:13-63, MicrofacetDielectricLayer.ih,
//   MicrofacetConductor.ih:17-146, GGXDistribution.ih:17-144,
//   MicrofacetDistribution.ih:10-22, Fresnel.ih:19-83,226-288, Optics.ih
//   render/bsdfs/MicrofacetAlbedo.ih, MicrofacetAlbedoTables.{ih,ispc},
//   math/interpolation.ih
//   lights/QuadLight.ispc:43-215, QuadLight.cpp:68-108,
//   lights/SphericalQuadSampling.ih, lights/AmbientLight.ispc:17-57
#pragma once
#include <cmath>
#include <vector>

#include "render.h"
#include "texture.h"

namespace orc {

constexpr float PI = 3.14159265358979323846f;
constexpr float EPS = 1e-6f;  // render/materials: EPS used by getBSDF thresholds

inline float sqr(float x) { return x * x; }
inline float cos2sin(float c) { return std::sqrt(std::fmax(0.f, 1.f - c * c)); }
inline float clamp01(float x) { return std::fmin(std::fmax(x, 0.f), 1.f); }
inline float rcp_safe(float x) { return 1.f / (std::fabs(x) < 1e-8f ? std::copysign(1e-8f, x) : x); }

// ---- interpolation (math/interpolation.ih)
inline float interp1D(float x, const float *f, int size) {
  const float xc = clampf(x, 0.f, float(size - 1));
  const float s = xc - std::floor(xc);
  const int x0 = std::min(int(xc), size - 1), x1 = std::min(x0 + 1, size - 1);
  return lerpf(s, f[x0], f[x1]);
}
inline float interp2D(float px, float py, const float *f, int sx, int sy) {
  const float xc = clampf(px, 0.f, float(sx - 1)), yc = clampf(py, 0.f, float(sy - 1));
  const float fx = xc - std::floor(xc), fy = yc - std::floor(yc);
  const int x0 = std::min(int(xc), sx - 1), x1 = std::min(x0 + 1, sx - 1);
  const int y0 = std::min(int(yc), sy - 1), y1 = std::min(y0 + 1, sy - 1);
  const float f0 = lerpf(fx, f[x0 + y0 * sx], f[x1 + y0 * sx]);
  const float f1 = lerpf(fx, f[x0 + y1 * sx], f[x1 + y1 * sx]);
  return lerpf(fy, f0, f1);
}
inline float interp3D(float px, float py, float pz, const float *f, int n) {
  const float zc = clampf(pz, 0.f, float(n - 1));
  const float fz = zc - std::floor(zc);
  const int z0 = std::min(int(zc), n - 1), z1 = std::min(z0 + 1, n - 1);
  const float a = interp2D(px, py, f + size_t(z0) * n * n, n, n);
  const float b = interp2D(px, py, f + size_t(z1) * n * n, n, n);
  return lerpf(fz, a, b);
}

// ---- GGX (isotropic alpha; anisotropy 0 in these materials)
struct GGX {
  float ax, ay;
};
inline GGX makeGGX(float roughness) {
  const float a = std::fmax(sqr(roughness), 0.001f);
  return {a, a};
}
inline float ggxEval(const GGX &m, V3 wh) {
  const float c2 = sqr(wh.z);
  const float e = (sqr(wh.x / m.ax) + sqr(wh.y / m.ay)) / c2;
  return 1.f / (PI * m.ax * m.ay * sqr(c2 * (1.f + e)));
}
inline float ggxLambda(const GGX &m, V3 wo) {
  const float c2 = sqr(wo.z);
  const float inv = (sqr(wo.x * m.ax) + sqr(wo.y * m.ay)) / c2;
  return 0.5f * (-1.f + std::sqrt(1.f + inv));
}
inline float ggxG1(const GGX &m, V3 wo, float cosOH) {
  if (wo.z * cosOH <= 0.f) return 0.f;
  return 1.f / (1.f + ggxLambda(m, wo));
}
inline float ggxG2(const GGX &m, V3 wo, V3 wi, float cosOH, float cosIH) {
  if (wo.z * cosOH <= 0.f || wi.z * cosIH <= 0.f) return 0.f;
  return 1.f / (1.f + ggxLambda(m, wo) + ggxLambda(m, wi));
}
inline float ggxEvalVisible(const GGX &m, V3 wh, V3 wo, float cosOH, float &pdf) {
  const float D = ggxEval(m, wh);
  pdf = ggxG1(m, wo, cosOH) * std::fabs(cosOH) * D / std::fabs(wo.z);
  return D;
}
inline V3 ggxSampleVisible(const GGX &m, V3 wo, float &pdf, V2 s) {
  const V3 V = normalize(v3(m.ax * wo.x, m.ay * wo.y, wo.z));
  const V3 T1 = V.z < 0.9999f ? normalize(cross(V, v3(0, 0, 1))) : v3(1, 0, 0);
  const V3 T2 = cross(T1, V);
  const float a = 1.f / (1.f + V.z);
  const float r = std::sqrt(s.x);
  const float phi = s.y < a ? s.y / a * PI : PI + (s.y - a) / (1.f - a) * PI;
  const float P1 = r * std::cos(phi);
  const float P2 = r * std::sin(phi) * (s.y < a ? 1.f : V.z);
  V3 wh = P1 * T1 + P2 * T2 + std::sqrt(std::fmax(0.f, 1.f - P1 * P1 - P2 * P2)) * V;
  wh = normalize(v3(m.ax * wh.x, m.ay * wh.y, std::fmax(0.f, wh.z)));
  pdf = ggxG1(m, wo, dot(wo, wh)) * std::fabs(dot(wo, wh)) * ggxEval(m, wh) / std::fabs(wo.z);
  return wh;
}

// ---- Fresnel / optics
inline V3 reflectV(V3 I, V3 N, float cosI) { return (2.f * cosI) * N - I; }
inline float sqrCosT(float cosI, float eta) { return 1.f - sqr(eta) * (1.f - sqr(cosI)); }
inline float refractCos(float cosI, float eta) { return std::sqrt(std::fmax(sqrCosT(cosI, eta), 0.f)); }
inline float fresnelDielectric(float cosI, float cosT, float eta) {
  const float Rper = (eta * cosI - cosT) / (eta * cosI + cosT);
  const float Rpar = (cosI - eta * cosT) / (cosI + eta * cosT);
  return 0.5f * (sqr(Rpar) + sqr(Rper));
}
inline float fresnelDielectric(float cosI, float eta) {
  const float c = sqrCosT(cosI, eta);
  if (c < 0.f) return 1.f;
  return fresnelDielectric(cosI, std::sqrt(c), eta);
}
// fresnelDielectricEx (bsdfs/Fresnel.ih:38-47)
inline float fresnelDielectricEx(float cosI, float &cosT, float eta) {
  const float k = sqrCosT(cosI, eta);
  if (k < 0.f) {
    cosT = 0.f;
    return 1.f;
  }
  cosT = std::sqrt(k);
  return fresnelDielectric(cosI, cosT, eta);
}
inline float fresnelDielectricAvg(float eta) {
  if (eta < 1.f) eta = 1.f / eta;
  return (eta - 1.f) / (4.08567f + 1.00071f * eta);
}
inline float fresnelConductor1(float cosI, float eta, float k) {
  const float tmp = sqr(eta) + sqr(k);
  const float Rpar = (tmp * sqr(cosI) - 2.f * eta * cosI + 1.f) / (tmp * sqr(cosI) + 2.f * eta * cosI + 1.f);
  const float Rper = (tmp - 2.f * eta * cosI + sqr(cosI)) / (tmp + 2.f * eta * cosI + sqr(cosI));
  return 0.5f * (Rpar + Rper);
}

// ---- microfacet albedo tables (computed once, like precomputeMicrofacetAlbedoTables)
struct AlbedoTables {
  static constexpr int N = 32, ND = 16;
  std::vector<float> dir, avg;            // N*N (cosThetaO fastest), N
  std::vector<float> reflDir, reflAvg;    // ND^3 (cos, eta, roughness), ND^2
  AlbedoTables();
  float eval(float cosO, float roughness) const { return interp2D(cosO * (N - 1), roughness * (N - 1), dir.data(), N, N); }
  float evalAvg(float roughness) const { return interp1D(roughness * (N - 1), avg.data(), N); }
  float etaParam(float eta) const { return (eta - 1.f / 3.f) / (1.f - 1.f / 3.f); }
  float reflEval(float cosO, float eta, float roughness) const {
    return interp3D(cosO * (ND - 1), etaParam(eta) * (ND - 1), roughness * (ND - 1), reflDir.data(), ND);
  }
  float reflEvalAvg(float eta, float roughness) const {
    return interp2D(etaParam(eta) * (ND - 1), roughness * (ND - 1), reflAvg.data(), ND, ND);
  }
};
const AlbedoTables &albedoTables();

// ---- principled BSDF restricted to the plastic + conductor lobes
// scattering types (render/pathtracer/Scattering.ih:8-47)
enum : int { SCATTER_SPEC_R = 1, SCATTER_GLOSSY_R = 2, SCATTER_DIFFUSE_R = 4 };

// Principled.cpp:37-79 parameters of the base stack (transmission, thin,
// coat and sheen at their defaults)
struct PrincipledParams {
  V3 baseColor;
  float roughness, metallic;
  float specular = 1.f, ior = 1.f, diffuse = 1.f;
  V3 edgeColor = {1.f, 1.f, 1.f};
  bool specularMetallic = true;
  bool fromOutside = true;  // the path travels in the outside medium (vacuum)
};

struct BSDFEval {
  V3 value;
  float pdf;
};
struct BSDFSample {
  V3 wi, weight;
  float pdf;
  int type;
};

struct Principled {
  L3 frame;
  V3 N;
  float roughness;
  GGX ggx;
  // base MultiBSDF: child 0 conductor, child 2 plastic
  float wC, iC, wP, iP, impSum;
  // conductor
  V3 ceta, ck, cFmsScale;
  float cEavg;
  // plastic = dielectric layer (eta, weight = specular) over Oren-Nayar;
  // roughness 0: smooth DielectricLayer over Lambert and a smooth Conductor
  V3 diffuse;  // baseColor * diffuse
  float eta, lEavg, lFmsScale, lRavg, lWeight, lFavg;
  bool smoothBase = false, hasLayer = false, smooth = false;
  V3 lAlbedo;  // layer albedo (substrate albedo scaled)
  V3 albedo;   // BSDF albedo (for the shading AOV / coat pick)
  void init(const PrincipledParams &p, const L3 &shadingFrame);
  BSDFEval eval(V3 wo, V3 wi) const;
  BSDFSample sample(V3 wo, V2 s, float ss) const;
  // children
  BSDFEval evalConductor(V3 wo, V3 wi) const;
  BSDFSample sampleConductor(V3 wo, V2 s) const;
  BSDFEval evalOrenNayar(V3 wo, V3 wi) const;
  BSDFSample sampleDiffuse(V3 wo, V2 s) const;
  BSDFEval evalPlastic(V3 wo, V3 wi) const;
  BSDFSample samplePlastic(V3 wo, V2 s, float ss) const;
};

// ---- lights
struct LightSample {
  V3 weight, dir;
  float dist, pdf;
};
struct LightEval {
  V3 radiance;
  float pdf;
};
struct QuadLight {
  V3 position, edge1, edge2, nnormal, radiance;
  float ppdf;
  bool visible;
  void init(V3 pos, V3 e1, V3 e2, V3 rad);
  LightSample sample(const DG &dg, V2 s) const;
  LightEval eval(const DG &dg, V3 dir, float minDist, float maxDist) const;
};
struct AmbientLight {
  V3 radiance;
  bool visible;
  LightSample sample(const DG &dg, V2 s) const;
  LightEval eval(const DG &dg, V3 dir, float minDist, float maxDist) const;
};
// DirectionalLight (lights/DirectionalLight.ispc:14-90, .cpp:77-105):
// dir towards the light, cone of half the angular diameter, irradiance
struct DistantLight {
  V3 dir, irradiance;
  float cosAngle, pdf;
  bool visible;
  void init(V3 direction, float angularDiameterDeg, V3 irr);
  LightSample sample(const DG &dg, V2 s) const;
  LightEval eval(const DG &dg, V3 dir, float minDist, float maxDist) const;
};
// PointLight (lights/PointLight.ispc:32-158, .cpp:68-121) with
// intensityQuantity INTENSITY and no intensity distribution
// SpotLight (lights/SpotLight.ispc:26-170, .cpp:76-140), intensityQuantity
// INTENSITY, no intensity distribution
struct SpotLight {
  V3 position, dir, c0, c90, radiance, intensity;
  float cosAngleMax, cosAngleScale, radius, innerRadius, areaPdf;
  bool visible;
  void init(V3 pos, V3 direction, float openingDeg, float penumbraDeg, float r, float ri, V3 coloredIntensity);
  LightSample sample(const DG &dg, V2 s) const;
  LightEval eval(const DG &dg, V3 dir, float minDist, float maxDist) const;
};
struct SphereLight {
  V3 position, radiance, intensity;
  float radius;
  bool visible;
  void init(V3 pos, float r, V3 coloredIntensity);
  LightSample sample(const DG &dg, V2 s) const;
  LightEval eval(const DG &dg, V3 dir, float minDist, float maxDist) const;
};

// ---- materials of the path tracer beyond the principled stack
//   render/materials/Principled.ispc:81-455 (root MultiBSDF with the cut-out)
//   render/materials/OBJ.ispc:29-126, OBJ.cpp:28-65; bsdfs/Lambert.ih,
//     Specular.ih, Transmission.ih, math/sampling.ih
//   render/materials/Metal.ispc:16-48, Metal.cpp:27-70; bsdfs/Conductor.ih,
//     MicrofacetConductor.ih, Fresnel.ih (FresnelConductorRGBUniform)
//   render/materials/Glass.ispc:16-60, Glass.cpp:27-50; bsdfs/RobustDielectric.ih
//   render/materials/ThinGlass.ispc:16-70, ThinGlass.cpp:27-45;
//     bsdfs/RobustThinDielectric.ih
//   render/materials/Medium.ih
enum : int { MAT_PRINCIPLED = 0, MAT_OBJ = 1, MAT_METAL = 2, MAT_GLASS = 3, MAT_THINGLASS = 4 };
enum : int {
  SCATTER_SPEC_T = 8,
  SCATTER_GLOSSY_T = 16,
  SCATTER_DIFFUSE_T = 32,
  SCATTER_REFLECTION = SCATTER_SPEC_R | SCATTER_GLOSSY_R | SCATTER_DIFFUSE_R,
  SCATTER_TRANSMISSION = SCATTER_SPEC_T | SCATTER_GLOSSY_T | SCATTER_DIFFUSE_T,
  SCATTER_SPECULAR = SCATTER_SPEC_R | SCATTER_SPEC_T,
  SCATTER_SMOOTH = SCATTER_GLOSSY_R | SCATTER_DIFFUSE_R | SCATTER_GLOSSY_T | SCATTER_DIFFUSE_T
};

struct Medium {
  float ior;
  V3 att;
};
inline bool sameMedium(const Medium &a, const Medium &b) {
  return a.ior == b.ior && a.att.x == b.att.x && a.att.y == b.att.y && a.att.z == b.att.z;
}
inline Medium vacuum() { return {1.f, v3(0.f)}; }

// a material after its type's commit
struct MaterialParams {
  int type = MAT_PRINCIPLED;
  V3 baseColor = v3(0.8f);  // principled baseColor; obj kd (energy-scaled)
  float roughness = 0.f, metallic = 0.f, opacity = 1.f;
  V3 ks = v3(0.f), tf = v3(0.f);  // obj (energy-scaled)
  float ns = 10.f;
  V3 eta = v3(0.f), k = v3(0.f);  // metal
  Medium inside = {1.f, v3(0.f)}, outside = {1.f, v3(0.f)};  // glass
  float thinEta = 1.f;  // thin glass: 1 / eta
  V3 thinAtt = v3(0.f);
  // principled base-stack parameters
  float specular = 1.f, ior = 1.f, diffuse = 1.f;
  V3 edgeColor = v3(1.f);
  bool specularMetallic = true;
  // principled map_baseColor / obj map_kd (null: none); mapAlpha: it has alpha
  const Texture *map = nullptr;
  bool mapAlpha = false;
};
// p: baseColor[3], roughness, metallic, opacity, ks[3], ns, tf[3], eta[3],
// k[3], attenuationColor[3], attenuationDistance, thickness, specular, ior,
// diffuse, edgeColor[3], specularMetallic (31 floats, the b200_material
// fields after its type without the colour map)
MaterialParams commitMaterial(int type, const float *p);
bool transparentMaterial(const MaterialParams &m);

struct SurfaceBSDF {
  int type = MAT_PRINCIPLED;
  bool smooth = false;
  V3 albedo = v3(0.f), N = v3(0.f);
  // principled: base stack + root (transmission importance tr, stack weight op)
  Principled st;
  float op = 0.f, tr = 0.f, impSum = 0.f;
  bool hasStack = false, hasCut = false;
  // obj
  L3 fr;
  V3 Kd = v3(0.f), T = v3(0.f), ksN = v3(0.f), specW = v3(0.f);
  float nsB = 0.f, iL = 0.f, iT = 0.f, iS = 0.f;
  // metal
  V3 ceta = v3(0.f), ck = v3(0.f);
  float rough = 0.f;
  GGX ggx = {0.f, 0.f};
  bool specular = false;
  // glass (RobustDielectric) and thin glass
  float geta = 1.f;
  V3 Ns = v3(0.f), Ng = v3(0.f), tatt = v3(0.f);
  BSDFEval eval(V3 wo, V3 wi) const;
  BSDFSample sample(V3 wo, V2 s, float ss) const;
};
// Material_dispatch_getBSDF for a hit with differential geometry dg; dPds the
// instance's x axis (makeShadingFrame), cur the path's current medium,
// footprint the hit's pixel footprint for the colour map's level selection
SurfaceBSDF makeBSDF(const MaterialParams &m, const DG &dg, V3 dPds, const Medium &cur, float footprint = 0.f);
// Material_getTransparency for a shadow ray of direction rayDir
V3 materialTransparency(const MaterialParams &m, const DG &dg, V3 rayDir, const Medium &cur, float footprint = 0.f);
// Material_selectNextMedium (glass; the others keep the medium)
Medium nextMedium(const MaterialParams &m, const Medium &cur);

}  // namespace orc
