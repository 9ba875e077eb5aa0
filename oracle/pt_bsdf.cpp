// Oracle (test infrastructure only): BSDF and light implementations; see
// pt_bsdf.h for the reference files each part restates.
#include "pt_bsdf.h"

#include <algorithm>

namespace orc {

namespace {
// MicrofacetAlbedo_sample / MicrofacetDielectricReflectionAlbedo_sample
float albedoSample(float cosO, const GGX &m, V2 s, bool dielectric, float eta) {
  cosO = std::fmax(cosO, 1e-6f);
  const V3 wo = v3(cos2sin(cosO), 0.f, cosO);
  float whPdf;
  const V3 wh = ggxSampleVisible(m, wo, whPdf, s);
  const float cosOH = dot(wo, wh);
  const V3 wi = reflectV(wo, wh, cosOH);
  if (wi.z <= 0.f) return 0.f;
  const float G = ggxG2(m, wo, wi, cosOH, dot(wi, wh));
  const float w = G * rcp_safe(ggxG1(m, wo, cosOH));
  return dielectric ? fresnelDielectric(cosOH, eta) * w : w;
}
float integrate(float cosO, float roughness, bool dielectric, float eta) {
  const GGX m = makeGGX(roughness);
  const int n = 32;  // sqrt(1024) stratified samples
  float sum = 0.f;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      const V2 s = {std::fmin((i + 0.5f) / n, 1.f - 1e-6f), std::fmin((j + 0.5f) / n, 1.f - 1e-6f)};
      sum += albedoSample(cosO, m, s, dielectric, eta);
    }
  return std::fmin(sum / (n * n), 1.f);
}
// MicrofacetAlbedoTable_integrateAvg
float integrateAvg(const float *f, int size) {
  const int n = 1025;
  float sum = 0.f;
  for (int i = 0; i < n; i++) {
    const float c = float(i) / (n - 1);
    sum += interp1D(c * (size - 1), f, size) * c * ((i == 0 || i == n - 1) ? 0.5f : 1.f);
  }
  return std::fmin(2.f * (sum / (n - 1)), 1.f);
}
}  // namespace

AlbedoTables::AlbedoTables() {
  dir.resize(N * N);
  avg.resize(N);
  for (int j = 0; j < N; j++) {
    const float r = float(j) / (N - 1);
    for (int i = 0; i < N; i++) dir[j * N + i] = integrate(float(i) / (N - 1), r, false, 1.f);
    avg[j] = integrateAvg(&dir[j * N], N);
  }
  reflDir.resize(ND * ND * ND);
  reflAvg.resize(ND * ND);
  const float minEta = 1.f / 3.f, maxEta = 1.f;
  for (int k = 0; k < ND; k++) {
    const float r = float(k) / (ND - 1);
    for (int j = 0; j < ND; j++) {
      const float t = float(j) / (ND - 1);
      const float eta = (1.f - t) * minEta + t * maxEta;
      float *row = &reflDir[(size_t(k) * ND + j) * ND];
      for (int i = 0; i < ND; i++) row[i] = integrate(float(i) / (ND - 1), r, true, eta);
      reflAvg[k * ND + j] = integrateAvg(row, ND);
    }
  }
}

const AlbedoTables &albedoTables() {
  static const AlbedoTables t;
  return t;
}

// The principled base stack (Principled.ispc:110-331) without
// transmission, coat or sheen: a MultiBSDF of the conductor (child 0) and
// the plastic layer (child 2).  roughness 0 (the parameter, < EPS): a smooth
// DielectricLayer over Lambert (bsdfs/DielectricLayer.ih) and a smooth
// Conductor (bsdfs/Conductor.ih); else MicrofacetDielectricLayer over
// Oren-Nayar and MicrofacetConductor.  specular 0: a PassthroughLayer.
void Principled::init(const PrincipledParams &p, const L3 &f) {
  frame = f;
  N = f.vz;
  const AlbedoTables &T = albedoTables();
  const V3 baseColor = {clamp01(p.baseColor.x), clamp01(p.baseColor.y), clamp01(p.baseColor.z)};
  const float metallic = clamp01(p.metallic), specular = clamp01(p.specular), diffuseW = clamp01(p.diffuse);
  roughness = clamp01(p.roughness);
  ggx = makeGGX(roughness);
  smoothBase = p.roughness < EPS;
  albedo = v3(0.f);
  wC = iC = wP = iP = impSum = 0.f;
  smooth = hasLayer = false;
  const float dielectric = 1.f - metallic;
  if (dielectric > EPS) {
    float ior = p.ior;
    if (ior < 1.f) ior = 1.f / ior;
    // eta = outside ior (vacuum, 1) / ior from outside, ior / outside ior inside
    float e = p.fromOutside ? 1.f * (1.f / ior) : ior * (1.f / 1.f);
    e = clampf(e, 1.f / 3.f, 3.f);
    const float plastic = dielectric;  // transmission 0
    if (plastic > EPS) {
      diffuse = baseColor * diffuseW;
      hasLayer = specular > EPS;
      // the layer keeps eta folded to <= 1.  (MicrofacetDielectricLayer_Constructor
      // reads self->eta before assigning it when computing Ravg; the assigned value
      // is used here.)
      eta = e <= 1.f ? e : 1.f / e;
      lWeight = specular;
      lAlbedo = diffuse;  // PassthroughLayer: the substrate's albedo
      if (hasLayer && smoothBase) {
        lFavg = fresnelDielectricAvg(e) * lWeight;
        lAlbedo = diffuse * ((1.f - lWeight) + 1.f * (1.f - lFavg));
      } else if (hasLayer) {
        lEavg = T.evalAvg(roughness);
        const float Favg = fresnelDielectricAvg(e);
        lFmsScale = Favg * (1.f - lEavg) / (1.f - Favg * lEavg);
        lRavg = (T.reflEvalAvg(eta, roughness) + lFmsScale * (1.f - lEavg)) * lWeight;
        lAlbedo = diffuse * ((1.f - lWeight) + 1.f * (1.f - Favg));
      }
      wP = plastic;
      iP = plastic * std::fmax(diffuseW, specular);
      impSum += iP;
      albedo = albedo + lAlbedo * wP;
      smooth = true;
    }
  }
  const float conductor = metallic * (p.specularMetallic ? specular : 1.f);
  if (conductor > EPS) {
    // FresnelConductorArtistic_create (bsdfs/Fresnel.ih): n between n_min and
    // n_max by the edge colour, k from the reflectivity
    const V3 r = vmin(baseColor, v3(0.99f));
    const V3 g = {clamp01(p.edgeColor.x), clamp01(p.edgeColor.y), clamp01(p.edgeColor.z)};
    const float rr[3] = {r.x, r.y, r.z}, gg[3] = {g.x, g.y, g.z};
    float ne[3], nk[3], favg[3];
    for (int c = 0; c < 3; c++) {
      const float nmin = (1.f - rr[c]) / (1.f + rr[c]);
      const float nmax = (1.f + std::sqrt(rr[c])) / (1.f - std::sqrt(rr[c]));
      const float n = gg[c] * nmin + (1.f - gg[c]) * nmax;
      const float k2 = (sqr(n + 1.f) * rr[c] - sqr(n - 1.f)) / (1.f - rr[c]);
      ne[c] = n;
      nk[c] = std::sqrt(std::fmax(k2, 0.f));
      const float R = rr[c], R2 = R * R, R3 = R2 * R, G = gg[c], G2 = G * G, G3 = G2 * G;
      favg[c] = 0.087237f + 0.0230685f * G - 0.0864902f * G2 + 0.0774594f * G3 + 0.782654f * R - 0.136432f * R2 +
                0.278708f * R3 + 0.19744f * G * R + 0.0360605f * G2 * R - 0.2586f * G * R2;
    }
    ceta = {ne[0], ne[1], ne[2]};
    ck = {nk[0], nk[1], nk[2]};
    const V3 Favg = {favg[0], favg[1], favg[2]};
    wC = conductor;
    iC = conductor;
    impSum += iC;
    if (smoothBase) {
      albedo = albedo + Favg * wC;  // Conductor: albedo = the Fresnel average
    } else {
      cEavg = T.evalAvg(roughness);
      // Stephen Hill's multiple-scattering tweak (MicrofacetConductor_Constructor)
      cFmsScale = {sqr(Favg.x) * cEavg / (1.f - Favg.x * (1.f - cEavg)),
                   sqr(Favg.y) * cEavg / (1.f - Favg.y * (1.f - cEavg)),
                   sqr(Favg.z) * cEavg / (1.f - Favg.z * (1.f - cEavg))};
      albedo = albedo + (Favg * cEavg) * wC;
      smooth = true;
    }
  }
}

static V3 toLocal(const L3 &f, V3 v) { return {dot(v, f.vx), dot(v, f.vy), dot(v, f.vz)}; }

BSDFEval Principled::evalConductor(V3 wo, V3 wi) const {
  if (smoothBase) return {v3(0.f), 0.f};  // Dirac
  const float cosO = dot(wo, N), cosI = dot(wi, N);
  if (cosO <= 0.f || cosI <= 0.f) return {v3(0.f), 0.f};
  const V3 wh = normalize(wi + wo);
  const float cosOH = dot(wo, wh), cosIH = dot(wi, wh);
  const V3 wo0 = toLocal(frame, wo), wi0 = toLocal(frame, wi), wh0 = toLocal(frame, wh);
  const V3 F = {fresnelConductor1(cosOH, ceta.x, ck.x), fresnelConductor1(cosOH, ceta.y, ck.y),
                fresnelConductor1(cosOH, ceta.z, ck.z)};
  float whPdf;
  const float D = ggxEvalVisible(ggx, wh0, wo0, cosOH, whPdf);
  const float G = ggxG2(ggx, wo0, wi0, cosOH, cosIH);
  const AlbedoTables &T = albedoTables();
  const float Eo = T.eval(cosO, roughness), Ei = T.eval(cosI, roughness);
  const V3 fms = cFmsScale * ((1.f - Eo) * (1.f - Ei) / (PI * (1.f - cEavg)) * cosI);
  return {F * (D * G / (4.f * cosO)) + fms, whPdf / (4.f * std::fabs(cosOH))};
}

BSDFSample Principled::sampleConductor(V3 wo, V2 s) const {
  BSDFSample res = {v3(0.f), v3(0.f), 0.f, 0};
  if (smoothBase) {  // Conductor_sample: mirror direction, weight = Fresnel
    const float c = dot(wo, N);
    res.wi = reflectV(wo, N, c);
    res.pdf = INFINITY;
    res.type = SCATTER_SPEC_R;
    res.weight = {fresnelConductor1(c, ceta.x, ck.x), fresnelConductor1(c, ceta.y, ck.y),
                  fresnelConductor1(c, ceta.z, ck.z)};
    return res;
  }
  const float cosO = dot(wo, N);
  if (cosO <= 0.f) return res;
  const V3 wo0 = toLocal(frame, wo);
  float whPdf;
  const V3 wh = xfmVector(frame, ggxSampleVisible(ggx, wo0, whPdf, s));
  res.wi = reflectV(wo, wh, dot(wo, wh));
  const float cosI = dot(res.wi, N);
  if (cosI <= 0.f) return {v3(0.f), v3(0.f), 0.f, 0};
  const float cosOH = dot(wo, wh), cosIH = dot(res.wi, wh);
  const V3 wi0 = toLocal(frame, res.wi);
  const V3 F = {fresnelConductor1(cosOH, ceta.x, ck.x), fresnelConductor1(cosOH, ceta.y, ck.y),
                fresnelConductor1(cosOH, ceta.z, ck.z)};
  const float G = ggxG2(ggx, wo0, wi0, cosOH, cosIH);
  const AlbedoTables &T = albedoTables();
  const float Eo = T.eval(cosO, roughness), Ei = T.eval(cosI, roughness);
  const V3 fms = cFmsScale * ((1.f - Eo) * (1.f - Ei) / (PI * (1.f - cEavg)) * cosI);
  res.type = SCATTER_GLOSSY_R;
  res.pdf = whPdf / (4.f * std::fabs(cosOH));
  res.weight = F * (G * rcp_safe(ggxG1(ggx, wo0, cosOH))) + fms * (1.f / res.pdf);
  return res;
}

// Oren-Nayar (bsdfs/OrenNayar.ih:13-63); Lambert at roughness 0
BSDFEval Principled::evalOrenNayar(V3 wo, V3 wi) const {
  const float cosO = std::fmax(dot(wo, N), 0.f), cosI = std::fmax(dot(wi, N), 0.f);
  const float s = dot(wo, wi) - cosO * cosI;
  const float sInvt = s > 0.f ? s * rcp_safe(std::fmax(cosO, cosI)) : s;
  const V3 v = diffuse * (cosI * (1.f + roughness * sInvt) / (PI + (PI / 2.f - 2.f / 3.f) * roughness));
  return {v, cosI / PI};
}

BSDFSample Principled::sampleDiffuse(V3 wo, V2 s) const {
  BSDFSample res;
  // cosine hemisphere in the shading frame
  const float phi = 2.f * PI * s.x;
  const float cosT = std::sqrt(s.y), sinT = std::sqrt(1.f - s.y);
  const V3 local = {std::cos(phi) * sinT, std::sin(phi) * sinT, cosT};
  res.wi = xfmVector(frame, local);
  const BSDFEval e = evalOrenNayar(wo, res.wi);
  res.pdf = e.pdf;
  res.type = SCATTER_DIFFUSE_R;
  res.weight = e.value * (1.f / e.pdf);
  return res;
}

// MICROFACETDIELECTRICLAYER_EVAL / DIELECTRICLAYER_EVAL with a diffuse substrate
BSDFEval Principled::evalPlastic(V3 wo, V3 wi) const {
  if (!hasLayer) return evalOrenNayar(wo, wi);  // PassthroughLayer
  const float cosO = dot(wo, N);
  if (cosO <= 0.f) return {v3(0.f), 0.f};
  const float cosI = dot(wi, N);
  BSDFEval sub = evalOrenNayar(wo, wi);
  if (smoothBase) {
    float cosO1, cosI1;
    const float F = fresnelDielectricEx(cosO, cosO1, eta);
    const float Fo = F * lWeight, Fi = fresnelDielectricEx(std::fabs(cosI), cosI1, eta) * lWeight;
    sub.value = sub.value * ((1.f - Fo) * (1.f - Fi) * (1.f / (1.f - lFavg)));
    const float coatPick = Fo / ((1.f - F) * reduce_max(lAlbedo) + Fo);
    sub.pdf *= 1.f - coatPick;
    return sub;
  }
  // substrate MultiBSDF (one child, weight 1, importance 1)
  // coating absorption: transmittance 1 -> factor 1 (lerp of equal values)
  const AlbedoTables &T = albedoTables();
  const float Eo = T.eval(cosO, roughness), Ei = T.eval(std::fabs(cosI), roughness);
  const float Ro = (T.reflEval(cosO, eta, roughness) + lFmsScale * (1.f - Eo)) * lWeight;
  const float Ri = (T.reflEval(std::fabs(cosI), eta, roughness) + lFmsScale * (1.f - Ei)) * lWeight;
  const float Tr = (1.f - Ro) * (1.f - Ri) / (1.f - lRavg);
  sub.value = sub.value * Tr;
  const float coatPick = lWeight * Ro / ((1.f - Ro) * reduce_max(lAlbedo) + lWeight * Ro);
  const float subPick = 1.f - coatPick;
  if (cosI > 0.f) {
    const V3 wh = normalize(wo + wi);
    const float cosOH = dot(wo, wh);
    const float F = fresnelDielectric(cosOH, eta) * lWeight;
    const float cosIH = dot(wi, wh);
    const V3 wo0 = toLocal(frame, wo), wi0 = toLocal(frame, wi), wh0 = toLocal(frame, wh);
    float whPdf;
    const float D = ggxEvalVisible(ggx, wh0, wo0, cosOH, whPdf);
    const float G = ggxG2(ggx, wo0, wi0, cosOH, cosIH);
    const float fms = lFmsScale * ((1.f - Eo) * (1.f - Ei) / (PI * (1.f - lEavg)) * cosI);
    const float coatPdf = whPdf / (4.f * cosOH);
    const float coatVal = F * D * G / (4.f * cosO) + fms;
    sub.pdf = coatPick * coatPdf + subPick * sub.pdf;
    sub.value = v3(coatVal) + sub.value;
  } else {
    sub.pdf *= subPick;
  }
  return sub;
}

// MICROFACETDIELECTRICLAYER_SAMPLE / DIELECTRICLAYER_SAMPLE with a diffuse substrate
BSDFSample Principled::samplePlastic(V3 wo, V2 s, float ss) const {
  BSDFSample res = {v3(0.f), v3(0.f), 0.f, 0};
  if (!hasLayer) return sampleDiffuse(wo, s);  // PassthroughLayer
  const float cosO = dot(wo, N);
  if (cosO <= 0.f) return res;
  if (smoothBase) {
    float cosO1;
    const float F = fresnelDielectricEx(cosO, cosO1, eta);
    const float Fo = F * lWeight;
    const float coatPick = Fo / ((1.f - F) * reduce_max(lAlbedo) + Fo);
    if (ss < coatPick) {
      res.type = SCATTER_SPEC_R;
      res.wi = reflectV(wo, N, cosO);
      res.pdf = INFINITY;
      res.weight = v3(Fo / coatPick);
      return res;
    }
    res = sampleDiffuse(wo, s);
    if (reduce_max(res.weight) <= 0.f) return res;
    float cosI1;
    const float Fi = fresnelDielectricEx(std::fabs(dot(res.wi, N)), cosI1, eta) * lWeight;
    const float Tr = (1.f - Fo) * (1.f - Fi) * (1.f / (1.f - lFavg));
    res.weight = res.weight * (Tr * (1.f / (1.f - coatPick)));
    res.pdf *= 1.f - coatPick;
    return res;
  }
  const V3 wo0 = toLocal(frame, wo);
  const AlbedoTables &T = albedoTables();
  const float Eo = T.eval(cosO, roughness);
  // (the reference's sample weighs only the multiple-scattering term here)
  const float Ro = T.reflEval(cosO, eta, roughness) + lFmsScale * (1.f - Eo) * lWeight;
  const float coatPick = lWeight * Ro / ((1.f - Ro) * reduce_max(lAlbedo) + lWeight * Ro);
  const float subPick = 1.f - coatPick;
  V3 wh;
  BSDFEval sub;
  if (ss < coatPick) {
    float whPdf;
    wh = xfmVector(frame, ggxSampleVisible(ggx, wo0, whPdf, s));
    res.type = SCATTER_GLOSSY_R;
    res.wi = reflectV(wo, wh, dot(wo, wh));
    sub = evalOrenNayar(wo, res.wi);
  } else {
    res = sampleDiffuse(wo, s);
    if (reduce_max(res.weight) <= 0.f) return res;
    sub.pdf = res.pdf;
    sub.value = res.weight * res.pdf;
    wh = normalize(wo + res.wi);
  }
  const float cosI = dot(res.wi, N);
  const float cosOH = dot(wo, wh);
  const float Ei = T.eval(std::fabs(cosI), roughness);
  const float Ri = (T.reflEval(std::fabs(cosI), eta, roughness) + lFmsScale * (1.f - Ei)) * lWeight;
  const float Tr = (1.f - Ro) * (1.f - Ri) / (1.f - lRavg);
  sub.value = sub.value * Tr;
  if (cosI <= 0.f) {
    res.pdf = subPick * sub.pdf;
    res.weight = sub.value * (1.f / res.pdf);
  } else {
    const float F = fresnelDielectric(cosOH, eta) * lWeight;
    const float cosIH = dot(res.wi, wh);
    const V3 wi0 = toLocal(frame, res.wi), wh0 = toLocal(frame, wh);
    float whPdf;
    const float D = ggxEvalVisible(ggx, wh0, wo0, cosOH, whPdf);
    const float G = ggxG2(ggx, wo0, wi0, cosOH, cosIH);
    const float fms = lFmsScale * ((1.f - Eo) * (1.f - Ei) / (PI * (1.f - lEavg)) * cosI);
    const float coatPdf = whPdf / (4.f * cosOH);
    const float coatVal = F * D * G / (4.f * cosO) + fms;
    res.pdf = coatPick * coatPdf + subPick * sub.pdf;
    res.weight = (v3(coatVal) + sub.value) * (1.f / res.pdf);
  }
  return res;
}

// MultiBSDF eval over {conductor (0), plastic (2)}
BSDFEval Principled::eval(V3 wo, V3 wi) const {
  BSDFEval r = {v3(0.f), 0.f};
  if (iC > 0.f) {
    const BSDFEval c = evalConductor(wo, wi);
    r.value = r.value + c.value * wC;
    r.pdf += c.pdf * iC;
  }
  if (iP > 0.f) {
    const BSDFEval c = evalPlastic(wo, wi);
    r.value = r.value + c.value * wP;
    r.pdf += c.pdf * iP;
  }
  r.pdf *= 1.f / impSum;
  return r;
}

// MultiBSDF sample over {conductor (0), plastic (2)} (MultiBSDF.ih:81-127):
// a Dirac lobe returns alone, scaled by 1 / its selection probability
BSDFSample Principled::sample(V3 wo, V2 s, float ss) const {
  BSDFSample res = {v3(0.f), v3(0.f), 0.f, 0};
  if (impSum == 0.f) return res;
  const float x = ss * impSum;
  float prefix = 0.f;
  int choice = -1;
  if (x < (prefix += iC)) {
    choice = 0;
    res = sampleConductor(wo, s);
    res.weight = res.weight * wC;
  } else if (x < (prefix += iP)) {
    choice = 2;
    const float ss1 = (x + iP - prefix) / iP;
    res = samplePlastic(wo, s, ss1);
    res.weight = res.weight * wP;
  }
  if (choice < 0 || (res.weight.x == 0.f && res.weight.y == 0.f && res.weight.z == 0.f) || res.pdf == 0.f)
    return {v3(0.f), v3(0.f), 0.f, 0};
  if (res.type & (SCATTER_SPEC_R | SCATTER_SPEC_T)) {
    res.weight = res.weight * (impSum * (1.f / (choice == 0 ? iC : iP)));
    return res;
  }
  V3 value = res.weight * res.pdf;
  float pdf = res.pdf * (choice == 0 ? iC : iP);
  if (choice != 0 && iC > 0.f) {
    const BSDFEval c = evalConductor(wo, res.wi);
    value = value + c.value * wC;
    pdf += c.pdf * iC;
  }
  if (choice != 2 && iP > 0.f) {
    const BSDFEval c = evalPlastic(wo, res.wi);
    value = value + c.value * wP;
    pdf += c.pdf * iP;
  }
  res.pdf = pdf * (1.f / impSum);
  res.weight = value * (1.f / res.pdf);
  return res;
}

// ---------------------------------------------------------------- lights
void QuadLight::init(V3 pos, V3 e1, V3 e2, V3 rad) {
  position = pos;
  edge1 = e1;
  edge2 = e2;
  const V3 nd = cross(e2, e1);
  ppdf = 1.f / length(nd);
  nnormal = nd * ppdf;
  radiance = rad;
  visible = true;
}

namespace {
struct SphQuad {
  V3 e0, e1, z;
  float S, k, n0z, n2z, x0, x1, y0, y1, z0;
};
SphQuad sphQuad(V3 q0, V3 e0, V3 e1, V3 n, V3 P) {
  const float e0l = length(e0), e1l = length(e1);
  SphQuad q;
  q.e0 = e0 / e0l;
  q.e1 = e1 / e1l;
  q.z = n;
  const V3 d = q0 - P;
  q.z0 = dot(d, q.z);
  q.z = q.z0 > 0.f ? -q.z : q.z;
  q.z0 = -std::fabs(q.z0);
  q.x0 = dot(d, q.e0);
  q.y0 = dot(d, q.e1);
  q.x1 = q.x0 + e0l;
  q.y1 = q.y0 + e1l;
  const V3 v00 = {q.x0, q.y0, q.z0}, v01 = {q.x0, q.y1, q.z0}, v10 = {q.x1, q.y0, q.z0}, v11 = {q.x1, q.y1, q.z0};
  const V3 n0 = normalize(cross(v00, v10)), n1 = normalize(cross(v10, v11));
  const V3 n2 = normalize(cross(v11, v01)), n3 = normalize(cross(v01, v00));
  q.n0z = n0.z;
  q.n2z = n2.z;
  const float g0 = std::acos(clampf(-dot(n0, n1), -1.f, 1.f));
  const float g1 = std::acos(clampf(-dot(n1, n2), -1.f, 1.f));
  const float g2 = std::acos(clampf(-dot(n2, n3), -1.f, 1.f));
  const float g3 = std::acos(clampf(-dot(n3, n0), -1.f, 1.f));
  q.k = 2.f * PI - g2 - g3;
  q.S = std::fmax(0.f, g0 + g1 - q.k);
  return q;
}
float signf(float x) { return float(0.f < x) - float(x < 0.f); }
V3 sampleSphQuad(const SphQuad &q, V2 s) {
  const float au = s.x * q.S + q.k;
  const float sinau = std::sin(au), cosau = std::cos(au);
  const float fu = (cosau * q.n0z - q.n2z) / sinau;
  const float cu = clampf(1.f / std::sqrt(fu * fu + sqr(q.n0z)) * signf(fu), -1.f, 1.f);
  const float x0 = -(cu * q.z0) / std::sqrt(1.f - cu * cu);
  const float xu = clampf(x0, q.x0, q.x1);
  const float ds = std::sqrt(sqr(xu) + sqr(q.z0));
  const float ds2 = sqr(ds);
  const float h0 = q.y0 / std::sqrt(ds2 + sqr(q.y0));
  const float h1 = q.y1 / std::sqrt(ds2 + sqr(q.y1));
  const float hv = s.y * (h1 - h0) + h0;
  const float hv2 = sqr(hv);
  const float yv = hv2 < 1.f - 1e-4f ? (hv * ds) / std::sqrt(1.f - hv2) : q.y1;
  return xu * q.e0 + yv * q.e1 + q.z0 * q.z;
}
float solveQuadratic(float A, float B, float C) {
  if (A == 0.f) return -C / B;
  float rad = B * B - 4.f * A * C;
  if (rad < 0.f) return 0.f;
  rad = std::sqrt(rad);
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
// Hart et al. 2020 bilinear cosine warp (SphericalQuadSampling.ih)
V3 cosineWeightedRNG(V3 q0, V3 e0, V3 e1, V3 P, V3 Ng, V2 s) {
  const V3 wp[4] = {q0, q0 + e0, q0 + e1, q0 + e0 + e1};
  float prob[4];
  for (int i = 0; i < 4; i++) prob[i] = std::fmax(0.f, dot(normalize(wp[i] - P), Ng));
  if (prob[0] + prob[2] == 0.f) return {s.x, s.y, 1.f};
  const float tot = prob[0] + prob[2] + prob[1] + prob[3];
  const float W00 = prob[0], W01 = prob[2], W10 = prob[1], W11 = prob[3];
  float u;
  {
    const float A = W10 + W11 - W01 - W00, B = 2.f * (W01 + W00);
    u = (A + B == 0.f) ? s.x : solveQuadratic(A, B, -(W00 + W01 + W10 + W11) * s.x);
  }
  float v;
  {
    const float A = (1.f - u) * W01 + u * W11 - (1.f - u) * W00 - u * W10;
    const float B = 2.f * (1.f - u) * W00 + 2.f * u * W10;
    v = (A + B == 0.f) ? s.y
                       : solveQuadratic(A, B, -((1.f - u) * W01 + u * W11 + (1.f - u) * W00 + u * W10) * s.y);
  }
  const float pdf = 4.f * ((1.f - u) * (1.f - v) * prob[0] + u * (1.f - v) * prob[1] + u * v * prob[3] +
                           (1.f - u) * v * prob[2]) / tot;
  return {u, v, pdf};
}
}  // namespace

LightSample QuadLight::sample(const DG &dg, V2 s) const {
  LightSample res;
  if (s.x == 0.f && s.y == 0.f) {
    // SampleArea at the quad centre
    const V3 p = position + edge1 * 0.5f + edge2 * 0.5f;
    const V3 d = p - dg.P;
    const float dist = length(d);
    res.dir = d / dist;
    res.dist = dist;
    const float cosd = dot(nnormal, res.dir);
    res.pdf = ppdf * sqr(dist) / std::fabs(cosd);
    res.weight = radiance * (cosd > 0.f ? 1.f / res.pdf : 0.f);
    return res;
  }
  const SphQuad q = sphQuad(position, edge1, edge2, -nnormal, dg.P);
  const V3 cw = cosineWeightedRNG(position, edge1, edge2, dg.P, dg.Ng, s);
  const V3 d = sampleSphQuad(q, {cw.x, cw.y});
  const float dist = length(d);
  res.dir = d / dist;
  res.dist = dist;
  const float cosd = dot(nnormal, res.dir);
  res.pdf = q.S == 0.f ? 0.f : cw.z / q.S;
  res.weight = (cosd > 0.f && res.pdf != 0.f) ? radiance * (1.f / res.pdf) : v3(0.f);
  return res;
}

LightEval QuadLight::eval(const DG &dg, V3 dir, float minDist, float maxDist) const {
  LightEval res = {v3(0.f), 0.f};
  const float cosd = dot(nnormal, dir);
  if (cosd <= 0.f) return res;
  const V3 c = position - dg.P;
  const V3 r = cross(c, dir);
  const float rcosd = 1.f / cosd;
  const float u = dot(r, edge1) * rcosd;
  const float v = -dot(r, edge2) * rcosd;
  if (std::fmin(u, v) < 0.f || std::fmax(u, v) * ppdf > 1.f) return res;
  const float dist = dot(nnormal, c) * rcosd;
  if (dist <= minDist || dist > maxDist) return res;
  const SphQuad q = sphQuad(position, edge1, edge2, -nnormal, dg.P);
  if (q.S > 0.f) {
    res.radiance = radiance;
    res.pdf = 1.f / q.S;
  }
  return res;
}

LightSample AmbientLight::sample(const DG &dg, V2 s) const {
  LightSample res;
  const float phi = 2.f * PI * s.x;
  const float cosT = std::sqrt(s.y), sinT = std::sqrt(1.f - s.y);
  const V3 local = {std::cos(phi) * sinT, std::sin(phi) * sinT, cosT};
  res.dir = xfmVector(frame(dg.Ns), local);
  res.pdf = local.z / PI;
  res.dist = INFINITY;
  res.weight = radiance * (1.f / res.pdf);
  return res;
}

LightEval AmbientLight::eval(const DG &dg, V3 dir, float, float maxDist) const {
  LightEval res;
  res.radiance = INFINITY <= maxDist ? radiance : v3(0.f);
  res.pdf = std::fmax(dot(dg.Ns, dir), 0.f) / PI;
  return res;
}


// uniformSampleCone (math/sampling.ih:92-97) about axis n
static V3 sampleCone(V3 n, float cosAngle, V2 s) {
  const float phi = 2.f * PI * s.x;
  const float cosT = 1.f - s.y * (1.f - cosAngle);
  const float sinT = std::sqrt(std::fmax(0.f, 1.f - cosT * cosT));
  return xfmVector(frame(n), {std::cos(phi) * sinT, std::sin(phi) * sinT, cosT});
}

void DistantLight::init(V3 direction, float angularDiameterDeg, V3 irr) {
  dir = -normalize(direction);
  const float ad = std::fmin(std::fmax(angularDiameterDeg, 0.f), 180.f);
  cosAngle = std::cos(ad * 0.5f * float(M_PI / 180.0));
  pdf = cosAngle < 0.99999988f ? 1.f / (2.f * PI * (1.f - cosAngle)) : INFINITY;
  irradiance = irr;
  visible = true;
}

LightSample DistantLight::sample(const DG &, V2 s) const {
  LightSample res;
  res.dir = dir;
  res.dist = INFINITY;
  res.pdf = pdf;
  if (cosAngle < 0.99999988f) res.dir = sampleCone(dir, cosAngle, s);
  res.weight = irradiance;
  return res;
}

LightEval DistantLight::eval(const DG &, V3 d, float, float maxDist) const {
  LightEval res;
  res.radiance = v3(0.f);
  res.pdf = 0.f;
  if (INFINITY <= maxDist && cosAngle < 0.99999988f && dot(dir, d) > cosAngle) {
    res.radiance = irradiance * pdf;
    res.pdf = pdf;
  }
  return res;
}

void SpotLight::init(V3 pos, V3 direction, float openingDeg, float penumbraDeg, float r, float ri, V3 ci) {
  position = pos;
  dir = normalize(direction);
  const V3 a = std::fabs(direction.x) < std::fabs(direction.y) ? V3{0.f, direction.z, direction.y}
                                                                : V3{direction.z, 0.f, direction.x};
  c90 = normalize(cross(a, dir));
  c0 = cross(dir, c90);
  const float opening = std::fmin(std::fmax(openingDeg, 0.f), 360.f);
  const float penumbra = std::fmin(std::fmax(penumbraDeg, 0.f), 0.5f * opening);
  const float deg = float(M_PI / 180.0);
  cosAngleMax = std::cos(deg * 0.5f * opening);
  cosAngleScale = 1.f / (std::cos(deg * (0.5f * opening - penumbra)) - cosAngleMax);
  radius = std::fmax(0.f, r);
  innerRadius = std::fmin(std::fmax(ri, 0.f), 0.999f * radius);
  const float ring = PI * (radius * radius - innerRadius * innerRadius);
  areaPdf = 1.f / ring;
  intensity = ci;
  radiance = radius > 0.f ? ci * (1.f / ring) : v3(0.f);
  visible = true;
}

LightSample SpotLight::sample(const DG &dg, V2 s) const {
  LightSample res;
  res.dir = position - dg.P;
  if (radius > 0.f) {
    const float rr = std::sqrt((1.f - s.x) * (innerRadius * innerRadius) + s.x * (radius * radius));
    const float phi = 2.f * PI * s.y;
    res.dir = c0 * (rr * std::cos(phi)) + c90 * (rr * std::sin(phi)) + res.dir;
  }
  const float dist2 = dot(res.dir, res.dir);
  const float invdist = 1.f / std::sqrt(dist2);
  res.dir = res.dir * invdist;
  res.dist = dist2 * invdist;
  const float cosAngle = -dot(dir, res.dir);
  float w = clampf((cosAngle - cosAngleMax) * cosAngleScale, 0.f, 1.f);
  if (radius > 0.f) {
    res.pdf = areaPdf * (dist2 / std::fabs(cosAngle));
    w = w / res.pdf;
    res.weight = radiance * w;
  } else {
    res.pdf = INFINITY;
    w *= std::fabs(cosAngle);
    res.weight = intensity * ((invdist * invdist) * w);
  }
  return res;
}

LightEval SpotLight::eval(const DG &dg, V3 d, float minDist, float maxDist) const {
  LightEval res;
  res.radiance = v3(0.f);
  res.pdf = 0.f;
  if (radius > 0.f) {
    const float cosAngle = -dot(dir, d);
    if (cosAngle > cosAngleMax) {
      const V3 vp = dg.P - position;
      const float t = dot(vp, dir) * (1.f / cosAngle);
      if (t > minDist && t <= maxDist) {
        const V3 vd = vp + d * t;
        const float d2 = dot(vd, vd);
        if (d2 < radius * radius && d2 > innerRadius * innerRadius) {
          res.radiance = radiance * clampf((cosAngle - cosAngleMax) * cosAngleScale, 0.f, 1.f);
          res.pdf = areaPdf * (t * t / std::fabs(cosAngle));
        }
      }
    }
  }
  return res;
}

void SphereLight::init(V3 pos, float r, V3 coloredIntensity) {
  position = pos;
  radius = r;
  intensity = coloredIntensity;
  radiance = r > 0.f ? coloredIntensity * (1.f / (PI * r * r)) : v3(0.f);
  visible = true;
}

LightSample SphereLight::sample(const DG &dg, V2 s) const {
  LightSample res;
  const V3 d = position - dg.P;
  const float dist2 = dot(d, d);
  const float invdist = 1.f / std::sqrt(dist2);
  res.dir = d * invdist;
  res.dist = dist2 * invdist;
  res.pdf = INFINITY;
  const float sinTheta = radius * invdist;
  if (radius > 0.f && sinTheta > 0.005f) {
    if (sinTheta < 1.f) {
      const float cosTheta = std::sqrt(1.f - sinTheta * sinTheta);
      const float phi = 2.f * PI * s.x;
      const float c = 1.f - s.y * (1.f - cosTheta);
      const float sn = std::sqrt(std::fmax(0.f, 1.f - c * c));
      res.dir = xfmVector(frame(res.dir), {std::cos(phi) * sn, std::sin(phi) * sn, c});
      res.pdf = 1.f / (2.f * PI * (1.f - cosTheta));
      res.dist = c * res.dist - std::sqrt(std::fmax(0.f, radius * radius - (1.f - c * c) * dist2));
      res.weight = radiance * (1.f / res.pdf);
    } else {
      res.weight = v3(0.f);
    }
  } else {
    res.weight = intensity * (invdist * invdist);
  }
  return res;
}

LightEval SphereLight::eval(const DG &dg, V3 dir, float minDist, float maxDist) const {
  LightEval res;
  res.radiance = v3(0.f);
  res.pdf = 0.f;
  const V3 A = position - dg.P;
  const float sinTheta2 = radius * radius / dot(A, A);
  if (radius > 0.f && std::sqrt(sinTheta2) > 0.005f) {
    const float rd2 = 1.f / dot(dir, dir);
    const float projCO = dot(A, dir) * rd2;
    const V3 perp = A - dir * projCO;
    const float l2 = dot(perp, perp);
    if (l2 <= radius * radius) {
      const float t = projCO - std::sqrt((radius * radius - l2) * rd2);
      if (t > minDist && t < maxDist) {
        res.pdf = 1.f / (2.f * PI * (1.f - std::sqrt(1.f - sinTheta2)));
        res.radiance = radiance;
      }
    }
  }
  return res;
}

}  // namespace orc
