// Oracle (test infrastructure only): the path tracer's material types other
// than the principled base stack, restated from the reference:
//   Principled root MultiBSDF with the cut-out  render/materials/Principled.ispc:81-455
//   OBJ          render/materials/OBJ.ispc:29-126, OBJ.cpp:28-65
//                bsdfs/Lambert.ih, Specular.ih, Transmission.ih, math/sampling.ih
//   Metal        render/materials/Metal.ispc:16-48, Metal.cpp:27-70
//                bsdfs/Conductor.ih, MicrofacetConductor.ih, Fresnel.ih
//   Glass        render/materials/Glass.ispc:16-60, Glass.cpp:27-50, bsdfs/RobustDielectric.ih
//   ThinGlass    render/materials/ThinGlass.ispc:16-70, ThinGlass.cpp:27-45,
//                bsdfs/RobustThinDielectric.ih
//   MultiBSDF    bsdfs/MultiBSDF.ih (eval / sample macros)
#include <algorithm>

#include "pt_bsdf.h"

namespace orc {

namespace {
constexpr float ONE_OVER_PI = 0.31830988618379067154f;
constexpr float ONE_OVER_TWO_PI = 0.15915494309189533577f;
constexpr float ONE_OVER_FOUR_PI = 0.07957747154594766788f;
constexpr float LN2_OVER_2 = 0.34657359027997265471f;

inline float luminance(V3 c) { return 0.212671f * c.x + 0.715160f * c.y + 0.072169f * c.z; }
inline V3 vexp(V3 a) { return {std::exp(a.x), std::exp(a.y), std::exp(a.z)}; }
inline V3 vlog(V3 a) { return {std::log(a.x), std::log(a.y), std::log(a.z)}; }
inline V3 toLocalF(const L3 &f, V3 v) { return {dot(v, f.vx), dot(v, f.vy), dot(v, f.vz)}; }
inline bool isZero(V3 v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f; }
inline BSDFSample zeroSample() { return {v3(0.f), v3(0.f), 0.f, 0}; }

// cartesian(phi, sinTheta, cosTheta) of math/sampling.ih
inline V3 cartesian(float phi, float sinT, float cosT) { return {std::cos(phi) * sinT, std::sin(phi) * sinT, cosT}; }

V3 fresnelConductorRGB(float c, V3 eta, V3 k) {
  return {fresnelConductor1(c, eta.x, k.x), fresnelConductor1(c, eta.y, k.y), fresnelConductor1(c, eta.z, k.z)};
}



// RobustThinDielectric reflection R and transmission T of the slab
void thinSlab(float cosO, float eta, V3 att, V3 &R, V3 &T) {
  float cosT;
  const float Fo = fresnelDielectricEx(cosO, cosT, eta);
  const float Ft = fresnelDielectric(cosT, 1.f / eta);
  const V3 A = vexp(att * (1.f / cosT));
  const V3 FA = A * Ft;
  const V3 FA2 = FA * FA;
  const V3 inv = {1.f / (1.f - FA2.x), 1.f / (1.f - FA2.y), 1.f / (1.f - FA2.z)};
  R = v3(Fo) + (A * A) * ((1.f - Fo) * (1.f - Ft) * Ft) * inv;
  T = A * ((1.f - Fo) * (1.f - Ft)) * (v3(1.f) + FA2 * inv);
}
}  // namespace

MaterialParams commitMaterial(int type, const float *p) {
  MaterialParams m;
  m.type = type;
  const V3 base = {p[0], p[1], p[2]};
  const float roughness = p[3], metallic = p[4], opacity = p[5];
  const V3 ks = {p[6], p[7], p[8]};
  const float ns = p[9];
  const V3 tf = {p[10], p[11], p[12]}, eta = {p[13], p[14], p[15]}, k = {p[16], p[17], p[18]};
  const V3 attColor = {p[19], p[20], p[21]};
  const float attDist = p[22], thickness = p[23];
  m.specular = p[24];
  m.ior = p[25];
  m.diffuse = p[26];
  m.edgeColor = {p[27], p[28], p[29]};
  m.specularMetallic = p[30] != 0.f;
  constexpr float eps = 1e-6f;
  switch (type) {
    case MAT_OBJ: {
      // OBJMaterial::commit: kd + ks + tf scaled down to at most 1
      V3 kd = base, s = ks, t = tf;
      const float total = std::max({kd.x + s.x + t.x, kd.y + s.y + t.y, kd.z + s.z + t.z});
      if (total > 1.f) {
        kd = kd / total;
        s = s / total;
        t = t / total;
      }
      m.baseColor = kd;
      m.ks = s;
      m.tf = t;
      m.ns = ns;
      m.opacity = opacity;
      break;
    }
    case MAT_METAL:
      m.roughness = roughness;
      m.eta = eta;
      m.k = k;
      break;
    case MAT_GLASS:
      m.inside = {eta.x, vlog(attColor) / std::max(attDist, eps)};
      m.outside = {eta.y, v3(0.f)};
      break;
    case MAT_THINGLASS:
      m.thinEta = 1.f / eta.x;
      m.thinAtt = vlog(attColor) * (thickness * (1.f / std::max(attDist, eps)));
      break;
    default:
      m.baseColor = base;
      m.roughness = roughness;
      m.metallic = metallic;
      m.opacity = opacity;
      break;
  }
  return m;
}

bool transparentMaterial(const MaterialParams &m) {
  if (m.mapAlpha && (m.type == MAT_PRINCIPLED || m.type == MAT_OBJ)) return true;
  switch (m.type) {
    case MAT_PRINCIPLED: return 1.f - m.opacity > EPS;
    case MAT_OBJ: {
      const V3 T = m.tf * m.opacity + v3(1.f - m.opacity);
      return T.x > 0.f || T.y > 0.f || T.z > 0.f;
    }
    case MAT_GLASS:
    case MAT_THINGLASS: return true;
    default: return false;
  }
}

// makeShadingFrame (common/DifferentialGeometry.ih) with dPds
static L3 shadingFrameOf(const DG &dg, V3 dPds) {
  const V3 N = dg.Ns;
  V3 U = normalize(dPds);
  V3 V = cross(N, U);
  if (dot(V, V) > 0.f) {
    V = normalize(V);
    U = cross(V, N);
    return {U, V, N};
  }
  return frame(N);
}

static bool glassFromOutside(const MaterialParams &m, const Medium &cur) { return sameMedium(cur, m.outside); }

// The colour map's texel at the hit (1 without a map)
static V4 mapTexel(const MaterialParams &m, const DG &dg, float footprint) {
  return m.map ? m.map->get(dg.st, footprint) : V4{1.f, 1.f, 1.f, 1.f};
}

// Principled.ispc:110-135 (baseColor x map.rgb x colour.rgb, clamped; opacity
// x map alpha) and OBJ.ispc:52-66 (d x colour alpha x map alpha, kd x map.rgb
// x colour.rgb): the material at this hit; `opacity` principled's effective one
static MaterialParams atHit(const MaterialParams &m0, const DG &dg, float footprint, float &opacity) {
  MaterialParams m = m0;
  opacity = clamp01(m0.opacity);
  if (m0.type == MAT_PRINCIPLED) {
    const V4 t = mapTexel(m0, dg, footprint);
    m.baseColor = {clamp01(m0.baseColor.x * t.x * dg.color.x), clamp01(m0.baseColor.y * t.y * dg.color.y),
                   clamp01(m0.baseColor.z * t.z * dg.color.z)};
    if (m0.mapAlpha) opacity *= t.w;
  } else if (m0.type == MAT_OBJ) {
    const V4 t = mapTexel(m0, dg, footprint);
    m.opacity = m0.opacity * dg.color.w * t.w;
    m.baseColor = {m0.baseColor.x * t.x * dg.color.x, m0.baseColor.y * t.y * dg.color.y,
                   m0.baseColor.z * t.z * dg.color.z};
  }
  return m;
}

SurfaceBSDF makeBSDF(const MaterialParams &m0, const DG &dg, V3 dPds, const Medium &cur, float footprint) {
  float opacity;
  const MaterialParams m = atHit(m0, dg, footprint, opacity);
  SurfaceBSDF b;
  b.type = m.type;
  switch (m.type) {
    case MAT_OBJ: {
      b.fr = shadingFrameOf(dg, dPds);
      b.N = b.fr.vz;
      const float d = m.opacity;
      b.Kd = m.baseColor * d;
      b.T = m.tf * d + v3(1.f - d);
      const V3 Ks = m.ks * d;
      b.impSum = 0.f;
      if (reduce_max(b.Kd) > 0.f) {
        b.iL = luminance(b.Kd);
        b.impSum += b.iL;
        b.albedo = b.albedo + b.Kd;
      }
      if (reduce_max(b.T) > 0.f) {
        b.iT = luminance(b.T);
        b.impSum += b.iT;
        b.albedo = b.albedo + b.T;
      }
      // Specular_Constructor: Phong exponent to Blinn, normalisation
      b.nsB = m.ns * 4.f;
      const float tmp = (b.nsB + 2.f) * (1.f / (2.f - std::exp(b.nsB * -LN2_OVER_2)));
      b.ksN = Ks * (ONE_OVER_FOUR_PI * tmp);
      b.specW = Ks * (2.f * tmp * (1.f / (b.nsB + 1.f)));
      if (reduce_max(Ks) > 0.f) {
        b.iS = luminance(Ks);
        b.impSum += b.iS;
        b.albedo = b.albedo + Ks;
      }
      b.smooth = b.iL > 0.f || b.iS > 0.f;
      break;
    }
    case MAT_METAL: {
      b.fr = frame(dg.Ns);
      b.N = dg.Ns;
      b.ceta = m.eta;
      b.ck = m.k;
      b.rough = m.roughness;
      b.ggx = makeGGX(m.roughness);
      b.specular = m.roughness == 0.f;
      b.smooth = !b.specular;
      b.albedo = v3(0.f);  // the RGB conductor Fresnel's average is 0
      break;
    }
    case MAT_GLASS: {
      const bool out = glassFromOutside(m, cur);
      b.geta = out ? m.outside.ior * (1.f / m.inside.ior) : m.inside.ior * (1.f / m.outside.ior);
      b.Ns = dg.Ns;
      b.Ng = dg.Ng;
      b.N = dg.Ns;
      b.albedo = v3(1.f);
      b.smooth = false;
      break;
    }
    case MAT_THINGLASS: {
      b.N = dg.Ns;
      b.geta = m.thinEta;
      b.tatt = m.thinAtt;
      b.albedo = vexp(m.thinAtt);
      b.smooth = false;
      break;
    }
    default: {
      const L3 f = shadingFrameOf(dg, dPds);
      b.op = opacity;
      b.tr = 1.f - b.op;
      b.hasStack = m.opacity > EPS;
      b.hasCut = 1.f - m.opacity > EPS || m.mapAlpha;
      b.N = f.vz;
      b.st.frame = f;
      b.st.N = f.vz;
      b.st.impSum = 0.f;
      if (b.hasStack) {
        PrincipledParams pp;
        pp.baseColor = m.baseColor;
        pp.roughness = m.roughness;
        pp.metallic = m.metallic;
        pp.specular = m.specular;
        pp.ior = m.ior;
        pp.diffuse = m.diffuse;
        pp.edgeColor = m.edgeColor;
        pp.specularMetallic = m.specularMetallic;
        pp.fromOutside = sameMedium(cur, vacuum());  // Principled's outside medium: vacuum
        b.st.init(pp, f);
        b.albedo = b.st.albedo * b.op;
        b.smooth = b.st.smooth;
      }
      b.impSum = 0.f;
      if (b.hasCut) {
        b.albedo = b.albedo + v3(b.tr);
        b.impSum += b.tr;
      }
      if (b.hasStack) b.impSum += b.op;
      break;
    }
  }
  return b;
}

BSDFEval SurfaceBSDF::eval(V3 wo, V3 wi) const {
  BSDFEval r = {v3(0.f), 0.f};
  switch (type) {
    case MAT_OBJ: {
      if (iL > 0.f) {  // Lambert_eval
        const float c = std::fmax(dot(wi, N), 0.f);
        r.value = r.value + Kd * (ONE_OVER_PI * c);
        r.pdf += c * ONE_OVER_PI * iL;
      }
      if (iS > 0.f) {  // Specular_eval
        const float cosO = dot(wo, N), cosI = dot(wi, N);
        if (cosO > 0.f && cosI > 0.f) {
          const V3 wh = normalize(wo + wi);
          const float cosH = dot(wh, N);
          const float pdf = (nsB + 1.f) * ONE_OVER_TWO_PI * std::pow(cosH, nsB) * (1.f / (4.f * dot(wo, wh)));
          r.value = r.value + ksN * std::pow(cosH, nsB);
          r.pdf += pdf * iS;
        }
      }
      r.pdf *= 1.f / impSum;
      return r;
    }
    case MAT_METAL: {
      if (specular) return r;
      const float cosO = dot(wo, N), cosI = dot(wi, N);
      if (cosO <= 0.f || cosI <= 0.f) return r;
      const V3 wh = normalize(wi + wo);
      const float cosOH = dot(wo, wh), cosIH = dot(wi, wh);
      const V3 wo0 = toLocalF(fr, wo), wi0 = toLocalF(fr, wi), wh0 = toLocalF(fr, wh);
      float whPdf;
      const float D = ggxEvalVisible(ggx, wh0, wo0, cosOH, whPdf);
      const float G = ggxG2(ggx, wo0, wi0, cosOH, cosIH);
      return {fresnelConductorRGB(cosOH, ceta, ck) * (D * G * (1.f / (4.f * cosO))),
              whPdf * (1.f / (4.f * std::fabs(cosOH)))};
    }
    case MAT_GLASS:
    case MAT_THINGLASS: return r;
    default: {
      if (hasStack && op > 0.f) {
        const BSDFEval e = st.eval(wo, wi);
        r.value = e.value * op;
        r.pdf = e.pdf * op;
      }
      r.pdf *= 1.f / impSum;
      return r;
    }
  }
}

BSDFSample SurfaceBSDF::sample(V3 wo, V2 s, float ss) const {
  BSDFSample r = zeroSample();
  switch (type) {
    case MAT_OBJ: {
      if (impSum == 0.f) return r;
      const float x = ss * impSum;
      float prefix = 0.f, imp = 0.f;
      int choice;
      if (x < (prefix += iL)) {  // Lambert_sample
        choice = 0;
        imp = iL;
        const V3 l = cartesian(2.f * PI * s.x, std::sqrt(1.f - s.y), std::sqrt(s.y));
        r.wi = xfmVector(fr, l);
        r.pdf = l.z * ONE_OVER_PI;
        r.type = SCATTER_DIFFUSE_R;
        r.weight = Kd;
      } else if (x < (prefix += iT)) {  // Transmission_sample
        choice = 1;
        imp = iT;
        r.wi = -wo;
        r.pdf = INFINITY;
        r.type = SCATTER_SPEC_T;
        r.weight = T;
      } else if (x < (prefix += iS)) {  // Specular_sample
        choice = 2;
        imp = iS;
        const float cosT = std::pow(s.y, 1.f / (nsB + 1.f));
        const V3 whl = cartesian(2.f * PI * s.x, cos2sin(cosT), cosT);
        const V3 wh = xfmVector(fr, whl);
        const float cosOH = dot(wo, wh);
        r.wi = reflectV(wo, wh, cosOH);
        if (dot(r.wi, N) <= 0.f) return zeroSample();
        r.pdf = (nsB + 1.f) * ONE_OVER_TWO_PI * std::pow(whl.z, nsB) * (1.f / (4.f * cosOH));
        r.type = SCATTER_GLOSSY_R;
        r.weight = specW * cosOH;
      } else {
        return r;
      }
      if (isZero(r.weight) || r.pdf == 0.f) return zeroSample();
      if (r.type & SCATTER_SPECULAR) {
        r.weight = r.weight * (impSum * (1.f / imp));
        return r;
      }
      V3 value = r.weight * r.pdf;
      float pdf = r.pdf * imp;
      if (choice != 0 && iL > 0.f) {
        const float c = std::fmax(dot(r.wi, N), 0.f);
        value = value + Kd * (ONE_OVER_PI * c);
        pdf += c * ONE_OVER_PI * iL;
      }
      if (choice != 2 && iS > 0.f) {
        const float cosO = dot(wo, N), cosI = dot(r.wi, N);
        if (cosO > 0.f && cosI > 0.f) {
          const V3 wh = normalize(wo + r.wi);
          const float cosH = dot(wh, N);
          value = value + ksN * std::pow(cosH, nsB);
          pdf += (nsB + 1.f) * ONE_OVER_TWO_PI * std::pow(cosH, nsB) * (1.f / (4.f * dot(wo, wh))) * iS;
        }
      }
      r.pdf = pdf * (1.f / impSum);
      r.weight = value * (1.f / r.pdf);
      return r;
    }
    case MAT_METAL: {
      if (specular) {  // Conductor_sample
        const float c = dot(wo, N);
        r.wi = reflectV(wo, N, c);
        r.pdf = INFINITY;
        r.type = SCATTER_SPEC_R;
        r.weight = fresnelConductorRGB(c, ceta, ck);
        return r;
      }
      // MicrofacetConductor_sample (fmsScale 0)
      const float cosO = dot(wo, N);
      if (cosO <= 0.f) return r;
      const V3 wo0 = toLocalF(fr, wo);
      float whPdf;
      const V3 wh = xfmVector(fr, ggxSampleVisible(ggx, wo0, whPdf, s));
      const V3 wi = reflectV(wo, wh, dot(wo, wh));
      const float cosI = dot(wi, N);
      if (cosI <= 0.f) return r;
      const float cosOH = dot(wo, wh), cosIH = dot(wi, wh);
      const float G = ggxG2(ggx, wo0, toLocalF(fr, wi), cosOH, cosIH);
      r.wi = wi;
      r.type = SCATTER_GLOSSY_R;
      r.pdf = whPdf * (1.f / (4.f * std::fabs(cosOH)));
      r.weight = fresnelConductorRGB(cosOH, ceta, ck) * (G * rcp_safe(ggxG1(ggx, wo0, cosOH)));
      return r;
    }
    case MAT_GLASS: {  // RobustDielectric_sample
      r.pdf = INFINITY;
      r.weight = v3(1.f);
      const V3 inc = -wo;
      V3 sn = Ns, gn = Ng;
      const float e = 1.f / geta;
      const float geps = 1e-6f;
      const bool canReflect = e < 1.f - geps || e > 1.f + geps;
      if (dot(inc, sn) > 0.f) sn = -sn;
      if (dot(inc, gn) > 0.f) gn = -gn;
      const V3 par = sn * dot(inc, sn);
      const V3 dirR = (inc - par) - par;  // ReflectionDirection
      V3 dirT;
      float FR;
      bool mustReflect = false;
      {  // RefractionDirection
        const float cos1 = dot(inc, sn);
        const float c1 = std::fabs(cos1);
        const bool headOn = 1.f - 1e-6f < c1 && c1 < 1.f - 1e-6f;
        if (headOn) {
          FR = sqr((e - 1.f) / (e + 1.f));
          dirT = inc;
        } else {
          const V3 dpar = sn * cos1;
          const V3 dperp = inc - dpar;
          const V3 b = normalize(dperp);
          const float sin1 = dot(dperp, b);
          const float sin2 = sin1 / e;
          if (sin2 > 1.f) {
            dirT = v3(0.f);
            FR = 1.f;
            mustReflect = true;
          } else {
            const float cos2 = std::sqrt(clamp01(1.f - sin2 * sin2));
            const V3 N2 = normalize(dpar);
            dirT = N2 * cos2 + b * sin2;
            const float q1 = (e * c1 - cos2) / (e * c1 + cos2);
            const float q2 = (c1 - e * cos2) / (c1 + e * cos2);
            FR = 0.5f * (q1 * q1 + q2 * q2);
          }
        }
        FR = clamp01(FR);
      }
      if ((ss < FR && canReflect) || mustReflect) {
        r.wi = dirR;
        r.type = SCATTER_SPEC_R;
        const float gc = dot(r.wi, gn);
        if (gc >= 0.f) {
          if (gc < geps) r.wi = normalize(r.wi + gn * geps);
        } else {
          r.wi = r.wi - gn * (2.f * gc);
        }
      } else {
        r.wi = dirT;
        r.type = SCATTER_SPEC_T;
        const float gc = dot(r.wi, gn);
        if (gc <= 0.f) {
          if (gc > -geps) r.wi = normalize(r.wi - gn * geps);
        } else {
          r.type = SCATTER_SPEC_R;
        }
      }
      return r;
    }
    case MAT_THINGLASS: {  // RobustThinDielectric_sample
      const float cosO = std::fmax(dot(wo, N), 0.f);
      V3 R, T2;
      thinSlab(cosO, geta, tatt, R, T2);
      const float pR = luminance(R), pT = luminance(T2);
      const float p = std::fmin(std::fmax(pR * (1.f / (pR + pT)), 0.25f), 0.75f);
      if (ss <= p) {
        r.wi = reflectV(wo, N, cosO);
        r.type = SCATTER_SPEC_R;
        r.weight = R * (1.f / p);
      } else {
        r.wi = -wo;
        r.type = SCATTER_SPEC_T;
        r.weight = T2 * (1.f / (1.f - p));
      }
      r.pdf = INFINITY;
      return r;
    }
    default: {  // Principled_BSDF_sample: root MultiBSDF
      if (impSum == 0.f) return r;
      const float x = ss * impSum;
      float prefix = 0.f;
      if (hasCut && x < (prefix += tr)) {
        r.wi = -wo;
        r.pdf = INFINITY;
        r.type = SCATTER_SPEC_T;
        r.weight = v3(tr) * (impSum * (1.f / tr));
        return r;
      }
      if (!hasStack) return r;
      prefix += op;
      r = st.sample(wo, s, (x + op - prefix) * (1.f / op));
      r.weight = r.weight * op;
      if (isZero(r.weight) || r.pdf == 0.f) return zeroSample();
      if (r.type & SCATTER_SPECULAR) {
        r.weight = r.weight * (impSum * (1.f / op));
        return r;
      }
      const V3 value = r.weight * r.pdf;
      r.pdf = r.pdf * op * (1.f / impSum);
      r.weight = value * (1.f / r.pdf);
      return r;
    }
  }
}

V3 materialTransparency(const MaterialParams &m, const DG &dg, V3 rayDir, const Medium &cur, float footprint) {
  switch (m.type) {
    case MAT_PRINCIPLED: {  // Principled_getTransparency (Principled.ispc:432-580), no glass lobe
      float op = clamp01(m.opacity);
      if (m.mapAlpha) op *= mapTexel(m, dg, footprint).w;
      const float tr = 1.f - op;
      if (tr <= EPS) return v3(0.f);
      return v3(tr);
    }
    case MAT_OBJ: {  // OBJ_getTransparency (OBJ.ispc:93-110)
      float d = m.opacity * dg.color.w;
      if (m.mapAlpha) d *= mapTexel(m, dg, footprint).w;
      return m.tf * d + v3(1.f - d);
    }
    case MAT_GLASS: {
      const float eta = glassFromOutside(m, cur) ? m.outside.ior * (1.f / m.inside.ior)
                                                 : m.inside.ior * (1.f / m.outside.ior);
      const float cosO = std::fmax(-dot(rayDir, dg.Ns), 0.f);
      return v3(1.f - fresnelDielectric(cosO, eta));
    }
    case MAT_THINGLASS: {
      V3 R, T;
      thinSlab(std::fmax(-dot(rayDir, dg.Ns), 0.f), m.thinEta, m.thinAtt, R, T);
      return T;
    }
    default: return v3(0.f);
  }
}

Medium nextMedium(const MaterialParams &m, const Medium &cur) {
  if (m.type != MAT_GLASS) return cur;
  return glassFromOutside(m, cur) ? m.inside : m.outside;
}

}  // namespace orc
