// Oracle (test infrastructure only): CPU restatement of the path tracer.
//   PathTracer_renderPixel  render/pathtracer/PathTracer.ispc:75-216
//   samplePath              render/pathtracer/PathSampler.ispc:109-415
//   nextEventEstimation     render/pathtracer/NextEventEstimation.ispc:25-160
//   evaluateVirtualLights   render/pathtracer/VirtualLight.ispc:38-107
//   transparentShadow       render/pathtracer/TransparentShadow.ispc:18-85
//   misHeuristic            render/pathtracer/PathTracerUtil.ih:30-46
//   light list + CDF        render/pathtracer/PathTracerData.cpp:32-82
//   parameters              render/pathtracer/PathTracer.cpp:29-51
//   ray cones               common/World.ih:458-464, camera/*Camera.ispc
//                           initRay, PathTracer.ispc:183-187,
//                           NextEventEstimation.ispc:103-106
//   backplate               render/Renderer.ispc:19-29, PathSampler.ispc:200-215
#include <cstring>

#include "pt_bsdf.h"

namespace orc {

extern thread_local uint64_t tl_rays;

struct PtParams {
  int spp, maxPathLength, roulettePathLength, maxScatteringEvents, lightSamples, limitIndirectLightSamples;
  float minContribution, maxContribution;
  V4 bg;
  const Texture *backplate = nullptr;  // map_backplate
  float mipBiasFactor = 1.f;           // 2^mipMapBias
  const Texture *maxDepth = nullptr;   // map_maxDepth
};

struct PtLights {
  std::vector<int> kind;  // 0 quad, 1 ambient, 2 distant, 3 sphere, 4 spot
  std::vector<QuadLight> quads;
  std::vector<AmbientLight> ambients;
  std::vector<DistantLight> distants;
  std::vector<SphereLight> spheres;
  std::vector<SpotLight> spots;
  std::vector<int> index;
  std::vector<float> cdf;
  void finalize() {
    cdf.assign(kind.size(), 1.f);
    if (cdf.empty()) return;
    float sum = cdf[0];
    for (size_t i = 1; i < cdf.size(); i++) cdf[i] = sum += cdf[i];
    const float r = 1.f / sum;
    for (auto &c : cdf) c = c >= sum ? 0x1.000002p+0f : c * r;
  }
  LightSample sample(int i, const DG &dg, V2 s) const {
    switch (kind[i]) {
      case 0: return quads[index[i]].sample(dg, s);
      case 2: return distants[index[i]].sample(dg, s);
      case 3: return spheres[index[i]].sample(dg, s);
      case 4: return spots[index[i]].sample(dg, s);
      default: return ambients[index[i]].sample(dg, s);
    }
  }
  LightEval eval(int i, const DG &dg, V3 dir, float lo, float hi) const {
    switch (kind[i]) {
      case 0: return quads[index[i]].eval(dg, dir, lo, hi);
      case 2: return distants[index[i]].eval(dg, dir, lo, hi);
      case 3: return spheres[index[i]].eval(dg, dir, lo, hi);
      case 4: return spots[index[i]].eval(dg, dir, lo, hi);
      default: return ambients[index[i]].eval(dg, dir, lo, hi);
    }
  }
  bool visible(int i) const {
    switch (kind[i]) {
      case 0: return quads[index[i]].visible;
      case 2: return distants[index[i]].visible;
      case 3: return spheres[index[i]].visible;
      case 4: return spots[index[i]].visible;
      default: return ambients[index[i]].visible;
    }
  }
};

namespace {

inline float luminance(V3 c) { return 0.212671f * c.x + 0.715160f * c.y + 0.072169f * c.z; }
inline float mis(float p1, float p2) {
  const float p = sqr(p1) / (sqr(p1) + sqr(p2));
  return p1 > 1e17f ? 1.f : p;
}

struct Vertex {
  DG dg;
  float pdf_w;
  int numLightSamples;
  bool env;
};

struct Ctx {
  const Scene &sc;
  const PtLights &L;
  const std::vector<MaterialParams> &mats;
  const PtParams &p;
  int nFirst, nIndirect;
  bool transparentShadows;  // some material lets shadow rays through
};

const MaterialParams *materialOf(const Ctx &c, const Hit &hit) {
  const InstanceEntry &e = c.sc.entries[hit.entry];
  if (e.material < 0 || size_t(e.material) >= c.mats.size()) return nullptr;
  return &c.mats[e.material];
}

// transparentShadow (render/pathtracer/TransparentShadow.ispc:18-85): the
// shadow ray's closest hits in turn, each multiplying the contribution by
// the material's transparency and the medium's Beer attenuation over the
// segment, until the light is reached (the remaining contribution) or the
// contribution drops to minContribution / maxPathLength surfaces were crossed
// (0).  Without transparent materials the first hit blocks the light.
// coneWidth: the path's ray cone width at the shadow ray's origin; the
// shadow cone narrows to 0 at the light and restarts from that width after
// every surface crossed.
V3 transparentShadow(const Ctx &c, V3 lightContrib, Ray shadowRay, Medium medium, float coneWidth) {
  if (!c.transparentShadows) {
    tl_rays++;
    return c.sc.occluded(shadowRay) ? v3(0.f) : lightContrib;
  }
  int maxDepth = c.p.maxPathLength;
  const float tOriginal = shadowRay.tfar;
  const float dwdt = -coneWidth * (1.f / tOriginal);
  for (;;) {
    Hit hit;
    tl_rays++;
    if (!c.sc.intersect(shadowRay, hit)) return lightContrib;
    const DG dg = postIntersect(c.sc, shadowRay, hit, true);
    const MaterialParams *m = materialOf(c, hit);
    const float fp = m && m->map ? pixelFootprint(coneWidth + dwdt * hit.t, shadowRay.dir, dg, c.p.mipBiasFactor) : 0.f;
    const V3 T = m ? materialTransparency(*m, dg, shadowRay.dir, medium, fp) : v3(0.f);
    lightContrib = lightContrib * T;
    if (medium.att.x != 0.f || medium.att.y != 0.f || medium.att.z != 0.f) {
      const V3 a = medium.att * (hit.t - shadowRay.tnear);
      lightContrib = lightContrib * V3{std::exp(a.x), std::exp(a.y), std::exp(a.z)};
    }
    if (reduce_max(lightContrib) <= c.p.minContribution || --maxDepth <= 0) return v3(0.f);
    if (m) medium = nextMedium(*m, medium);
    shadowRay = {shadowRay.org, hit.t + dg.epsilon, shadowRay.dir, tOriginal};
  }
}

V3 virtualLights(const Ctx &c, bool straightPath, const Vertex &last, bool env, const Ray &ray, float t,
                 V3 throughput) {
  V3 L = v3(0.f);
  const float lo = length(last.dg.P - ray.org);
  const float hi = env ? INFINITY : length(last.dg.P - (ray.org + t * ray.dir));
  const float selPdf = float(last.numLightSamples) / float(c.L.kind.size());
  for (size_t i = 0; i < c.L.kind.size(); i++) {
    if (straightPath && !c.L.visible(int(i))) continue;
    const LightEval le = c.L.eval(int(i), last.dg, ray.dir, lo, hi);
    if (reduce_max(le.radiance) > 0.f) {
      const float w = selPdf != 0.f ? mis(last.pdf_w, selPdf * le.pdf) : 1.f;
      L = L + throughput * le.radiance * w;
    }
  }
  return L;
}

V3 nee(const Ctx &c, LDSampler &ld, const DG &dg, const SurfaceBSDF &bsdf, V3 wo, V3 throughput, int numLS,
       const Medium &medium, float coneWidth) {
  V3 L = v3(0.f);
  const int nl = int(c.L.kind.size());
  for (int i = 0; i < numLS; i++) {
    float ss;
    const V2 s = ld.get3LightSamples(uint32_t(i), numLS > 1, ss);
    // Distribution1D_sample over the light CDF
    int first = 0, len = nl;
    while (len > 0) {
      const int half = len >> 1, mid = first + half;
      if (ss < c.L.cdf[mid]) {
        len = half;
      } else {
        first = mid + 1;
        len -= half + 1;
      }
    }
    const float prob = c.L.cdf[first] - (first == 0 ? 0.f : c.L.cdf[first - 1]);
    const float selProb = prob * float(numLS);
    LightSample ls = c.L.sample(first, dg, s);
    ls.weight = ls.weight / selProb;
    ls.pdf *= selProb;
    if (reduce_max(ls.weight) <= 0.f || ls.pdf <= 0.f) continue;
    const BSDFEval fe = bsdf.eval(wo, ls.dir);
    if (reduce_max(fe.value) <= 0.f) continue;
    V3 org = dg.P;
    if (dot(dg.Ng, ls.dir) < 0.f) org = org - (2.f * dg.epsilon) * dg.Ng;
    const V3 contrib =
        transparentShadow(c, throughput * fe.value * ls.weight, {org, 0.f, ls.dir, ls.dist}, medium, coneWidth);
    if (reduce_max(contrib) > 0.f) L = L + contrib * mis(ls.pdf, fe.pdf);
  }
  return L;
}

struct PathOut {
  V3 rgb;
  float alpha, z;
  uint32_t primID, geomID, instID;
  V3 normal, albedo;
};

// cone: the camera ray's cone (width, dwdt) in units of the frame height;
// screen: the pixel centre (the backplate's lookup position)
PathOut samplePath(const Ctx &c, LDSampler &ld, Ray ray, V2 cone, V2 screen) {
  float coneWidth = cone.x;
  PathOut out = {v3(0.f), 1.f, INFINITY, INVALID_ID, INVALID_ID, INVALID_ID, v3(0.f), v3(0.f)};
  V3 throughput = v3(1.f), contribution = v3(0.f);
  int depth = 0, scatteringEvents = 0;
  bool straightPath = true, firstBounceLight = true;
  Medium medium = vacuum();
  Vertex last;
  last.env = false;
  last.pdf_w = INFINITY;
  last.dg.P = ray.org;
  last.dg.epsilon = reduce_max(vabs(ray.org)) * ulpEpsilon;
  last.dg.Ns = last.dg.Ng = ray.dir;
  last.numLightSamples = 0;
  do {
    Hit hit;
    tl_rays++;
    const bool h = c.sc.intersect(ray, hit);
    const float t = h ? hit.t : ray.tfar;
    const V3 wo = -ray.dir;
    if (depth == 0) out.z = t;
    if (!h && straightPath) {
      const V4 bg = c.p.backplate ? c.p.backplate->getScreen(screen) : c.p.bg;
      out.alpha -= luminance(throughput) * (1.f - bg.w);
      contribution = contribution + throughput * v3(bg.x, bg.y, bg.z);
    }
    contribution = contribution + virtualLights(c, straightPath, last, !h, ray, t, throughput);
    if (!h) break;
    if (depth >= c.p.maxPathLength) break;  // no geometry lights
    const DG dg = postIntersect(c.sc, ray, hit, true);
    coneWidth += cone.y * hit.t;  // propagated to the hit
    if (depth == 0) {
      out.primID = dg.primID;
      out.geomID = dg.geomID;
      out.instID = dg.instID;
    }
    if (depth >= c.p.maxPathLength || scatteringEvents >= c.p.maxScatteringEvents) break;
    const MaterialParams *mat = materialOf(c, hit);
    if (!mat) break;  // no material: no BSDF
    const float fp = mat->map ? pixelFootprint(coneWidth, ray.dir, dg, c.p.mipBiasFactor) : 0.f;
    const SurfaceBSDF bsdf = makeBSDF(*mat, dg, dg.dPds, medium, fp);
    ld.nextGroup();
    int numLS = 0;
    if (bsdf.smooth) {
      if (scatteringEvents == 0) {  // updateAuxilliaryData (PathTracerUtil.ih:48-60)
        out.albedo = throughput * bsdf.albedo;
        out.normal = throughput * bsdf.N;
      }
      numLS = firstBounceLight ? c.nFirst : c.nIndirect;
      contribution = contribution + nee(c, ld, dg, bsdf, wo, throughput, numLS, medium, coneWidth);
      firstBounceLight = false;
    }
    float ss;
    uint32_t uu3;
    const V2 s = ld.getNext4Samples(ss, uu3);
    BSDFSample fs = bsdf.sample(wo, s, ss);
    // consistent side of the surface (light leaks)
    const bool sameSide = dot(fs.wi, dg.Ng) >= 0.f;
    const bool reflection = (fs.type & SCATTER_REFLECTION) != 0;
    if (sameSide != reflection) fs.weight = v3(0.f);
    if (reduce_max(fs.weight) <= 0.f || fs.pdf <= 0.f) break;
    throughput = throughput * fs.weight;
    if (depth >= c.p.roulettePathLength) {
      const float rr = ld.finalizeDim3(uu3);
      const float contProb = std::fmin(reduce_max(throughput), 0.95f);
      if (rr > contProb) break;
      throughput = throughput * (1.f / contProb);
    }
    // Beer's law over the segment that reached this vertex
    if (std::fmin(std::fmin(medium.att.x, medium.att.y), medium.att.z) < 0.f) {
      const V3 a = medium.att * t;
      throughput = throughput * V3{std::exp(a.x), std::exp(a.y), std::exp(a.z)};
    }
    V3 org = dg.P;
    if (fs.type & SCATTER_TRANSMISSION) {
      org = org - (2.f * dg.epsilon) * dg.Ng;
      medium = nextMedium(*mat, medium);
    }
    // a specular transmission keeps the last vertex (MIS through transparencies)
    if (fs.type & ~SCATTER_SPEC_T) {
      last.dg = dg;
      last.pdf_w = fs.pdf;
      last.numLightSamples = numLS;
    }
    if (!(ray.dir.x == fs.wi.x && ray.dir.y == fs.wi.y && ray.dir.z == fs.wi.z)) straightPath = false;
    ray = {org, 0.f, fs.wi, INFINITY};
    depth++;
    if (fs.type & SCATTER_SMOOTH) scatteringEvents++;
  } while (reduce_max(throughput) > c.p.minContribution);
  out.rgb = contribution;
  if (std::isnan(contribution.x) || std::isnan(contribution.y) || std::isnan(contribution.z)) {
    out.rgb = v3(0.f);
    out.alpha = 1.f;
  }
  return out;
}

}  // namespace

void renderPT(const Scene &sc, const PtLights &lights, const std::vector<MaterialParams> &mats, const Camera &cam,
              const PixelFilter &pf, const PtParams &p, FrameBuffer &fb, int nthreads, int y0, int y1) {
  const int W = fb.W;
  const int nl = int(lights.kind.size());
  const int nFirst = p.lightSamples >= 0 && nl > 0 ? p.lightSamples : std::min(1024, nl);
  const int nIndirect = p.limitIndirectLightSamples && nFirst >= 1 ? 1 : nFirst;
  // shadow rays loop over closest hits when a material lets them through or
  // vertex colours with alpha < 1 meet an obj material (d x alpha)
  bool transparent = false, anyObj = false, colorAlpha = false;
  for (const MaterialParams &m : mats) {
    transparent = transparent || transparentMaterial(m);
    anyObj = anyObj || m.type == MAT_OBJ;
  }
  for (const Geometry &g : sc.geoms)
    for (const V4 &col : g.colors) colorAlpha = colorAlpha || col.w != 1.f;
  transparent = transparent || (colorAlpha && anyObj);
  const Ctx c = {sc, lights, mats, p, nFirst, nIndirect, transparent};
  const V2 rcpSize = {1.f / float(fb.W), 1.f / float(fb.H)};
  const uint32_t accumID = uint32_t(fb.frameID);
  parallelRows(y1 - y0, nthreads, [&](int yy) {
    const int y = y0 + yy;
    for (int x = 0; x < W; x++) {
      ScreenSample acc;
      const uint32_t seed = 0x49c5f37eu ^ uint32_t(W * y + x);
      for (int s = 0; s < p.spp; s++) {
        const uint32_t sampleID = accumID * uint32_t(p.spp) + uint32_t(s);
        LDSampler ld;
        ld.init(seed, sampleID, sampleID * uint32_t(nFirst), 16, 16);
        uint32_t ss234[3];
        const V2 ps = ld.getNext5Samples(ss234);
        const V2 pfs = pf.sample(ps);
        const V2 center = {(float(x) + 0.5f) * rcpSize.x, (float(y) + 0.5f) * rcpSize.y};
        const V2 screen = {center.x + pfs.x * rcpSize.x, center.y + pfs.y * rcpSize.y};
        V2 mapped = screen;
        const float eye = cameraScreen(cam, mapped, center);
        // the lens sample from the sample stream when the camera has an aperture (PathTracer.ispc:172-175)
        Ray ray = cameraRay(cam, mapped, cam.scaledAperture > 0.f ? ld.finalizeDim23(ss234) : V2{0.5f, 0.5f}, eye);
        // the camera sample's time (PathTracer.ispc:177-180, Camera_shutterTime)
        rayTime = shutterTime(cam, mapped, cam.needTime ? ld.finalizeDim4(ss234) : 0.5f);
        // Renderer_getMaxDepth at the sample's (unmapped) screen position (PathTracer.ispc:189-192)
        if (p.maxDepth) ray.tfar = std::fmin(ray.tfar, std::fmax(0.f, p.maxDepth->get(screen, 0.f).x));
        const PathOut o = samplePath(c, ld, ray, cameraCone(cam, mapped, rcpSize.y), center);
        ScreenSample smp;
        smp.rgb = vmin(o.rgb, v3(p.maxContribution));
        smp.alpha = o.alpha;
        smp.z = o.z;
        smp.primID = o.primID;
        smp.geomID = o.geomID;
        smp.instID = o.instID;
        smp.normal = o.normal;
        smp.albedo = o.albedo;
        accumulateScreen(acc, smp);
      }
      const float rspp = 1.f / float(p.spp);
      acc.rgb = acc.rgb * rspp;
      acc.alpha *= rspp;
      acc.normal = acc.normal * rspp;
      acc.albedo = acc.albedo * rspp;
      fbAccumulate(fb, x, y, acc);
    }
    g_rayCount.fetch_add(tl_rays);
    tl_rays = 0;
  });
}

}  // namespace orc

using namespace orc;

struct OrCameraPT {
  float pos[3], dir[3], up[3];
  float fovy, aspect, nearClip;
  int type;  // 0 perspective, 1 orthographic, 2 panoramic
  float height;  // orthographic image height
  float shutter[2];
  int shutterType;
  float rollingDuration;
  float apertureRadius, focusDistance;
  int architectural;
  float imageStart[2], imageEnd[2];  // the sub-image (all zero: whole)
  int stereoMode;
  float interpupillaryDistance;
};

struct OrPtScene {
  PtLights lights;
  std::vector<MaterialParams> mats;
};

extern "C" {

void *or_pt_new() { return new OrPtScene(); }
void or_pt_free(void *p) { delete static_cast<OrPtScene *>(p); }
int or_pt_add_material(void *p, const float *baseColor, float roughness, float metallic) {
  OrPtScene &s = *static_cast<OrPtScene *>(p);
  float f[31] = {baseColor[0], baseColor[1], baseColor[2], roughness, metallic, 1.f};
  for (int k = 24; k < 31; k++) f[k] = 1.f;  // specular, ior, diffuse, edgeColor, specularMetallic
  s.mats.push_back(commitMaterial(MAT_PRINCIPLED, f));
  return int(s.mats.size() - 1);
}
// type MAT_*, params: 31 floats in b200_material order after its type field (no colour map)
int or_pt_add_material2(void *p, int type, const float *params) {
  OrPtScene &s = *static_cast<OrPtScene *>(p);
  s.mats.push_back(commitMaterial(type, params));
  return int(s.mats.size() - 1);
}
// material `mat`'s colour map (principled map_baseColor / obj map_kd): a
// Texture from or_texture_new
void or_pt_set_material_map(void *p, int mat, const void *tex) {
  OrPtScene &s = *static_cast<OrPtScene *>(p);
  MaterialParams &m = s.mats[size_t(mat)];
  if (m.type != MAT_PRINCIPLED && m.type != MAT_OBJ) return;
  m.map = static_cast<const Texture *>(tex);
  m.mapAlpha = m.map && m.map->hasAlpha;
}
// position, edge1, edge2 (3 floats each), radiance rgb
void or_pt_add_quad_light(void *p, const float *pos, const float *e1, const float *e2, const float *radiance) {
  OrPtScene &s = *static_cast<OrPtScene *>(p);
  QuadLight q;
  q.init({pos[0], pos[1], pos[2]}, {e1[0], e1[1], e1[2]}, {e2[0], e2[1], e2[2]},
         {radiance[0], radiance[1], radiance[2]});
  s.lights.kind.push_back(0);
  s.lights.index.push_back(int(s.lights.quads.size()));
  s.lights.quads.push_back(q);
  s.lights.finalize();
}
void or_pt_add_ambient_light(void *p, const float *radiance) {
  OrPtScene &s = *static_cast<OrPtScene *>(p);
  s.lights.kind.push_back(1);
  s.lights.index.push_back(int(s.lights.ambients.size()));
  s.lights.ambients.push_back({{radiance[0], radiance[1], radiance[2]}, true});
  s.lights.finalize();
}

// direction the light travels, angular diameter (degrees), irradiance rgb
void or_pt_add_distant_light(void *p, const float *direction, float angularDiameter, const float *irradiance) {
  OrPtScene &s = *static_cast<OrPtScene *>(p);
  DistantLight d;
  d.init({direction[0], direction[1], direction[2]}, angularDiameter, {irradiance[0], irradiance[1], irradiance[2]});
  s.lights.kind.push_back(2);
  s.lights.index.push_back(int(s.lights.distants.size()));
  s.lights.distants.push_back(d);
  s.lights.finalize();
}
// centre, radius, radiative intensity rgb (color * intensity)
void or_pt_add_sphere_light(void *p, const float *pos, float radius, const float *intensity) {
  OrPtScene &s = *static_cast<OrPtScene *>(p);
  SphereLight l;
  l.init({pos[0], pos[1], pos[2]}, radius, {intensity[0], intensity[1], intensity[2]});
  s.lights.kind.push_back(3);
  s.lights.index.push_back(int(s.lights.spheres.size()));
  s.lights.spheres.push_back(l);
  s.lights.finalize();
}

// position, direction, opening / penumbra angles (degrees), radius, inner
// radius, radiative intensity rgb
void or_pt_add_spot_light(void *p, const float *pos, const float *dir, float opening, float penumbra, float radius,
                          float innerRadius, const float *intensity) {
  OrPtScene &s = *static_cast<OrPtScene *>(p);
  SpotLight l;
  l.init({pos[0], pos[1], pos[2]}, {dir[0], dir[1], dir[2]}, opening, penumbra, radius, innerRadius,
         {intensity[0], intensity[1], intensity[2]});
  s.lights.kind.push_back(4);
  s.lights.index.push_back(int(s.lights.spots.size()));
  s.lights.spots.push_back(l);
  s.lights.finalize();
}

struct OrPtParams {
  int spp, maxPathLength, roulettePathLength, maxScatteringEvents, lightSamples, limitIndirectLightSamples;
  float minContribution, maxContribution;
  float bg[4];
  int pixelFilter;
  const void *backplate;  // a Texture from or_texture_new, or null
  float mipMapBias;
  const void *maxDepth;   // a Texture or null
};

// Renders `frames` accumulated frames of rows [y0, y1) (y1 <= 0: all rows).
void or_render_pt(void *scp, void *ptp, const OrCameraPT *cam, const OrPtParams *pp, int W, int H, int frames,
                  int y0, int y1, float *color, float *depth, uint32_t *ids, int nthreads) {
  const Scene &sc = *static_cast<Scene *>(scp);
  const OrPtScene &pt = *static_cast<OrPtScene *>(ptp);
  Camera c = makeCamera({cam->pos[0], cam->pos[1], cam->pos[2]}, {cam->dir[0], cam->dir[1], cam->dir[2]},
                        {cam->up[0], cam->up[1], cam->up[2]}, cam->fovy, cam->aspect, cam->nearClip, cam->type, cam->height,
                        cam->apertureRadius, cam->focusDistance, cam->architectural != 0, cam->stereoMode,
                        cam->interpupillaryDistance);
  setShutter(c, cam->shutter[0], cam->shutter[1], cam->shutterType, cam->rollingDuration);
  setSubImage(c, cam->imageStart, cam->imageEnd, cam->stereoMode);
  PixelFilter pf;
  pf.init(pp->pixelFilter);
  PtParams p = {pp->spp, pp->maxPathLength, pp->roulettePathLength, pp->maxScatteringEvents, pp->lightSamples,
                pp->limitIndirectLightSamples, pp->minContribution, pp->maxContribution,
                {pp->bg[0], pp->bg[1], pp->bg[2], pp->bg[3]}, static_cast<const Texture *>(pp->backplate),
                std::pow(2.f, pp->mipMapBias), static_cast<const Texture *>(pp->maxDepth)};
  if (y1 <= 0) {
    y0 = 0;
    y1 = H;
  }
  FrameBuffer fb;
  fb.resize(W, H);
  for (int f = 0; f < frames; f++) {
    renderPT(sc, pt.lights, pt.mats, c, pf, p, fb, nthreads, y0, y1);
    fb.frameID++;
  }
  const size_t N = size_t(W) * H;
  if (color) std::memcpy(color, fb.color.data(), N * 16);
  copyAux(fb);
  if (depth) std::memcpy(depth, fb.depth.data(), N * 4);
  if (ids) {
    std::memcpy(ids, fb.primID.data(), N * 4);
    std::memcpy(ids + N, fb.geomID.data(), N * 4);
    std::memcpy(ids + 2 * N, fb.instID.data(), N * 4);
  }
}

}  // extern "C"
