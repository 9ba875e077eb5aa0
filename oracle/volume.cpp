// Oracle (test infrastructure only): SciVis volume rendering of one
// structured-regular volume through a piecewise-linear transfer function.
//   SciVis_renderSample              render/scivis/SciVis.ispc:24-222
//   integrateVolumeIntervalsGradient render/scivis/volumes.ispc:302-439
//     (the single-volume variant, with gradient shading: SciVis_computeShading
//     of each sample with Ns = -normalize(gradient), blended by
//     gradientShadingScale)
//   LinearTransferFunction_get       volume/transferFunction/LinearTransferFunction.ispc:11-43
//   value ranges / max opacity       volume/transferFunction/LinearTransferFunction.cpp:40-155
// Volume sampling and interval iteration are Open VKL 2.0.1 (not vendored).
// They are restated with this project's definitions, shared with the CUDA
// renderer: vertex-centred trilinear sampling of the grid, NaN outside it;
// intervals are the maximal runs of non-empty 16^3-voxel macrocells along
// the ray (empty: the transfer function's maximum opacity over the cell's
// value range is 0); nominalDeltaT = the smallest grid spacing.
#include <cmath>
#include <cstring>
#include <vector>

#include "pt_bsdf.h"
#include "render.h"

namespace orc {

extern thread_local uint64_t tl_rays;

struct Volume {
  int nx, ny, nz;
  V3 origin, spacing;
  std::vector<float> data;
  static constexpr int CELL = 16;
  int cx, cy, cz;
  std::vector<float> cmin, cmax;
  std::vector<uint8_t> cellEmpty;
  float at(int i, int j, int k) const { return data[(size_t(k) * ny + j) * nx + i]; }
  void buildCells() {
    cx = (nx - 1 + CELL - 1) / CELL;
    cy = (ny - 1 + CELL - 1) / CELL;
    cz = (nz - 1 + CELL - 1) / CELL;
    cx = cx < 1 ? 1 : cx;
    cy = cy < 1 ? 1 : cy;
    cz = cz < 1 ? 1 : cz;
    cmin.assign(size_t(cx) * cy * cz, INFINITY);
    cmax.assign(size_t(cx) * cy * cz, -INFINITY);
    for (int c = 0; c < cz; c++)
      for (int b = 0; b < cy; b++)
        for (int a = 0; a < cx; a++) {
          float lo = INFINITY, hi = -INFINITY;
          for (int k = c * CELL; k <= std::min(nz - 1, (c + 1) * CELL); k++)
            for (int j = b * CELL; j <= std::min(ny - 1, (b + 1) * CELL); j++)
              for (int i = a * CELL; i <= std::min(nx - 1, (a + 1) * CELL); i++) {
                const float v = at(i, j, k);
                lo = std::fmin(lo, v);
                hi = std::fmax(hi, v);
              }
          const size_t ci = (size_t(c) * cy + b) * cx + a;
          cmin[ci] = lo;
          cmax[ci] = hi;
        }
  }
  // vertex-centred trilinear sample at world point p (identity transform)
  float sample(V3 p) const {
    const float u = (p.x - origin.x) / spacing.x, v = (p.y - origin.y) / spacing.y, w = (p.z - origin.z) / spacing.z;
    if (!(u >= 0.f && v >= 0.f && w >= 0.f && u <= float(nx - 1) && v <= float(ny - 1) && w <= float(nz - 1)))
      return NAN;
    const int i = std::min(int(u), nx - 2), j = std::min(int(v), ny - 2), k = std::min(int(w), nz - 2);
    const float fx = u - float(i), fy = v - float(j), fz = w - float(k);
    const float c00 = lerpf(fx, at(i, j, k), at(i + 1, j, k));
    const float c10 = lerpf(fx, at(i, j + 1, k), at(i + 1, j + 1, k));
    const float c01 = lerpf(fx, at(i, j, k + 1), at(i + 1, j, k + 1));
    const float c11 = lerpf(fx, at(i, j + 1, k + 1), at(i + 1, j + 1, k + 1));
    return lerpf(fz, lerpf(fy, c00, c10), lerpf(fy, c01, c11));
  }
  // Volume_getGradient (volume/Volume.ih:26-56) over Open VKL's gradient,
  // restated as finite differences of the trilinear sample at one grid
  // spacing: forward, or backward where the forward point leaves the grid;
  // a NaN component becomes 1 (as Volume_getGradient does).
  V3 gradient(V3 p, float s0) const {
    const float h[3] = {spacing.x, spacing.y, spacing.z};
    float g[3];
    for (int a = 0; a < 3; a++) {
      V3 q = p;
      (a == 0 ? q.x : a == 1 ? q.y : q.z) += h[a];
      const float f = sample(q);
      if (!std::isnan(f)) {
        g[a] = (f - s0) / h[a];
      } else {
        V3 r = p;
        (a == 0 ? r.x : a == 1 ? r.y : r.z) -= h[a];
        g[a] = (s0 - sample(r)) / h[a];
      }
      if (std::isnan(g[a])) g[a] = 1.f;
    }
    return {g[0], g[1], g[2]};
  }
};

struct TransferFunction {
  std::vector<V3> color;
  std::vector<float> opacity;
  float lo, hi;
  V4 get(float value) const {
    value = (value - lo) * (1.f / (hi - lo));
    value = clampf(value, 0.f, 0x1.fffffep-1f);
    const int maxC = int(color.size()) - 1;
    const float fc = value * float(maxC);
    const int ic = int(fc);
    const V3 col = lerp3(fc - std::floor(fc), color[ic], color[std::min(maxC, ic + 1)]);
    const int maxO = int(opacity.size()) - 1;
    const float fo = value * float(maxO);
    const int io = int(fo);
    const float op = lerpf(fo - std::floor(fo), opacity[io], opacity[std::min(maxO, io + 1)]);
    return {col.x, col.y, col.z, op};
  }
  // maximum opacity of the piecewise-linear ramp over [a, b]
  float maxOpacity(float a, float b) const {
    const int maxO = int(opacity.size()) - 1;
    float ta = clampf((a - lo) / (hi - lo), 0.f, 1.f) * maxO, tb = clampf((b - lo) / (hi - lo), 0.f, 1.f) * maxO;
    float m = 0.f;
    const int ia = int(std::floor(ta)), ib = std::min(maxO, int(std::ceil(tb)));
    for (int i = ia; i <= ib; i++) m = std::fmax(m, opacity[i]);
    return m;
  }
};

struct VolumeModel {
  Volume vol;
  TransferFunction tf;
  float densityScale = 1.f;
  float gradientShadingScale = 0.f;  // VolumetricModel::commit volume/VolumetricModel.cpp:76
  bool identity = true;  // the instance transform of the volume (rays go to volume space by rcp)
  A3 rcp;
  // transformRay(tRay, instance->rcp_xfm) (render/scivis/volumes.ispc:311-313)
  Ray toVolume(const Ray &r) const {
    if (identity) return r;
    return {xfmPoint(rcp, r.org), r.tnear, xfmVector(rcp.l, r.dir), r.tfar};
  }
  void finalize() {
    vol.buildCells();
    vol.cellEmpty.resize(vol.cmin.size());
    for (size_t i = 0; i < vol.cmin.size(); i++)
      vol.cellEmpty[i] = tf.maxOpacity(vol.cmin[i], vol.cmax[i]) <= 0.f ? 1 : 0;
  }
};

// Iterates maximal runs of non-empty macrocells along a ray (3D DDA).
struct IntervalIter {
  const Volume *v;
  V3 uo, ud;       // ray in voxel units
  float tEnd;      // exit of the grid box
  float t;         // current position
  int c[3], step[3];
  float tMax[3], tDelta[3];
  bool done;
  void init(const Volume &vol, V3 org, V3 dir, float t0, float t1) {
    v = &vol;
    done = false;
    uo = {(org.x - vol.origin.x) / vol.spacing.x, (org.y - vol.origin.y) / vol.spacing.y,
          (org.z - vol.origin.z) / vol.spacing.z};
    ud = {dir.x / vol.spacing.x, dir.y / vol.spacing.y, dir.z / vol.spacing.z};
    const float hi[3] = {float(vol.nx - 1), float(vol.ny - 1), float(vol.nz - 1)};
    const float o[3] = {uo.x, uo.y, uo.z}, d[3] = {ud.x, ud.y, ud.z};
    float ta = t0, tb = t1;
    for (int k = 0; k < 3; k++) {
      const float r = 1.f / d[k];
      float n = (0.f - o[k]) * r, f = (hi[k] - o[k]) * r;
      if (n > f) std::swap(n, f);
      ta = n > ta ? n : ta;
      tb = f < tb ? f : tb;
    }
    if (!(ta < tb)) {
      done = true;
      return;
    }
    t = ta;
    tEnd = tb;
    const int ncell[3] = {vol.cx, vol.cy, vol.cz};
    for (int k = 0; k < 3; k++) {
      const float p = o[k] + t * d[k];
      int ci = int(std::floor(p / Volume::CELL));
      ci = std::min(std::max(ci, 0), ncell[k] - 1);
      c[k] = ci;
      if (d[k] > 0.f) {
        step[k] = 1;
        tMax[k] = (float((ci + 1) * Volume::CELL) - o[k]) / d[k];
        tDelta[k] = float(Volume::CELL) / d[k];
      } else if (d[k] < 0.f) {
        step[k] = -1;
        tMax[k] = (float(ci * Volume::CELL) - o[k]) / d[k];
        tDelta[k] = -float(Volume::CELL) / d[k];
      } else {
        step[k] = 0;
        tMax[k] = INFINITY;
        tDelta[k] = INFINITY;
      }
    }
  }
  bool cellEmpty() const { return v->cellEmpty[(size_t(c[2]) * v->cy + c[1]) * v->cx + c[0]] != 0; }
  // advance to the next cell; false when leaving the grid
  bool advance() {
    int k = 0;
    if (tMax[1] < tMax[k]) k = 1;
    if (tMax[2] < tMax[k]) k = 2;
    t = tMax[k];
    if (!(t < tEnd)) return false;
    c[k] += step[k];
    const int ncell[3] = {v->cx, v->cy, v->cz};
    if (c[k] < 0 || c[k] >= ncell[k]) return false;
    tMax[k] += tDelta[k];
    return true;
  }
  bool next(float &lo, float &hi) {
    if (done) return false;
    for (int g = 0; g < 1 << 20; g++) {  // skip empty cells
      if (!cellEmpty()) break;
      if (!advance()) {
        done = true;
        return false;
      }
    }
    lo = t;
    for (int g = 0; g < 1 << 20; g++) {  // extend through non-empty cells
      if (!advance()) {
        done = true;
        break;
      }
      if (cellEmpty()) break;
    }
    hi = std::fmin(t, tEnd);
    if (done) hi = tEnd;
    return true;
  }
};

V4 integrateVolume(const VolumeModel &m, const Ray &wray, float jitter, float samplingRate, float minContribution,
                   uint64_t &samples) {
  const Ray ray = m.toVolume(wray);
  IntervalIter it;
  it.init(m.vol, ray.org, ray.dir, ray.tnear, ray.tfar);
  const float nominalDeltaT = std::fmin(m.vol.spacing.x, std::fmin(m.vol.spacing.y, m.vol.spacing.z));
  V3 color = v3(0.f);
  float T = 1.f;
  float distance = INFINITY, iuDistance = jitter, iuLength = 0.f, step = 0.f;
  float ilo = 0.f, ihi = INFINITY;
  for (int g = 0; g < (1 << 24) && T > minContribution; g++) {
    float emptySpace = 0.f;
    while (iuDistance > iuLength) {
      const float prevUpper = ihi;
      if (it.next(ilo, ihi)) {
        emptySpace += std::fmax(ilo - prevUpper, 0.f);
        iuDistance -= iuLength;
        step = nominalDeltaT / samplingRate;
        iuLength = (ihi - ilo) / step;
        distance = distance == INFINITY ? ilo : distance;
      } else {
        return {color.x, color.y, color.z, T};
      }
    }
    const float newDistance = ilo + iuDistance * step;
    const V3 p = ray.org + newDistance * ray.dir;
    const float v = m.vol.sample(p);
    samples++;
    if (!std::isnan(v)) {
      V4 c = m.tf.get(v);
      const float dt = newDistance - distance - emptySpace;
      c.w = std::exp(-c.w * dt * m.densityScale);
      color = color + (T * (1.f - c.w)) * v3(c.x, c.y, c.z);
      T *= c.w;
    }
    iuDistance += 1.f;
    distance = newDistance;
  }
  return {color.x, color.y, color.z, T};
}

// ---------------------------------------------------------------- SciVis with surfaces
//   SciVis_renderSample        render/scivis/SciVis.ispc:24-222
//   SciVis_computeAO           render/scivis/SciVis.ispc:224-281
//   directIllumination, SciVis_computeShading, evaluateLights
//                              render/scivis/surfaces.ispc:17-128
//   evalMaterial               render/scivis/surfaces.ih:44-84
//   lightAlpha                 render/scivis/lightAlpha.ispc:19-122
//   integrateVolumeIntervals   render/ao/volumes.ispc:32-240 (shadow/AO rays)
//   light list and aoColorPi   render/scivis/SciVisData.cpp:15-105
//   ray cones / map_maxDepth    render/RendererRenderTaskFn.inl:40-72
//   background / backplate      render/Renderer.ispc:19-40
// dg.color is the mesh's interpolated vertex colour (1 without one);
// gradient-shaded volume samples pass their transfer-function colour.

struct SvMaterial {
  int isObj;
  V3 kd, ks;
  float ns, d;
  V3 tf;
  const Texture *kdMap = nullptr;  // obj map_kd
};

struct SvBSDF {
  V3 diffuse, specular;
  float shininess;
  V3 transmission, albedo;
  float opacity;
};

// dg (with footprint fp) addresses the obj map_kd; null: no lookup
SvBSDF svEvalMaterial(const SvMaterial *m, V4 color = {1.f, 1.f, 1.f, 1.f}, const DG *dg = nullptr, float fp = 0.f) {
  SvBSDF r;
  r.diffuse = v3(color.x, color.y, color.z);
  r.specular = v3(0.f);
  r.shininess = 10.f;
  r.transmission = v3(1.f - color.w);
  r.opacity = color.w;
  if (m && m->isObj) {
    float d = m->d * color.w;
    r.diffuse = r.diffuse * m->kd;
    if (m->kdMap && dg) {
      const V4 t = m->kdMap->get(dg->st, fp);
      r.diffuse = r.diffuse * v3(t.x, t.y, t.z);
      d *= t.w;
    }
    r.diffuse = r.diffuse * d;
    r.specular = d * m->ks;
    r.shininess = m->ns;
    r.transmission = m->tf * d + v3(1.f - d);
    r.opacity = d;
  }
  r.albedo = r.diffuse + r.specular;
  r.shininess *= 4.f;
  r.diffuse = r.diffuse * float(1.0 / M_PI);
  r.specular = r.specular * ((r.shininess + 2.f) * float(0.25 / M_PI) *
                             (1.f / (2.f - std::exp(r.shininess * -float(M_LN2 / 2.0)))));
  return r;
}

struct SvLight {
  int kind;  // 0 quad, 1 ambient, 2 distant, 3 sphere, 4 spot
  bool visible;
  QuadLight quad;
  AmbientLight amb;
  DistantLight dist;
  SphereLight sph;
  SpotLight spot;
  LightSample sample(const DG &dg, V2 s) const {
    switch (kind) {
      case 0: return quad.sample(dg, s);
      case 2: return dist.sample(dg, s);
      case 3: return sph.sample(dg, s);
      case 4: return spot.sample(dg, s);
      default: return amb.sample(dg, s);
    }
  }
  LightEval eval(const DG &dg, V3 dir, float lo, float hi) const {
    switch (kind) {
      case 0: return quad.eval(dg, dir, lo, hi);
      case 2: return dist.eval(dg, dir, lo, hi);
      case 3: return sph.eval(dg, dir, lo, hi);
      case 4: return spot.eval(dg, dir, lo, hi);
      default: return amb.eval(dg, dir, lo, hi);
    }
  }
};

struct SvParams {
  int spp;
  float samplingRate;
  V4 bg;
  int shadows, visibleLights, aoSamples;
  float aoRadius, minContribution;
  const Texture *backplate = nullptr, *maxDepth = nullptr;
  float mipBiasFactor = 1.f;
};

struct SvWorld {
  const Scene *scene;
  const VolumeModel *vm;  // may be null
  std::vector<SvLight> lights;  // SciVisData order: visible-only (ambient) lights first
  uint32_t numVisibleOnly = 0;
  V3 aoColor = v3(0.f);  // sum of the ambient radiances (aoColorPi = aoColor * pi)
  std::vector<SvMaterial> mats;
  // SciVisData::SciVisData / addVisibleOnlyToArray: an ambient light goes to
  // slot numVisibleOnly (the light there moves to the end) and adds its
  // radiance to the AO colour
  void addLight(const SvLight &L) {
    if (L.kind == 1) {
      if (numVisibleOnly == lights.size()) {
        lights.push_back(L);
      } else {
        lights.push_back(lights[numVisibleOnly]);
        lights[numVisibleOnly] = L;
      }
      numVisibleOnly++;
      aoColor = aoColor + L.amb.radiance;
    } else {
      lights.push_back(L);
    }
  }
  const SvMaterial *material(const Hit &h) const {
    const int m = scene->entries[h.entry].material;
    return (m >= 0 && m < int(mats.size())) ? &mats[size_t(m)] : nullptr;
  }
};

// does [ray.tnear, ray.tfar] overlap the volume's grid box (the test that
// starts IntervalIter)
bool svVolumeOverlaps(const VolumeModel &m, const Ray &wray) {
  const Ray ray = m.toVolume(wray);
  IntervalIter it;
  it.init(m.vol, ray.org, ray.dir, ray.tnear, ray.tfar);
  return !it.done;
}

// integrateVolumeIntervals (render/ao/volumes.ispc:251-352): colour and
// opacity accumulated front to back until 0.99; NaN samples are skipped
// inside the sample search.  The SciVis shadow and AO rays use the opacity,
// the AO renderer both.
V4 aoVolumeIntegrate(const VolumeModel &m, const Ray &wray, float jitter, float samplingRate) {
  const Ray ray = m.toVolume(wray);
  IntervalIter it;
  it.init(m.vol, ray.org, ray.dir, ray.tnear, ray.tfar);
  const float nominalDeltaT = std::fmin(m.vol.spacing.x, std::fmin(m.vol.spacing.y, m.vol.spacing.z));
  float alpha = 0.f, distance = INFINITY, iuDistance = jitter, iuLength = 0.f, step = 0.f;
  float ilo = 0.f, ihi = INFINITY;
  V3 color = v3(0.f);
  for (int g = 0; g < (1 << 24) && alpha < 0.99f; g++) {
    float dt = 0.f, val = NAN;
    for (int h = 0; h < (1 << 24) && std::isnan(val); h++) {
      float emptySpace = 0.f;
      while (iuDistance > iuLength) {
        const float prevUpper = ihi;
        if (!it.next(ilo, ihi)) return {color.x, color.y, color.z, alpha};
        emptySpace += std::fmax(ilo - prevUpper, 0.f);
        iuDistance -= iuLength;
        step = nominalDeltaT / samplingRate;
        iuLength = (ihi - ilo) / step;
        distance = distance == INFINITY ? ilo : distance;
      }
      const float newDistance = ilo + iuDistance * step;
      val = m.vol.sample(ray.org + newDistance * ray.dir);
      iuDistance += 1.f;
      dt = newDistance - distance - emptySpace;
      distance = newDistance;
    }
    const V4 c = m.tf.get(val);
    const float op = 1.f - std::exp(-c.w * dt * m.densityScale);
    color = color + ((1.f - alpha) * op) * v3(c.x, c.y, c.z);
    alpha = alpha + (1.f - alpha) * op;
  }
  return {color.x, color.y, color.z, alpha};
}

float svVolumeAlpha(const VolumeModel &m, const Ray &ray, float jitter, float samplingRate) {
  return aoVolumeIntegrate(m, ray, jitter, samplingRate).w;
}

inline float svLuminance(V3 c) { return 0.212671f * c.x + 0.715160f * c.y + 0.072169f * c.z; }

// cone: the shadow cone (width at the origin, dwdt); its width restarts
// from the origin's after every surface (lightAlpha.ispc:30,105)
V3 svLightAlpha(const SvWorld &w, const SvParams &p, Ray ray, RandomSampler &rs, V3 weight, float quality,
                V2 cone = {0.f, 0.f}) {
  V3 alpha = v3(1.f);
  const float orgTMax = ray.tfar;
  for (int g = 0; g < 1024; g++) {
    Hit hit;
    tl_rays++;
    const bool h = w.scene && w.scene->intersect(ray, hit);
    if (w.vm) {
      Ray vr = ray;
      vr.tfar = h ? hit.t : ray.tfar;
      if (svVolumeOverlaps(*w.vm, vr)) {
        const float jitter = rs.getFloat();
        alpha = alpha * (1.f - svVolumeAlpha(*w.vm, vr, jitter, p.samplingRate * quality));
      }
    }
    if (!h) break;
    const DG dg = postIntersect(*w.scene, ray, hit, true);
    const SvMaterial *m = w.material(hit);
    const float fp = m && m->kdMap ? pixelFootprint(cone.x + cone.y * hit.t, ray.dir, dg, p.mipBiasFactor) : 0.f;
    alpha = alpha * svEvalMaterial(m, dg.color, &dg, fp).transmission;
    ray.tnear = hit.t + dg.epsilon;
    ray.tfar = orgTMax;
    if (svLuminance(alpha * weight) < p.minContribution) {
      alpha = v3(0.f);
      break;
    }
  }
  return alpha;
}

V3 svComputeAO(const SvWorld &w, const SvParams &p, const DG &dg, int px, int py, uint32_t sampleZ,
                RandomSampler &rs, float coneWidth) {
  const uint32_t accumID = sampleZ * uint32_t(p.aoSamples);
  uint32_t t0 = uint32_t(px), t1 = uint32_t(py);
  tea8(t0, t1);
  const V2 rot = {to_float_unorm(t0), to_float_unorm(t1)};
  V3 hits = v3(0.f);
  const L3 l2w = frame(dg.Ns);
  for (int i = 0; i < p.aoSamples; i++) {
    const float hx = PermHalton_sample5(accumID + uint32_t(i)), hy = PermHalton_sample7(accumID + uint32_t(i));
    const float rx = CranleyPattersonRotation(hx, rot.x), ry = CranleyPattersonRotation(hy, rot.y);
    const float phi = float(2.0 * M_PI) * rx;
    const float cosT = std::sqrt(ry), sinT = std::sqrt(1.f - ry);
    const V3 dir = xfmVector(l2w, {std::cos(phi) * sinT, std::sin(phi) * sinT, cosT});
    if (dot(dir, dg.Ns) < 0.01f) {
      hits = hits + v3(1.f);
      continue;
    }
    const Ray aoRay = {dg.P, dg.epsilon, dir, p.aoRadius};
    hits = hits + (v3(1.f) - svLightAlpha(w, p, aoRay, rs, v3(1.f), 0.1f, {coneWidth, 0.f}));
  }
  return v3(1.f) - hits * (1.f / float(p.aoSamples));
}

struct SvShading {
  V3 shadedColor, transmission;
  float opacity;
  V3 albedo;
};

// coneWidth: the ray cone's width at this hit; fp: the hit's footprint
SvShading svComputeShading(const SvWorld &w, const SvParams &p, const DG &dg, const SvMaterial *mat, V4 dgColor,
                           V3 inDir, int px, int py, uint32_t sampleZ, RandomSampler &rs, float coneWidth = 0.f,
                           float fp = 0.f) {
  const SvBSDF bsdf = svEvalMaterial(mat, dgColor, &dg, fp);
  V3 color = v3(0.f);
  for (size_t i = w.numVisibleOnly; i < w.lights.size(); i++) {
    const LightSample ls = w.lights[i].sample(dg, {0.f, 0.f});  // area lights at their centre
    if (std::fmax(ls.weight.x, std::fmax(ls.weight.y, ls.weight.z)) > 0.f) {
      const float cosNL = dot(ls.dir, dg.Ns);
      if (cosNL < 0.f) continue;
      const V3 H = normalize(ls.dir - inDir);
      const float cosNH = dot(H, dg.Ns);
      const V3 specular = bsdf.specular * std::pow(cosNH, bsdf.shininess);
      const V3 diffuse = bsdf.diffuse * cosNL;
      const V3 contrib = (diffuse + specular) * ls.weight;
      if (p.shadows) {
        if (svLuminance(contrib) > p.minContribution) {
          V3 P = dg.P;
          if (dot(dg.Ng, ls.dir) < 0.f) P = P - (2.f * dg.epsilon) * dg.Ng;
          const V3 la = svLightAlpha(w, p, {P, 0.f, ls.dir, ls.dist}, rs, contrib, 0.25f,
                                     {coneWidth, -coneWidth * (1.f / ls.dist)});
          color = color + la * contrib;
        }
      } else {
        color = color + contrib;
      }
    }
  }
  V3 ao = v3(1.f);
  if (p.aoSamples > 0 && svLuminance(w.aoColor * float(M_PI)) > p.minContribution)
    ao = svComputeAO(w, p, dg, px, py, sampleZ, rs, coneWidth);
  color = color + bsdf.diffuse * ao * (w.aoColor * float(M_PI));
  return {color, bsdf.transmission, bsdf.opacity, bsdf.albedo};
}

// integrateVolumeIntervalsGradient (render/scivis/volumes.ispc:302-439) with
// gradient shading: a sample of non-zero opacity whose gradient is not
// vanishing is shaded like a surface with no material, colour = its
// transfer-function RGBA, Ns = Ng = -normalize(gradient), epsilon = dt / 2,
// and blended into the sample by gradientShadingScale before the Beer-law
// opacity.  Shadow and AO rays of the shading draw from the ray's sampler.
V4 integrateVolumeShaded(const SvWorld &w, const SvParams &p, const Ray &wray, float jitter, int px, int py,
                         uint32_t sid, RandomSampler &rs, uint64_t &samples) {
  const VolumeModel &m = *w.vm;
  const Ray ray = m.toVolume(wray);
  IntervalIter it;
  it.init(m.vol, ray.org, ray.dir, ray.tnear, ray.tfar);
  const float nominalDeltaT = std::fmin(m.vol.spacing.x, std::fmin(m.vol.spacing.y, m.vol.spacing.z));
  V3 color = v3(0.f);
  float T = 1.f;
  float distance = INFINITY, iuDistance = jitter, iuLength = 0.f, step = 0.f;
  float ilo = 0.f, ihi = INFINITY;
  for (int g = 0; g < (1 << 24) && T > p.minContribution; g++) {
    float emptySpace = 0.f;
    while (iuDistance > iuLength) {
      const float prevUpper = ihi;
      if (it.next(ilo, ihi)) {
        emptySpace += std::fmax(ilo - prevUpper, 0.f);
        iuDistance -= iuLength;
        step = nominalDeltaT / p.samplingRate;
        iuLength = (ihi - ilo) / step;
        distance = distance == INFINITY ? ilo : distance;
      } else {
        return {color.x, color.y, color.z, T};
      }
    }
    const float newDistance = ilo + iuDistance * step;
    const V3 pos = ray.org + newDistance * ray.dir;
    const float v = m.vol.sample(pos);
    samples++;
    if (!std::isnan(v)) {
      V4 c = m.tf.get(v);
      const float dt = newDistance - distance - emptySpace;
      if (c.w > 0.f) {
        const V3 grad = m.vol.gradient(pos, v);
        if (dot(grad, grad) > 1e-6f) {
          DG dg;
          dg.epsilon = dt / 2.f;
          dg.Ns = dg.Ng = normalize(m.identity ? -grad : xfmVector(transposed(m.rcp.l), -grad));
          dg.P = wray.org + newDistance * wray.dir;  // world space
          dg.primID = dg.geomID = dg.instID = 0xFFFFFFFFu;
          const SvShading sh = svComputeShading(w, p, dg, nullptr, c, wray.dir, px, py, sid, rs);
          const float a = 1.f - svLuminance(sh.transmission), f = m.gradientShadingScale;
          c = {lerpf(f, c.x, sh.shadedColor.x), lerpf(f, c.y, sh.shadedColor.y), lerpf(f, c.z, sh.shadedColor.z),
               lerpf(f, c.w, a)};
        }
      }
      c.w = std::exp(-c.w * dt * m.densityScale);
      color = color + (T * (1.f - c.w)) * v3(c.x, c.y, c.z);
      T *= c.w;
    }
    iuDistance += 1.f;
    distance = newDistance;
  }
  return {color.x, color.y, color.z, T};
}

// cone: the camera ray's (width, dwdt); center: the pixel centre (backplate
// and maxDepth lookups)
ScreenSample svRenderSample(const SvWorld &w, const SvParams &p, Ray ray, int x, int y, int W, uint32_t sid,
                            uint64_t &samples, V2 cone = {0.f, 0.f}, V2 center = {0.f, 0.f}) {
  RandomSampler rs;
  rs.init(uint32_t(x + W * y), sid);
  ScreenSample smp;
  if (p.maxDepth) ray.tfar = std::fmin(ray.tfar, std::fmax(0.f, p.maxDepth->get(center, 0.f).x));
  float coneWidth = cone.x;
  bool firstHit = true, allTrans = true;
  const float originalTFar = ray.tfar;
  V3 outColor = v3(0.f), outT = v3(1.f);
  for (int g = 0; g < 1024; g++) {
    Hit hit;
    tl_rays++;
    const bool h = w.scene && w.scene->intersect(ray, hit);
    const float rayT = h ? hit.t : ray.tfar;
    if (w.vm) {
      Ray vr = ray;
      vr.tfar = rayT;
      if (svVolumeOverlaps(*w.vm, vr)) {
        const float jitter = rs.getFloat();
        const V4 vc = w.vm->gradientShadingScale > 0.f
                          ? integrateVolumeShaded(w, p, vr, jitter, x, y, sid, rs, samples)
                          : integrateVolume(*w.vm, vr, jitter, p.samplingRate, p.minContribution, samples);
        outColor = outColor + outT * v3(vc.x, vc.y, vc.z);
        outT = outT * vc.w;
      }
    }
    if (p.visibleLights) {
      DG ldg;
      ldg.P = ray.org;
      V3 lc = v3(0.f);
      for (const SvLight &L : w.lights)
        if (L.visible) lc = lc + L.eval(ldg, ray.dir, ray.tnear, rayT).radiance;
      outColor = outColor + outT * lc;
    }
    if (firstHit || allTrans) smp.z = rayT;
    if (h) {
      const DG dg = postIntersect(*w.scene, ray, hit, true);
      coneWidth += cone.y * hit.t;  // World.ih postIntersect, t from the ray's origin
      const SvMaterial *m = w.material(hit);
      const float fp = m && m->kdMap ? pixelFootprint(coneWidth, ray.dir, dg, p.mipBiasFactor) : 0.f;
      const SvShading sh = svComputeShading(w, p, dg, m, dg.color, ray.dir, x, y, sid, rs, coneWidth, fp);
      if (firstHit || allTrans) {
        smp.normal = dg.Ns;
        smp.albedo = sh.albedo;
        smp.primID = dg.primID;
        smp.geomID = dg.geomID;
        smp.instID = dg.instID;
        firstHit = false;
      }
      allTrans = allTrans && sh.opacity < p.minContribution;
      outColor = outColor + outT * sh.shadedColor;
      outT = outT * sh.transmission;
      if (svLuminance(outT) < p.minContribution) {
        outT = v3(0.f);
        break;
      }
      ray.tnear = hit.t + dg.epsilon;
      ray.tfar = originalTFar;
    } else {
      const V4 bg = p.backplate ? p.backplate->getScreen(center) : p.bg;
      outColor = outColor + outT * v3(bg.x, bg.y, bg.z);
      outT = outT * (1.f - bg.w);
      break;
    }
  }
  smp.rgb = outColor;
  smp.alpha = 1.f - svLuminance(outT);
  return smp;
}

}  // namespace orc

using namespace orc;

std::atomic<uint64_t> g_volSamples{0};

extern "C" {

void *or_volume_new(const float *data, int nx, int ny, int nz, const float *origin, const float *spacing,
                    const float *colors, int ncolors, const float *opacity, int nopacity, float vlo, float vhi,
                    float densityScale) {
  VolumeModel *m = new VolumeModel();
  m->vol.nx = nx;
  m->vol.ny = ny;
  m->vol.nz = nz;
  m->vol.origin = {origin[0], origin[1], origin[2]};
  m->vol.spacing = {spacing[0], spacing[1], spacing[2]};
  m->vol.data.assign(data, data + size_t(nx) * ny * nz);
  for (int i = 0; i < ncolors; i++) m->tf.color.push_back({colors[3 * i], colors[3 * i + 1], colors[3 * i + 2]});
  m->tf.opacity.assign(opacity, opacity + nopacity);
  m->tf.lo = vlo;
  m->tf.hi = vhi;
  m->densityScale = densityScale;
  m->finalize();
  return m;
}

void or_volume_free(void *m) { delete static_cast<VolumeModel *>(m); }

// the AO renderer's volume and volumeSamplingRate for later or_render_ao calls (null: none)
void or_set_ao_volume(void *m, float samplingRate) {
  g_aoVolume.vm = m;
  g_aoVolume.samplingRate = samplingRate;
  g_aoVolume.overlaps = [](const void *vm, const Ray &r) {
    return svVolumeOverlaps(*static_cast<const VolumeModel *>(vm), r);
  };
  g_aoVolume.integrate = [](const void *vm, const Ray &r, float jitter, float rate) {
    return aoVolumeIntegrate(*static_cast<const VolumeModel *>(vm), r, jitter, rate);
  };
}

// the volume's instance transform, 3x4 row-major (null: identity)
void or_volume_set_transform(void *mp, const float *X) {
  VolumeModel &m = *static_cast<VolumeModel *>(mp);
  m.identity = X == nullptr;
  if (X) {
    A3 a;
    a.l.vx = {X[0], X[4], X[8]};
    a.l.vy = {X[1], X[5], X[9]};
    a.l.vz = {X[2], X[6], X[10]};
    a.p = {X[3], X[7], X[11]};
    m.rcp = rcpAffine(a);
  }
}

void or_volume_set_gradient_shading(void *m, float scale) { static_cast<VolumeModel *>(m)->gradientShadingScale = scale; }

uint64_t or_volume_sample_count(int reset) {
  const uint64_t n = g_volSamples.load();
  if (reset) g_volSamples.store(0);
  return n;
}

struct OrCameraV {
  float pos[3], dir[3], up[3];
  float fovy, aspect, nearClip;
  int type;  // 0 perspective, 1 orthographic, 2 panoramic
  float height;  // orthographic image height
  float shutter[2];  // (unused: a volume-only world does not move)
  int shutterType;
  float rollingDuration;
  float apertureRadius, focusDistance;  // (unused: SciVis uses a pinhole)
  int architectural;
  float imageStart[2], imageEnd[2];  // the sub-image (all zero: whole)
  int stereoMode;
  float interpupillaryDistance;
};

// the camera of an OrCameraV with its stereo mode and sub-image
static Camera volumeCamera(const OrCameraV *c) {
  Camera cam = makeCamera({c->pos[0], c->pos[1], c->pos[2]}, {c->dir[0], c->dir[1], c->dir[2]},
                          {c->up[0], c->up[1], c->up[2]}, c->fovy, c->aspect, c->nearClip, c->type, c->height, 0.f,
                          1.f, c->architectural != 0, c->stereoMode, c->interpupillaryDistance);
  setSubImage(cam, c->imageStart, c->imageEnd, c->stereoMode);
  return cam;
}

// SciVis frames of a volume-only world; rows [y0, y1) (y1 <= 0: all)
void or_render_scivis_volume(void *mp, const OrCameraV *c, int pixelFilter, int W, int H, int spp, float samplingRate,
                             const float *bg, int frames, int y0, int y1, float *color, int nthreads) {
  const VolumeModel &m = *static_cast<VolumeModel *>(mp);
  const Camera cam = volumeCamera(c);
  PixelFilter pf;
  pf.init(pixelFilter);
  FrameBuffer fb;
  fb.resize(W, H);
  if (y1 <= 0) {
    y0 = 0;
    y1 = H;
  }
  const V2 rcpSize = {1.f / float(W), 1.f / float(H)};
  const float minContribution = 0.001f;
  for (int f = 0; f < frames; f++) {
    const uint32_t start = uint32_t(fb.frameID * spp + 1);
    parallelRows(y1 - y0, nthreads, [&](int yy) {
      const int y = y0 + yy;
      uint64_t samples = 0;
      for (int x = 0; x < W; x++) {
        ScreenSample acc;
        for (int s = 0; s < spp; s++) {
          const uint32_t sid = start + s;
          const V2 ps = {Halton_sample2(sid), CranleyPattersonRotation(Halton_sample3(sid), 1.f / 6.f)};
          const V2 pfs = pf.sample(ps);
          const V2 center = {(float(x) + 0.5f) * rcpSize.x, (float(y) + 0.5f) * rcpSize.y};
          V2 screen = {center.x + pfs.x * rcpSize.x, center.y + pfs.y * rcpSize.y};
          const float eye = cameraScreen(cam, screen, center);
          const Ray ray = cameraRay(cam, screen, {0.f, 0.f}, eye);
          RandomSampler rs;
          rs.init(uint32_t(x + W * y), sid);
          const float jitter = rs.getFloat();
          tl_rays++;
          const V4 vc = integrateVolume(m, ray, jitter, samplingRate, minContribution, samples);
          V3 out = {vc.x, vc.y, vc.z};
          float T = vc.w;
          out = out + T * v3(bg[0], bg[1], bg[2]);
          T = T * (1.f - bg[3]);
          ScreenSample smp;
          smp.rgb = out;
          smp.alpha = 1.f - (0.212671f * T + 0.715160f * T + 0.072169f * T);
          smp.z = INFINITY;
          accumulateScreen(acc, smp);
        }
        const float rspp = 1.f / float(spp);
        acc.rgb = acc.rgb * rspp;
        acc.alpha *= rspp;
        acc.normal = acc.normal * rspp;
        acc.albedo = acc.albedo * rspp;
        fbAccumulate(fb, x, y, acc);
      }
      g_volSamples.fetch_add(samples);
      g_rayCount.fetch_add(tl_rays);
      tl_rays = 0;
    });
    fb.frameID++;
  }
  std::memcpy(color, fb.color.data(), size_t(W) * H * 16);
}

struct OrScivisLight {
  int kind, visible;
  float pos[3], e1[3], e2[3], radiance[3];
  float dir[3], angularDiameter, radius;  // distant / sphere / spot lights
  float openingAngle, penumbraAngle, innerRadius;  // spot lights
};
struct OrScivisMaterial {
  int isObj;
  float kd[3], ks[3], ns, d, tf[3];
  const void *kdMap;  // a Texture or null
};
struct OrScivisParams {
  int spp;
  float samplingRate;
  float bg[4];
  int shadows, visibleLights, aoSamples;
  float aoRadius, minContribution;
  int pixelFilter;
  const void *backplate, *maxDepth;  // Textures or null
  float mipMapBias;
};

// SciVis frames of a world with surfaces (and optionally the volume mp);
// rows [y0, y1) (y1 <= 0: all); color RGBA, depth, ids = primID|geomID|instID planes
void or_render_scivis(void *scp, void *mp, const OrCameraV *c, const OrScivisParams *pp, const OrScivisLight *lights,
                      int nlights, const OrScivisMaterial *mats, int nmats, int W, int H, int frames, int y0, int y1,
                      float *color, float *depth, uint32_t *ids, int nthreads) {
  SvWorld w;
  w.scene = static_cast<Scene *>(scp);
  w.vm = static_cast<VolumeModel *>(mp);
  for (int i = 0; i < nlights; i++) {
    const OrScivisLight &l = lights[i];
    SvLight L;
    L.kind = l.kind;
    L.visible = l.visible != 0;
    const V3 rad = {l.radiance[0], l.radiance[1], l.radiance[2]};
    if (l.kind == 0) {
      L.quad.init({l.pos[0], l.pos[1], l.pos[2]}, {l.e1[0], l.e1[1], l.e1[2]}, {l.e2[0], l.e2[1], l.e2[2]}, rad);
      L.quad.visible = L.visible;
    } else if (l.kind == 2) {
      L.dist.init({l.dir[0], l.dir[1], l.dir[2]}, l.angularDiameter, rad);
      L.dist.visible = L.visible;
    } else if (l.kind == 3) {
      L.sph.init({l.pos[0], l.pos[1], l.pos[2]}, l.radius, rad);
      L.sph.visible = L.visible;
    } else if (l.kind == 4) {
      L.spot.init({l.pos[0], l.pos[1], l.pos[2]}, {l.dir[0], l.dir[1], l.dir[2]}, l.openingAngle, l.penumbraAngle,
                  l.radius, l.innerRadius, rad);
      L.spot.visible = L.visible;
    } else {
      L.amb = {rad, L.visible};
    }
    w.addLight(L);
  }
  for (int i = 0; i < nmats; i++) {
    const OrScivisMaterial &m = mats[i];
    w.mats.push_back({m.isObj, {m.kd[0], m.kd[1], m.kd[2]}, {m.ks[0], m.ks[1], m.ks[2]}, m.ns, m.d,
                      {m.tf[0], m.tf[1], m.tf[2]}, static_cast<const Texture *>(m.kdMap)});
  }
  SvParams p = {pp->spp, pp->samplingRate, {pp->bg[0], pp->bg[1], pp->bg[2], pp->bg[3]}, pp->shadows,
                pp->visibleLights, pp->aoSamples, pp->aoRadius, pp->minContribution,
                static_cast<const Texture *>(pp->backplate), static_cast<const Texture *>(pp->maxDepth),
                std::pow(2.f, pp->mipMapBias)};
  const Camera cam = volumeCamera(c);
  PixelFilter pf;
  pf.init(pp->pixelFilter);
  FrameBuffer fb;
  fb.resize(W, H);
  if (y1 <= 0) {
    y0 = 0;
    y1 = H;
  }
  const V2 rcpSize = {1.f / float(W), 1.f / float(H)};
  for (int f = 0; f < frames; f++) {
    const uint32_t start = uint32_t(fb.frameID * p.spp + 1);
    parallelRows(y1 - y0, nthreads, [&](int yy) {
      const int y = y0 + yy;
      uint64_t samples = 0;
      for (int x = 0; x < W; x++) {
        ScreenSample acc;
        for (int s = 0; s < p.spp; s++) {
          const uint32_t sid = start + uint32_t(s);
          const V2 ps = {Halton_sample2(sid), CranleyPattersonRotation(Halton_sample3(sid), 1.f / 6.f)};
          const V2 pfs = pf.sample(ps);
          const V2 center = {(float(x) + 0.5f) * rcpSize.x, (float(y) + 0.5f) * rcpSize.y};
          V2 screen = {center.x + pfs.x * rcpSize.x, center.y + pfs.y * rcpSize.y};
          const float eye = cameraScreen(cam, screen, center);
          const Ray ray = cameraRay(cam, screen, {0.f, 0.f}, eye);
          accumulateScreen(acc, svRenderSample(w, p, ray, x, y, W, sid, samples, cameraCone(cam, screen, rcpSize.y),
                                               center));
        }
        const float rspp = 1.f / float(p.spp);
        acc.rgb = acc.rgb * rspp;
        acc.alpha *= rspp;
        acc.normal = acc.normal * rspp;
        acc.albedo = acc.albedo * rspp;
        fbAccumulate(fb, x, y, acc);
      }
      g_volSamples.fetch_add(samples);
      g_rayCount.fetch_add(tl_rays);
      tl_rays = 0;
    });
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
