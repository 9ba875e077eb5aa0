#include <cstring>
// Oracle (test infrastructure only): camera, pixel filter, postIntersect,
// framebuffer accumulation and the AO renderer; see render.h for citations.
#include "render.h"

#include <algorithm>

namespace orc {

const Tables &tables() {
  static const Tables t;
  return t;
}

std::atomic<uint64_t> g_rayCount{0};
thread_local uint64_t tl_rays = 0;  // flushed into g_rayCount once per image row

void setShutter(Camera &c, float lower, float upper, int type, float duration) {
  auto cl = [](float v) { return std::fmin(std::fmax(v, 0.f), 1.f); };
  float lo = cl(lower), hi = cl(upper);
  if (lo > hi) lo = hi;
  const float dur = std::fmin(std::fmax(duration, 0.f), hi - lo);
  c.needTime = type == 0 ? hi - lo != 0.f : dur != 0.f;
  if (type != 0) {
    hi -= dur;
    if (type == 2 || type == 3) std::swap(lo, hi);
  }
  c.shutterLo = lo;
  c.shutterHi = hi;
  c.rollingDuration = dur;
  c.shutterMode = type == 0 ? 0 : (type == 1 || type == 2 ? 1 : 2);
}

Camera makeCamera(V3 pos, V3 dir, V3 up, float fovy, float aspect, float nearClip, int type, float height,
                  float apertureRadius, float focusDistance, bool architectural, int stereoMode,
                  float interpupillaryDistance) {
  Camera c;
  c.type = type;
  c.nearClip = nearClip;
  if (type == 1) {
    const V3 d = normalize(dir);
    V3 du = normalize(cross(d, up));
    V3 dv = cross(du, d) * height;
    du = du * (height * aspect);
    c.dir_00 = d;
    c.du_size = du;
    c.dv_up = dv;
    c.org = pos - 0.5f * du - 0.5f * dv;
    return c;
  }
  if (type == 2) {
    const V3 vz = -normalize(dir);
    const V3 vx = normalize(cross(up, vz));
    c.du_size = vx;
    c.dv_up = cross(vz, vx);
    c.dir_00 = vz;
    c.org = pos;
    // PanoramicCamera::commit (camera/PanoramicCamera.cpp:45-52): the offset
    // negated for top / bottom; left / right keep a fixed eye
    const float h = 0.5f * interpupillaryDistance;
    c.ipdOffset = {stereoMode == 4 ? -h : h, 0.f, 0.f};
    c.monoEye = stereoMode == 1 ? -1.f : stereoMode == 2 ? 1.f : 0.f;
    c.split = stereoMode == 3 ? 1 : stereoMode == 4 ? 2 : 0;
    return c;
  }
  // PerspectiveCamera::commit (camera/PerspectiveCamera.cpp:37-91): side by
  // side halves the aspect, top / bottom doubles it; left / right move the
  // origin by half the interpupillary distance along the film's x axis
  if (stereoMode == 3) aspect = aspect * 0.5f;
  if (stereoMode == 4) aspect = aspect * 2.f;
  const float deg2rad = float(1.745329251994329576923690768489e-2);
  const float ipy = 2.f * std::tan(deg2rad * (0.5f * fovy));
  const float ipx = ipy * aspect;
  V3 d00 = normalize(dir);
  V3 du = normalize(cross(d00, up));
  V3 dv = architectural ? normalize(up) : cross(du, d00);
  V3 ipd = (0.5f * interpupillaryDistance) * du;
  if (stereoMode == 1) pos = pos - ipd;
  if (stereoMode == 2) pos = pos + ipd;
  if (stereoMode == 4) ipd = -1.f * ipd;
  c.ipdOffset = ipd;
  c.split = stereoMode == 3 ? 1 : stereoMode == 4 ? 2 : 0;
  du = du * ipx;
  dv = dv * ipy;
  d00 = d00 - 0.5f * du - 0.5f * dv;
  c.scaledAperture = apertureRadius != 0.f ? apertureRadius / (ipx * focusDistance) : 0.f;
  if (c.scaledAperture > 0.f) {  // prescaled to the focal plane
    du = du * focusDistance;
    dv = dv * focusDistance;
    d00 = d00 * focusDistance;
  }
  c.aspect = aspect;
  c.imgPlaneY = ipy;
  c.org = pos;
  c.dir_00 = d00;
  c.du_size = du;
  c.dv_up = dv;
  c.nearClip = nearClip;
  return c;
}

void setSubImage(Camera &c, const float lo[2], const float hi[2], int stereoMode) {
  const bool whole = lo[0] == 0.f && lo[1] == 0.f && hi[0] == 0.f && hi[1] == 0.f;
  c.subLo = whole ? V2{0.f, 0.f} : V2{lo[0], lo[1]};
  c.subHi = whole ? V2{1.f, 1.f} : V2{hi[0], hi[1]};
  c.coneScale = std::fabs(c.subHi.y - c.subLo.y) * (c.type != 1 && stereoMode == 4 ? 2.f : 1.f);
}

namespace {
float create1D(int n, float *cdf) {
  float sum = cdf[0];
  for (int i = 1; i < n; i++) cdf[i] = sum += cdf[i];
  const float rcpSum = 1.f / sum;
  const float nextAfter1 = 0x1.000002p+0f;
  for (int i = 0; i < n; i++) cdf[i] = cdf[i] >= sum ? nextAfter1 : cdf[i] * rcpSum;
  return sum;
}
struct S1 {
  int idx;
  float frac;
};
S1 sample1D(int size, const float *cdf, float s) {
  int first = 0, len = size;
  while (len > 0) {
    const int half = len >> 1, mid = first + half;
    if (s < cdf[mid]) {
      len = half;
    } else {
      first = mid + 1;
      len -= half + 1;
    }
  }
  const float bef = first == 0 ? 0.f : cdf[first - 1];
  const float dpdf = cdf[first] - bef;
  return {first, (s - bef) / dpdf};
}
}  // namespace

void PixelFilter::init(int t) {
  type = t;
  if (t == PF_POINT) {
    width = 0.f;
    return;
  }
  if (t == PF_BOX) {
    width = 1.f;
    return;
  }
  width = t == PF_MITCHELL ? 4.f : 3.f;
  lutW = int(std::ceil(width)) * 5;
  cdf_x.assign(size_t(lutW) * lutW, 0.f);
  cdf_y.assign(lutW, 0.f);
  for (int y = 0; y < lutW; y++) {
    const float fy = (y + 0.5f) * (1.f / float(lutW));
    for (int x = 0; x < lutW; x++) {
      const float fx = (x + 0.5f) * (1.f / float(lutW));
      const V2 c = {(fx - 0.5f) * width, (fy - 0.5f) * width};
      float e = 0.f;
      if (t == PF_GAUSS) {
        const float sigma = (0.5f * width) / 3.f;
        e = std::exp(-0.5f * ((c.x * c.x + c.y * c.y) / (sigma * sigma)));
      } else if (t == PF_MITCHELL) {
        const float B = 1.f / 3.f, C = 1.f / 3.f;
        const float tx = c.x / width * 4.f, ty = c.y / width * 4.f;
        const float f = std::sqrt(tx * tx + ty * ty), f2 = f * f, f3 = f2 * f;
        if (f < 1.f)
          e = (1.f / 6.f) * ((12.f - 9.f * B - 6.f * C) * f3 + (-18.f + 12.f * B + 6.f * C) * f2 +
                             (6.f - 2.f * B));
        else if (f < 2.f)
          e = (1.f / 6.f) * ((-B - 6.f * C) * f3 + (6.f * B + 30.f * C) * f2 +
                             (-12.f * B - 48.f * C) * f + (8.f * B + 24.f * C));
      } else {
        const float f = std::sqrt(c.x * c.x + c.y * c.y) + width / 2.f;
        const float w = 1.f / width;
        const float pi2 = float(2.0 * M_PI);
        e = 0.35875f - 0.48829f * std::cos(pi2 * f * w) + 0.14128f * std::cos(2.f * pi2 * f * w) -
            0.01168f * std::cos(3.f * pi2 * f * w);
      }
      cdf_x[size_t(y) * lutW + x] = std::max(0.f, e);
    }
    cdf_y[y] = create1D(lutW, &cdf_x[size_t(y) * lutW]);
  }
  create1D(lutW, cdf_y.data());
}

V2 PixelFilter::sample(V2 s) const {
  if (type == PF_POINT) return {0.f, 0.f};
  if (type == PF_BOX) return {(s.x - 0.5f) * width, (s.y - 0.5f) * width};
  const S1 sy = sample1D(lutW, cdf_y.data(), s.y);
  const S1 sx = sample1D(lutW, &cdf_x[size_t(sy.idx) * lutW], s.x);
  const float r = 1.f / float(lutW);
  const V2 uv = {(sx.idx + sx.frac) * r, (sy.idx + sy.frac) * r};
  return {(uv.x - 0.5f) * width, (uv.y - 0.5f) * width};
}

DG postIntersect(const Scene &s, const Ray &ray, const Hit &hit, bool attrs) {
  DG dg;
  dg.st = {hit.u, hit.v};
  dg.primID = hit.primID;
  dg.geomID = hit.geomID;
  dg.instID = hit.instID;
  dg.P = ray.org + hit.t * ray.dir;
  // find the entry of this (instance, model)
  const InstanceEntry *e = &s.entries[hit.entry];
  const Geometry &g = s.geoms[e->geom];
  V3 Ng = hit.Ng, Ns = hit.Ng;
  V3 dPds = v3(1.f, 0.f, 0.f);  // World.ih postIntersect default tangent
  float eps;
  if (g.type == 0 && g.boxFaces) {
    eps = 0.f;  // Boxes_postIntersect (geometry/Boxes.ispc) sets no geometry epsilon
  } else if (g.type == 0 && !g.quadIndex.empty()) {
    // QuadMesh_postIntersect (geometry/Mesh.ispc:67-176): calcEpsilon over the 4 vertices, dPds = vb - va
    const uint32_t *q = &g.quadIndex[4 * size_t(hit.primID)];
    const V3 a = g.verts[q[0]], b = g.verts[q[1]], c = g.verts[q[2]], d = g.verts[q[3]];
    eps = reduce_max(vmax(vmax(vabs(a), vabs(b)), vmax(vabs(c), vabs(d)))) * ulpEpsilon;
    dPds = b - a;
    dg.dPdt = d - a;
  } else if (g.type == 0) {
    // TriangleMesh_postIntersect (geometry/Mesh.ispc:178-276): dPds = vb - va without texcoords
    const uint32_t i0 = g.index[3 * hit.primID], i1 = g.index[3 * hit.primID + 1], i2 = g.index[3 * hit.primID + 2];
    const V3 a = g.verts[i0], b = g.verts[i1], c = g.verts[i2];
    eps = reduce_max(vmax(vmax(vabs(a), vabs(b)), vabs(c))) * ulpEpsilon;
    dPds = b - a;
    dg.dPdt = c - a;
    if (attrs && !g.boxFaces) {
      const float w0 = 1.f - hit.u - hit.v, w1 = hit.u, w2 = hit.v;
      if (!g.normals.empty()) Ns = w0 * g.normals[i0] + w1 * g.normals[i1] + w2 * g.normals[i2];
      if (!g.colors.empty()) {
        const V4 c0 = g.colors[i0], c1 = g.colors[i1], c2 = g.colors[i2];
        dg.color = {w0 * c0.x + w1 * c1.x + w2 * c2.x, w0 * c0.y + w1 * c1.y + w2 * c2.y,
                    w0 * c0.z + w1 * c1.z + w2 * c2.z, w0 * c0.w + w1 * c1.w + w2 * c2.w};
      }
      if (!g.texcoords.empty()) {
        const V2 t0 = g.texcoords[i0], t1 = g.texcoords[i1], t2 = g.texcoords[i2];
        dg.st = {w0 * t0.x + w1 * t1.x + w2 * t2.x, w0 * t0.y + w1 * t1.y + w2 * t2.y};
        const V2 d02 = {t0.x - t2.x, t0.y - t2.y}, d12 = {t1.x - t2.x, t1.y - t2.y};
        const float det = d02.x * d12.y - d02.y * d12.x;
        if (det != 0.f) {
          const float inv = 1.f / det;
          const V3 p02 = a - c, p12 = b - c;
          dPds = (d12.y * p02 - d02.y * p12) * inv;
          dg.dPdt = (d02.x * p12 - d12.x * p02) * inv;
        }
      }
    }
  } else if (g.type == 3) {
    eps = 0.f;  // Planes_postIntersect (geometry/Planes.ispc:115-121) sets no geometry epsilon
  } else {
    eps = g.spheres[hit.primID].w * ulpEpsilon;  // Spheres_postIntersect, also for discs
  }
  // the instance transform (motion blur: at the ray time, Instance.ih:57-91)
  const bool moving = e->motion.size() >= 24;
  const A3 X = moving ? e->xfmAt(rayTime) : e->xfm;
  const A3 R = moving ? rcpAffine(X) : e->rcp;
  dg.dPds = xfmVector(X.l, dPds);  // Instance_postIntersect (common/Instance.ih:95-98)
  dg.dPdt = xfmVector(X.l, dg.dPdt);
  if (g.type != 0 || g.boxFaces) dg.st = {0.f, 0.f};  // spheres, boxes: no texture coordinates in these scenes
  // Instance_postIntersect: normals by the inverse transpose, epsilon by the
  // largest diagonal scale
  const L3 it = transposed(R.l);
  Ns = xfmVector(it, Ns);
  Ng = xfmVector(it, Ng);
  eps *= std::fmax(std::fabs(X.l.vx.x), std::fmax(std::fabs(X.l.vy.y), std::fabs(X.l.vz.z)));
  // calcEpsilon(P, dir, t)
  const float e2 = std::fmax(reduce_max(vabs(dg.P)), reduce_max(vabs(ray.dir)) * hit.t) * ulpEpsilon;
  dg.epsilon = std::fmax(eps, e2);
  V3 ffnng = normalize(Ng);
  Ng = ffnng;
  Ns = normalize(Ns);
  if (dot(ray.dir, Ng) >= 0.f) {
    ffnng = -ffnng;
    Ng = -Ng;
  }
  if (dot(Ng, Ns) < 0.f) Ns = -Ns;
  dg.Ng = Ng;
  dg.Ns = Ns;
  dg.P = dg.P + dg.epsilon * ffnng;
  return dg;
}

void fbAccumulate(FrameBuffer &fb, int x, int y, const ScreenSample &s) {
  const size_t i = size_t(y) * fb.W + x;
  const float accScale = 1.f / float(fb.frameID + 1);
  const float c[4] = {s.rgb.x, s.rgb.y, s.rgb.z, s.alpha};
  for (int k = 0; k < 4; k++)
    fb.color[4 * i + k] = accScale > 0.8f ? c[k] : lerpf(accScale, fb.color[4 * i + k], c[k]);
  const float a[6] = {s.normal.x, s.normal.y, s.normal.z, s.albedo.x, s.albedo.y, s.albedo.z};
  for (int k = 0; k < 3; k++) {
    fb.normal[3 * i + k] = accScale > 0.8f ? a[k] : lerpf(accScale, fb.normal[3 * i + k], a[k]);
    fb.albedo[3 * i + k] = accScale > 0.8f ? a[3 + k] : lerpf(accScale, fb.albedo[3 * i + k], a[3 + k]);
  }
  bool upd = fb.frameID == 0;
  if (fb.frameID > 0 && std::fabs(s.z) < std::fabs(fb.depth[i])) upd = true;
  if (upd) {
    fb.depth[i] = s.z;
    fb.primID[i] = s.primID;
    fb.geomID[i] = s.geomID;
    fb.instID[i] = s.instID;
  }
}

float *g_auxNormal = nullptr, *g_auxAlbedo = nullptr;
AOVolume g_aoVolume;
void copyAux(const FrameBuffer &fb) {
  if (g_auxNormal) std::memcpy(g_auxNormal, fb.normal.data(), fb.normal.size() * 4);
  if (g_auxAlbedo) std::memcpy(g_auxAlbedo, fb.albedo.data(), fb.albedo.size() * 4);
}

// ---------------------------------------------------------------- AO renderer
// AORenderer_renderSample (render/ao/AORenderer.ispc:23-149),
// AORenderer_computeShading (render/ao/surfaces.ispc:44-74),
// computeAO (render/util.ispc:12-54).
static float computeAO(const Scene &s, const DG &dg, int sampleCnt, float aoRadius, int px, int py,
                       uint32_t sampleZ) {
  const uint32_t accumID = sampleZ * uint32_t(sampleCnt);
  uint32_t t0 = uint32_t(px), t1 = uint32_t(py);
  tea8(t0, t1);
  const V2 rot = {to_float_unorm(t0), to_float_unorm(t1)};
  int hits = 0;
  const L3 l2w = frame(dg.Ns);
  for (int i = 0; i < sampleCnt; i++) {
    const float hx = PermHalton_sample5(accumID + i), hy = PermHalton_sample7(accumID + i);
    const float rx = CranleyPattersonRotation(hx, rot.x), ry = CranleyPattersonRotation(hy, rot.y);
    // cosineSampleHemisphere (math/sampling.ih:49-56)
    const float phi = float(2.0 * M_PI) * rx;
    const float cosT = std::sqrt(ry), sinT = std::sqrt(1.f - ry);
    const V3 local = {std::cos(phi) * sinT, std::sin(phi) * sinT, cosT};
    const V3 dir = xfmVector(l2w, local);
    if (dot(dir, dg.Ns) < 0.01f) {
      hits++;
      continue;
    }
    tl_rays++;
    if (s.occluded({dg.P, dg.epsilon, dir, aoRadius})) hits++;
  }
  return 1.f - float(hits) / float(sampleCnt);
}

void renderAO(const Scene &s, const Camera &cam, const PixelFilter &pf, const AOParams &p, FrameBuffer &fb,
              int nthreads) {
  const int W = fb.W, H = fb.H;
  const V2 rcpSize = {1.f / float(W), 1.f / float(H)};
  const uint32_t startSampleID = uint32_t(fb.frameID * p.spp + 1);
  parallelRows(H, nthreads, [&](int y) {
    for (int x = 0; x < W; x++) {
      ScreenSample acc;
      for (int sp = 0; sp < p.spp; sp++) {
        const uint32_t sid = startSampleID + sp;
        const V2 ps = {Halton_sample2(sid), CranleyPattersonRotation(Halton_sample3(sid), 1.f / 6.f)};
        const V2 pfs = pf.sample(ps);
        const V2 center = {(float(x) + 0.5f) * rcpSize.x, (float(y) + 0.5f) * rcpSize.y};
        V2 screen = {center.x + pfs.x * rcpSize.x, center.y + pfs.y * rcpSize.y};
        const float eye = cameraScreen(cam, screen, center);
        Ray ray = cameraRay(cam, screen, {0.f, 0.f}, eye);
        rayTime = shutterTime(cam, screen, 0.5f);  // RendererRenderTaskFn.inl:64: time sample 0.5
        // Renderer_getMaxDepth at the pixel centre (RendererRenderTaskFn.inl:41-42)
        if (p.maxDepth) ray.tfar = std::fmin(ray.tfar, std::fmax(0.f, p.maxDepth->get(center, 0.f).x));
        const V2 cone = cameraCone(cam, screen, rcpSize.y);
        float coneWidth = cone.x;
        ScreenSample smp;
        V4 out = {0, 0, 0, 0};
        bool first = true;
        const float tfar0 = ray.tfar;
        RandomSampler rs;
        rs.init(uint32_t(x + W * y), sid);
        while (out.w < 0.99f) {
          Hit hit;
          tl_rays++;
          const bool h = s.intersect(ray, hit);
          if (g_aoVolume.vm) {
            Ray vr = ray;
            vr.tfar = h ? hit.t : ray.tfar;
            if (g_aoVolume.overlaps(g_aoVolume.vm, vr)) {
              const float jitter = rs.getFloat();
              const V4 vc = g_aoVolume.integrate(g_aoVolume.vm, vr, jitter, g_aoVolume.samplingRate);
              const float f = 1.f - out.w;
              out = {out.x + f * vc.x, out.y + f * vc.y, out.z + f * vc.z, out.w + f * vc.w};
            }
          }
          V4 blended;
          if (h) {
            const DG dg = postIntersect(s, ray, hit, true);
            coneWidth += cone.y * hit.t;
            // getSurfaceColor (render/ao/surfaces.ispc:17-42)
            V3 color = v3(1.f);
            float opacity = 1.f;
            const int mi = s.entries[hit.entry].material;
            if (mi >= 0 && size_t(mi) < p.mats.size() && p.mats[size_t(mi)].isObj) {
              const AOMaterial &m = p.mats[size_t(mi)];
              color = m.kd;
              if (m.kdMap) {
                const V4 t = m.kdMap->get(dg.st, pixelFootprint(coneWidth, ray.dir, dg, p.mipBiasFactor));
                color = color * v3(t.x, t.y, t.z);
                opacity *= t.w;
              }
              opacity *= m.d;
            }
            color = color * v3(dg.color.x, dg.color.y, dg.color.z);
            opacity *= dg.color.w;
            const float eye = std::fabs(dot(dg.Ns, ray.dir)) * opacity;
            float intensity = eye;
            if (p.aoSamples > 0 && p.aoIntensity > 0.01f) {
              const float ao = computeAO(s, dg, p.aoSamples, p.aoRadius, x, y, sid);
              intensity *= (1.f - p.aoIntensity) + ao * p.aoIntensity;
            }
            blended = {color.x * intensity, color.y * intensity, color.z * intensity, opacity};
            if (first) {
              smp.albedo = color;  // AORenderer_computeShading: the surface colour
              smp.normal = dg.Ns;
              smp.z = hit.t;
              smp.primID = dg.primID;
              smp.geomID = dg.geomID;
              smp.instID = dg.instID;
            }
            ray.tnear = hit.t + dg.epsilon;
            ray.tfar = tfar0;
          } else {
            blended = p.backplate ? p.backplate->getScreen(center) : p.bgColor;
            if (first) {
              smp.z = ray.tfar;
              smp.albedo = {blended.x, blended.y, blended.z};
              smp.normal = ray.dir;
            }
          }
          const float f = 1.f - out.w;
          out = {out.x + f * blended.x, out.y + f * blended.y, out.z + f * blended.z, out.w + f * blended.w};
          first = false;
          if (!h) break;
        }
        smp.rgb = {out.x, out.y, out.z};
        smp.alpha = out.w;
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
  fb.frameID++;
}

}  // namespace orc
