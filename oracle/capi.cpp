// Oracle (test infrastructure only): flat C interface used by the tests and
// by bench.py's CPU-baseline leg through ctypes.  Nothing in the product
// links or loads this library.
#include <cstring>

#include "render.h"
#include "texture.h"

using namespace orc;

// rkcommon rcp(AffineSpace3f): adjoint / det in float, p' = -(l' p)
A3 orc::rcpAffine(const A3 &a) {
  const L3 &l = a.l;
  const float det = dot(l.vx, cross(l.vy, l.vz));
  const L3 adjT = {cross(l.vy, l.vz), cross(l.vz, l.vx), cross(l.vx, l.vy)};
  const L3 adj = transposed(adjT);
  L3 il = {adj.vx / det, adj.vy / det, adj.vz / det};
  A3 r;
  r.l = il;
  r.p = -xfmVector(il, a.p);
  return r;
}
namespace {
A3 fromRowMajor(const float *X) {
  A3 a;
  a.l.vx = {X[0], X[4], X[8]};
  a.l.vy = {X[1], X[5], X[9]};
  a.l.vz = {X[2], X[6], X[10]};
  a.p = {X[3], X[7], X[11]};
  return a;
}
}  // namespace

struct OrCamera {
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

extern "C" {

void *or_scene_new() { return new Scene(); }
void or_scene_free(void *s) { delete static_cast<Scene *>(s); }

int or_scene_add_mesh(void *sp, const float *verts, int nverts, const uint32_t *index, int ntris) {
  Scene &s = *static_cast<Scene *>(sp);
  Geometry g;
  g.type = 0;
  g.verts.resize(nverts);
  std::memcpy(g.verts.data(), verts, sizeof(float) * 3 * nverts);
  g.index.assign(index, index + 3 * size_t(ntris));
  s.geoms.push_back(std::move(g));
  return int(s.geoms.size() - 1);
}

// quad (v0, v1, v2, v3) -> triangles (v0, v1, v3), (v2, v3, v1) (Embree's
// quad decomposition), both reporting the quad's primID
int or_scene_add_quad_mesh(void *sp, const float *verts, int nverts, const uint32_t *index, int nquads) {
  Scene &s = *static_cast<Scene *>(sp);
  Geometry g;
  g.type = 0;
  g.verts.resize(nverts);
  std::memcpy(g.verts.data(), verts, sizeof(float) * 3 * nverts);
  g.quadIndex.assign(index, index + 4 * size_t(nquads));
  g.primDiv = 2;
  for (int q = 0; q < nquads; q++) {
    const uint32_t *v = index + 4 * size_t(q);
    for (uint32_t k : {v[0], v[1], v[3], v[2], v[3], v[1]}) g.index.push_back(k);
  }
  s.geoms.push_back(std::move(g));
  return int(s.geoms.size() - 1);
}

// box3f (lower, upper) -> 8 corners and 12 face triangles (corner c =
// (x: c & 1, y: c >> 1 & 1, z: c >> 2)), all reporting the box's primID
int or_scene_add_boxes(void *sp, const float *boxes, int n) {
  Scene &s = *static_cast<Scene *>(sp);
  Geometry g;
  g.type = 0;
  g.primDiv = 12;
  g.boxFaces = true;
  static const int F[6][4] = {{0, 4, 6, 2}, {1, 3, 7, 5}, {0, 1, 5, 4}, {2, 6, 7, 3}, {0, 2, 3, 1}, {4, 5, 7, 6}};
  for (int b = 0; b < n; b++) {
    const float *lo = boxes + 6 * size_t(b), *hi = lo + 3;
    const uint32_t o = uint32_t(g.verts.size());
    for (int c = 0; c < 8; c++) g.verts.push_back({(c & 1) ? hi[0] : lo[0], (c & 2) ? hi[1] : lo[1], (c & 4) ? hi[2] : lo[2]});
    for (int f = 0; f < 6; f++)
      for (int k : {0, 1, 2, 0, 2, 3}) g.index.push_back(o + uint32_t(F[f][k]));
  }
  s.geoms.push_back(std::move(g));
  return int(s.geoms.size() - 1);
}

// per-vertex normals (3), colours (4) and texture coordinates (2) of
// triangle mesh `geom`, each null or one per vertex
void or_scene_set_mesh_attributes(void *sp, int geom, const float *normals, const float *colors,
                                  const float *texcoords) {
  Geometry &g = static_cast<Scene *>(sp)->geoms[size_t(geom)];
  const size_t n = g.verts.size();
  g.normals.clear();
  g.colors.clear();
  g.texcoords.clear();
  for (size_t i = 0; normals && i < n; i++) g.normals.push_back({normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]});
  for (size_t i = 0; colors && i < n; i++)
    g.colors.push_back({colors[4 * i], colors[4 * i + 1], colors[4 * i + 2], colors[4 * i + 3]});
  for (size_t i = 0; texcoords && i < n; i++) g.texcoords.push_back({texcoords[2 * i], texcoords[2 * i + 1]});
}

// 2D textures: w x h texels of an OSPTextureFormat, rows from the bottom
void *or_texture_new(int w, int h, int format, int filter, int wrapS, int wrapT, int mipmaps, const void *data) {
  return makeTexture(w, h, format, filter, wrapS, wrapT, mipmaps != 0, data);
}
void or_texture_free(void *t) { delete static_cast<Texture *>(t); }
int or_texture_levels(const void *t) { return int(static_cast<const Texture *>(t)->levels.size()); }
// copies level `level`'s texels into dst (bytes must cover them); returns the bytes copied
size_t or_texture_read_level(const void *tp, int level, void *dst, size_t bytes) {
  const Texture &t = *static_cast<const Texture *>(tp);
  const std::vector<uint8_t> &l = t.levels[size_t(level)];
  if (bytes < l.size()) return 0;
  std::memcpy(dst, l.data(), l.size());
  return l.size();
}
// Texture2D_get at n texture coordinates st (2 floats each) with footprints fp
void or_texture_sample(const void *tp, int n, const float *st, const float *fp, float *out) {
  const Texture &t = *static_cast<const Texture *>(tp);
  for (int i = 0; i < n; i++) {
    const V4 v = t.get({st[2 * i], st[2 * i + 1]}, fp[i]);
    out[4 * i] = v.x;
    out[4 * i + 1] = v.y;
    out[4 * i + 2] = v.z;
    out[4 * i + 3] = v.w;
  }
}

int or_scene_add_spheres(void *sp, const float *xyzr, int n) {
  Scene &s = *static_cast<Scene *>(sp);
  Geometry g;
  g.type = 1;
  g.spheres.resize(n);
  std::memcpy(g.spheres.data(), xyzr, sizeof(float) * 4 * n);
  s.geoms.push_back(std::move(g));
  return int(s.geoms.size() - 1);
}

// discs: xyzr per disc; normals null (ray-facing discs) or 3 per disc (oriented discs)
int or_scene_add_discs(void *sp, const float *xyzr, int n, const float *normals) {
  Scene &s = *static_cast<Scene *>(sp);
  Geometry g;
  g.type = 1;
  g.sphereKind = normals ? 2 : 1;
  g.spheres.resize(n);
  std::memcpy(g.spheres.data(), xyzr, sizeof(float) * 4 * n);
  for (int i = 0; normals && i < n; i++) g.discNormals.push_back({normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]});
  s.geoms.push_back(std::move(g));
  return int(s.geoms.size() - 1);
}

// planes: (a, b, c, d) per plane (a x + b y + c z = d); bounds null or 6 per plane (lower, upper)
int or_scene_add_planes(void *sp, const float *coeffs, int n, const float *bounds) {
  Scene &s = *static_cast<Scene *>(sp);
  Geometry g;
  g.type = 3;
  g.planeBounded = bounds != nullptr;
  for (int i = 0; i < n; i++) {
    g.planes.push_back({coeffs[4 * i], coeffs[4 * i + 1], coeffs[4 * i + 2], coeffs[4 * i + 3]});
    if (bounds) {
      const float *b = bounds + 6 * i;
      g.planeBounds.push_back({{b[0], b[1], b[2]}, {b[3], b[4], b[5]}});
    }
  }
  s.geoms.push_back(std::move(g));
  return int(s.geoms.size() - 1);
}

// xfm: row-major 3x4 affine or null for identity
void or_scene_add_instance(void *sp, int geom, uint32_t instID, uint32_t geomID, const float *xfm, int material) {
  Scene &s = *static_cast<Scene *>(sp);
  InstanceEntry e;
  e.material = material;
  e.geom = geom;
  e.instID = instID;
  e.geomID = geomID;
  static const float I[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
  e.identity = xfm == nullptr;
  e.xfm = fromRowMajor(xfm ? xfm : I);
  e.rcp = rcpAffine(e.xfm);
  s.entries.push_back(e);
}

// xfms: nkeys >= 2 row-major 3x4 keys over [t0, t1]
void or_scene_add_instance_motion(void *sp, int geom, uint32_t instID, uint32_t geomID, const float *xfms, int nkeys,
                                  float t0, float t1, int material) {
  Scene &s = *static_cast<Scene *>(sp);
  InstanceEntry e;
  e.material = material;
  e.geom = geom;
  e.instID = instID;
  e.geomID = geomID;
  e.identity = false;
  e.xfm = fromRowMajor(xfms);
  e.rcp = rcpAffine(e.xfm);
  e.motion.assign(xfms, xfms + 12 * size_t(nkeys));
  e.t0 = t0;
  e.t1 = t1 < t0 ? t0 : t1;
  s.entries.push_back(e);
}

void or_scene_commit(void *sp) { static_cast<Scene *>(sp)->commit(); }

// rays: n x 8 floats (org xyz, tnear, dir xyz, tfar).
// out_f: n x 6 floats (t, u, v, Ng xyz); out_id: n x 3 uint32 (prim, geom, inst).
// occlusion != 0: out_f[6i] = 1 when occluded else 0, ids untouched.
void or_trace(void *sp, const float *rays, int n, int occlusion, float *out_f, uint32_t *out_id, int nthreads) {
  const Scene &s = *static_cast<Scene *>(sp);
  const int rowsz = 1024;
  const int nrows = (n + rowsz - 1) / rowsz;
  parallelRows(nrows, nthreads, [&](int r) {
    for (int i = r * rowsz; i < std::min(n, (r + 1) * rowsz); i++) {
      const float *R = rays + 8 * size_t(i);
      const Ray ray = {{R[0], R[1], R[2]}, R[3], {R[4], R[5], R[6]}, R[7]};
      if (occlusion) {
        out_f[6 * size_t(i)] = s.occluded(ray) ? 1.f : 0.f;
        continue;
      }
      Hit h;
      const bool hit = s.intersect(ray, h);
      float *F = out_f + 6 * size_t(i);
      uint32_t *I = out_id + 3 * size_t(i);
      if (!hit) {
        F[0] = INFINITY;
        F[1] = F[2] = F[3] = F[4] = F[5] = 0.f;
        I[0] = I[1] = I[2] = INVALID_ID;
        continue;
      }
      F[0] = h.t;
      F[1] = h.u;
      F[2] = h.v;
      F[3] = h.Ng.x;
      F[4] = h.Ng.y;
      F[5] = h.Ng.z;
      I[0] = h.primID;
      I[1] = h.geomID;
      I[2] = h.instID;
    }
  });
}

// Primary camera rays for a W x H image at frame `frameID` with `spp`
// samples per pixel (sample s of pixel (x,y) at index ((y*W)+x)*spp+s),
// exactly as the renderers generate them.  out: 8 floats per ray.
void or_camera_rays(const OrCamera *c, int pixelFilter, int W, int H, int spp, int frameID, float *out) {
  Camera cam = makeCamera({c->pos[0], c->pos[1], c->pos[2]}, {c->dir[0], c->dir[1], c->dir[2]},
                          {c->up[0], c->up[1], c->up[2]}, c->fovy, c->aspect, c->nearClip, c->type, c->height,
                          0.f, 1.f, false, c->stereoMode, c->interpupillaryDistance);
  setSubImage(cam, c->imageStart, c->imageEnd, c->stereoMode);
  PixelFilter pf;
  pf.init(pixelFilter);
  const V2 rcpSize = {1.f / float(W), 1.f / float(H)};
  const uint32_t start = uint32_t(frameID * spp + 1);
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++)
      for (int sp = 0; sp < spp; sp++) {
        const uint32_t sid = start + sp;
        const V2 ps = {Halton_sample2(sid), CranleyPattersonRotation(Halton_sample3(sid), 1.f / 6.f)};
        const V2 pfs = pf.sample(ps);
        const V2 center = {(float(x) + 0.5f) * rcpSize.x, (float(y) + 0.5f) * rcpSize.y};
        V2 screen = {center.x + pfs.x * rcpSize.x, center.y + pfs.y * rcpSize.y};
        const float eye = cameraScreen(cam, screen, center);
        const Ray r = cameraRay(cam, screen, {0.f, 0.f}, eye);
        float *o = out + 8 * ((size_t(y) * W + x) * spp + sp);
        o[0] = r.org.x;
        o[1] = r.org.y;
        o[2] = r.org.z;
        o[3] = r.tnear;
        o[4] = r.dir.x;
        o[5] = r.dir.y;
        o[6] = r.dir.z;
        o[7] = r.tfar;
      }
}

// the renderers' next calls also copy the accumulated normal / albedo
// channels (3 floats per pixel) to these (null: not wanted)
void or_set_aux_output(float *normal, float *albedo) {
  g_auxNormal = normal;
  g_auxAlbedo = albedo;
}

struct OrFrame {
  float *color;      // W*H*4
  float *depth;      // W*H
  uint32_t *primID;  // W*H
  uint32_t *geomID;
  uint32_t *instID;
};

// the AO renderer's optional inputs: map_backplate, map_maxDepth (Textures
// or null), mipMapBias, and obj materials (isObj, kd[3], ks[3], ns, d,
// tf[3], map_kd as in b200_scivis_material; null / 0: white surfaces)
struct OrAoExtra {
  const void *backplate, *maxDepth;
  float mipMapBias;
  const void *materials;
  int nmaterials;
};
struct OrAoMaterial {
  int isObj;
  float kd[3], ks[3], ns, d, tf[3];
  const void *kdMap;
};

// Renders `frames` accumulated frames of the AO renderer; outputs the final
// accumulation buffers.
void or_render_ao(void *sp, const OrCamera *c, int pixelFilter, int W, int H, int spp, int aoSamples,
                  float aoRadius, float aoIntensity, const float *bg, int frames, OrFrame *out, int nthreads,
                  const OrAoExtra *extra) {
  const Scene &s = *static_cast<Scene *>(sp);
  Camera cam = makeCamera({c->pos[0], c->pos[1], c->pos[2]}, {c->dir[0], c->dir[1], c->dir[2]},
                          {c->up[0], c->up[1], c->up[2]}, c->fovy, c->aspect, c->nearClip, c->type, c->height,
                          c->apertureRadius, c->focusDistance, c->architectural != 0, c->stereoMode,
                          c->interpupillaryDistance);
  setShutter(cam, c->shutter[0], c->shutter[1], c->shutterType, c->rollingDuration);
  setSubImage(cam, c->imageStart, c->imageEnd, c->stereoMode);
  PixelFilter pf;
  pf.init(pixelFilter);
  FrameBuffer fb;
  fb.resize(W, H);
  AOParams p;
  p.spp = spp;
  p.aoSamples = aoSamples;
  p.aoRadius = aoRadius;
  p.aoIntensity = aoIntensity;
  p.bgColor = {bg[0], bg[1], bg[2], bg[3]};
  if (extra) {
    p.backplate = static_cast<const Texture *>(extra->backplate);
    p.maxDepth = static_cast<const Texture *>(extra->maxDepth);
    p.mipBiasFactor = std::pow(2.f, extra->mipMapBias);
    const OrAoMaterial *m = static_cast<const OrAoMaterial *>(extra->materials);
    for (int i = 0; i < extra->nmaterials; i++)
      p.mats.push_back({m[i].isObj, {m[i].kd[0], m[i].kd[1], m[i].kd[2]}, m[i].d,
                        static_cast<const Texture *>(m[i].kdMap)});
  }
  for (int f = 0; f < frames; f++) renderAO(s, cam, pf, p, fb, nthreads);
  const size_t N = size_t(W) * H;
  std::memcpy(out->color, fb.color.data(), N * 4 * sizeof(float));
  std::memcpy(out->depth, fb.depth.data(), N * sizeof(float));
  std::memcpy(out->primID, fb.primID.data(), N * 4);
  std::memcpy(out->geomID, fb.geomID.data(), N * 4);
  std::memcpy(out->instID, fb.instID.data(), N * 4);
  copyAux(fb);
}

uint64_t or_ray_count(int reset) {
  const uint64_t n = g_rayCount.load();
  if (reset) g_rayCount.store(0);
  return n;
}

// Sampler tables for the pinning test against the reference's tables.
void or_tables(uint32_t *perm3, uint32_t *perm5, uint32_t *perm7, uint32_t *sobolRev) {
  const Tables &t = tables();
  std::memcpy(perm3, t.perm3, sizeof(t.perm3));
  std::memcpy(perm5, t.perm5, sizeof(t.perm5));
  std::memcpy(perm7, t.perm7, sizeof(t.perm7));
  std::memcpy(sobolRev, t.sobolRev, sizeof(t.sobolRev));
}

}  // extern "C"
