// Camera ray generation, pixel-filter sampling, differential geometry and
// framebuffer accumulation for the b200 renderers.
//   PerspectiveCamera_initRay  modules/cpu/camera/PerspectiveCamera.ispc:16-64
//   pixel loop                 modules/cpu/render/RendererRenderTaskFn.inl:30-80
//   LUTPixelFilter_sample      modules/cpu/pf/LUTPixelFilter.ispc:10-17,
//                              math/Distribution1D.ih, Distribution2D.ispc
//   postIntersect              modules/cpu/common/World.ih:389-465,
//                              common/Instance.ih:44-107, geometry/Mesh.ispc:178+,
//                              geometry/Spheres.ispc:24-42
//   LocalFB_accumulateSample   modules/cpu/fb/LocalFB.ispc:14-78
#pragma once
#include "samplers.cuh"
#include "traverse.cuh"

namespace b200 {

// type 0 perspective; 1 orthographic (org = lower-left corner of the image
// plane, dir_00 = view direction); 2 panoramic (frame vx, vy, vz in
// du_size, dv_up, dir_00)
struct CameraD {
  V3 org, dir_00, du_size, dv_up;
  float nearClip;
  int type;
};

struct PixelFilterD {
  int type;  // 0 point, 1 box, 2.. LUT
  float width;
  int lutW;
  const float *cdf_x;  // lutW * lutW
  const float *cdf_y;  // lutW
};

struct FrameD {
  float4 *color;
  float *depth;
  uint32_t *primID, *geomID, *instID;
  float4 *variance;  // optional: accumulates the frames picked by accumVariance
  float3 *normal, *albedo;
  int W, H, frameID;
  float *aux;                 // NORMAL/ALBEDO requested: per pixel the path tracer's sums of this frame (6 floats)
  int accumVariance;          // this frame goes into the variance buffer (FrameBuffer::beginFrame)
  const uint8_t *taskActive;  // adaptive accumulation: per 8x8 task, render it? (null: all)
  int tasksX;
};

// Is pixel (x, y) in a render task of this frame (LocalFrameBuffer::getRenderTaskIDs)?
B200_D bool pixelActive(const FrameD &fb, int x, int y) {
  return !fb.taskActive || fb.taskActive[(y >> 3) * fb.tasksX + (x >> 3)] != 0;
}

B200_D Ray cameraRay(const CameraD &c, float sx, float sy) {
  Ray r;
  r.tnear = c.nearClip;
  r.tfar = INFINITY;
  if (c.type == 1) {  // OrthographicCamera_initRay (camera/OrthographicCamera.ispc:11-49)
    r.org = add(add(c.org, mul(sx, c.du_size)), mul(sy, c.dv_up));
    r.dir = c.dir_00;
    return r;
  }
  if (c.type == 2) {  // PanoramicCamera_initRay (camera/PanoramicCamera.ispc:12-90), mono
    float sp, cp, st, ct;
    sincosf(6.28318530717958647692f * sx, &sp, &cp);
    sincosf(3.14159265358979323846f * sy, &st, &ct);
    const V3 l = mk(cp * st, sp * st, ct);
    r.org = c.org;
    r.dir = add(add(mul(c.du_size, -l.y), mul(c.dv_up, -l.z)), mul(c.dir_00, l.x));
    return r;
  }
  const V3 d = add(add(c.dir_00, mul(sx, c.du_size)), mul(sy, c.dv_up));
  r.org = c.org;
  r.dir = normalize(d);
  return r;
}

B200_D void sample1D(int size, const float *cdf, float s, int &idx, float &frac) {
  int first = 0, len = size;
  while (len > 0) {
    const int half = len >> 1, mid = first + half;
    if (s < __ldg(cdf + mid)) {
      len = half;
    } else {
      first = mid + 1;
      len -= half + 1;
    }
  }
  const float bef = first == 0 ? 0.f : __ldg(cdf + first - 1);
  const float dpdf = fsub(__ldg(cdf + first), bef);
  idx = first;
  frac = fdiv(fsub(s, bef), dpdf);
}

B200_D float2 filterSample(const PixelFilterD &pf, float sx, float sy) {
  if (pf.type == 0) return make_float2(0.f, 0.f);
  if (pf.type == 1) return make_float2(fmul(fsub(sx, 0.5f), pf.width), fmul(fsub(sy, 0.5f), pf.width));
  int iy, ix;
  float fy, fx;
  sample1D(pf.lutW, pf.cdf_y, sy, iy, fy);
  sample1D(pf.lutW, pf.cdf_x + iy * pf.lutW, sx, ix, fx);
  const float r = fdiv(1.f, float(pf.lutW));
  const float u = fmul(fadd(float(ix), fx), r), v = fmul(fadd(float(iy), fy), r);
  return make_float2(fmul(fsub(u, 0.5f), pf.width), fmul(fsub(v, 0.5f), pf.width));
}

// screen position of sample `sid` of pixel (x, y): Halton(2), rotated
// Halton(3), through the pixel filter
B200_D Ray primaryRay(const SamplerTables *T, const CameraD &cam, const PixelFilterD &pf, int x, int y, float rcpW, float rcpH,
                      uint32_t sid) {
  const float ps_x = Halton_sample2(sid);
  const float ps_y = cpRotate(Halton_sample3(T, sid), 1.f / 6.f);
  const float2 pfs = filterSample(pf, ps_x, ps_y);
  const float cx = fmul(fadd(float(x), 0.5f), rcpW), cy = fmul(fadd(float(y), 0.5f), rcpH);
  return cameraRay(cam, fadd(cx, fmul(pfs.x, rcpW)), fadd(cy, fmul(pfs.y, rcpH)));
}

struct DG {
  V3 P, Ng, Ns;
  V3 dPds;  // surface tangent (DG_TANGENTS): the triangle's first edge, else (1, 0, 0), in world space
  float epsilon;
  uint32_t entry;
};

// postIntersect with DG_NG | DG_NS | DG_NORMALIZE | DG_FACEFORWARD
B200_D DG postIntersect(const Scene &sc, const Ray &ray, const HitRec &hit) {
  DG dg;
  dg.entry = hit.entry;
  const Entry &e = sc.entries[hit.entry];
  dg.P = add(ray.org, mul(hit.t, ray.dir));
  V3 Ng = hit.Ng, Ns = hit.Ng;
  // DG_TANGENTS: meshes take their first edge (TriangleMesh_postIntersect
  // geometry/Mesh.ispc:172-175, QuadMesh_postIntersect :171-174), other
  // geometry keeps the default (1, 0, 0) (World.ih postIntersect)
  V3 dPds = mk(1.f, 0.f, 0.f);
  float eps;
  if (e.type == GEOM_TRIANGLES && e.meshKind == MESH_BOXES) {
    eps = 0.f;  // Boxes_postIntersect (geometry/Boxes.ispc) sets no geometry epsilon
  } else if (e.type == GEOM_TRIANGLES && e.meshKind == MESH_QUADS) {
    // QuadMesh_postIntersect (geometry/Mesh.ispc:67-176): epsilon over the 4 vertices
    const uint4 q = __ldg(reinterpret_cast<const uint4 *>(e.index) + hit.primID);
    const uint32_t ix[4] = {q.x, q.y, q.z, q.w};
    V3 m = splat(0.f), v[2];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const V3 p = mk(__ldg(e.verts + 3 * ix[k]), __ldg(e.verts + 3 * ix[k] + 1), __ldg(e.verts + 3 * ix[k] + 2));
      if (k < 2) v[k] = p;
      m = vmax(m, vabs(p));
    }
    eps = fmul(reduce_max(m), ULP_EPSILON);
    dPds = sub(v[1], v[0]);
  } else if (e.type == GEOM_TRIANGLES) {
    const uint32_t i0 = __ldg(e.index + 3 * hit.primID), i1 = __ldg(e.index + 3 * hit.primID + 1),
                   i2 = __ldg(e.index + 3 * hit.primID + 2);
    const V3 a = mk(__ldg(e.verts + 3 * i0), __ldg(e.verts + 3 * i0 + 1), __ldg(e.verts + 3 * i0 + 2));
    const V3 b = mk(__ldg(e.verts + 3 * i1), __ldg(e.verts + 3 * i1 + 1), __ldg(e.verts + 3 * i1 + 2));
    const V3 c = mk(__ldg(e.verts + 3 * i2), __ldg(e.verts + 3 * i2 + 1), __ldg(e.verts + 3 * i2 + 2));
    eps = fmul(reduce_max(vmax(vmax(vabs(a), vabs(b)), vabs(c))), ULP_EPSILON);
    dPds = sub(b, a);
  } else {
    eps = fmul(__ldg(&e.spheres[hit.primID].w), ULP_EPSILON);
  }
  if (!e.identity) {
    Ns = xfmVectorT(e.rcp, Ns);
    Ng = xfmVectorT(e.rcp, Ng);
    eps = fmul(eps, e.epsScale);
    dPds = xfmVector(e.xfm, dPds);  // Instance_postIntersect (common/Instance.ih:95-98)
  }
  dg.dPds = dPds;
  const float e2 = fmul(fmaxf(reduce_max(vabs(dg.P)), fmul(reduce_max(vabs(ray.dir)), hit.t)), ULP_EPSILON);
  dg.epsilon = fmaxf(eps, e2);
  V3 ffnng = normalize(Ng);
  Ng = ffnng;
  Ns = normalize(Ns);
  if (dot(ray.dir, Ng) >= 0.f) {
    ffnng = neg(ffnng);
    Ng = neg(Ng);
  }
  if (dot(Ng, Ns) < 0.f) Ns = neg(Ns);
  dg.Ng = Ng;
  dg.Ns = Ns;
  dg.P = add(dg.P, mul(dg.epsilon, ffnng));
  return dg;
}

// Shading frame around N (rkcommon frame(N))
B200_D void frame(V3 N, V3 &dx, V3 &dy) {
  const V3 dx0 = mk(0.f, N.z, -N.y), dx1 = mk(-N.z, 0.f, N.x);
  dx = normalize(fabsf(N.x) < fabsf(N.y) ? dx0 : dx1);
  dy = normalize(cross(N, dx));
}
B200_D V3 toWorld(V3 dx, V3 dy, V3 N, V3 l) { return add(add(mul(dx, l.x), mul(dy, l.y)), mul(N, l.z)); }

// computeAO's sampling (render/util.ispc:12-54): a TEA-hashed Cranley-
// Patterson rotation per pixel over permuted Halton (bases 5, 7), mapped to a
// cosine-weighted direction about Ns
struct AOBasis {
  V3 dx, dy;
  float rx0, ry0;
};

B200_D AOBasis aoBasis(const DG &dg, int px, int py) {
  AOBasis B;
  uint32_t t0 = uint32_t(px), t1 = uint32_t(py);
  tea8(t0, t1);
  B.rx0 = to_float_unorm(t0);
  B.ry0 = to_float_unorm(t1);
  frame(dg.Ns, B.dx, B.dy);
  return B;
}

B200_D V3 aoDirection(const SamplerTables *T, const AOBasis &B, V3 Ns, uint32_t index) {
  const float rx = cpRotate(PermHalton_sample5(T, index), B.rx0);
  const float ry = cpRotate(PermHalton_sample7(T, index), B.ry0);
  const float phi = fmul(6.283185307179586f, rx);
  const float cosT = fsqrt(ry), sinT = fsqrt(fsub(1.f, ry));
  float sp, cp;
  sincosf(phi, &sp, &cp);
  return toWorld(B.dx, B.dy, Ns, mk(fmul(cp, sinT), fmul(sp, sinT), cosT));
}


struct PixelOut {
  float r, g, b, a;
  float z;
  uint32_t primID, geomID, instID;
  V3 n, al;  // normal and albedo channels (ScreenSample.normal / .albedo)
};

// FRAMEBUFFER_ACCUMULATE_VALUE's lerp, (1 - f) * old + f * new, rounded per operation
B200_D float lerpAcc(float f, float o, float v) { return fadd(fmul(fsub(1.f, f), o), fmul(f, v)); }

B200_D void fbAccumulate(const FrameD &fb, int x, int y, const PixelOut &s) {
  const size_t i = size_t(y) * fb.W + x;
  const float accScale = fdiv(1.f, float(fb.frameID + 1));
  float4 c = make_float4(s.r, s.g, s.b, s.a);
  if (fb.color) {
    if (!(accScale > 0.8f)) {
      const float4 o = fb.color[i];
      const float k = fsub(1.f, accScale);
      c.x = fadd(fmul(k, o.x), fmul(accScale, c.x));
      c.y = fadd(fmul(k, o.y), fmul(accScale, c.y));
      c.z = fadd(fmul(k, o.z), fmul(accScale, c.z));
      c.w = fadd(fmul(k, o.w), fmul(accScale, c.w));
    }
    fb.color[i] = c;
  }
  if (fb.variance && fb.accumVariance) {
    const float vs = fdiv(1.f, float(fb.frameID / 2 + 1));
    float4 v = make_float4(s.r, s.g, s.b, s.a);
    if (!(vs > 0.8f)) {
      const float4 o = fb.variance[i];
      const float k = fsub(1.f, vs);
      v.x = fadd(fmul(k, o.x), fmul(vs, v.x));
      v.y = fadd(fmul(k, o.y), fmul(vs, v.y));
      v.z = fadd(fmul(k, o.z), fmul(vs, v.z));
      v.w = fadd(fmul(k, o.w), fmul(vs, v.w));
    }
    fb.variance[i] = v;
  }
  if (fb.normal) {
    const float3 o = fb.normal[i];
    fb.normal[i] = accScale > 0.8f ? make_float3(s.n.x, s.n.y, s.n.z)
                                   : make_float3(lerpAcc(accScale, o.x, s.n.x), lerpAcc(accScale, o.y, s.n.y),
                                                 lerpAcc(accScale, o.z, s.n.z));
  }
  if (fb.albedo) {
    const float3 o = fb.albedo[i];
    fb.albedo[i] = accScale > 0.8f ? make_float3(s.al.x, s.al.y, s.al.z)
                                   : make_float3(lerpAcc(accScale, o.x, s.al.x), lerpAcc(accScale, o.y, s.al.y),
                                                 lerpAcc(accScale, o.z, s.al.z));
  }
  bool upd = fb.frameID == 0;
  if (fb.depth) {
    if (fb.frameID > 0 && fabsf(s.z) < fabsf(fb.depth[i])) upd = true;
    if (upd) fb.depth[i] = s.z;
  }
  if (upd) {
    if (fb.primID) fb.primID[i] = s.primID;
    if (fb.geomID) fb.geomID[i] = s.geomID;
    if (fb.instID) fb.instID[i] = s.instID;
  }
}

}  // namespace b200
