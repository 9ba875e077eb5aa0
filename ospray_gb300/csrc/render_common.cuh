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
  // shutter after Camera::commit (rolling: upper reduced by the duration,
  // swapped for the left / down types); mode 0 global, 1 rolling along
  // screen x, 2 rolling along screen y; needTime: the path tracer draws a
  // time sample
  float shutterLo, shutterHi, rollingDuration;
  int shutterMode, needTime;
  // perspective: lens radius over the image plane (0: pinhole; the frame is
  // then prescaled to the focal plane), aspect, image-plane height
  float scaledAperture, aspect, imgPlaneY;
  // the sub-image ("imageStart" / "imageEnd", Camera::commit
  // camera/Camera.cpp:42-43,108-109): screen positions map to
  // (1 - s) lo + s hi
  float subLoX, subLoY, subHiX, subHiY;
  // stereo: split 0 none, 1 side by side (screen x), 2 top / bottom (screen
  // y); monoEye the fixed eye of a panoramic left (-1) / right (+1) camera
  // (a perspective one has it folded into org); ipdOffset half the
  // interpupillary distance, perspective along the film's x axis, panoramic
  // in x, negated for top / bottom; coneScale |imageEnd.y - imageStart.y|,
  // doubled for top / bottom
  int split;
  float monoEye;
  V3 ipdOffset;
  float coneScale;
};

// The stereo split and Camera_subRegion (PerspectiveCamera.ispc:28-41,
// PanoramicCamera.ispc:24-45, Camera.ih:28-31): maps the screen position
// (sx, sy) of a sample of the pixel with centre (cx, cy) in place and
// returns its eye (-1 left, +1 right, 0 mono)
B200_D float cameraScreen(const CameraD &c, float &sx, float &sy, float cx, float cy) {
  float eye = c.monoEye;
  if (c.split) {
    float &s = c.split == 1 ? sx : sy;
    s = fmul(s, 2.f);
    if ((c.split == 1 ? cx : cy) < 0.5f) {
      eye = -1.f;
    } else {
      eye = 1.f;
      s = fsub(s, 1.f);
    }
  }
  sx = fadd(fmul(fsub(1.f, sx), c.subLoX), fmul(sx, c.subHiX));
  sy = fadd(fmul(fsub(1.f, sy), c.subLoY), fmul(sy, c.subHiY));
  return eye;
}

// Camera_shutterTime (camera/Camera.ih:33-42): the ray time of a camera
// sample with time sample `time` at screen position (sx, sy); rkcommon's
// lerp(f, a, b) = (1 - f) a + f b
B200_D float shutterTime(const CameraD &c, float sx, float sy, float time) {
  if (c.shutterMode == 0) return fadd(fmul(fsub(1.f, time), c.shutterLo), fmul(time, c.shutterHi));
  const float t = fmul(time, c.rollingDuration);
  const float pos = c.shutterMode == 1 ? sx : sy;
  const float v = fadd(t, fadd(fmul(fsub(1.f, pos), c.shutterLo), fmul(pos, c.shutterHi)));
  return fminf(fmaxf(v, 0.f), 1.f);
}

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

// lens: the lens sample (PerspectiveCamera_initRay, camera/PerspectiveCamera.ispc:44-52:
// uniformSampleDisk over scaledAperture, the offset along du and aspect x dv)
// (sx, sy): the mapped screen position (cameraScreen); eye: its eye
B200_D Ray cameraRay(const CameraD &c, float sx, float sy, float2 lens = make_float2(0.f, 0.f), float eye = 0.f) {
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
    r.dir = add(add(mul(c.du_size, -l.y), mul(c.dv_up, -l.z)), mul(c.dir_00, l.x));
    // stereo: the eye's offset across the view direction (frame.vy = dv_up)
    r.org = eye != 0.f ? add(c.org, mul(fmul(eye, c.ipdOffset.x), cross(r.dir, c.dv_up))) : c.org;
    return r;
  }
  V3 d = add(add(c.dir_00, mul(sx, c.du_size)), mul(sy, c.dv_up));
  r.org = eye < 0.f ? sub(c.org, c.ipdOffset) : eye > 0.f ? add(c.org, c.ipdOffset) : c.org;
  if (c.scaledAperture > 0.f) {
    const float rr = fmul(sqrtf(lens.x), c.scaledAperture);
    float sp, cp;
    sincosf(fmul(6.28318530717958647692f, lens.y), &sp, &cp);
    const V3 lp = add(mul(fmul(rr, cp), c.du_size), mul(fmul(fmul(rr, sp), c.aspect), c.dv_up));
    r.org = add(r.org, lp);
    d = sub(d, lp);
  }
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
                      uint32_t sid, float2 *screen = nullptr) {
  const float ps_x = Halton_sample2(sid);
  const float ps_y = cpRotate(Halton_sample3(T, sid), 1.f / 6.f);
  const float2 pfs = filterSample(pf, ps_x, ps_y);
  const float cx = fmul(fadd(float(x), 0.5f), rcpW), cy = fmul(fadd(float(y), 0.5f), rcpH);
  float sx = fadd(cx, fmul(pfs.x, rcpW)), sy = fadd(cy, fmul(pfs.y, rcpH));
  const float eye = cameraScreen(cam, sx, sy, cx, cy);
  if (screen) *screen = make_float2(sx, sy);  // mapped: shutter time and ray cone
  return cameraRay(cam, sx, sy, make_float2(0.f, 0.f), eye);
}

// The camera ray's cone at screen position (sx, sy), in units of the frame
// height (PathTracer.ispc:186-187): perspective 0 wide, widening by the
// image plane height x rsqrt(|unnormalised direction|^2)
// (PerspectiveCamera.ispc:58-63); orthographic as wide as the image height,
// parallel (OrthographicCamera.ispc:52-53); panoramic pi sin(theta)
// (PanoramicCamera.ispc:86-90); all scaled by the sub-image height, twice
// that for top / bottom stereo.  (sx, sy): the mapped screen position.
B200_D float2 cameraCone(const CameraD &c, float sx, float sy, float rcpH) {
  if (c.type == 1) return make_float2(sqrtf(dot(c.dv_up, c.dv_up)) * c.coneScale * rcpH, 0.f);
  if (c.type == 2)
    return make_float2(0.f, 3.14159265358979323846f * sinf(3.14159265358979323846f * sy) * c.coneScale * rcpH);
  const V3 d = add(add(c.dir_00, mul(sx, c.du_size)), mul(sy, c.dv_up));
  return make_float2(0.f, c.imgPlaneY * c.coneScale * rsqrtf(dot(d, d)) * rcpH);
}


struct DG {
  V3 P, Ng, Ns;
  V3 dPds;  // surface tangent (DG_TANGENTS): the triangle's first edge, else (1, 0, 0), in world space
  float epsilon;
  uint32_t entry;
};

// What the path tracer's materials read beyond DG (DG_COLOR, DG_TEXCOORD and
// the second tangent of DG_TANGENTS): the interpolated vertex colour (1 when
// the mesh has none), the texture coordinates (the hit's u, v when the mesh
// has none, World.ih postIntersect) and dPdt, in world space.
// The hit's barycentric u, v are recomputed here from the hit point rather
// than carried from traversal (the closest-hit kernel stays as small as it
// is): triangles (a, b, c) give P = a + u (b - a) + v (c - a); quads
// (v0, v1, v2, v3) the same over (v0, v1, v3), which is the quad's bilinear
// (u, v) for a parallelogram; spheres and boxes 0.
struct DGAttr {
  float4 color;
  float s, t;
  V3 dPdt;
};

// (u, v) with P = a + u (b - a) + v (c - a) for the hit at distance t, in the
// entry's object space: least squares over the plane of (a, b, c)
B200_D float2 hitBarycentrics(bool identity, const Xfm &R, const Ray &ray, float t, V3 a, V3 b, V3 c) {
  V3 P = add(ray.org, mul(t, ray.dir));
  if (!identity) P = xfmPoint(R, P);
  const V3 e1 = sub(b, a), e2 = sub(c, a), d = sub(P, a);
  const float d11 = dot(e1, e1), d12 = dot(e1, e2), d22 = dot(e2, e2);
  const float r1 = dot(d, e1), r2 = dot(d, e2);
  const float det = d11 * d22 - d12 * d12;
  if (!(det > 0.f)) return make_float2(0.f, 0.f);
  const float inv = 1.f / det;
  return make_float2((d22 * r1 - d12 * r2) * inv, (d11 * r2 - d12 * r1) * inv);
}

// postIntersect with DG_NG | DG_NS | DG_NORMALIZE | DG_FACEFORWARD (and with
// ATTR also DG_COLOR | DG_TEXCOORD and the mesh's vertex normals:
// TriangleMesh_postIntersect geometry/Mesh.ispc:178-276)
//
// MOTION: the entry is motion-blurred, its transform taken at the ray's time
// (Instance_postIntersect, common/Instance.ih:57-91, with Embree's
// interpolated transform).
template <bool ATTR, bool MOTION>
B200_D DG postIntersectT(const Entry &e, const Ray &ray, const HitRec &hit, DGAttr *at, float time) {
  DG dg;
  dg.entry = hit.entry;
  Xfm mx, mr;
  float mEps = 0.f;
  if (MOTION) {
    mx = motionXfm(e.motionKeys, e.motionCount, e.motionT0, e.motionT1, time);
    mr = rcpXfm(mx);
    mEps = fmaxf(fabsf(mx.m[0]), fmaxf(fabsf(mx.m[5]), fabsf(mx.m[10])));
  }
  const Xfm &X = MOTION ? mx : e.xfm;
  const Xfm &R = MOTION ? mr : e.rcp;
  const bool identity = !MOTION && e.identity;
  dg.P = add(ray.org, mul(hit.t, ray.dir));
  V3 Ng = hit.Ng, Ns = hit.Ng;
  // DG_TANGENTS: meshes take their first edge (TriangleMesh_postIntersect
  // geometry/Mesh.ispc:172-175, QuadMesh_postIntersect :171-174), other
  // geometry keeps the default (1, 0, 0) (World.ih postIntersect)
  V3 dPds = mk(1.f, 0.f, 0.f), dPdt = mk(0.f, 1.f, 0.f);
  if (ATTR) {
    at->color = make_float4(1.f, 1.f, 1.f, 1.f);
    at->s = at->t = 0.f;
  }
  float eps;
  if (e.type == GEOM_TRIANGLES && e.meshKind == MESH_BOXES) {
    eps = 0.f;  // Boxes_postIntersect (geometry/Boxes.ispc) sets no geometry epsilon
  } else if (e.type == GEOM_TRIANGLES && e.meshKind == MESH_QUADS) {
    // QuadMesh_postIntersect (geometry/Mesh.ispc:67-176): epsilon over the 4 vertices
    const uint4 q = __ldg(reinterpret_cast<const uint4 *>(e.index) + hit.primID);
    const uint32_t ix[4] = {q.x, q.y, q.z, q.w};
    V3 m = splat(0.f), v[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const V3 p = mk(__ldg(e.verts + 3 * ix[k]), __ldg(e.verts + 3 * ix[k] + 1), __ldg(e.verts + 3 * ix[k] + 2));
      v[k] = p;
      m = vmax(m, vabs(p));
    }
    eps = fmul(reduce_max(m), ULP_EPSILON);
    dPds = sub(v[1], v[0]);
    if (ATTR) {
      dPdt = sub(v[3], v[0]);
      const float2 uv = hitBarycentrics(identity, R, ray, hit.t, v[0], v[1], v[3]);
      at->s = uv.x;
      at->t = uv.y;
    }
  } else if (e.type == GEOM_TRIANGLES) {
    const uint32_t i0 = __ldg(e.index + 3 * hit.primID), i1 = __ldg(e.index + 3 * hit.primID + 1),
                   i2 = __ldg(e.index + 3 * hit.primID + 2);
    const V3 a = mk(__ldg(e.verts + 3 * i0), __ldg(e.verts + 3 * i0 + 1), __ldg(e.verts + 3 * i0 + 2));
    const V3 b = mk(__ldg(e.verts + 3 * i1), __ldg(e.verts + 3 * i1 + 1), __ldg(e.verts + 3 * i1 + 2));
    const V3 c = mk(__ldg(e.verts + 3 * i2), __ldg(e.verts + 3 * i2 + 1), __ldg(e.verts + 3 * i2 + 2));
    eps = fmul(reduce_max(vmax(vmax(vabs(a), vabs(b)), vabs(c))), ULP_EPSILON);
    dPds = sub(b, a);
    if (ATTR) {
      dPdt = sub(c, a);
      // barycentric weights (1 - u - v, u, v) of vertices (i0, i1, i2)
      const float2 uv = hitBarycentrics(identity, R, ray, hit.t, a, b, c);
      at->s = uv.x;
      at->t = uv.y;
      const float w0 = 1.f - uv.x - uv.y, w1 = uv.x, w2 = uv.y;
      if (e.normals) {
        const float *n = e.normals;
        Ns = mk(w0 * __ldg(n + 3 * i0) + w1 * __ldg(n + 3 * i1) + w2 * __ldg(n + 3 * i2),
                w0 * __ldg(n + 3 * i0 + 1) + w1 * __ldg(n + 3 * i1 + 1) + w2 * __ldg(n + 3 * i2 + 1),
                w0 * __ldg(n + 3 * i0 + 2) + w1 * __ldg(n + 3 * i1 + 2) + w2 * __ldg(n + 3 * i2 + 2));
      }
      if (e.colors) {
        const float4 *cl = reinterpret_cast<const float4 *>(e.colors);
        const float4 c0 = __ldg(cl + i0), c1 = __ldg(cl + i1), c2 = __ldg(cl + i2);
        at->color = make_float4(w0 * c0.x + w1 * c1.x + w2 * c2.x, w0 * c0.y + w1 * c1.y + w2 * c2.y,
                                w0 * c0.z + w1 * c1.z + w2 * c2.z, w0 * c0.w + w1 * c1.w + w2 * c2.w);
      }
      if (e.texcoords) {
        const float2 *tc = reinterpret_cast<const float2 *>(e.texcoords);
        const float2 t0 = __ldg(tc + i0), t1 = __ldg(tc + i1), t2 = __ldg(tc + i2);
        at->s = w0 * t0.x + w1 * t1.x + w2 * t2.x;
        at->t = w0 * t0.y + w1 * t1.y + w2 * t2.y;
        // tangents along the texture axes where the texture map is not degenerate
        const float ds02 = t0.x - t2.x, dt02 = t0.y - t2.y, ds12 = t1.x - t2.x, dt12 = t1.y - t2.y;
        const float det = ds02 * dt12 - dt02 * ds12;
        if (det != 0.f) {
          const float inv = 1.f / det;
          const V3 dp02 = sub(a, c), dp12 = sub(b, c);
          dPds = mul(sub(mul(dt12, dp02), mul(dt02, dp12)), inv);
          dPdt = mul(sub(mul(ds02, dp12), mul(ds12, dp02)), inv);
        }
      }
    }
  } else if (e.type == GEOM_PLANES) {
    eps = 0.f;  // Planes_postIntersect (geometry/Planes.ispc:115-121) sets no geometry epsilon
  } else {
    // Spheres_postIntersect (geometry/Spheres.ispc:24-42): radius x ulpEpsilon, also for discs
    eps = fmul(__ldg(&e.spheres[hit.primID].w), ULP_EPSILON);
  }
  if (!identity) {
    Ns = xfmVectorT(R, Ns);
    Ng = xfmVectorT(R, Ng);
    eps = fmul(eps, MOTION ? mEps : e.epsScale);
    dPds = xfmVector(X, dPds);  // Instance_postIntersect (common/Instance.ih:95-98)
    if (ATTR) dPdt = xfmVector(X, dPdt);
  }
  dg.dPds = dPds;
  if (ATTR) at->dPdt = dPdt;
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

// the motion-blurred case out of line (the shading kernels keep their
// registers); a hit the wavefront trace kernels left unevaluated
// (Traverser::finish with DEFER; `slot` its leaf slot) is re-evaluated here
// first
template <bool ATTR>
static __device__ __noinline__ DG postIntersectMotion(const Entry &e, Ray ray, HitRec hit, DGAttr *at, float time,
                                                      uint32_t slot) {
  if (slot != INVALID_ID) {
    const HitSurface f = finishMotion(e, time, ray, hit.t, slot);
    hit.u = f.u;
    hit.v = f.v;
    hit.Ng = f.Ng;
  }
  return postIntersectT<ATTR, true>(e, ray, hit, at, time);
}

// postIntersect at the ray's `time` (motion-blurred instances only; a
// negative time: the scene's); deferredSlot: the leaf slot of a hit whose
// motion-blurred evaluation the trace kernel deferred
template <bool ATTR = false, bool MOTION = true>
B200_D DG postIntersect(const Scene &sc, const Ray &ray, const HitRec &hit, DGAttr *at = nullptr, float time = -1.f,
                        uint32_t deferredSlot = INVALID_ID) {
  const Entry &e = sc.entries[hit.entry];
  if (MOTION && sc.hasUser && e.motionCount > 1)
    return postIntersectMotion<ATTR>(e, ray, hit, at, time >= 0.f ? time : sc.time, deferredSlot);
  return postIntersectT<ATTR, false>(e, ray, hit, at, time);
}

// the pixel footprint of a hit for texture level selection (World.ih
// postIntersect: the ray cone's width projected onto the surface, in texture
// space, times 2^mipMapBias); coneWidth: the cone's width at the hit
B200_D float pixelFootprint(float coneWidth, V3 rayDir, const DG &dg, const DGAttr &at, float mipBias) {
  const V3 x = cross(dg.dPds, at.dPdt);
  const float texArea = sqrtf(dot(x, x));
  return coneWidth / -dot(rayDir, dg.Ng) * (1.f / sqrtf(texArea)) * mipBias;
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
