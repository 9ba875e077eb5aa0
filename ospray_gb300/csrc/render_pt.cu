// Path tracer as a wavefront over device-side path queues, for one frame
// (launchRenderPT) or a batch of many requests (launchBatchWave), following
//   PathTracer_renderPixel  render/pathtracer/PathTracer.ispc:75-216
//   samplePath              render/pathtracer/PathSampler.ispc:109-415
//   nextEventEstimation     render/pathtracer/NextEventEstimation.ispc:25-160
//   evaluateVirtualLights   render/pathtracer/VirtualLight.ispc:38-107
//   transparentShadow       render/pathtracer/TransparentShadow.ispc:18-85
//     (scenes whose materials are all opaque trace shadow rays as any-hit queries)
//   ray cones               common/World.ih:458-464 (postIntersect), camera
//                           initRay (camera/*Camera.ispc), PathTracer.ispc:186-187
//   misHeuristic            render/pathtracer/PathTracerUtil.ih:30-46
// and, for AO requests of a batch, AORenderer_renderSample
// (render/ao/AORenderer.ispc:23-149) with its AO rays in the shadow queue.
#include <algorithm>
#include <cstring>
#include <stdexcept>

#include "kernels.h"
#include "lights.cuh"
#include "pt_bsdf.cuh"

namespace b200 {

namespace {

struct PtCtx {
  const SamplerTables *T;
  Scene sc;
  PtParamsD p;
  const MaterialD *mats;
  const LightD *lights;
  const float *lightCdf;
  const AlbedoTablesD *AT;
  int frameID;
  float *aux;  // per pixel: sums of the first vertices' normal and albedo (null: not wanted)
  int W;       // single frames: framebuffer width and reciprocal size (backplate lookups)
  float rcpW, rcpH;
};

struct PathResult {
  V3 rgb;
  float alpha, z;
  uint32_t primID, geomID, instID;
};

// ---------------------------------------------------------------- wavefront path tracer
// A frame's paths (pixel x sample) live in a workspace of 128-byte records.
// Each bounce runs three kernels over queues of path indices: a persistent
// closest-hit trace of the extension rays, a shading kernel (the body of
// samplePath's loop) that appends shadow rays and continuing paths to new
// queues, and a persistent any-hit trace of the shadow rays, whose unblocked
// contributions are added to their paths.  A final kernel averages each
// pixel's samples into the framebuffer.  Queue lengths stay on the device,
// so a frame is a fixed sequence of launches (graph-capturable).

struct __align__(16) PathRec {
  float4 org;   // ray origin, first-hit depth z
  float4 dir;   // ray direction, last vertex BSDF pdf
  float4 thr;   // throughput, alpha
  float4 con;   // contribution, medium id (bits)
  float4 lastP; // previous vertex position, tnear of the next ray
  float4 lastN; // previous vertex shading normal, ray cone width at the last hit (at the camera before)
  uint4 meta;   // LDSampler scramble, flags, first-hit primID, geomID
  uint4 meta2;  // first-hit instID, request (batch) / ray cone dwdt bits (single frame), sampleID,
                // pixel / radiance-cache training slot
};
static_assert(sizeof(PathRec) == 128, "PathRec must be 128 bytes");

struct __align__(16) HitBuf {
  float4 a;  // t, primID bits, entry bits, hit flag
  float4 b;  // unnormalised object-space Ng
};

struct __align__(16) ShadowRec {
  float4 a;  // origin, tfar
  float4 b;  // direction, path index bits
  float4 c;  // contribution if unblocked, (unused)
};

// flags: depth 0..7, straightPath bit 8, firstBounceLight bit 9, ended bit 10,
// (11, 12 below), auxiliary data recorded bit 13, scattering events 14..20,
// lastNLS 21..31
constexpr uint32_t F_STRAIGHT = 1u << 8, F_FIRST = 1u << 9, F_ENDED = 1u << 10, F_AUXDONE = 1u << 13;
constexpr int F_SCATTER_SHIFT = 14, F_NLS_SHIFT = 21;
constexpr uint32_t F_SCATTER_MAX = 127u, F_NLS_MAX = 2047u;

struct Workspace {
  PathRec *paths;
  HitBuf *hits;
  uint32_t *qa, *qb;  // path queues
  ShadowRec *shadows;
  // a bounce's misses (k_partition), in the last 4 bytes per path of the
  // shadow records' space: a bounce's shading writes at most 2 records per
  // hit, so with n paths of which m miss, the records end at 96 (n - m)
  // bytes and the misses start at 92 npaths + 4 (n - m) bytes, never below
  uint32_t *misses;
  // each path's ray time (scenes with motion-blurred instances; else null)
  float *times;
  // [0] qa count, [1] qb count, [2] shadow count, [3] closest fetch, [4]
  // shadow fetch, [5..7] partition part sizes
  uint32_t *counters;
};

struct FrameInfo {
  int W, H, spp, frameID;
  float rcpW, rcpH;
  long long npaths;
};

// a request of a batch, as the kernels read it (device table)
struct ReqD {
  PtCtx c;
  CameraD cam;
  PixelFilterD pf;
  FrameInfo fi;
  FrameD fb;
  AOParamsD ao;
  int kind;
};

// a run of path slots of one wave that belongs to one request
struct SegD {
  long long start;     // first path slot in the wave
  long long first;     // first path of the request (pixel-major)
  long long pixStart;  // first pixel slot in the wave
  int rid, pad;
};

// path flags: AO request hit its first surface; the path bounced off a
// diffuse surface (radiance-cache mode)
constexpr uint32_t F_AOHIT = 1u << 11, F_DIFFUSE = 1u << 12;

// the camera ray of sample s of pixel (x, y) of a path-traced frame, as a
// fresh path record (meta2: first-hit instID, request, sampleID, pixel)
B200_D PathRec genPT(const PtCtx &c, const CameraD &cam, const PixelFilterD &pf, const FrameInfo &fi, int x, int y,
                     int s, uint32_t rid, float2 *screen = nullptr, float *time = nullptr) {
  const uint32_t seed = 0x49c5f37eu ^ uint32_t(fi.W * y + x);
  const uint32_t sampleID = uint32_t(fi.frameID) * uint32_t(fi.spp) + uint32_t(s);
  LDSampler ld;
  ld.init(c.T, seed, sampleID, sampleID * uint32_t(c.p.nFirst), 16, 16);
  uint32_t ss234[3];
  const float2 ps = ld.getNext5Samples(ss234);
  const float2 pfs = filterSample(pf, ps.x, ps.y);
  const float cx = fmul(fadd(float(x), 0.5f), fi.rcpW), cy = fmul(fadd(float(y), 0.5f), fi.rcpH);
  const float sx = fadd(cx, fmul(pfs.x, fi.rcpW)), sy = fadd(cy, fmul(pfs.y, fi.rcpH));
  if (screen) *screen = make_float2(sx, sy);  // unmapped: Renderer_getMaxDepth (PathTracer.ispc:189-190)
  float mx = sx, my = sy;
  const float eye = cameraScreen(cam, mx, my, cx, cy);
  // the lens sample (PathTracer.ispc:172-175): from the sample stream when
  // the camera has an aperture
  const Ray ray = cameraRay(cam, mx, my, cam.scaledAperture > 0.f ? ld.finalizeDim23(ss234) : make_float2(0.5f, 0.5f),
                            eye);
  if (screen) screen[1] = make_float2(mx, my);
  // the camera sample's time (PathTracer.ispc:177-180, Camera_shutterTime)
  if (time) *time = shutterTime(cam, mx, my, cam.needTime ? ld.finalizeDim4(ss234) : 0.5f);
  PathRec r;
  r.org = make_float4(ray.org.x, ray.org.y, ray.org.z, INFINITY);
  r.dir = make_float4(ray.dir.x, ray.dir.y, ray.dir.z, INFINITY);
  r.thr = make_float4(1.f, 1.f, 1.f, 1.f);
  r.con = make_float4(0.f, 0.f, 0.f, __uint_as_float(MEDIUM_VACUUM));  // w: the medium the path travels in
  r.lastP = make_float4(ray.org.x, ray.org.y, ray.org.z, ray.tnear);
  r.lastN = make_float4(ray.dir.x, ray.dir.y, ray.dir.z, 0.f);
  r.meta = make_uint4(ld.scramble, F_STRAIGHT | F_FIRST, INVALID_ID, INVALID_ID);
  r.meta2 = make_uint4(INVALID_ID, rid, sampleID, uint32_t(fi.W * y + x));
  return r;
}

// appends one entry per lane that wants to, with one atomic per warp
B200_D uint32_t warpAppend(bool want, uint32_t *counter) {
  const unsigned m = __ballot_sync(__activemask(), want);
  if (!m) return 0;
  const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(counter, uint32_t(__popc(m)));
  base = __shfl_sync(__activemask(), base, leader);
  return base + uint32_t(__popc(m & ((1u << lane) - 1u)));
}

// nrcStride > 0: the radiance-cache training paths of this frame get their
// slot in meta2.w (INVALID_ID for the others)
//
// Adaptive accumulation (fb.taskActive set): only the paths of pixels in
// selected tasks are generated, appended to queue `active` (counted in
// ws.counters[0], zeroed beforehand); the first bounce then reads that queue.
__global__ void k_pt_generate(PtCtx c, CameraD cam, PixelFilterD pf, FrameInfo fi, Workspace ws, uint32_t nrcStride,
                              uint32_t nrcOffset, uint32_t nrcSlots, FrameD fb, uint32_t *active) {
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p == 0 && !active) {
    ws.counters[0] = uint32_t(fi.npaths);
    for (int k = 1; k < 16; k++) ws.counters[k] = 0;
  }
  const int pix = int(p / fi.spp), s = int(p % fi.spp);
  const bool live = p < fi.npaths && (!active || pixelActive(fb, pix % fi.W, pix / fi.W));
  if (active) {
    const uint32_t slot = warpAppend(live, ws.counters);
    if (live) active[slot] = uint32_t(p);
  }
  if (!live) return;
  float2 scr[2];  // the sample's screen position, unmapped and mapped
  float time;
  PathRec r = genPT(c, cam, pf, fi, pix % fi.W, pix / fi.W, s, 0u, scr, ws.times ? &time : nullptr);
  if (ws.times) ws.times[p] = time;
  // Renderer_getMaxDepth at the sample's screen position (PathTracer.ispc:189-192):
  // the camera ray's tfar, carried in org.w until the first hit sets the depth there
  if (c.p.maxDepth) r.org.w = texMaxDepth(c.p.maxDepth, scr[0].x, scr[0].y);
  const float2 cone = cameraCone(cam, scr[1].x, scr[1].y, fi.rcpH);
  r.lastN.w = cone.x;
  r.meta2.y = __float_as_uint(cone.y);
  if (nrcStride) {
    const uint32_t k = uint32_t(p) + nrcOffset;
    r.meta2.w = (k % nrcStride == 0 && k / nrcStride < nrcSlots) ? k / nrcStride : INVALID_ID;
  }
  ws.paths[p] = r;
}

// What the transparent-shadow trace needs of the materials
// (TransparentShadow.ispc:18-85): the material list, the renderer's
// minContribution and its maxPathLength as the limit of surfaces crossed.
struct ShadowMatD {
  const MaterialD *mats;
  int nmats, maxDepth;
  float minContribution;
  float mipBiasFactor;
};

// Persistent any/closest-hit tracing over a queue with per-lane dynamic
// fetch: whenever lanes of a warp finish their rays, the warp takes that many
// new ones with one atomic, so no lane idles while work remains.
// In a batch (BATCH) every ray traverses its own request's scene.
// TRANSP (shadow rays of scenes with transparent materials): each shadow ray
// is a loop of closest-hit queries; at every hit its contribution is
// multiplied by the material's transparency (and the medium's attenuation
// over the segment), and the lane restarts the same ray just past the hit,
// until it reaches the light or is blocked.  The shadow record's fourth
// contribution word then carries the path's medium (tnear is 0).
#ifndef B200_REFILL_LANES
#define B200_REFILL_LANES 8
#endif
#ifndef B200_TRACE_CARVEOUT
#define B200_TRACE_CARVEOUT -1
#endif
#ifndef B200_SHADE_CARVEOUT
#define B200_SHADE_CARVEOUT -1
#endif
// the same threshold for the shadow (any-hit) instantiations (4: 1,050, 8:
// 1,051, 16: 1,035 Mrays/s with the closest-hit threshold at 8)
#ifndef B200_REFILL_LANES_SHADOW
#define B200_REFILL_LANES_SHADOW B200_REFILL_LANES
#endif

// The body is a device function so that the persistent batch kernel runs it
// as one of its stages; a batch reads its queue with coherent loads (in the
// persistent kernel the queue was written earlier in the same launch).
template <bool SHADOW, bool STATS, bool BATCH, bool TRANSP = false, bool USER = true>
__device__ __forceinline__ void traceQueue(Scene sc, Workspace ws, const uint32_t *queue, const uint32_t *count,
                                           uint32_t *fetch, const ReqD *reqs, ShadowMatD sm) {
  static_assert(!(BATCH && STATS), "batched traversal keeps no per-scene statistics");
  static_assert(!TRANSP || (SHADOW && !BATCH), "transparent shadows: single-request shadow rays only");
  const int lane = threadIdx.x & 31;
  const uint32_t n = *(volatile const uint32_t *)count;
  TraceStats ts = {0, 0, 0, 0};
  Scene bsc = sc;  // this lane's scene in a batch
  const Scene &S = BATCH ? bsc : sc;
  Traverser tv;
  TraceSpill spill;
  if (USER) spill.time = 0.f;
  bool has = false, exhausted = false;
  uint32_t item = 0;
  // transparent shadows: the ray, its remaining contribution, medium and crossing budget
  Ray tray;
  V3 tcon = splat(0.f);
  uint32_t tmed = MEDIUM_VACUUM;
  int tdepth = 0;
  float tcone = 0.f;  // the path's ray cone width at the shadow ray's origin
  for (int guard = 0; guard < (1 << 30); guard++) {
    // refill once at least B200_REFILL_LANES lanes wait (or no lane has a
    // ray left), so the warp does not stop for every lane that finishes
    const unsigned need = __ballot_sync(0xffffffffu, !has && !exhausted);
    if (need && (__popc(need) >= (SHADOW ? B200_REFILL_LANES_SHADOW : B200_REFILL_LANES) ||
                 !__any_sync(0xffffffffu, has))) {
      const int leader = __ffs(need) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(fetch, uint32_t(__popc(need)));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (!has && !exhausted) {
        const uint32_t idx = base + uint32_t(__popc(need & ((1u << lane) - 1u)));
        if (idx < n) {
          Ray r;
          if (SHADOW) {
            // a shadow queue, when given, holds record indices
            item = queue ? (BATCH ? queue[idx] : __ldg(queue + idx)) : idx;
            const ShadowRec s = ws.shadows[item];
            r.org = mk(s.a.x, s.a.y, s.a.z);
            r.tnear = TRANSP ? 0.f : s.c.w;
            r.dir = mk(s.b.x, s.b.y, s.b.z);
            r.tfar = s.a.w;
            if (TRANSP) {
              tray = r;
              tcon = mk(s.c.x, s.c.y, s.c.z);
              tmed = __float_as_uint(s.c.w);
              tdepth = sm.maxDepth;
              tcone = ws.paths[__float_as_uint(s.b.w)].lastN.w;
            }
            if (BATCH) bsc = reqs[ws.paths[__float_as_uint(s.b.w)].meta2.y].c.sc;
            if (USER && !BATCH && ws.times) spill.time = ws.times[__float_as_uint(s.b.w)];
          } else {
            item = queue ? (BATCH ? queue[idx] : __ldg(queue + idx)) : idx;
            const float4 o = ws.paths[item].org, d = ws.paths[item].dir;
            r.org = mk(o.x, o.y, o.z);
            r.tnear = ws.paths[item].lastP.w;  // camera rays: nearClip; bounces: 0
            r.dir = mk(d.x, d.y, d.z);
            // camera rays: the maxDepth limit in org.w (infinite without one)
            r.tfar = (ws.paths[item].meta.y & 0xffu) == 0u ? o.w : INFINITY;
            if (BATCH) bsc = reqs[ws.paths[item].meta2.y].c.sc;
            if (USER && !BATCH && ws.times) spill.time = ws.times[item];
          }
          tv.init(S, r, SHADOW && !TRANSP, &spill);
          if (STATS) ts.rays++;
          has = true;
        } else {
          exhausted = true;
        }
      }
    }
    if (!__any_sync(0xffffffffu, has)) break;
    // the batch keeps whole primitive groups per step (its height-field
    // scenes: 1,505 vs 1,469 Mrays/s with one test per step)
    if (has && tv.step<STATS, USER, BATCH ? B200_PRIMS_PER_STEP : B200_QUEUE_PRIMS_PER_STEP,
                       BATCH ? B200_POSTPONE_LANES : B200_QUEUE_POSTPONE_LANES>(S, &ts)) {
      if (TRANSP) {
        bool done = true;
        if (!tv.found) {
          float *con = &ws.paths[__float_as_uint(ws.shadows[item].b.w)].con.x;
          atomicAdd(con + 0, tcon.x);
          atomicAdd(con + 1, tcon.y);
          atomicAdd(con + 2, tcon.z);
        } else {
          tv.finish<true, true>(S);
          DGAttr at;
          const DG dg = postIntersect<true>(S, tray, tv.hit, &at, spill.time, tv.hslot);
          const uint32_t mi = S.entries[tv.hit.entry].materialID;
          const bool hasMat = mi < uint32_t(sm.nmats);
          // the shadow cone narrows from the path's width to 0 at the light
          // (NextEventEstimation.ispc:103-106), re-widened at every surface
          const float w = tcone + (-tcone * (1.f / tray.tfar)) * tv.hit.t;
          const float fp = hasMat && sm.mats[mi].map ? pixelFootprint(w, tray.dir, dg, at, sm.mipBiasFactor) : 0.f;
          tcon = tcon * (hasMat ? materialTransparency(sm.mats, mi, tray.dir, dg.Ns, tmed, at, fp) : splat(0.f));
          const MediumD md = mediumOf(sm.mats, tmed);
          if (md.att.x != 0.f || md.att.y != 0.f || md.att.z != 0.f)
            tcon = tcon * expV(md.att * (tv.hit.t - tray.tnear));
          if (!(maxc(tcon) <= sm.minContribution || --tdepth <= 0)) {
            if (hasMat && sm.mats[mi].kind == MAT_GLASS)
              tmed = glassFromOutside(sm.mats, mi, tmed) ? 2u * mi : 2u * mi + 1u;
            tray.tnear = tv.hit.t + dg.epsilon;
            tv.init(S, tray, false, &spill);  // the same ray again, past this surface
            if (STATS) ts.rays++;
            done = false;
          }
        }
        has = !done;
      } else {
        if (SHADOW) {
          if (!tv.found) {
            const ShadowRec s = ws.shadows[item];
            float *con = &ws.paths[__float_as_uint(s.b.w)].con.x;
            atomicAdd(con + 0, s.c.x);
            atomicAdd(con + 1, s.c.y);
            atomicAdd(con + 2, s.c.z);
          }
        } else {
          tv.finish<true, true>(S);
          HitBuf hb;
          hb.a = make_float4(tv.hit.t, __uint_as_float(tv.hit.primID), __uint_as_float(tv.hit.entry),
                             tv.found ? 1.f : 0.f);
          // w: the leaf slot (a deferred motion-blurred hit is re-evaluated from it)
          hb.b = make_float4(tv.hit.Ng.x, tv.hit.Ng.y, tv.hit.Ng.z, USER ? __uint_as_float(tv.hslot) : 0.f);
          ws.hits[item] = hb;
        }
        has = false;
      }
    }
  }
  if (STATS) flushStats(sc, ts);
}

// USER = false: an instantiation for scenes without discs, planes or
// motion-blurred instances (Scene::hasUser), without their code
template <bool SHADOW, bool STATS, bool BATCH, bool TRANSP = false, bool USER = true>
__global__ void __launch_bounds__(TRACE_BLOCK, BATCH ? B200_BATCH_TRACE_MINBLOCKS : B200_TRACE_MINBLOCKS)
    k_trace_queue(Scene sc, Workspace ws, const uint32_t *queue, const uint32_t *count, uint32_t *fetch,
                  const ReqD *reqs, ShadowMatD sm) {
  traceQueue<SHADOW, STATS, BATCH, TRANSP, USER>(sc, ws, queue, count, fetch, reqs, sm);
}


// The shading step of an AO request's camera sample (AORenderer_renderSample,
// render/ao/AORenderer.ispc:23-149, with computeAO render/util.ispc:12-54):
// postIntersect, the eye-light term |Ns . dir| into thr.x, and the AO rays:
// those below the surface count as occluded and are not traced, the first two
// go to the shadow queue (contribution 1 to con.x when unblocked), further
// ones are traced here.  The pixel's AO value and colour are formed at
// finalize from these integer counts, with the same arithmetic as the
// single-frame AO kernel.
B200_D void aoShade(const PtCtx &C, const AOParamsD &A, int W, PathRec &pr, const HitBuf &hb, uint32_t p,
                    ShadowRec *sh, int &nsh) {
  uint32_t flags = F_ENDED;
  float unblocked = 0.f;
  if (hb.a.w != 0.f) {
    Ray ray;
    ray.org = mk(pr.org.x, pr.org.y, pr.org.z);
    ray.tnear = pr.lastP.w;
    ray.dir = mk(pr.dir.x, pr.dir.y, pr.dir.z);
    ray.tfar = INFINITY;
    HitRec h;
    h.t = hb.a.x;
    h.primID = __float_as_uint(hb.a.y);
    h.entry = __float_as_uint(hb.a.z);
    h.Ng = mk(hb.b.x, hb.b.y, hb.b.z);
    const Entry &e = C.sc.entries[h.entry];
    h.geomID = e.geomID;
    h.instID = e.instID;
    const DG dg = postIntersect<false, false>(C.sc, ray, h);  // batches hold no motion-blurred instances
    pr.org.w = h.t;
    pr.meta.z = h.primID;
    pr.meta.w = h.geomID;
    pr.meta2.x = h.instID;
    pr.thr.x = fabsf(dot(dg.Ns, ray.dir));
    flags |= F_AOHIT;
    if (A.aoSamples > 0 && A.aoIntensity > 0.01f) {
      const uint32_t pixel = pr.meta2.w;
      const AOBasis B = aoBasis(dg, int(pixel % uint32_t(W)), int(pixel / uint32_t(W)));
      const uint32_t accumID = pr.meta2.z * uint32_t(A.aoSamples);
      for (int i = 0; i < A.aoSamples; i++) {
        const V3 dir = aoDirection(C.T, B, dg.Ns, accumID + i);
        if (dot(dir, dg.Ns) < 0.01f) continue;
        if (nsh < 2) {
          sh[nsh].a = make_float4(dg.P.x, dg.P.y, dg.P.z, A.aoRadius);
          sh[nsh].b = make_float4(dir.x, dir.y, dir.z, __uint_as_float(p));
          sh[nsh].c = make_float4(1.f, 0.f, 0.f, dg.epsilon);
          nsh++;
        } else {
          Ray r;
          r.org = dg.P;
          r.tnear = dg.epsilon;
          r.dir = dir;
          r.tfar = A.aoRadius;
          HitRec hh;
          if (!traceRay<false, false, false>(C.sc, r, hh, true, true, nullptr)) unblocked += 1.f;
        }
      }
    }
  }
  pr.con = make_float4(unblocked, 0.f, 0.f, 0.f);
  pr.meta.y = flags;
}

// The mutable state of a path between bounces (PathState,
// render/pathtracer/PathStructs.ih), unpacked from its record.
struct PathVars {
  V3 throughput, contribution;
  int depth, scatter, lastNLS;
  bool straightPath, firstBounceLight, diffuseSeen, auxDone, cont;
  uint32_t medium;
  float cone;  // ray cone width at this vertex
  float time;  // the path's ray time (motion blur; negative: none)
};

// transparentShadow (render/pathtracer/TransparentShadow.ispc:18-85) for one
// shadow ray traced in place: closest hits in turn, each multiplying the
// contribution by its material's transparency (and the medium's Beer
// attenuation over the segment), until the ray reaches tfar (unblocked) or
// the contribution drops to minContribution or maxPathLength surfaces were
// crossed.  Opaque scenes use one any-hit query.
template <bool TRANSP, bool MOTION>
B200_D V3 shadowInPlace(const PtCtx &C, Ray sr, V3 contrib, uint32_t medium, float cone, float time) {
  HitRec h;
  if (!TRANSP) return traceRay<false, false, MOTION>(C.sc, sr, h, true, true, nullptr, time) ? splat(0.f) : contrib;
  const float tfar = sr.tfar;
  int maxDepth = C.p.maxPathLength;
  for (int guard = 0; guard < 4096; guard++) {
    if (!traceRay<false, false, MOTION>(C.sc, sr, h, false, true, nullptr, time)) return contrib;
    const Entry &e = C.sc.entries[h.entry];
    h.geomID = e.geomID;
    h.instID = e.instID;
    DGAttr at;
    const DG dg = postIntersect<true, MOTION>(C.sc, sr, h, &at, time);
    const uint32_t mi = e.materialID;
    const bool hasMat = mi < uint32_t(C.p.numMaterials);
    const float w = cone + (-cone * (1.f / tfar)) * h.t;
    const float fp = hasMat && C.mats[mi].map ? pixelFootprint(w, sr.dir, dg, at, C.p.mipBiasFactor) : 0.f;
    contrib = contrib * (hasMat ? materialTransparency(C.mats, mi, sr.dir, dg.Ns, medium, at, fp) : splat(0.f));
    const MediumD md = mediumOf(C.mats, medium);
    if (md.att.x != 0.f || md.att.y != 0.f || md.att.z != 0.f) contrib = contrib * expV(md.att * (h.t - sr.tnear));
    if (maxc(contrib) <= C.p.minContribution || --maxDepth <= 0) return splat(0.f);
    if (hasMat && C.mats[mi].kind == MAT_GLASS)
      medium = glassFromOutside(C.mats, mi, medium) ? 2u * mi : 2u * mi + 1u;
    sr.tnear = h.t + dg.epsilon;
    sr.tfar = tfar;
  }
  return splat(0.f);
}

// The shading part of one samplePath iteration at a surface with BSDF `bsdf`
// (render/pathtracer/PathSampler.ispc:290-411): auxiliary data, next-event
// estimation at smooth vertices (shadow rays to the shadow queue), BSDF
// sampling with the same-side check, Russian roulette, Beer attenuation in
// the current medium, medium change on transmission, and the continuation
// ray.  A specular transmission keeps the previous vertex for MIS.
// The path record is read and written field by field (gp: the record in
// memory; org4 / dir4 / meta: the fields the kernel keeps in registers), so
// the whole 128-byte record is never live at once.
template <class B, bool NRC, bool ALLMAT, bool MOTION = false>
B200_D void scatterSurface(const PtCtx &C, const B &bsdf, const MaterialD &mat, uint32_t mi, const DG &dg,
                           const Ray &ray, float t, V3 wo, PathRec *gp, float4 &org4, float4 &dir4, uint4 &meta,
                           PathVars &v, uint32_t p, ShadowRec *sh, int &nsh, const NrcFrameD &nf) {
  const int nl = C.p.numLights;
  const bool transparentShadows = ALLMAT && C.p.transparentShadows != 0;
  if (ALLMAT) gp->lastN.w = v.cone;  // this vertex's cone width (shadow rays, the next bounce)
  if (bsdf.smooth && v.scatter == 0 && !v.auxDone && C.aux) {
    // updateAuxilliaryData (render/pathtracer/PathTracerUtil.ih:48-60) at the
    // first smooth vertex: throughput x BSDF albedo and x shading normal
    float *a = C.aux + size_t(p / uint32_t(C.p.spp)) * 6;
    const V3 an = v.throughput * bsdf.N(), aa = v.throughput * bsdf.albedoV();
    atomicAdd(a + 0, an.x);
    atomicAdd(a + 1, an.y);
    atomicAdd(a + 2, an.z);
    atomicAdd(a + 3, aa.x);
    atomicAdd(a + 4, aa.y);
    atomicAdd(a + 5, aa.z);
    v.auxDone = true;
  }
  bool cached = false;
  if (NRC) {
    const uint32_t slot = gp->meta2.w;
    if (slot != INVALID_ID) {  // training path: record the vertex
      float *q = nf.trainVerts + (size_t(slot) * nf.maxLen1 + v.depth) * 20;
      const float rv[20] = {dg.P.x, dg.P.y, dg.P.z, wo.x, wo.y, wo.z, dg.Ns.x, dg.Ns.y, dg.Ns.z,
                            mat.roughness, mat.r, mat.g, mat.b, v.throughput.x, v.throughput.y, v.throughput.z,
                            v.contribution.x, v.contribution.y, v.contribution.z, __uint_as_float(p)};
      for (int k = 0; k < 20; k++) q[k] = rv[k];
    } else if (nf.useCache && v.depth >= 1 && v.diffuseSeen && bsdf.smooth) {  // end in the cache
      const uint32_t qn = atomicAdd(nf.counters, 1u);
      float *q = nf.queries + size_t(qn) * 16;
      const float qv[16] = {dg.P.x, dg.P.y, dg.P.z, wo.x, wo.y, wo.z, dg.Ns.x, dg.Ns.y, dg.Ns.z,
                            mat.roughness, mat.r, mat.g, mat.b, v.throughput.x, v.throughput.y, v.throughput.z};
      for (int k = 0; k < 16; k++) q[k] = qv[k];
      nf.qpath[qn] = p;
      cached = true;
    }
  }
  if (cached) return;
  // LDSampler of this path at its current group; advanced unconditionally
  const uint32_t sampleID = gp->meta2.z;
  LDSampler ld;
  ld.init(C.T, meta.x, sampleID, sampleID * uint32_t(C.p.nFirst), 16, 16);
  ld.nextGroup();
  int numLS = 0;
  if (bsdf.smooth) {
    numLS = v.firstBounceLight ? C.p.nFirst : C.p.nIndirect;
    for (int i = 0; i < numLS; i++) {
      float ss;
      const float2 sl = ld.get3LightSamples(uint32_t(i), numLS > 1, ss);
      int first = 0, len = nl;
      while (len > 0) {
        const int half = len >> 1, mid = first + half;
        if (ss < __ldg(C.lightCdf + mid)) {
          len = half;
        } else {
          first = mid + 1;
          len -= half + 1;
        }
      }
      first = min(first, nl - 1);
      const float prob = __ldg(C.lightCdf + first) - (first == 0 ? 0.f : __ldg(C.lightCdf + first - 1));
      const float selProb = prob * float(numLS);
      LightSampleD ls = sampleLight(C.lights[first], dg.P, dg.Ng, dg.Ns, sl.x, sl.y);
      ls.weight = ls.weight * (1.f / selProb);
      ls.pdf *= selProb;
      if (maxc(ls.weight) <= 0.f || ls.pdf <= 0.f) continue;
      const BsdfEval fe = bsdf.eval(wo, ls.dir, C.AT);
      if (maxc(fe.value) <= 0.f) continue;
      V3 org = dg.P;
      if (fdot(dg.Ng, ls.dir) < 0.f) org = org - (2.f * dg.epsilon) * dg.Ng;
      const V3 cval = v.throughput * fe.value * ls.weight * misH(ls.pdf, fe.pdf);
      if (nsh < 2) {
        sh[nsh].a = make_float4(org.x, org.y, org.z, ls.dist);
        sh[nsh].b = make_float4(ls.dir.x, ls.dir.y, ls.dir.z, __uint_as_float(p));
        // transparent shadows carry the path's medium in place of tnear (0)
        sh[nsh].c = make_float4(cval.x, cval.y, cval.z, transparentShadows ? __uint_as_float(v.medium) : 0.f);
        nsh++;
      } else {
        // beyond two light samples per vertex: trace in place
        Ray sr;
        sr.org = org;
        sr.tnear = 0.f;
        sr.dir = ls.dir;
        sr.tfar = ls.dist;
        v.contribution = v.contribution + (transparentShadows
                                               ? shadowInPlace<ALLMAT, MOTION>(C, sr, cval, v.medium, v.cone, v.time)
                                               : shadowInPlace<false, MOTION>(C, sr, cval, v.medium, 0.f, v.time));
      }
    }
    v.firstBounceLight = false;
  }
  float ss;
  uint32_t uu3;
  const float2 sb = ld.getNext4Samples(ss, uu3);
  BsdfSample fs = bsdf.sample(wo, sb.x, sb.y, ss, C.AT);
  // consistent side of the surface (light leaks)
  const bool sameSide = fdot(fs.wi, dg.Ng) >= 0.f;
  if (sameSide != ((fs.type & ST_REFLECTION) != 0)) fs.weight = splat(0.f);
  bool cont = !(maxc(fs.weight) <= 0.f || fs.pdf <= 0.f);
  if (cont) {
    v.throughput = v.throughput * fs.weight;
    if (v.depth >= C.p.roulettePathLength) {
      const float rr = ld.finalizeDim3(uu3);
      const float contProb = fminf(maxc(v.throughput), 0.95f);
      if (rr > contProb)
        cont = false;
      else
        v.throughput = v.throughput * (1.f / contProb);
    }
  }
  if (cont) {
    V3 org = dg.P;
    if (ALLMAT) {  // (opaque principled materials neither change nor attenuate the medium)
      // Beer's law over the segment that reached this vertex
      const MediumD md = mediumOf(C.mats, v.medium);
      if (fminf(fminf(md.att.x, md.att.y), md.att.z) < 0.f) v.throughput = v.throughput * expV(md.att * t);
    }
    if (ALLMAT && (fs.type & ST_TRANSMISSION)) {
      org = org - (2.f * dg.epsilon) * dg.Ng;
      if (mat.kind == MAT_GLASS) v.medium = glassFromOutside(C.mats, mi, v.medium) ? 2u * mi : 2u * mi + 1u;
    }
    // a rough or non-metallic vertex counts as the path's diffuse bounce
    if (mat.kind == MAT_PRINCIPLED ? (mat.metallic < 0.5f || mat.roughness > 0.3f) : (fs.type & ST_DIFFUSE_R) != 0)
      v.diffuseSeen = true;
    if (!(ray.dir.x == fs.wi.x && ray.dir.y == fs.wi.y && ray.dir.z == fs.wi.z)) v.straightPath = false;
    if (fs.type & ~ST_SPEC_T) {  // the new last vertex for MIS
      gp->lastP = make_float4(dg.P.x, dg.P.y, dg.P.z, 0.f);
      gp->lastN = make_float4(dg.Ns.x, dg.Ns.y, dg.Ns.z, ALLMAT ? v.cone : 0.f);
      dir4.w = fs.pdf;
      v.lastNLS = numLS;
    } else if (ALLMAT && v.depth == 0) {
      gp->lastP.w = 0.f;  // the continuation ray starts at this surface, not at the camera's near clip
    }
    org4 = make_float4(org.x, org.y, org.z, org4.w);
    dir4 = make_float4(fs.wi.x, fs.wi.y, fs.wi.z, dir4.w);
    v.depth++;
    if (fs.type & ST_SMOOTH) v.scatter++;
    if (!(maxc(v.throughput) > C.p.minContribution)) cont = false;
  }
  meta.x = ld.scramble;
  v.cont = cont;
}

// One bounce of samplePath for every queued path (render/pathtracer/
// PathSampler.ispc:109-415): environment and virtual lights, postIntersect,
// the material's BSDF, NEE light samples (to the shadow queue), BSDF sample
// and Russian roulette (to the next queue).
// NRC: the radiance-cache mode (training paths record their vertices; the
// others end in a cache query at their first vertex after a diffuse bounce).
// ALLMAT: the material list has types other than principled (obj, metal,
// glass, thin glass) or lets shadow rays through; without it the kernel
// carries the opaque principled BSDF only (a smaller kernel for the common
// case).
// (A device function, a stage of the persistent batch kernel too.)
// MOTION: the scene has motion-blurred instances.
template <bool BATCH, bool NRC, bool ALLMAT = true, bool MOTION = false>
// qmiss (a partitioned queue, k_partition): the queue is [diffuse hits |
// other hits | misses] with the first two parts in qin (other hits at its
// end) and the misses at the end of qmiss (Workspace::misses); cpart holds
// the part sizes.
__device__ __forceinline__ void ptShade(PtCtx c, Workspace ws, const uint32_t *qin, const uint32_t *cin, uint32_t *qout,
                                        uint32_t *cout, uint32_t *cshadow, const ReqD *reqs, NrcFrameD nf,
                                        const uint32_t *qmiss, const uint32_t *cpart) {
  static_assert(!(BATCH && NRC), "the radiance cache runs on single-request frames");
  const uint32_t n = *(volatile const uint32_t *)cin;
  const uint32_t nd = qmiss ? cpart[0] : 0u, nm = qmiss ? cpart[2] : 0u;
  const uint32_t stride = gridDim.x * blockDim.x;
  // warp-uniform loop so the appends can use warp votes
  const uint32_t nround = (n + stride - 1) / stride;
  for (uint32_t r = 0; r < nround; r++) {
    const uint32_t qi = r * stride + blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = qi < n;
    uint32_t p = 0u;
    if (valid) {
      if (qmiss)
        p = qi < nd ? qin[qi] : (qi < n - nm ? qin[qi + nm] : qmiss[qi]);
      else
        p = qin ? (BATCH ? qin[qi] : __ldg(qin + qi)) : qi;
    }
    bool cont = false;
    // shadow requests of this lane (numLS <= MAX_NEE per bounce in the queue)
    int nsh = 0;
    ShadowRec sh[2];
    if (valid) {
      PathRec *gp = ws.paths + p;
      const HitBuf hb = ws.hits[p];
      const ReqD *R = BATCH ? reqs + gp->meta2.y : nullptr;
      const PtCtx &C = BATCH ? R->c : c;
      if (BATCH && R->kind == BATCH_AO) {
        PathRec pr = *gp;
        aoShade(C, R->ao, R->fi.W, pr, hb, p, sh, nsh);
        *gp = pr;
      } else {
      const int nl = C.p.numLights;
      float4 org4 = gp->org, dir4 = gp->dir;
      const float4 thr4 = gp->thr, con4 = gp->con;
      uint4 meta = gp->meta;
      const uint32_t flags = meta.y;
      PathVars v;
      v.diffuseSeen = (flags & F_DIFFUSE) != 0;
      v.auxDone = (flags & F_AUXDONE) != 0;
      v.depth = int(flags & 0xffu);
      v.scatter = int((flags >> F_SCATTER_SHIFT) & F_SCATTER_MAX);
      v.straightPath = (flags & F_STRAIGHT) != 0;
      v.firstBounceLight = (flags & F_FIRST) != 0;
      v.lastNLS = int(flags >> F_NLS_SHIFT);
      v.throughput = mk(thr4.x, thr4.y, thr4.z);
      v.contribution = mk(con4.x, con4.y, con4.z);
      v.medium = __float_as_uint(con4.w);
      v.cont = false;
      v.cone = 0.f;
      v.time = ws.times ? ws.times[p] : -1.f;
      float alpha = thr4.w;
      Ray ray;
      ray.org = mk(org4.x, org4.y, org4.z);
      ray.tnear = 0.f;
      ray.dir = mk(dir4.x, dir4.y, dir4.z);
      ray.tfar = INFINITY;
      const bool hit = hb.a.w != 0.f;
      const float t = hit ? hb.a.x : (v.depth == 0 ? org4.w : INFINITY);  // a miss of the camera ray: its tfar
      const V3 wo = -ray.dir;
      if (v.depth == 0) org4.w = t;
      if (!hit && v.straightPath) {
        // Renderer_getBackground (render/Renderer.ispc:19-29) at the pixel centre
        float4 bg = make_float4(C.p.bg[0], C.p.bg[1], C.p.bg[2], C.p.bg[3]);
        if (ALLMAT && !BATCH && C.p.backplate) {
          const uint32_t pix = p / uint32_t(C.p.spp);
          bg = texGetScreen(*C.p.backplate, (float(pix % uint32_t(C.W)) + 0.5f) * C.rcpW,
                            (float(pix / uint32_t(C.W)) + 0.5f) * C.rcpH);
        }
        alpha -= luminance(v.throughput) * (1.f - bg.w);
        v.contribution = v.contribution + v.throughput * mk(bg.x, bg.y, bg.z);
      }
      if (nl > 0) {  // evaluateVirtualLights
        const float4 lp = gp->lastP, ln = gp->lastN;
        const V3 lastP = mk(lp.x, lp.y, lp.z), lastNs = mk(ln.x, ln.y, ln.z);
        const float lastPdf = dir4.w;
        const V3 d0 = lastP - ray.org;
        const float lo = sqrtf(fdot(d0, d0));
        float hiD = INFINITY;
        if (hit) {
          const V3 d1 = lastP - (ray.org + t * ray.dir);
          hiD = sqrtf(fdot(d1, d1));
        }
        const float selPdf = float(v.lastNLS) / float(nl);
        for (int i = 0; i < nl; i++) {
          const LightD &L = C.lights[i];
          if (v.straightPath && !L.visible) continue;
          float lpdf;
          const V3 rad = evalLight(L, lastP, lastNs, ray.dir, lo, hiD, lpdf);
          if (maxc(rad) > 0.f) {
            const float w = selPdf != 0.f ? misH(lastPdf, selPdf * lpdf) : 1.f;
            v.contribution = v.contribution + v.throughput * rad * w;
          }
        }
      }
      if (hit && v.depth < C.p.maxPathLength) {
        HitRec h;
        h.t = t;
        h.primID = __float_as_uint(hb.a.y);
        h.entry = __float_as_uint(hb.a.z);
        h.Ng = mk(hb.b.x, hb.b.y, hb.b.z);
        const Entry &e = C.sc.entries[h.entry];
        h.geomID = e.geomID;
        h.instID = e.instID;
        DGAttr at;
        // hb.b.w: the leaf slot (a motion-blurred hit is re-evaluated from it)
        const DG dg = ALLMAT ? postIntersect<true, MOTION>(C.sc, ray, h, &at, v.time, __float_as_uint(hb.b.w))
                             : postIntersect<false, MOTION>(C.sc, ray, h, nullptr, v.time, __float_as_uint(hb.b.w));
        if (ALLMAT && !BATCH) v.cone = gp->lastN.w + __uint_as_float(gp->meta2.y) * t;
        if (v.depth == 0) {
          meta.z = h.primID;
          meta.w = h.geomID;
          gp->meta2.x = h.instID;
        }
        const uint32_t mi = e.materialID;
        if (v.scatter < C.p.maxScatteringEvents && mi < uint32_t(C.p.numMaterials)) {
          // the colour map and vertex colour applied (principled, obj)
          float opacity = 0.f;
          MaterialD mloc;
          if (ALLMAT) {
            const MaterialD &mrec = C.mats[mi];
            mloc = shadedMaterial(
                mrec, at, mrec.map ? pixelFootprint(v.cone, ray.dir, dg, at, C.p.mipBiasFactor) : 0.f, opacity);
          }
          const MaterialD &mat = ALLMAT ? mloc : C.mats[mi];
          switch (ALLMAT ? mat.kind : MAT_PRINCIPLED) {
            case MAT_OBJ:
            case MAT_PRINCIPLED: {
              // makeShadingFrame (common/DifferentialGeometry.ih) with the surface tangent dPds
              const V3 U = fnormalize(dg.dPds);
              const V3 Vv = fcross(dg.Ns, U);
              V3 fxv, fyv;
              if (fdot(Vv, Vv) > 0.f) {
                fyv = fnormalize(Vv);
                fxv = fcross(fyv, dg.Ns);
              } else {
                frame(dg.Ns, fxv, fyv);
              }
              if (ALLMAT && mat.kind == MAT_OBJ) {
                ObjBsdf b;
                b.init(mat, fxv, fyv, dg.Ns);
                scatterSurface<ObjBsdf, NRC, ALLMAT, MOTION>(C, b, mat, mi, dg, ray, t, wo, gp, org4, dir4, meta, v, p, sh,
                                                     nsh, nf);
              } else {
                PrincipledBsdfT<ALLMAT> b;
                if (ALLMAT)
                  b.init(mat, fxv, fyv, dg.Ns, C.AT, opacity,
                         sameMedium(mediumOf(C.mats, v.medium), MediumD{1.f, splat(0.f)}));
                else
                  b.init(mat, fxv, fyv, dg.Ns, C.AT);
                scatterSurface<PrincipledBsdfT<ALLMAT>, NRC, ALLMAT, MOTION>(C, b, mat, mi, dg, ray, t, wo, gp, org4, dir4,
                                                                    meta, v, p, sh, nsh, nf);
              }
              break;
            }
            case MAT_METAL: {
              if (ALLMAT) {
                MetalBsdf b;
                b.init(mat, dg.Ns);
                scatterSurface<MetalBsdf, NRC, ALLMAT, MOTION>(C, b, mat, mi, dg, ray, t, wo, gp, org4, dir4, meta, v, p, sh,
                                                       nsh, nf);
              }
              break;
            }
            case MAT_GLASS: {
              if (ALLMAT) {
                GlassBsdf b;
                const bool out = glassFromOutside(C.mats, mi, v.medium);
                b.init(out ? mat.iorOut * (1.f / mat.iorIn) : mat.iorIn * (1.f / mat.iorOut), dg.Ns, dg.Ng);
                scatterSurface<GlassBsdf, NRC, ALLMAT, MOTION>(C, b, mat, mi, dg, ray, t, wo, gp, org4, dir4, meta, v, p, sh,
                                                       nsh, nf);
              }
              break;
            }
            case MAT_THINGLASS: {
              if (ALLMAT) {
                ThinGlassBsdf b;
                b.init(mat, dg.Ns);
                scatterSurface<ThinGlassBsdf, NRC, ALLMAT, MOTION>(C, b, mat, mi, dg, ray, t, wo, gp, org4, dir4, meta, v, p,
                                                           sh, nsh, nf);
              }
              break;
            }
            default:
              break;
          }
          cont = v.cont;
        }
      }
      meta.y = uint32_t(v.depth) | (v.straightPath ? F_STRAIGHT : 0u) | (v.firstBounceLight ? F_FIRST : 0u) |
               (cont ? 0u : F_ENDED) | (v.diffuseSeen ? F_DIFFUSE : 0u) | (v.auxDone ? F_AUXDONE : 0u) |
               (uint32_t(min(v.scatter, int(F_SCATTER_MAX))) << F_SCATTER_SHIFT) |
               (uint32_t(min(v.lastNLS, int(F_NLS_MAX))) << F_NLS_SHIFT);
      gp->org = org4;
      gp->dir = dir4;
      gp->thr = make_float4(v.throughput.x, v.throughput.y, v.throughput.z, alpha);
      gp->con = make_float4(v.contribution.x, v.contribution.y, v.contribution.z, __uint_as_float(v.medium));
      gp->meta = meta;
      }
    }
    // queue appends (warp-uniform region)
    const uint32_t oi = warpAppend(cont, cout);
    if (cont) qout[oi] = p;
    for (int k = 0; k < 2; k++) {
      const bool want = k < nsh;
      const uint32_t si = warpAppend(want, cshadow);
      if (want) ws.shadows[si] = sh[k];
    }
  }
}

#ifndef B200_SHADE_MINBLOCKS
#define B200_SHADE_MINBLOCKS 2
#endif
template <bool BATCH, bool NRC, bool ALLMAT = true, bool MOTION = false>
__global__ void __launch_bounds__(128, B200_SHADE_MINBLOCKS)
    k_pt_shade(PtCtx c, Workspace ws, const uint32_t *qin, const uint32_t *cin, uint32_t *qout, uint32_t *cout,
               uint32_t *cshadow, const ReqD *reqs, NrcFrameD nf, const uint32_t *qmiss, const uint32_t *cpart) {
  ptShade<BATCH, NRC, ALLMAT, MOTION>(c, ws, qin, cin, qout, cout, cshadow, reqs, nf, qmiss, cpart);
}

// averages each pixel's samples into the framebuffer (ScreenSample_accumulate
// / normalize, maxContribution clamp, NaN -> 0 with alpha 1)
B200_D PixelOut finalizePT(const PathRec *paths, int spp, float maxContribution) {
  PixelOut acc = {0.f, 0.f, 0.f, 0.f, INFINITY, INVALID_ID, INVALID_ID, INVALID_ID};
  for (int s = 0; s < spp; s++) {
    const PathRec &pr = paths[s];
    float r = pr.con.x, g = pr.con.y, b = pr.con.z, a = pr.thr.w;
    if (isnan(r) || isnan(g) || isnan(b)) {
      r = g = b = 0.f;
      a = 1.f;
    }
    acc.r += fminf(r, maxContribution);
    acc.g += fminf(g, maxContribution);
    acc.b += fminf(b, maxContribution);
    acc.a += a;
    const float z = pr.org.w;
    if (fabsf(z) < fabsf(acc.z)) {
      acc.z = z;
      acc.primID = pr.meta.z;
      acc.geomID = pr.meta.w;
      acc.instID = pr.meta2.x;
    }
  }
  const float rspp = 1.f / float(spp);
  acc.r *= rspp;
  acc.g *= rspp;
  acc.b *= rspp;
  acc.a *= rspp;
  return acc;
}

// an AO pixel from its samples' eye-light terms and unblocked-ray counts, in
// the operation order of the single-frame AO kernel (bit-identical results)
B200_D PixelOut finalizeAO(const PathRec *paths, int spp, const AOParamsD &A) {
  PixelOut acc = {0.f, 0.f, 0.f, 0.f, INFINITY, INVALID_ID, INVALID_ID, INVALID_ID};
  float ar = 0.f, ag = 0.f, ab = 0.f, aa = 0.f;
  for (int s = 0; s < spp; s++) {
    const PathRec &pr = paths[s];
    float bl[4];
    if (pr.meta.y & F_AOHIT) {
      float intensity = pr.thr.x;
      if (A.aoSamples > 0 && A.aoIntensity > 0.01f) {
        const int hits = A.aoSamples - int(pr.con.x);
        const float ao = 1.f - float(hits) / float(A.aoSamples);
        intensity = fmul(intensity, fadd(fsub(1.f, A.aoIntensity), fmul(ao, A.aoIntensity)));
      }
      bl[0] = bl[1] = bl[2] = intensity;
      bl[3] = 1.f;
    } else {
      for (int k = 0; k < 4; k++) bl[k] = A.bg[k];
    }
    const float f = fsub(1.f, 0.f);
    ar = fadd(ar, fadd(0.f, fmul(f, bl[0])));
    ag = fadd(ag, fadd(0.f, fmul(f, bl[1])));
    ab = fadd(ab, fadd(0.f, fmul(f, bl[2])));
    aa = fadd(aa, fadd(0.f, fmul(f, bl[3])));
    const float z = pr.org.w;
    if (fabsf(z) < fabsf(acc.z)) {
      acc.z = z;
      acc.primID = pr.meta.z;
      acc.geomID = pr.meta.w;
      acc.instID = pr.meta2.x;
    }
  }
  const float rspp = fdiv(1.f, float(spp));
  acc.r = fmul(ar, rspp);
  acc.g = fmul(ag, rspp);
  acc.b = fmul(ab, rspp);
  acc.a = fmul(aa, rspp);
  return acc;
}

__global__ void k_pt_finalize(PtCtx c, Workspace ws, FrameInfo fi, FrameD fb) {
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= fi.W * fi.H || !pixelActive(fb, pix % fi.W, pix / fi.W)) return;
  PixelOut o = finalizePT(ws.paths + size_t(pix) * fi.spp, fi.spp, c.p.maxContribution);
  if (c.aux) {  // the frame's normal / albedo sums; cleared for the next frame
    float *a = c.aux + size_t(pix) * 6;
    const float rspp = 1.f / float(fi.spp);
    o.n = mk(a[0], a[1], a[2]) * rspp;
    o.al = mk(a[3], a[4], a[5]) * rspp;
    for (int k = 0; k < 6; k++) a[k] = 0.f;
  }
  fbAccumulate(fb, pix % fi.W, pix / fi.W, o);
}

// ---------------------------------------------------------------- batch kernels
// the segment of a wave slot (segments sorted by `key`)
template <class KeyFn>
B200_D int findSeg(const SegD *segs, int nseg, long long slot, KeyFn key) {
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (key(segs[mid]) <= slot)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// path slot p of a wave: its request's camera ray (PT) or AO camera sample
B200_D void batchGenerate(const ReqD *reqs, const SegD *segs, int nseg, long long p, const Workspace &ws) {
  const SegD &sg = segs[findSeg(segs, nseg, p, [](const SegD &q) { return q.start; })];
  const ReqD &R = reqs[sg.rid];
  const long long lp = sg.first + (p - sg.start);
  const int pix = int(lp / R.fi.spp), s = int(lp % R.fi.spp);
  const int x = pix % R.fi.W, y = pix / R.fi.W;
  if (R.kind == BATCH_PT) {
    ws.paths[p] = genPT(R.c, R.cam, R.pf, R.fi, x, y, s, uint32_t(sg.rid));
    return;
  }
  // AO: the Halton camera sample of AORenderer (sample IDs from frameID * spp + 1)
  const uint32_t sid = uint32_t(R.fi.frameID * R.fi.spp + 1 + s);
  const Ray ray = primaryRay(R.c.T, R.cam, R.pf, x, y, R.fi.rcpW, R.fi.rcpH, sid);
  PathRec r;
  r.org = make_float4(ray.org.x, ray.org.y, ray.org.z, ray.tfar);
  r.dir = make_float4(ray.dir.x, ray.dir.y, ray.dir.z, 0.f);
  r.thr = make_float4(0.f, 0.f, 0.f, 1.f);
  r.con = make_float4(0.f, 0.f, 0.f, 0.f);
  r.lastP = make_float4(0.f, 0.f, 0.f, ray.tnear);
  r.lastN = make_float4(0.f, 0.f, 0.f, 0.f);
  r.meta = make_uint4(0u, 0u, INVALID_ID, INVALID_ID);
  r.meta2 = make_uint4(INVALID_ID, uint32_t(sg.rid), sid, uint32_t(R.fi.W * y + x));
  ws.paths[p] = r;
}

// pixel slot q of a wave: its samples averaged into its request's framebuffer
B200_D void batchFinalize(const ReqD *reqs, const SegD *segs, int nseg, long long q, const Workspace &ws) {
  const SegD &sg = segs[findSeg(segs, nseg, q, [](const SegD &g) { return g.pixStart; })];
  const ReqD &R = reqs[sg.rid];
  const int spp = R.fi.spp;
  const long long pix = sg.first / spp + (q - sg.pixStart);
  const PathRec *paths = ws.paths + sg.start + (pix - sg.first / spp) * spp;
  const PixelOut o = R.kind == BATCH_PT ? finalizePT(paths, spp, R.c.p.maxContribution) : finalizeAO(paths, spp, R.ao);
  fbAccumulate(R.fb, int(pix % R.fi.W), int(pix / R.fi.W), o);
}

__global__ void k_batch_generate(const ReqD *reqs, const SegD *segs, int nseg, long long npaths, Workspace ws) {
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p == 0) {
    ws.counters[0] = uint32_t(npaths);
    for (int k = 1; k < 8; k++) ws.counters[k] = 0;
  }
  if (p < npaths) batchGenerate(reqs, segs, nseg, p, ws);
}

__global__ void k_batch_finalize(const ReqD *reqs, const SegD *segs, int nseg, long long npix, Workspace ws) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q < npix) batchFinalize(reqs, segs, nseg, q, ws);
}

B200_D unsigned long long globalTimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__global__ void k_stamp(unsigned long long *stamps, int first, int end) {
  const unsigned long long t = globalTimer();
  for (int i = first + int(threadIdx.x); i < end; i += blockDim.x) stamps[i] = t;
}

// ---------------------------------------------------------------- persistent batch kernel
// A whole batch frame in one cooperative launch.  The reference hands render
// tasks to threads through its tile scheduler (render/LoadBalancer.cpp:13-32);
// here the work items are the waves' (request, pixel range) segments and
// their queues: per wave, generate -> per bounce (closest trace -> shade ->
// shadow trace) -> finalize, each stage a grid-stride loop or a dynamically
// fetched queue over the whole resident grid, the stages separated by
// grid-wide barriers.  The requests a wave completes are post-processed in
// the next stage (beside the next wave's generation) and stamped after it.

// a wave as the persistent kernel reads it (device table)
struct WaveD {
  long long npaths, npix;
  int segOffset, nseg, maxBounces, completeFirst, completeEnd, pad;
};

// a request's post-processing (device table)
struct PostD {
  const float4 *color;
  void *out;
  long long n;
  ToneMapD tm;
  int format, tonemap;
};

struct BatchRunD {
  const ReqD *reqs;
  const SegD *segs;
  const WaveD *waves;
  const PostD *post;
  int nwaves, nreqs;
  Workspace ws;
  uint32_t *bar;  // [0] arrivals, [1] generation, [2] error (a wait timed out)
  unsigned long long *rays, *stamps;
  unsigned long long timeoutNs;  // the bound of a barrier wait
};


B200_D uint32_t loadAcquire(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid-wide barrier of the cooperative launch.  A wait longer than
// timeoutNs sets the error word, and a block that finds the error word set
// does not wait: every block then leaves the kernel (false) instead of
// spinning on.
B200_D bool gridBarrier(uint32_t *bar, uint32_t &gen, unsigned long long timeoutNs) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = *(volatile uint32_t *)(bar + 2) == 0u;
    if (ok) {
      const uint32_t next = gen + 1u;
      __threadfence();
      if (atomicAdd(bar, 1u) == gridDim.x - 1u) {
        atomicExch(bar, 0u);
        __threadfence();
        atomicExch(bar + 1, next);
      } else {
        const unsigned long long t0 = globalTimer();
        while (loadAcquire(bar + 1) != next) {
          if (*(volatile uint32_t *)(bar + 2) != 0u || globalTimer() - t0 > timeoutNs) {
            atomicExch(bar + 2, 1u);
            ok = 0;
            break;
          }
          __nanosleep(64);
        }
      }
      __threadfence();
    }
    s_ok = ok;
  }
  __syncthreads();
  gen++;
  return s_ok != 0;
}

// the colour conversion of requests [first, end) (framePostProcess; batched
// frames keep no variance estimate)
B200_D void batchPost(const BatchRunD &R, int first, int end, long long tid, long long nthreads) {
  for (int r = first; r >= 0 && r < end; r++) {
    const PostD &P = R.post[r];
    if (P.format == B200_FB_NONE) continue;
    for (long long i = tid; i < P.n; i += nthreads) postPixel(P.color, i, P.format, P.tonemap, P.tm, P.out);
  }
}

#ifndef B200_PERSIST_MINBLOCKS
#define B200_PERSIST_MINBLOCKS 3
#endif
// B200_PERSIST_CALLS: the trace and shade stages as out-of-line functions,
// each register-allocated on its own (within the kernel's budget) rather
// than inlined into one body whose live ranges all compete (1,302 vs 1,263
// Mrays/s on the 64-request batch; 4 blocks per SM: 1,278 / 1,270)
#ifndef B200_PERSIST_CALLS
#define B200_PERSIST_CALLS 1
#endif
#if B200_PERSIST_CALLS
#define B200_STAGE static __device__ __noinline__
#else
#define B200_STAGE static __device__ __forceinline__
#endif
template <bool SHADOW>
B200_STAGE void persistTrace(Workspace ws, const uint32_t *queue, const uint32_t *count, uint32_t *fetch,
                             const ReqD *reqs) {
  traceQueue<SHADOW, false, true>(Scene{}, ws, queue, count, fetch, reqs, ShadowMatD{});
}
B200_STAGE void persistShade(Workspace ws, const uint32_t *qin, const uint32_t *cin, uint32_t *qout, uint32_t *cout,
                             uint32_t *cshadow, const ReqD *reqs) {
  ptShade<true, false, true>(PtCtx{}, ws, qin, cin, qout, cout, cshadow, reqs, NrcFrameD{}, nullptr, nullptr);
}
__global__ void __launch_bounds__(TRACE_BLOCK, B200_PERSIST_MINBLOCKS) k_batch_persistent(BatchRunD R) {
  // little state lives across the stages (the wave's fields are re-read
  // from its table entry where a stage needs them), so the shading stage
  // keeps its registers
  const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
  uint32_t *ctr = R.ws.counters;
  volatile uint32_t *vctr = ctr;
  uint32_t gen = 0;
  if (lead) R.stamps[R.nreqs] = globalTimer();
  for (int wi = 0; wi <= R.nwaves; wi++) {
    // post-processing of the requests the previous wave completed, beside
    // this wave's generation
    {
      const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
      const long long nthreads = (long long)gridDim.x * blockDim.x;
      if (wi > 0) batchPost(R, R.waves[wi - 1].completeFirst, R.waves[wi - 1].completeEnd, tid, nthreads);
      if (wi < R.nwaves) {
        const WaveD &w = R.waves[wi];
        if (lead) {
          vctr[0] = uint32_t(w.npaths);
          for (int k = 1; k < 8; k++) vctr[k] = 0u;
        }
        for (long long p = tid; p < w.npaths; p += nthreads) batchGenerate(R.reqs, R.segs + w.segOffset, w.nseg, p, R.ws);
      }
    }
    if (!gridBarrier(R.bar, gen, R.timeoutNs)) return;
    if (lead && wi > 0)
      for (int r = R.waves[wi - 1].completeFirst; r >= 0 && r < R.waves[wi - 1].completeEnd; r++)
        R.stamps[r] = globalTimer();
    if (wi == R.nwaves) break;
    const int nb = R.waves[wi].maxBounces;
    for (int b = 0; b <= nb; b++) {
      const int cin = b & 1, cout = cin ^ 1;
      const uint32_t *qin = b == 0 ? nullptr : (cin ? R.ws.qb : R.ws.qa);
      // counter upkeep, each beside a stage that does not use that counter:
      // the rays of the last bounce are counted, the shadow queue and its
      // fetch counter cleared
      if (lead) {
        *R.rays += (unsigned long long)vctr[cin] + vctr[2];
        vctr[2] = 0u;
        vctr[4] = 0u;
      }
      persistTrace<false>(R.ws, qin, ctr + cin, ctr + 3, R.reqs);
      if (!gridBarrier(R.bar, gen, R.timeoutNs)) return;
      if (lead) vctr[3] = 0u;  // closest-hit fetch counter of the next bounce
      persistShade(R.ws, qin, ctr + cin, cout ? R.ws.qb : R.ws.qa, ctr + cout, ctr + 2, R.reqs);
      if (!gridBarrier(R.bar, gen, R.timeoutNs)) return;
      if (lead) vctr[cin] = 0u;  // the next bounce's output queue
      persistTrace<true>(R.ws, nullptr, ctr + 2, ctr + 4, R.reqs);
      if (!gridBarrier(R.bar, gen, R.timeoutNs)) return;
    }
    if (lead) *R.rays += vctr[2];
    {
      const WaveD &w = R.waves[wi];
      const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
      for (long long q = tid; q < w.npix; q += (long long)gridDim.x * blockDim.x)
        batchFinalize(R.reqs, R.segs + w.segOffset, w.nseg, q, R.ws);
    }
    if (!gridBarrier(R.bar, gen, R.timeoutNs)) return;
  }
}

// ---------------------------------------------------------------- radiance cache hooks
// adds throughput x cached radiance to the paths that ended in a query, then
// clears the query count for the next bounce (one thread per possible query;
// the count is read before any thread clears it: the last block to finish
// does the clearing)
__global__ void k_nrc_apply(NrcFrameD nf, PathRec *paths, uint32_t cap) {
  const uint32_t n = min(*(volatile const uint32_t *)nf.counters, cap);
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const float *q = nf.queries + size_t(i) * 16;
    const float *L = nf.qout + size_t(i) * 3;
    float *con = &paths[nf.qpath[i]].con.x;
    for (int k = 0; k < 3; k++) atomicAdd(con + k, q[13 + k] * fmaxf(L[k], 0.f));
  }
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(nf.counters + 2, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    nf.counters[0] = 0;
    nf.counters[2] = 0;
  }
}

// training samples from the recorded vertices: inputs and the radiance the
// rest of the path brought back, (C_end - C_i) / T_i per channel
__global__ void k_nrc_targets(NrcFrameD nf, const PathRec *paths, long long nv) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const float *v = nf.trainVerts + size_t(i) * 20;
  const uint32_t p = __float_as_uint(v[19]);
  if (p == 0xffffffffu) return;
  const float4 cend = paths[p].con;
  const float ce[3] = {cend.x, cend.y, cend.z};
  float tgt[3];
  bool ok = true;
  for (int k = 0; k < 3; k++) {
    const float T = v[13 + k];
    tgt[k] = T > 0.f ? fmaxf(ce[k] - v[16 + k], 0.f) / T : 0.f;
    ok = ok && isfinite(tgt[k]);
  }
  if (!ok) return;
  const uint32_t si = atomicAdd(nf.counters + 1, 1u);
  if (si >= nf.sampleCap) return;
  float *o = nf.samples + size_t(si) * 16;
  for (int k = 0; k < 13; k++) o[k] = v[k];
  for (int k = 0; k < 3; k++) o[13 + k] = tgt[k];
}

// ---------------------------------------------------------------- albedo tables
// MicrofacetAlbedo_integrate / MicrofacetDielectricReflectionAlbedo_integrate:
// 32x32 stratified visible-normal samples per entry.
B200_D float albedoIntegrate(float cosO, float roughness, bool dielectric, float eta) {
  const float a = fmaxf(sqrf(roughness), 0.001f);
  cosO = fmaxf(cosO, 1e-6f);
  const V3 wo = mk(sqrtf(fmaxf(0.f, 1.f - cosO * cosO)), 0.f, cosO);
  float sum = 0.f;
  for (int i = 0; i < 32; i++)
    for (int j = 0; j < 32; j++) {
      const float sx = fminf((i + 0.5f) / 32.f, 1.f - 1e-6f), sy = fminf((j + 0.5f) / 32.f, 1.f - 1e-6f);
      float whPdf;
      const V3 wh = ggxSampleVisible(a, wo, whPdf, sx, sy);
      const float cosOH = fdot(wo, wh);
      const V3 wi = reflectV(wo, wh, cosOH);
      if (wi.z <= 0.f) continue;
      const float w = ggxG2(a, wo, wi, cosOH, fdot(wi, wh)) * rcpSafe(ggxG1(a, wo, cosOH));
      sum += dielectric ? fresnelDiel(cosOH, eta) * w : w;
    }
  return fminf(sum / 1024.f, 1.f);
}

__global__ void k_albedo_dir(AlbedoTablesD *T) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 32 * 32) {
    T->dir[i] = albedoIntegrate(float(i % 32) / 31.f, float(i / 32) / 31.f, false, 1.f);
  } else if (i < 32 * 32 + 16 * 16 * 16) {
    const int k = i - 32 * 32;
    const float t = float((k / 16) % 16) / 15.f;
    const float eta = (1.f - t) * (1.f / 3.f) + t * 1.f;
    T->reflDir[k] = albedoIntegrate(float(k % 16) / 15.f, float(k / 256) / 15.f, true, eta);
  }
}

// MicrofacetAlbedoTable_integrateAvg over each table row
__global__ void k_albedo_avg(AlbedoTablesD *T) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const float *row;
  int n;
  float *out;
  if (r < 32) {
    row = T->dir + r * 32;
    n = 32;
    out = T->avg + r;
  } else if (r < 32 + 256) {
    row = T->reflDir + (r - 32) * 16;
    n = 16;
    out = T->reflAvg + (r - 32);
  } else {
    return;
  }
  float sum = 0.f;
  for (int i = 0; i < 1025; i++) {
    const float c = float(i) / 1024.f;
    sum += interp1(c * (n - 1), row, n) * c * ((i == 0 || i == 1024) ? 0.5f : 1.f);
  }
  *out = fminf(2.f * (sum / 1024.f), 1.f);
}

// Between bounces: counts the rays of the bounce about to run (its
// extension queue) and of the last one's shadow queue, then clears the
// output queue, shadow queue and fetch counters.
__global__ void k_bounce_reset(uint32_t *counters, int cin, int cout, unsigned long long *rays) {
  if (rays) *rays += (unsigned long long)counters[cin] + counters[2];
  counters[cout] = 0;
  counters[2] = 0;
  counters[3] = 0;
  counters[4] = 0;
  counters[5] = 0;
  counters[6] = 0;
  counters[7] = 0;
}

// Splits a bounce's queue of traced paths by what their shading runs: the
// front of `out` gets the hits on diffuse-based materials (principled with
// metallic < 0.5, obj), its back the other hits (conductors, metal, glass),
// and the misses go to the end of ws.misses, so that most warps of the
// shading kernel take one branch of the BSDF code.  cpart[0..2] count the
// three parts (cleared per bounce).  The shading kernel reads them in the
// order diffuse, other, misses.  (`out` is not the traced queue: this
// kernel reads that one throughout.)
// In a batch (BATCH) each path's request gives the scene and materials.
template <bool BATCH>
__global__ void k_partition(Scene sc, const MaterialD *mats, int nmats, Workspace ws, const uint32_t *qin,
                            const uint32_t *count, uint32_t *out, uint32_t *cpart, const ReqD *reqs) {
  const uint32_t n = *(volatile const uint32_t *)count;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t nround = (n + stride - 1) / stride;  // warp-uniform loop (warp appends)
  for (uint32_t r = 0; r < nround; r++) {
    const uint32_t i = r * stride + blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    uint32_t p = 0;
    bool diffuse = false, hit = false;
    if (valid) {
      p = qin ? qin[i] : i;
      const float4 a = ws.hits[p].a;
      hit = a.w != 0.f;
      if (hit) {
        const Entry *entries = sc.entries;
        const MaterialD *M = mats;
        int nm = nmats;
        if (BATCH) {
          const ReqD &R = reqs[ws.paths[p].meta2.y];
          entries = R.c.sc.entries;
          M = R.c.mats;
          nm = R.kind == BATCH_PT ? R.c.p.numMaterials : 0;
        }
        const uint32_t mi = __ldg(&entries[__float_as_uint(a.z)].materialID);
        if (mi >= uint32_t(nm)) {
          diffuse = true;
        } else {
          const uint32_t kind = __ldg(&M[mi].kind);
          diffuse = kind == MAT_OBJ || (kind == MAT_PRINCIPLED && __ldg(&M[mi].metallic) < 0.5f);
        }
      }
    }
    const uint32_t f = warpAppend(valid && diffuse, cpart);
    const uint32_t k = warpAppend(valid && hit && !diffuse, cpart + 1);
    const uint32_t m = warpAppend(valid && !hit, cpart + 2);
    if (valid) {
      if (diffuse)
        out[f] = p;
      else if (hit)
        out[n - 1u - k] = p;
      else
        ws.misses[n - 1u - m] = p;
    }
  }
}

__global__ void k_count_tail(const uint32_t *counters, unsigned long long *rays) { *rays += counters[2]; }

int persistentBlocks(const void *kernel, size_t smem) {
  int dev, sms, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, TRACE_BLOCK, smem);
  return sms * (per > 0 ? per : 1);
}

}  // namespace

namespace {
Workspace carveWorkspace(void *workspace, long long npaths) {
  Workspace ws;
  char *base = static_cast<char *>(workspace);
  auto carve = [&](size_t bytes) {
    char *q = base;
    base += (bytes + 255) & ~size_t(255);
    return q;
  };
  ws.paths = (PathRec *)carve(sizeof(PathRec) * npaths);
  ws.hits = (HitBuf *)carve(sizeof(HitBuf) * npaths);
  ws.qa = (uint32_t *)carve(4 * npaths);
  ws.qb = (uint32_t *)carve(4 * npaths);
  ws.shadows = (ShadowRec *)carve(sizeof(ShadowRec) * 2 * npaths);
  ws.misses = reinterpret_cast<uint32_t *>(ws.shadows + 2 * npaths) - npaths;
  ws.times = nullptr;
  ws.counters = (uint32_t *)carve(64);
  return ws;
}

int smCount() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}
}  // namespace

cudaError_t computeAlbedoTables(AlbedoTablesD *T, cudaStream_t st) {
  k_albedo_dir<<<(32 * 32 + 4096 + 127) / 128, 128, 0, st>>>(T);
  k_albedo_avg<<<(32 + 256 + 127) / 128, 128, 0, st>>>(T);
  return cudaGetLastError();
}

size_t ptWorkspaceBytes(long long npaths) {
  auto up = [](size_t x) { return (x + 255) & ~size_t(255); };
  return up(sizeof(PathRec) * npaths) + up(sizeof(HitBuf) * npaths) + 2 * up(4 * npaths) +
         up(sizeof(ShadowRec) * 2 * npaths) + up(64);
}

cudaError_t launchRenderPT(const SamplerTables *T, const Scene &sc, const CameraD &cam, const PixelFilterD &pf,
                           const PtParamsD &p, const MaterialD *mats, const LightD *lights, const float *lightCdf,
                           const AlbedoTablesD *AT, const FrameD &fb, bool stats, void *workspace, size_t wsBytes,
                           cudaStream_t st, const NrcFrameD *nrc, void (*nrcInfer)(void *, cudaStream_t),
                           void *nrcCtx, KernelTimer *kt, float *rayTimes) {
  FrameInfo fi;
  fi.W = fb.W;
  fi.H = fb.H;
  fi.spp = p.spp;
  fi.frameID = fb.frameID;
  fi.rcpW = fdiv(1.f, float(fb.W));
  fi.rcpH = fdiv(1.f, float(fb.H));
  fi.npaths = (long long)fb.W * fb.H * p.spp;
  if (ptWorkspaceBytes(fi.npaths) > wsBytes) return cudaErrorInvalidValue;
  if (nrc && (stats || !nrcInfer)) return cudaErrorInvalidValue;
  Workspace ws = carveWorkspace(workspace, fi.npaths);
  ws.times = rayTimes;
  PtCtx c = {T, sc, p, mats, lights, lightCdf, AT, fb.frameID, fb.aux, fb.W, fi.rcpW, fi.rcpH};
  static int traceBlocks = 0, shadowBlocks = 0, transpBlocks = 0, shadeBlocks = 0, shadeAllBlocks = 0,
             shadeNrcBlocks = 0;
  if (!traceBlocks) {
    // shared-memory carveout preferences (percent of the SM's shared memory;
    // the rest is L1, which caches the BVH nodes and the shading kernel's
    // spills); negative: the driver's choice, which measured as good as the
    // best setting (1,097 vs 1,098 Mrays/s at 50 % trace / 25 % shade; 100 %
    // for the trace kernels: 1,001; 0 % for the shading kernels: 948)
    if (B200_TRACE_CARVEOUT >= 0) {
      const void *tk[] = {(const void *)k_trace_queue<false, false, false>,
                          (const void *)k_trace_queue<true, false, false>,
                          (const void *)k_trace_queue<false, false, false, false, false>,
                          (const void *)k_trace_queue<true, false, false, false, false>};
      for (const void *k : tk)
        cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, B200_TRACE_CARVEOUT);
    }
    if (B200_SHADE_CARVEOUT >= 0) {
      const void *sk[] = {(const void *)k_pt_shade<false, false, false>, (const void *)k_pt_shade<false, false, true>};
      for (const void *k : sk)
        cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, B200_SHADE_CARVEOUT);
    }
    traceBlocks = persistentBlocks((const void *)k_trace_queue<false, false, false>, TRACE_SMEM_BYTES);
    shadowBlocks = persistentBlocks((const void *)k_trace_queue<true, false, false>, TRACE_SMEM_BYTES);
    transpBlocks = persistentBlocks((const void *)k_trace_queue<true, false, false, true>, TRACE_SMEM_BYTES);
    shadeBlocks = persistentBlocks((const void *)k_pt_shade<false, false, false>, TRACE_SMEM_BYTES);
    shadeAllBlocks = persistentBlocks((const void *)k_pt_shade<false, false, true>, TRACE_SMEM_BYTES);
    shadeNrcBlocks = persistentBlocks((const void *)k_pt_shade<false, true, false>, TRACE_SMEM_BYTES);
  }
  const NrcFrameD nf = nrc ? *nrc : NrcFrameD{};
  const ShadowMatD sm = {mats, p.numMaterials, p.maxPathLength, p.minContribution, p.mipBiasFactor};
  const bool transp = p.transparentShadows != 0;
  if (nrc) {
    cudaMemsetAsync(nf.counters, 0, 16, st);
    cudaMemsetAsync(nf.trainVerts, 0xff, size_t(nf.trainSlots) * nf.maxLen1 * 20 * 4, st);
  }
  const int gen = int((fi.npaths + 255) / 256);
  const bool adaptive = fb.taskActive != nullptr;
  if (adaptive) cudaMemsetAsync(ws.counters, 0, 16 * sizeof(uint32_t), st);
  k_pt_generate<<<gen, 256, 0, st>>>(c, cam, pf, fi, ws, nf.trainStride, nf.trainOffset, nf.trainSlots, fb,
                                     adaptive ? ws.qa : nullptr);
  // the queue a bounce traces (camera rays of a whole frame: none, the
  // identity); shading appends the continuing paths to another buffer, and
  // with the partition the partitioned copy takes the third role
  uint32_t *inBuf = adaptive ? ws.qa : nullptr;
  const bool partition = B200_SHADE_PARTITION != 0;
  static int partBlocks = 0;
  if (!partBlocks) partBlocks = smCount() * 8;
  for (int b = 0; b <= p.maxPathLength; b++) {
    const int cin = b & 1, cout = cin ^ 1;
    k_bounce_reset<<<1, 1, 0, st>>>(ws.counters, cin, cout, nullptr);
    const uint32_t *qin = inBuf;
    uint32_t *other = inBuf == ws.qb ? ws.qa : ws.qb;  // not the traced queue
    uint32_t *third = other == ws.qa ? ws.qb : ws.qa;  // the traced queue, or at bounce 0 the free buffer
    const uint32_t *qshade = qin;
    uint32_t *qnext = other;
    {
      KernelScope ks(kt, KK_TRACE_CLOSEST, st);
      if (stats)
        k_trace_queue<false, true, false><<<traceBlocks, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(
            sc, ws, qin, ws.counters + cin, ws.counters + 3, nullptr, sm);
      else if (sc.hasUser)
        k_trace_queue<false, false, false><<<traceBlocks, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(
            sc, ws, qin, ws.counters + cin, ws.counters + 3, nullptr, sm);
      else
        k_trace_queue<false, false, false, false, false><<<traceBlocks, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(
            sc, ws, qin, ws.counters + cin, ws.counters + 3, nullptr, sm);
    }
    const uint32_t *qmiss = nullptr, *cpart = nullptr;
    if (partition && b > 0) {
      k_partition<false><<<partBlocks, 256, 0, st>>>(sc, mats, p.numMaterials, ws, qin, ws.counters + cin, other,
                                                     ws.counters + 5, nullptr);
      qshade = other;
      qnext = third;
      qmiss = ws.misses;
      cpart = ws.counters + 5;
    }
    {
      KernelScope ks(kt, KK_SHADE, st);
      if (nrc && p.allMaterials)
        k_pt_shade<false, true, true><<<shadeNrcBlocks, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(
            c, ws, qshade, ws.counters + cin, qnext, ws.counters + cout, ws.counters + 2, nullptr, nf, qmiss, cpart);
      else if (nrc)
        k_pt_shade<false, true, false><<<shadeNrcBlocks, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(
            c, ws, qshade, ws.counters + cin, qnext, ws.counters + cout, ws.counters + 2, nullptr, nf, qmiss, cpart);
      else if (ws.times)  // motion-blurred instances: the general kernel with their code
        k_pt_shade<false, false, true, true><<<shadeAllBlocks, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(
            c, ws, qshade, ws.counters + cin, qnext, ws.counters + cout, ws.counters + 2, nullptr, nf, qmiss, cpart);
      else if (p.allMaterials)
        k_pt_shade<false, false, true><<<shadeAllBlocks, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(
            c, ws, qshade, ws.counters + cin, qnext, ws.counters + cout, ws.counters + 2, nullptr, nf, qmiss, cpart);
      else
        k_pt_shade<false, false, false><<<shadeBlocks, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(
            c, ws, qshade, ws.counters + cin, qnext, ws.counters + cout, ws.counters + 2, nullptr, nf, qmiss, cpart);
    }
    inBuf = qnext;
    const uint32_t *sq = nullptr;  // shadow records in queue order
    {
      KernelScope ks(kt, KK_TRACE_SHADOW, st);
      if (transp && stats)
        k_trace_queue<true, true, false, true><<<transpBlocks, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(
            sc, ws, sq, ws.counters + 2, ws.counters + 4, nullptr, sm);
      else if (transp)
        k_trace_queue<true, false, false, true><<<transpBlocks, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(
            sc, ws, sq, ws.counters + 2, ws.counters + 4, nullptr, sm);
      else if (stats)
        k_trace_queue<true, true, false><<<shadowBlocks, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(
            sc, ws, sq, ws.counters + 2, ws.counters + 4, nullptr, sm);
      else if (sc.hasUser)
        k_trace_queue<true, false, false><<<shadowBlocks, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(
            sc, ws, sq, ws.counters + 2, ws.counters + 4, nullptr, sm);
      else
        k_trace_queue<true, false, false, false, false><<<shadowBlocks, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(
            sc, ws, sq, ws.counters + 2, ws.counters + 4, nullptr, sm);
    }
    if (nrc && nf.useCache) {  // answer this bounce's cache queries
      nrcInfer(nrcCtx, st);
      k_nrc_apply<<<unsigned((fi.npaths + 255) / 256), 256, 0, st>>>(nf, ws.paths, uint32_t(fi.npaths));
    }
  }
  k_pt_finalize<<<(fb.W * fb.H + 127) / 128, 128, 0, st>>>(c, ws, fi, fb);
  if (nrc) {
    const long long nv = (long long)nf.trainSlots * nf.maxLen1;
    k_nrc_targets<<<unsigned((nv + 255) / 256), 256, 0, st>>>(nf, ws.paths, nv);
  }
  return cudaGetLastError();
}

void planBatch(const SamplerTables *T, const AlbedoTablesD *AT, const BatchReqH *reqs, int n, long long wavePaths,
               std::vector<unsigned char> &tables, std::vector<BatchWave> &waves, BatchLayout &layout) {
  std::vector<ReqD> rd(n);
  for (int i = 0; i < n; i++) {
    const BatchReqH &h = reqs[i];
    ReqD &r = rd[i];
    r = ReqD{};
    r.kind = h.kind;
    const int spp = h.kind == BATCH_PT ? h.pt.spp : h.ao.spp;
    r.c = PtCtx{T, h.sc, h.pt, h.mats, h.lights, h.lightCdf, AT, h.fb.frameID};
    r.cam = h.cam;
    r.pf = h.pf;
    r.fi.W = h.fb.W;
    r.fi.H = h.fb.H;
    r.fi.spp = spp;
    r.fi.frameID = h.fb.frameID;
    r.fi.rcpW = 1.f / float(h.fb.W);
    r.fi.rcpH = 1.f / float(h.fb.H);
    r.fi.npaths = (long long)h.fb.W * h.fb.H * spp;
    r.fb = h.fb;
    r.ao = h.ao;
  }
  std::vector<SegD> segs;
  waves.clear();
  BatchWave w = {};
  auto close = [&]() {
    if (w.npaths > 0) waves.push_back(w);
    w = BatchWave{};
    w.segOffset = int(segs.size());
    w.completeFirst = w.completeEnd = -1;
  };
  close();
  for (int i = 0; i < n; i++) {
    const int spp = rd[i].fi.spp;
    if (spp > wavePaths) throw std::runtime_error("batch: a wave must hold at least one pixel's samples");
    const long long npix = (long long)rd[i].fi.W * rd[i].fi.H;
    long long done = 0;
    while (done < npix) {
      long long fit = (wavePaths - w.npaths) / spp;
      if (fit == 0) {
        close();
        fit = wavePaths / spp;
      }
      const long long k = std::min(fit, npix - done);
      SegD sg;
      sg.start = w.npaths;
      sg.first = done * spp;
      sg.pixStart = w.npix;
      sg.rid = i;
      sg.pad = 0;
      segs.push_back(sg);
      w.nseg++;
      w.npaths += k * spp;
      w.npix += k;
      w.maxBounces = std::max(w.maxBounces, rd[i].kind == BATCH_PT ? rd[i].c.p.maxPathLength : 0);
      done += k;
      if (done == npix) {
        if (w.completeFirst < 0) w.completeFirst = i;
        w.completeEnd = i + 1;
      }
    }
  }
  close();
  std::vector<WaveD> wd(waves.size());
  for (size_t i = 0; i < waves.size(); i++) {
    const BatchWave &b = waves[i];
    wd[i] = WaveD{b.npaths, b.npix, b.segOffset, b.nseg, b.maxBounces, b.completeFirst, b.completeEnd, 0};
  }
  std::vector<PostD> pd(n);
  for (int i = 0; i < n; i++) {
    const BatchReqH &h = reqs[i];
    pd[i] = PostD{h.fb.color, h.postOut, (long long)h.fb.W * h.fb.H, h.postTm, h.postFormat, h.postTonemap};
  }
  auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
  layout.segs = up(sizeof(ReqD) * n);
  layout.waves = up(layout.segs + sizeof(SegD) * segs.size());
  layout.post = up(layout.waves + sizeof(WaveD) * wd.size());
  layout.nwaves = int(wd.size());
  tables.assign(layout.post + sizeof(PostD) * n, 0);
  std::memcpy(tables.data(), rd.data(), sizeof(ReqD) * n);
  std::memcpy(tables.data() + layout.segs, segs.data(), sizeof(SegD) * segs.size());
  if (!wd.empty()) std::memcpy(tables.data() + layout.waves, wd.data(), sizeof(WaveD) * wd.size());
  std::memcpy(tables.data() + layout.post, pd.data(), sizeof(PostD) * n);
}

cudaError_t launchBatchWave(const void *dtables, size_t segTableOffset, const BatchWave &w, const BatchTuning &tune,
                            void *workspace, size_t wsBytes, unsigned long long *rayCount, cudaStream_t st) {
  if (w.npaths > tune.wavePaths || ptWorkspaceBytes(tune.wavePaths) > wsBytes) return cudaErrorInvalidValue;
  const ReqD *reqs = static_cast<const ReqD *>(dtables);
  const SegD *segs = reinterpret_cast<const SegD *>(static_cast<const char *>(dtables) + segTableOffset) + w.segOffset;
  Workspace ws = carveWorkspace(workspace, tune.wavePaths);
  const int sms = smCount();
  const int traceBlocks = sms * std::max(1, tune.traceBlocksPerSM);
  const int shadeBlocks = sms * std::max(1, tune.shadeBlocksPerSM);
  const Scene noScene = {};
  const PtCtx noCtx = {};
  k_batch_generate<<<unsigned((w.npaths + 255) / 256), 256, 0, st>>>(reqs, segs, w.nseg, w.npaths, ws);
  // queue buffers as in launchRenderPT (the partition from the second bounce on)
  uint32_t *inBuf = nullptr;
  for (int b = 0; b <= w.maxBounces; b++) {
    const int cin = b & 1, cout = cin ^ 1;
    k_bounce_reset<<<1, 1, 0, st>>>(ws.counters, cin, cout, rayCount);
    const uint32_t *qin = inBuf;
    uint32_t *other = inBuf == ws.qb ? ws.qa : ws.qb;
    uint32_t *third = other == ws.qa ? ws.qb : ws.qa;
    const uint32_t *qshade = qin;
    uint32_t *qnext = other;
    k_trace_queue<false, false, true><<<traceBlocks, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(
        noScene, ws, qin, ws.counters + cin, ws.counters + 3, reqs, ShadowMatD{});
    const uint32_t *qmiss = nullptr, *cpart = nullptr;
    if (B200_SHADE_PARTITION && b > 0) {
      k_partition<true><<<unsigned(sms * 8), 256, 0, st>>>(noScene, nullptr, 0, ws, qin, ws.counters + cin, other,
                                                           ws.counters + 5, reqs);
      qshade = other;
      qnext = third;
      qmiss = ws.misses;
      cpart = ws.counters + 5;
    }
    k_pt_shade<true, false, true><<<shadeBlocks, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(
        noCtx, ws, qshade, ws.counters + cin, qnext, ws.counters + cout, ws.counters + 2, reqs, NrcFrameD{}, qmiss,
        cpart);
    inBuf = qnext;
    k_trace_queue<true, false, true><<<traceBlocks, TRACE_BLOCK, TRACE_SMEM_BYTES, st>>>(
        noScene, ws, nullptr, ws.counters + 2, ws.counters + 4, reqs, ShadowMatD{});
  }
  if (rayCount) k_count_tail<<<1, 1, 0, st>>>(ws.counters, rayCount);
  k_batch_finalize<<<unsigned((w.npix + 127) / 128), 128, 0, st>>>(reqs, segs, w.nseg, w.npix, ws);
  return cudaGetLastError();
}

int batchPersistentBlocksPerSM() {
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_persistent, TRACE_BLOCK, TRACE_SMEM_BYTES) !=
      cudaSuccess)
    return 0;
  return per;
}

cudaError_t launchBatchPersistent(const void *dtables, const BatchLayout &layout, int nreqs, const BatchTuning &tune,
                                  void *workspace, size_t wsBytes, unsigned long long *rayCount,
                                  unsigned long long *stamps, uint32_t *barrier, unsigned long long timeoutNs,
                                  cudaStream_t st) {
  if (ptWorkspaceBytes(tune.wavePaths) > wsBytes || !rayCount || !stamps || !barrier) return cudaErrorInvalidValue;
  const int per = batchPersistentBlocksPerSM();
  if (per < 1) return cudaErrorInvalidConfiguration;
  const char *t = static_cast<const char *>(dtables);
  BatchRunD R;
  R.reqs = reinterpret_cast<const ReqD *>(t);
  R.segs = reinterpret_cast<const SegD *>(t + layout.segs);
  R.waves = reinterpret_cast<const WaveD *>(t + layout.waves);
  R.post = reinterpret_cast<const PostD *>(t + layout.post);
  R.nwaves = layout.nwaves;
  R.nreqs = nreqs;
  R.ws = carveWorkspace(workspace, tune.wavePaths);
  R.bar = barrier;
  R.rays = rayCount;
  R.stamps = stamps;
  R.timeoutNs = timeoutNs;
  cudaError_t e = cudaMemsetAsync(barrier, 0, 4 * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  // all blocks resident at once (the cooperative attribute makes the launch
  // fail rather than run a grid that does not fit)
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(unsigned(smCount() * per));
  cfg.blockDim = dim3(TRACE_BLOCK);
  cfg.dynamicSmemBytes = TRACE_SMEM_BYTES;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_batch_persistent, R);
}

cudaError_t launchStamp(unsigned long long *stamps, int first, int end, cudaStream_t st) {
  if (end <= first) return cudaSuccess;
  k_stamp<<<1, 32, 0, st>>>(stamps, first, end);
  return cudaGetLastError();
}

}  // namespace b200
