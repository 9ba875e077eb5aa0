// Two-level ray traversal of the quantised 8-wide BVH with watertight
// triangle and geometric sphere tests.  Replaces rtcIntersectV / rtcOccludedV
// as called from traceGeometryRay / isOccluded
// (modules/cpu/common/World.ih:29-52,311-380).
//
// Triangle test: Woop, Benthin, Wald, "Watertight Ray/Triangle
// Intersection", JCGT 2013.  Sphere test: Haines et al., "Precision
// Improvements for Ray/Sphere Intersection", Ray Tracing Gems 2019, ch. 7.
// Both run on non-contracted IEEE operations so a scalar CPU evaluation of
// the same formulas gives the same t bit for bit.  Equal-t ties resolve to
// the smallest (instID, geomID, primID), independent of traversal order.
#pragma once
#include "common.cuh"

namespace b200 {


struct HitRec {
  float t, u, v;
  V3 Ng;
  uint32_t primID, geomID, instID, entry;
};

// Per-thread traversal counters, filled only by the STATS instantiations.
struct TraceStats {
  uint32_t rays, nodes, tris, spheres;
};

struct Scene {
  const Node8 *tlas;         // root at 0 (empty when ntlas == 0)
  const uint32_t *tlasLeaf;   // entry index per TLAS leaf slot
  const Entry *entries;
  int nentries;
  int ntlas;
  int hasUser;                // an entry holds discs or planes or is motion-blurred (the traversal's out-of-line calls)
  float time;                 // ray time of the lane's queries (renderers set it per sample; 0 by default)
  uint32_t *status;           // bit 0: traversal stack overflow seen
  unsigned long long *counters;  // [rays, node visits, triangle tests, sphere tests]
};

// Adds a warp's per-thread counters to the scene counters (one atomic per
// field per warp).
B200_D void flushStats(const Scene &sc, const TraceStats &t) {
  uint32_t v[4] = {t.rays, t.nodes, t.tris, t.spheres};
#pragma unroll
  for (int k = 0; k < 4; k++) {
    uint32_t x = v[k];
    for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(__activemask(), x, o);
    v[k] = x;
  }
  if ((threadIdx.x & 31) == __ffs(__activemask()) - 1)
    for (int k = 0; k < 4; k++)
      if (v[k]) atomicAdd(sc.counters + k, (unsigned long long)v[k]);
}

// Per-ray constants of the watertight test: the axis permutation (kx, ky,
// kz packed in two bits each) and the shear.
struct TriPre {
  uint32_t k;
  float Sx, Sy, Sz;
  B200_D int kx() const { return int(k & 3u); }
  B200_D int ky() const { return int((k >> 2) & 3u); }
  B200_D int kz() const { return int(k >> 4); }
};

B200_D TriPre triPre(V3 d) {
  TriPre p;
  const V3 a = vabs(d);
  int kz = 0;
  if (a.y > comp(a, kz)) kz = 1;
  if (a.z > comp(a, kz)) kz = 2;
  int kx = kz == 2 ? 0 : kz + 1;
  int ky = kx == 2 ? 0 : kx + 1;
  if (comp(d, kz) < 0.f) {
    const int t = kx;
    kx = ky;
    ky = t;
  }
  p.k = uint32_t(kx) | uint32_t(ky) << 2 | uint32_t(kz) << 4;
  p.Sx = fdiv(comp(d, kx), comp(d, kz));
  p.Sy = fdiv(comp(d, ky), comp(d, kz));
  p.Sz = fdiv(1.f, comp(d, kz));
  return p;
}

B200_D bool triTest(const TriPre &p, V3 org, float tnear, float tfar, V3 v0, V3 v1, V3 v2, float &t, float &u,
                    float &v) {
  const V3 A = sub(v0, org), B = sub(v1, org), C = sub(v2, org);
  const int kx = p.kx(), ky = p.ky(), kz = p.kz();
  const float Akz = comp(A, kz), Bkz = comp(B, kz), Ckz = comp(C, kz);
  const float Ax = fsub(comp(A, kx), fmul(p.Sx, Akz));
  const float Ay = fsub(comp(A, ky), fmul(p.Sy, Akz));
  const float Bx = fsub(comp(B, kx), fmul(p.Sx, Bkz));
  const float By = fsub(comp(B, ky), fmul(p.Sy, Bkz));
  const float Cx = fsub(comp(C, kx), fmul(p.Sx, Ckz));
  const float Cy = fsub(comp(C, ky), fmul(p.Sy, Ckz));
  float U = fsub(fmul(Cx, By), fmul(Cy, Bx));
  float V = fsub(fmul(Ax, Cy), fmul(Ay, Cx));
  float W = fsub(fmul(Bx, Ay), fmul(By, Ax));
  if (U == 0.f || V == 0.f || W == 0.f) {
    U = float(__dsub_rn(__dmul_rn(double(Cx), double(By)), __dmul_rn(double(Cy), double(Bx))));
    V = float(__dsub_rn(__dmul_rn(double(Ax), double(Cy)), __dmul_rn(double(Ay), double(Cx))));
    W = float(__dsub_rn(__dmul_rn(double(Bx), double(Ay)), __dmul_rn(double(By), double(Ax))));
  }
  if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
  const float det = fadd(fadd(U, V), W);
  if (det == 0.f) return false;
  const float Az = fmul(p.Sz, Akz), Bz = fmul(p.Sz, Bkz), Cz = fmul(p.Sz, Ckz);
  const float T = fadd(fadd(fmul(U, Az), fmul(V, Bz)), fmul(W, Cz));
  t = fdiv(T, det);
  if (!(t >= tnear && t <= tfar)) return false;
  u = fdiv(V, det);
  v = fdiv(W, det);
  return true;
}

B200_D bool sphTest(V3 org, V3 d, float tnear, float tfar, float4 s, float &t, V3 &Ng) {
  const float rd2 = fdiv(1.f, dot(d, d));
  const V3 c0 = sub(mk(s.x, s.y, s.z), org);
  const float projC0 = fmul(dot(c0, d), rd2);
  const V3 perp = sub(c0, mul(projC0, d));
  const float l2 = dot(perp, perp);
  const float r2 = fmul(s.w, s.w);
  if (!(l2 <= r2)) return false;
  const float td = fsqrt(fmul(fsub(r2, l2), rd2));
  const float tf = fsub(projC0, td), tb = fadd(projC0, td);
  if (tf >= tnear && tf <= tfar)
    t = tf;
  else if (tb >= tnear && tb <= tfar)
    t = tb;
  else
    return false;
  Ng = sub(mul(t, d), c0);
  return true;
}

// Ray-facing disc (Embree 4.3.3's DISC_POINT, the reference's OSP_DISC): the
// disc through the centre perpendicular to the ray, hit at the centre's
// projection onto the ray when the ray passes within the radius; Ng = -d.
B200_D bool discTest(V3 org, V3 d, float tnear, float tfar, float4 s, float &t) {
  const float rd2 = fdiv(1.f, dot(d, d));
  const V3 c0 = sub(mk(s.x, s.y, s.z), org);
  const float projC0 = fmul(dot(c0, d), rd2);
  if (!(projC0 >= tnear && projC0 <= tfar)) return false;
  const V3 perp = sub(c0, mul(projC0, d));
  if (!(dot(perp, perp) <= fmul(s.w, s.w))) return false;
  t = projC0;
  return true;
}

// Oriented disc (Embree's ORIENTED_DISC_POINT, OSP_ORIENTED_DISC): the plane
// through the centre with normal n, hit inside the radius; Ng = n.
B200_D bool orientedDiscTest(V3 org, V3 d, float tnear, float tfar, float4 s, float4 n4, float &t) {
  const V3 n = mk(n4.x, n4.y, n4.z);
  const float div = dot(d, n);
  if (div == 0.f) return false;
  const V3 c = mk(s.x, s.y, s.z);
  const float tt = fdiv(dot(sub(c, org), n), div);
  if (!(tt >= tnear && tt <= tfar)) return false;
  const V3 q = sub(add(org, mul(d, tt)), c);
  if (!(dot(q, q) < fmul(s.w, s.w))) return false;
  t = tt;
  return true;
}

// Planes_intersect_kernel (geometry/Planes.ispc:40-78, intersectPlane and
// intersectBox common/Intersect.ih:195-237, filterIntersectionSingle
// common/FilterIntersect.ih): the plane n . P = d, hit for tnear < t <= tfar,
// inside the plane's box when it has one; Ng = n.
B200_D bool planeTest(V3 org, V3 d, float tnear, float tfar, const float4 *p, float &t) {
  const float4 c = __ldg(p);
  const V3 n = mk(c.x, c.y, c.z);
  const float DdN = dot(d, n);
  if (DdN == 0.f) return false;
  const float tt = fdiv(fsub(c.w, dot(org, n)), DdN);
  if (!(tt > tnear && tt <= tfar)) return false;
  const float4 lo = __ldg(p + 1);
  if (lo.w != 0.f) {
    const float4 hi = __ldg(p + 2);
    // rcp_safe: reciprocals of near-zero components clamped to 1e-18
    auto rs = [](float x) { return fdiv(1.f, fabsf(x) < 1e-18f ? copysignf(1e-18f, x) : x); };
    const V3 r = mk(rs(d.x), rs(d.y), rs(d.z));
    const V3 m0 = mk(fmul(fsub(lo.x, org.x), r.x), fmul(fsub(lo.y, org.y), r.y), fmul(fsub(lo.z, org.z), r.z));
    const V3 m1 = mk(fmul(fsub(hi.x, org.x), r.x), fmul(fsub(hi.y, org.y), r.y), fmul(fsub(hi.z, org.z), r.z));
    const float en = fmaxf(fmaxf(fminf(m0.x, m1.x), fminf(m0.y, m1.y)), fminf(m0.z, m1.z));
    const float ex = fminf(fminf(fmaxf(m0.x, m1.x), fmaxf(m0.y, m1.y)), fmaxf(m0.z, m1.z));
    if (!(en < ex) || tt < en || tt > ex) return false;
  }
  t = tt;
  return true;
}

// the disc and plane tests by type (out of line: the triangle and sphere
// tests of the traversal loop keep their registers); the hit distance, NaN
// for no hit (a value, not a reference, so no local of the loop lives in
// memory); Ng from userNormal
static __device__ __noinline__ float userTest(uint32_t type, V3 org, V3 d, float tnear, float tfar,
                                              const float4 *prims, uint32_t slot) {
  float t = 0.f;
  bool h;
  if (type == GEOM_DISCS)
    h = discTest(org, d, tnear, tfar, __ldg(prims + slot), t);
  else if (type == GEOM_ORIENTED_DISCS)
    h = orientedDiscTest(org, d, tnear, tfar, __ldg(prims + 2 * slot), __ldg(prims + 2 * slot + 1), t);
  else
    h = planeTest(org, d, tnear, tfar, prims + 3 * slot, t);
  return h ? t : __int_as_float(0x7fffffff);
}
// the ray (origin, direction) in a motion-blurred entry's frame at `time`
// (out of line, as the disc and plane tests; returned by value, so no
// traversal state has its address taken)
struct RayFrame {
  V3 o, d;
};
static __device__ __noinline__ RayFrame motionFrame(const Entry &e, float time, V3 org, V3 dir) {
  const Xfm r = rcpXfm(motionXfm(e.motionKeys, e.motionCount, e.motionT0, e.motionT1, time));
  return RayFrame{xfmPoint(r, org), xfmVector(r, dir)};
}
static __device__ __noinline__ V3 userNormal(uint32_t type, V3 d, const float4 *prims, uint32_t slot);

// The closest hit's u, v and geometric normal on a motion-blurred entry,
// re-evaluated in the entry's frame at the ray's time (Traverser::finish
// for such entries, out of line so that the traversal kernels keep their
// registers)
struct HitSurface {
  float u, v;
  V3 Ng;
};
static __device__ __noinline__ HitSurface finishMotion(const Entry &e, float time, Ray ray, float ht,
                                                        uint32_t hslot) {
  const RayFrame f = motionFrame(e, time, ray.org, ray.dir);
  HitSurface r = {0.f, 0.f, mk(0.f, 0.f, 0.f)};
  float t;
  if (e.type == GEOM_TRIANGLES) {
    const float4 a = __ldg(e.prims + 3 * hslot), b = __ldg(e.prims + 3 * hslot + 1),
                 c = __ldg(e.prims + 3 * hslot + 2);
    const V3 v0 = mk(a.x, a.y, a.z), v1 = mk(b.x, b.y, b.z), v2 = mk(c.x, c.y, c.z);
    triTest(triPre(f.d), f.o, ray.tnear, ht, v0, v1, v2, t, r.u, r.v);
    r.Ng = cross(sub(v1, v0), sub(v2, v0));
  } else if (e.type == GEOM_SPHERES) {
    sphTest(f.o, f.d, ray.tnear, ht, __ldg(e.prims + hslot), t, r.Ng);
  } else {
    r.Ng = userNormal(e.type, f.d, e.prims, hslot);
  }
  return r;
}

static __device__ __noinline__ V3 userNormal(uint32_t type, V3 d, const float4 *prims, uint32_t slot) {
  if (type == GEOM_DISCS) return neg(d);
  const float4 n = __ldg(prims + (type == GEOM_ORIENTED_DISCS ? 2 * slot + 1 : 3 * slot));
  return mk(n.x, n.y, n.z);
}

// Is a hit at t of (entry e, prim) better than the current closest
// (ht, hentry, hprim)?  Equal t resolves to the smallest (instID, geomID,
// primID); the IDs are read from the entries only for such ties.
B200_D bool better(const Scene &sc, float t, uint32_t e, uint32_t prim, float ht, uint32_t hentry,
                   uint32_t hprim) {
  if (t != ht) return t < ht;
  if (hentry == INVALID_ID) return true;
  if (e != hentry) {
    const uint32_t i0 = sc.entries[e].instID, i1 = sc.entries[hentry].instID;
    if (i0 != i1) return i0 < i1;
    return sc.entries[e].geomID < sc.entries[hentry].geomID;
  }
  return prim < hprim;
}

// The 80-byte node as five 16-byte words in registers.
struct NodeView {
  uint4 q[5];
  B200_D float px() const { return __uint_as_float(q[0].x); }
  B200_D float py() const { return __uint_as_float(q[0].y); }
  B200_D float pz() const { return __uint_as_float(q[0].z); }
  B200_D uint32_t exw() const { return q[0].w; }  // ex | ey<<8 | ez<<16 | imask<<24
  B200_D uint32_t childBase() const { return q[1].x; }
  B200_D uint32_t primBase() const { return q[1].y; }
  B200_D uint32_t meta(int i) const { return ((i < 4 ? q[1].z : q[1].w) >> (8 * (i & 3))) & 0xffu; }
  // quantised byte b of the 48-byte box block (qlo[3][8] then qhi[3][8])
  B200_D uint32_t qbyte(int b) const {
    const int w = b >> 2;  // word in q[2..4]
    const uint4 v = q[2 + (w >> 2)];
    const uint32_t word = (w & 3) == 0 ? v.x : ((w & 3) == 1 ? v.y : ((w & 3) == 2 ? v.z : v.w));
    return (word >> (8 * (b & 3))) & 0xffu;
  }
};

B200_D NodeView loadNode(const Node8 *nodes, uint32_t i) {
  const uint4 *p = reinterpret_cast<const uint4 *>(nodes + i);
  NodeView n;
#pragma unroll
  for (int k = 0; k < 5; k++) n.q[k] = __ldg(p + k);
  return n;
}

B200_D float max3f(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
B200_D float min3f(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// byte b of w as a float (an integer-to-float conversion: forming it as a
// byte permute into the mantissa of 2^23 minus 2^23 instead cost the
// issue-bound path-tracer trace kernels 3 %)
B200_D float u8f(uint32_t w, int b) { return float((w >> (8 * b)) & 0xffu); }

// Intersects the node's 8 child boxes with the ray (direction octant oct).
// keys: the hit internal children, child slot i at bit i ^ oct, so the
// lowest set bit is the next child in the octant's visiting order.  prims:
// the leaf primitive slots (relative to primBase) of the hit leaf children.
//
// Slab distances are formed on the quantisation grid directly in t units,
// t = q * (2^e * rdir) + (p - org) * rdir, one FMA per plane; the near and
// far planes of each axis are chosen per ray octant on whole 4-child words.
// The comparison is widened by 8e-7 relative (about 7 ulp) on the exit and on
// tfar, so rounding never culls a box the ray touches.
B200_D void intersectChildren(const NodeView &n, V3 org, V3 rdir, float tnear, float tfar, uint32_t oct,
                              uint32_t &keys, uint32_t &prims) {
  const uint32_t e = n.exw();
  const float ax = __uint_as_float((e & 0xffu) << 23) * rdir.x;
  const float ay = __uint_as_float(((e >> 8) & 0xffu) << 23) * rdir.y;
  const float az = __uint_as_float(((e >> 16) & 0xffu) << 23) * rdir.z;
  const float bx = (n.px() - org.x) * rdir.x, by = (n.py() - org.y) * rdir.y, bz = (n.pz() - org.z) * rdir.z;
  const bool xn = rdir.x < 0.f, yn = rdir.y < 0.f, zn = rdir.z < 0.f;
  // box block words: qlo x/y/z = q2.xy, q2.zw, q3.xy; qhi x/y/z = q3.zw, q4.xy, q4.zw
  const uint32_t nx0 = xn ? n.q[3].z : n.q[2].x, nx1 = xn ? n.q[3].w : n.q[2].y;
  const uint32_t fx0 = xn ? n.q[2].x : n.q[3].z, fx1 = xn ? n.q[2].y : n.q[3].w;
  const uint32_t ny0 = yn ? n.q[4].x : n.q[2].z, ny1 = yn ? n.q[4].y : n.q[2].w;
  const uint32_t fy0 = yn ? n.q[2].z : n.q[4].x, fy1 = yn ? n.q[2].w : n.q[4].y;
  const uint32_t nz0 = zn ? n.q[4].z : n.q[3].x, nz1 = zn ? n.q[4].w : n.q[3].y;
  const uint32_t fz0 = zn ? n.q[3].x : n.q[4].z, fz1 = zn ? n.q[3].y : n.q[4].w;
  const float tmax = tfar * 1.0000008f;
  keys = 0;
  prims = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const uint32_t meta = n.meta(i);
    if (meta == 0) continue;
    const int by8 = i & 3;
    const float tnx = fmaf(u8f(i < 4 ? nx0 : nx1, by8), ax, bx);
    const float tfx = fmaf(u8f(i < 4 ? fx0 : fx1, by8), ax, bx);
    const float tny = fmaf(u8f(i < 4 ? ny0 : ny1, by8), ay, by);
    const float tfy = fmaf(u8f(i < 4 ? fy0 : fy1, by8), ay, by);
    const float tnz = fmaf(u8f(i < 4 ? nz0 : nz1, by8), az, bz);
    const float tfz = fmaf(u8f(i < 4 ? fz0 : fz1, by8), az, bz);
    const float t0 = max3f(tnx, tny, fmaxf(tnz, tnear));
    const float t1 = min3f(tfx, tfy, tfz) * 1.0000008f;
    if (t0 <= fminf(t1, tmax)) {
      if (meta & 0x80u)
        keys |= 1u << (uint32_t(i) ^ oct);
      else
        prims |= ((1u << (meta >> 5)) - 1u) << (meta & 31u);
    }
  }
}

B200_D uint32_t octantOf(V3 d) {
  return (d.x < 0.f ? 1u : 0u) | (d.y < 0.f ? 2u : 0u) | (d.z < 0.f ? 4u : 0u);
}

// ---------------------------------------------------------------- traversal
// Compressed-wide-BVH traversal after Ylitie, Karras, Laine, "Efficient
// Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs" (HPG 2017).
// Nothing is sorted at run time: a node's hit internal children form one
// node group (child base, 8 hit bits in the octant's visiting order, the
// node's internal-child mask) and its hit leaf primitives one primitive group
// (primitive base, 24 hit bits).  Each node visit pushes at most the rest of
// the current node group.  Primitive tests are postponed (the group pushed)
// while only a few lanes of the warp would run them and node work is
// pending, so lanes stay busy with node visits.
//
// Both levels share one stack.  Entries carry their kind in the top two bits
// of the second word: TLAS node group, BLAS node group, TLAS instance group
// (TLAS leaf slots) or BLAS primitive group.  Popping a TLAS entry while in a
// BLAS ends the current instance.
//
// The first STACK_SMEM entries of each thread live in shared memory, one
// column per thread (entry k of thread t at word k * TRACE_BLOCK + t, so a
// warp's accesses are conflict-free); deeper entries spill to a short local
// array.  Kernels that trace declare TRACE_SMEM_BYTES of dynamic shared
// memory and launch TRACE_BLOCK threads per block.
// The shared-memory stack depth and the trace kernels' minimum resident
// blocks per SM are build parameters (ospray_gb300/tuned.json, chosen by
// ospray_gb300/tune_build.py on the GPU).
#ifndef B200_STACK_SMEM
#define B200_STACK_SMEM 16
#endif
#ifndef B200_BATCH_TRACE_MINBLOCKS
#define B200_BATCH_TRACE_MINBLOCKS 6  // the batched wavefront's trace kernels (their own register budget)
#endif
#ifndef B200_TRACE_MINBLOCKS
#define B200_TRACE_MINBLOCKS 1
#endif
// Primitive tests per traversal step, and the lane count below which a
// lane postpones its primitive group while a node group is pending: the
// single-frame path tracer's persistent queue kernels (B200_QUEUE_*, whose
// warps refill finished lanes) run one test per step and never postpone the
// first (1,102 Mrays/s on the 1080p instanced-spheres frame; postponing
// below 8 lanes: 1,077, below 16: 1,073; 2 tests per step: 1,060, 4: 1,042,
// a whole group: 1,039).  The choice depends on the scene: on the batch's
// height fields whole groups are faster (1,505 vs 1,469 Mrays/s batched,
// 1,121 vs 1,103 for the same requests one at a time), so the batch keeps
// them, as does traceRay (whole warps that trace together, the AO and
// SciVis kernels: AO within its run-to-run spread either way).
#ifndef B200_PRIMS_PER_STEP
#define B200_PRIMS_PER_STEP 64
#endif
#ifndef B200_POSTPONE_LANES
#define B200_POSTPONE_LANES 8
#endif
#ifndef B200_QUEUE_PRIMS_PER_STEP
#define B200_QUEUE_PRIMS_PER_STEP 1
#endif
#ifndef B200_QUEUE_POSTPONE_LANES
#define B200_QUEUE_POSTPONE_LANES 0
#endif
constexpr int TRACE_BLOCK = 128;
constexpr int STACK_SMEM = B200_STACK_SMEM;
constexpr int STACK_LOCAL = STACK_SMEM < 40 ? 48 - STACK_SMEM : 8;  // 48 entries in all
constexpr size_t TRACE_SMEM_BYTES = size_t(STACK_SMEM) * TRACE_BLOCK * sizeof(uint2);

constexpr uint32_t G_TNODE = 0u << 30, G_BNODE = 1u << 30, G_TINST = 2u << 30, G_BPRIM = 3u << 30;
constexpr uint32_t G_KIND = 3u << 30, G_BLAS = 1u << 30, G_PRIMS = 2u << 30;

// Entries beyond the shared-memory column go to a per-thread overflow array
// that the caller declares (TraceSpill) and the stack points to; keeping that
// dynamically indexed array outside the traverser lets the compiler hold the
// traverser's own fields in registers.
struct TraceSpill {
  uint2 e[STACK_LOCAL];
  float time;  // the ray's time (motion-blurred instances), read by the traverser from here
};

struct TraceStack {
  uint2 *smem;   // this thread's column
  uint2 *local;  // this thread's overflow array
  int sp;
  B200_D void push(uint2 item, uint32_t *status) {
    if (sp < STACK_SMEM) {
      smem[sp * TRACE_BLOCK] = item;
    } else if (sp < STACK_SMEM + STACK_LOCAL) {
      local[sp - STACK_SMEM] = item;
    } else {
      atomicOr(status, 1u);  // overflow: the entry is dropped and reported
      return;
    }
    sp++;
  }
  B200_D uint2 pop() {
    --sp;
    return sp < STACK_SMEM ? smem[sp * TRACE_BLOCK] : local[sp - STACK_SMEM];
  }
};

// this thread's stack column in the kernel's dynamic shared memory
B200_D uint2 *traceStackBase() {
  extern __shared__ uint2 s_traceStack[];
  return s_traceStack + threadIdx.x;
}

// Resumable traversal of one ray: init() sets it up, each step() visits one
// node and tests the primitives it exposes, until it reports the ray
// finished.  Kernels drive the steps so that the lanes of a warp stay in
// lockstep and can replace finished rays with new ones.
struct Traverser {
  TraceStack st;
  Ray ray;
  V3 org, dir, rdir;  // current frame
  TriPre pre;
  const Node8 *nodes;
  const float4 *prims;
  const uint32_t *primIDs;
  uint32_t etype, eidx;
  uint32_t nbase, nbits;  // node group: child base; hit keys (bits 0-7) | imask << 8
  uint32_t pbase, pbits;  // primitive group: slot base; hit slots (bits 0-23)
  uint32_t oct;           // direction octant of the current frame
  bool inBlas, anyHit, found;
  // the closest hit so far: distance, primitive ID, entry, leaf slot; the
  // rest of the record is formed once by finish()
  float ht;
  uint32_t hprim, hentry, hslot;
  HitRec hit;

  B200_D void init(const Scene &sc, const Ray &r, bool any, TraceSpill *spill) {
    ray = r;
    anyHit = any;
    st.smem = traceStackBase();
    st.local = spill->e;
    st.sp = 0;
    ht = r.tfar;
    hprim = hentry = hslot = INVALID_ID;
    org = r.org;
    dir = r.dir;
    rdir = mk(1.f / r.dir.x, 1.f / r.dir.y, 1.f / r.dir.z);
    oct = octantOf(r.dir);
    nodes = sc.tlas;
    prims = nullptr;
    primIDs = nullptr;
    etype = eidx = 0;
    inBlas = false;
    found = false;
    // the TLAS root as a one-child group
    nbase = 0;
    nbits = sc.ntlas > 0 ? ((1u << oct) | (1u << 8)) : 0u;
    pbase = pbits = 0;
  }

  B200_D bool idle() const { return !(nbits & 0xffu) && !pbits && st.sp == 0; }

  // the ray's time, kept beside the local stack entries (TraceSpill)
  B200_D float rayTime() const { return reinterpret_cast<const TraceSpill *>(st.local)->time; }

  template <bool MOTION = true>
  B200_D void enterInstance(const Scene &sc, uint32_t entry) {
    eidx = entry;
    const Entry &e = sc.entries[eidx];
    nodes = e.nodes;
    prims = e.prims;
    primIDs = e.primIDs;
    etype = e.type;
    if (MOTION && e.motionCount > 1) {
      const RayFrame f = motionFrame(e, rayTime(), ray.org, ray.dir);
      org = f.o;
      dir = f.d;
      rdir = mk(1.f / dir.x, 1.f / dir.y, 1.f / dir.z);
    } else if (!e.identity) {
      const Xfm r = e.rcp;
      org = xfmPoint(r, ray.org);
      dir = xfmVector(r, ray.dir);
      rdir = mk(1.f / dir.x, 1.f / dir.y, 1.f / dir.z);
    }
    pre = triPre(dir);
    oct = octantOf(dir);
    inBlas = true;
    nbase = 0;
    nbits = (1u << oct) | (1u << 8);
  }

  B200_D void leaveInstance(const Scene &sc) {
    inBlas = false;
    nodes = sc.tlas;
    org = ray.org;
    dir = ray.dir;
    rdir = mk(1.f / ray.dir.x, 1.f / ray.dir.y, 1.f / ray.dir.z);
    oct = octantOf(ray.dir);
  }

  // The full hit record of the closest hit: u, v and the geometric normal
  // re-evaluated on the hit primitive in its entry's frame with the same
  // operations as during traversal (so identical values), and the IDs.
  // USER = false: the scene has no discs or planes (Scene::hasUser), so no
  // out-of-line call is compiled into the caller.  DEFER: u, v and Ng of a
  // hit on a motion-blurred entry are not valid (taken in the entry's static
  // frame); the caller hands the leaf slot hslot to postIntersect, which
  // re-evaluates them at the ray's time, so the wavefront trace kernels
  // carry no call here.
  // MOTION = false: no entry is motion-blurred (no motion code compiled in).
  template <bool USER = true, bool DEFER = false, bool MOTION = USER>
  B200_D void finish(const Scene &sc) {
    hit.t = ht;
    hit.primID = hprim;
    hit.entry = hentry;
    hit.u = hit.v = 0.f;
    hit.Ng = mk(0.f, 0.f, 0.f);
    hit.instID = hit.geomID = INVALID_ID;
    if (!found) return;
    const Entry &e = sc.entries[hentry];
    hit.instID = e.instID;
    hit.geomID = e.geomID;
    if (MOTION && !DEFER && e.motionCount > 1) {  // the whole re-evaluation out of line
      const HitSurface f = finishMotion(e, rayTime(), ray, ht, hslot);
      hit.u = f.u;
      hit.v = f.v;
      hit.Ng = f.Ng;
      return;
    }
    V3 o = ray.org, d = ray.dir;
    if (!e.identity) {
      const Xfm r = e.rcp;
      o = xfmPoint(r, ray.org);
      d = xfmVector(r, ray.dir);
    }
    float t;
    if (e.type == GEOM_TRIANGLES) {
      const float4 a = __ldg(e.prims + 3 * hslot), b = __ldg(e.prims + 3 * hslot + 1),
                   c = __ldg(e.prims + 3 * hslot + 2);
      const V3 v0 = mk(a.x, a.y, a.z), v1 = mk(b.x, b.y, b.z), v2 = mk(c.x, c.y, c.z);
      triTest(triPre(d), o, ray.tnear, ht, v0, v1, v2, t, hit.u, hit.v);
      hit.Ng = cross(sub(v1, v0), sub(v2, v0));
    } else if (!USER || e.type == GEOM_SPHERES) {
      sphTest(o, d, ray.tnear, ht, __ldg(e.prims + hslot), t, hit.Ng);
    } else {
      hit.Ng = userNormal(e.type, d, e.prims, hslot);
    }
  }

  // one traversal step; true when the ray is finished (USER as for finish;
  // PPS and POSTPONE as B200_PRIMS_PER_STEP and B200_POSTPONE_LANES)
  template <bool STATS, bool USER = true, int PPS = B200_PRIMS_PER_STEP, int POSTPONE = B200_POSTPONE_LANES,
            bool MOTION = USER>
  B200_D bool step(const Scene &sc, TraceStats *ts) {
    // 1) the next node of the current node group
    if (nbits & 0xffu) {
      const uint32_t key = uint32_t(__ffs(nbits & 0xffu) - 1);
      nbits &= ~(1u << key);
      const uint32_t slot = key ^ oct;
      const uint32_t child = nbase + uint32_t(__popc((nbits >> 8) & ((1u << slot) - 1u)));
      if (nbits & 0xffu) st.push(make_uint2(nbase, nbits | (inBlas ? G_BNODE : G_TNODE)), sc.status);
      const NodeView n = loadNode(nodes, child);
      if (STATS) ts->nodes++;
      uint32_t keys, hitPrims;
      intersectChildren(n, org, rdir, ray.tnear, ht, oct, keys, hitPrims);
      nbase = n.childBase();
      nbits = keys | (((n.exw() >> 24) & 0xffu) << 8);
      pbase = n.primBase();
      pbits = hitPrims;
    }
    // 2) the primitives of the current primitive group (at most PPS per
    // step: the rest wait for the next step, on the stack when a node group
    // is pending)
    for (int np = 0; pbits; np++) {
      if ((nbits & 0xffu) && (np >= PPS || __popc(__activemask()) < POSTPONE)) {
        st.push(make_uint2(pbase, pbits | (inBlas ? G_BPRIM : G_TINST)), sc.status);
        pbits = 0;
        break;
      }
      if (np >= PPS) break;
      const uint32_t k = uint32_t(__ffs(pbits) - 1);
      pbits &= pbits - 1u;
      const uint32_t slot = pbase + k;
      if (!inBlas) {
        // a TLAS leaf slot: enter its instance; the rest of this level waits
        // on the stack (remaining instances above the node group)
        if (nbits & 0xffu) st.push(make_uint2(nbase, nbits | G_TNODE), sc.status);
        if (pbits) st.push(make_uint2(pbase, pbits | G_TINST), sc.status);
        pbits = 0;
        enterInstance<MOTION>(sc, __ldg(sc.tlasLeaf + slot));
        break;
      }
      float t;
      uint32_t prim;
      bool h;
      if (STATS) (etype == GEOM_TRIANGLES ? ts->tris : ts->spheres)++;
      if (etype == GEOM_TRIANGLES) {
        const float4 a = __ldg(prims + 3 * slot), b = __ldg(prims + 3 * slot + 1), c = __ldg(prims + 3 * slot + 2);
        float u, v;
        h = triTest(pre, org, ray.tnear, ht, mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), mk(c.x, c.y, c.z), t, u, v);
        prim = __float_as_uint(a.w);
      } else {
        if (!USER || etype == GEOM_SPHERES) {
          V3 Ng;
          h = sphTest(org, dir, ray.tnear, ht, __ldg(prims + slot), t, Ng);
        } else {
          t = userTest(etype, org, dir, ray.tnear, ht, prims, slot);
          h = !isnan(t);
        }
        prim = __ldg(primIDs + slot);
      }
      if (h && better(sc, t, eidx, prim, ht, hentry, hprim)) {
        ht = t;
        hprim = prim;
        hentry = eidx;
        hslot = slot;
        found = true;
        if (anyHit) return true;
      }
    }
    // 3) both groups empty: the next group from the stack
    if (!(nbits & 0xffu) && !pbits) {
      if (st.sp == 0) return true;
      const uint2 s = st.pop();
      const uint32_t kind = s.y & G_KIND;
      if (inBlas && !(kind & G_BLAS)) leaveInstance(sc);
      if (kind & G_PRIMS) {
        pbase = s.x;
        pbits = s.y & 0xffffffu;
        nbits = 0;
      } else {
        nbase = s.x;
        nbits = s.y & 0xffffu;
      }
    }
    return false;
  }
};

// Closest hit or any hit over the whole scene, for one ray per lane.  anyHit
// selects occlusion (stop at the first hit) at run time, so a kernel that
// traces both kinds of rays needs one copy of the traversal code.
//
// The lanes that call together trace together: every step starts with a
// vote over those lanes, which is also where they reconverge; a lane whose
// ray is finished idles until the last lane of its group is done.  Without
// this the lanes of a warp drift to different points of the data-dependent
// loop and execute one at a time.  `active == false` makes a lane take part
// without tracing anything.
//
// SPLIT: two copies of the loop, one without the out-of-line disc and plane
// tests for scenes that have none (Scene::hasUser); without SPLIT one loop
// with them (smaller code, for callers inside large kernels).
// MOTION = false: the caller never sees motion-blurred instances.
template <bool STATS = false, bool SPLIT = true, bool MOTION = true>
B200_D bool traceRay(const Scene &sc, const Ray &ray, HitRec &hit, bool anyHit, bool active = true,
                     TraceStats *ts = nullptr, float time = -1.f) {
  if (STATS && active) ts->rays++;
  const unsigned group = __activemask();
  Traverser tv;
  TraceSpill spill;
  spill.time = time >= 0.f ? time : sc.time;  // (a negative time: the scene's)
  tv.init(sc, ray, anyHit, &spill);
  bool done = !active || tv.idle();
  // the lanes' scenes may differ in a batch: the choice is made for the group
  if (!SPLIT || __any_sync(group, sc.hasUser != 0)) {
    for (int guard = 0; guard < (1 << 18); guard++) {
      if (!__any_sync(group, !done)) break;
      if (!done) done = tv.step<STATS, true, B200_PRIMS_PER_STEP, B200_POSTPONE_LANES, MOTION>(sc, ts);
    }
    if (!anyHit) tv.finish<true, false, MOTION>(sc);
  } else {
    for (int guard = 0; guard < (1 << 18); guard++) {
      if (!__any_sync(group, !done)) break;
      if (!done) done = tv.step<STATS, false>(sc, ts);
    }
    if (!anyHit) tv.finish<false>(sc);
  }
  hit = tv.hit;
  return tv.found;
}

// Closest hit (ANY = false) or any hit (ANY = true), at the scene's ray time.
template <bool ANY, bool STATS = false>
B200_D bool traceScene(const Scene &sc, const Ray &ray, HitRec &hit, TraceStats *ts = nullptr) {
  return traceRay<STATS>(sc, ray, hit, ANY, true, ts);
}

}  // namespace b200
