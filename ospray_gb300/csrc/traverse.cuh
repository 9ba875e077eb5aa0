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

struct TriPre {
  int kx, ky, kz;
  float Sx, Sy, Sz;
};

B200_D TriPre triPre(V3 d) {
  TriPre p;
  const V3 a = vabs(d);
  p.kz = 0;
  if (a.y > comp(a, p.kz)) p.kz = 1;
  if (a.z > comp(a, p.kz)) p.kz = 2;
  p.kx = p.kz == 2 ? 0 : p.kz + 1;
  p.ky = p.kx == 2 ? 0 : p.kx + 1;
  if (comp(d, p.kz) < 0.f) {
    const int t = p.kx;
    p.kx = p.ky;
    p.ky = t;
  }
  p.Sx = fdiv(comp(d, p.kx), comp(d, p.kz));
  p.Sy = fdiv(comp(d, p.ky), comp(d, p.kz));
  p.Sz = fdiv(1.f, comp(d, p.kz));
  return p;
}

B200_D bool triTest(const TriPre &p, V3 org, float tnear, float tfar, V3 v0, V3 v1, V3 v2, float &t, float &u,
                    float &v) {
  const V3 A = sub(v0, org), B = sub(v1, org), C = sub(v2, org);
  const float Akz = comp(A, p.kz), Bkz = comp(B, p.kz), Ckz = comp(C, p.kz);
  const float Ax = fsub(comp(A, p.kx), fmul(p.Sx, Akz));
  const float Ay = fsub(comp(A, p.ky), fmul(p.Sy, Akz));
  const float Bx = fsub(comp(B, p.kx), fmul(p.Sx, Bkz));
  const float By = fsub(comp(B, p.ky), fmul(p.Sy, Bkz));
  const float Cx = fsub(comp(C, p.kx), fmul(p.Sx, Ckz));
  const float Cy = fsub(comp(C, p.ky), fmul(p.Sy, Ckz));
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

B200_D bool better(float t, uint32_t inst, uint32_t geom, uint32_t prim, const HitRec &h) {
  if (t != h.t) return t < h.t;
  if (inst != h.instID) return inst < h.instID;
  if (geom != h.geomID) return geom < h.geomID;
  return prim < h.primID;
}

// Loads a node and intersects its 8 child boxes.  Returns a bit mask of hit
// children; dist[i] holds the entry distance of hit child i.
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

B200_D uint32_t intersectChildren(const NodeView &n, V3 org, V3 rdir, float tnear, float tfar, float dist[8]) {
  const uint32_t e = n.exw();
  const float sx = __uint_as_float((e & 0xffu) << 23);
  const float sy = __uint_as_float(((e >> 8) & 0xffu) << 23);
  const float sz = __uint_as_float(((e >> 16) & 0xffu) << 23);
  // near/far planes chosen per axis from the ray octant; every byte index is
  // a compile-time constant so the node stays in registers
  const bool xn = rdir.x < 0.f, yn = rdir.y < 0.f, zn = rdir.z < 0.f;
  const float ox = n.px() - org.x, oy = n.py() - org.y, oz = n.pz() - org.z;
  uint32_t mask = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    dist[i] = INFINITY;
    if (n.meta(i) == 0) continue;
    const float lx = fmaf(float(n.qbyte(0 + i)), sx, ox), hx = fmaf(float(n.qbyte(24 + i)), sx, ox);
    const float ly = fmaf(float(n.qbyte(8 + i)), sy, oy), hy = fmaf(float(n.qbyte(32 + i)), sy, oy);
    const float lz = fmaf(float(n.qbyte(16 + i)), sz, oz), hz = fmaf(float(n.qbyte(40 + i)), sz, oz);
    const float t0x = (xn ? hx : lx) * rdir.x, t1x = (xn ? lx : hx) * rdir.x;
    const float t0y = (yn ? hy : ly) * rdir.y, t1y = (yn ? ly : hy) * rdir.y;
    const float t0z = (zn ? hz : lz) * rdir.z, t1z = (zn ? lz : hz) * rdir.z;
    const float t0 = fmaxf(fmaxf(t0x, t0y), fmaxf(t0z, tnear));
    const float t1 = fminf(fminf(t1x, t1y), t1z) * 1.0000004f;
    if (t0 <= fminf(t1, tfar)) {
      mask |= 1u << i;
      dist[i] = t0;
    }
  }
  return mask;
}

// a[i] for a runtime i without dynamic indexing (keeps `a` in registers)
B200_D float pick8(const float (&a)[8], int i) {
  float r = a[0];
#pragma unroll
  for (int k = 1; k < 8; k++) r = (i == k) ? a[k] : r;
  return r;
}

// ---------------------------------------------------------------- traversal
// One stack serves both levels.  Items carry a 2-bit tag in the top bits of
// the word: TLAS node, BLAS node of the instance being traversed, or an
// instance (entry index) still to enter.  BLAS items always sit above the
// TLAS/instance items pushed before their instance was entered, so popping a
// non-BLAS item means the current instance is finished.
//
// The first STACK_SMEM items of each thread live in shared memory, one
// column per thread (item k of thread t at word k * TRACE_BLOCK + t, so a
// warp's accesses are conflict-free); deeper items spill to a short local
// array.  Kernels that trace declare TRACE_SMEM_BYTES of dynamic shared
// memory and launch TRACE_BLOCK threads per block.
// The shared-memory stack depth and the trace kernels' minimum resident
// blocks per SM are build parameters (ospray_gb300/tuned.json, chosen by
// ospray_gb300/tune_build.py on the GPU).
#ifndef B200_STACK_SMEM
#define B200_STACK_SMEM 24
#endif
#ifndef B200_TRACE_MINBLOCKS
#define B200_TRACE_MINBLOCKS 1
#endif
constexpr int TRACE_BLOCK = 128;
constexpr int STACK_SMEM = B200_STACK_SMEM;
constexpr int STACK_LOCAL = STACK_SMEM < 56 ? 64 - STACK_SMEM : 8;  // 64 entries in all
constexpr size_t TRACE_SMEM_BYTES = size_t(STACK_SMEM) * TRACE_BLOCK * sizeof(uint2);

constexpr uint32_t TAG_TLAS = 0u, TAG_BLAS = 1u << 30, TAG_INST = 2u << 30, TAG_MASK = 3u << 30;

struct TraceStack {
  uint2 *smem;  // this thread's column
  uint2 local[STACK_LOCAL];
  int sp;
  B200_D bool push(uint32_t item, float dist, uint32_t *status) {
    if (sp < STACK_SMEM) {
      smem[sp * TRACE_BLOCK] = make_uint2(item, __float_as_uint(dist));
    } else if (sp < STACK_SMEM + STACK_LOCAL) {
      local[sp - STACK_SMEM] = make_uint2(item, __float_as_uint(dist));
    } else {
      atomicOr(status, 1u);  // overflow: the item is dropped and reported
      return false;
    }
    sp++;
    return true;
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

// Resumable traversal of one ray: init() sets it up, each step() pops or
// visits one node (testing the node's leaf primitives), until it reports the
// ray finished.  Kernels drive the steps so that the lanes of a warp stay in
// lockstep and can replace finished rays with new ones.
struct Traverser {
  TraceStack st;
  Ray ray;
  V3 wrdir, org, dir, rdir;  // world reciprocal direction; current frame
  TriPre pre;
  const Node8 *nodes;
  const float4 *prims;
  const uint32_t *primIDs;
  uint32_t etype, einst, egeom, eidx, node;
  bool inBlas, have, anyHit, found;
  HitRec hit;

  B200_D void init(const Scene &sc, const Ray &r, bool any) {
    ray = r;
    anyHit = any;
    st.smem = traceStackBase();
    st.sp = 0;
    hit.t = r.tfar;
    hit.u = hit.v = 0.f;
    hit.primID = hit.geomID = hit.instID = hit.entry = INVALID_ID;
    wrdir = mk(1.f / r.dir.x, 1.f / r.dir.y, 1.f / r.dir.z);
    org = r.org;
    dir = r.dir;
    rdir = wrdir;
    nodes = sc.tlas;
    prims = nullptr;
    primIDs = nullptr;
    etype = einst = egeom = eidx = 0;
    node = 0;
    inBlas = false;
    found = false;
    have = sc.ntlas > 0;
  }

  // one traversal step; true when the ray is finished
  template <bool STATS>
  B200_D bool step(const Scene &sc, TraceStats *ts) {
    if (!have) {
      // pop until an entry that can still hold a closer hit (culled entries
      // cost no step of their own)
      uint2 s;
      do {
        if (st.sp == 0) return true;
        s = st.pop();
      } while (__uint_as_float(s.y) > hit.t);
      const uint32_t tag = s.x & TAG_MASK;
      if (tag != TAG_BLAS && inBlas) {
        inBlas = false;
        nodes = sc.tlas;
        org = ray.org;
        dir = ray.dir;
        rdir = wrdir;
      }
      if (tag == TAG_INST) {
        eidx = s.x & ~TAG_MASK;
        const Entry &e = sc.entries[eidx];
        nodes = e.nodes;
        prims = e.prims;
        primIDs = e.primIDs;
        etype = e.type;
        einst = e.instID;
        egeom = e.geomID;
        if (!e.identity) {
          const Xfm r = e.rcp;
          org = xfmPoint(r, ray.org);
          dir = xfmVector(r, ray.dir);
          rdir = mk(1.f / dir.x, 1.f / dir.y, 1.f / dir.z);
        }
        pre = triPre(dir);
        inBlas = true;
        node = 0;
      } else {
        node = s.x & ~TAG_MASK;
      }
    }
    have = false;
    const NodeView n = loadNode(nodes, node);
    if (STATS) ts->nodes++;
    float dist[8];
    const uint32_t mask = intersectChildren(n, org, rdir, ray.tnear, hit.t, dist);
    if (!mask) return false;
    if (!inBlas) {
      // TLAS node: internal children and instances go on the stack, farthest
      // first, so the nearest is popped first and tightens hit.t early
      for (uint32_t m = mask; m;) {
        int i = __ffs(m) - 1;
        float di = pick8(dist, i);
        for (uint32_t r = m & (m - 1); r; r &= r - 1) {
          const int j = __ffs(r) - 1;
          const float dj = pick8(dist, j);
          if (dj > di) {
            i = j;
            di = dj;
          }
        }
        m &= ~(1u << i);
        const uint32_t meta = n.meta(i);
        if (meta & 0x80u) {
          st.push(TAG_TLAS | (n.childBase() + (meta & 7u)), di, sc.status);
        } else {
          const uint32_t cnt = meta >> 5, first = n.primBase() + (meta & 31u);
          for (uint32_t k = 0; k < cnt; k++) st.push(TAG_INST | __ldg(sc.tlasLeaf + first + k), di, sc.status);
        }
      }
      return false;
    }
    // BLAS node: leaves first (they tighten hit.t), then internal children
    for (uint32_t m = mask; m; m &= m - 1) {
      const int i = __ffs(m) - 1;
      const uint32_t meta = n.meta(i);
      if (meta & 0x80u) continue;
      const uint32_t cnt = meta >> 5, first = n.primBase() + (meta & 31u);
      for (uint32_t k = 0; k < cnt; k++) {
        const uint32_t slot = first + k;
        float t, u = 0.f, v = 0.f;
        V3 Ng;
        uint32_t prim;
        bool h;
        if (STATS) (etype == GEOM_TRIANGLES ? ts->tris : ts->spheres)++;
        if (etype == GEOM_TRIANGLES) {
          const float4 a = __ldg(prims + 3 * slot), b = __ldg(prims + 3 * slot + 1), c = __ldg(prims + 3 * slot + 2);
          const V3 v0 = mk(a.x, a.y, a.z), v1 = mk(b.x, b.y, b.z), v2 = mk(c.x, c.y, c.z);
          h = triTest(pre, org, ray.tnear, hit.t, v0, v1, v2, t, u, v);
          if (h) Ng = cross(sub(v1, v0), sub(v2, v0));
          prim = __float_as_uint(a.w);
        } else {
          h = sphTest(org, dir, ray.tnear, hit.t, __ldg(prims + slot), t, Ng);
          prim = __ldg(primIDs + slot);
        }
        if (h && better(t, einst, egeom, prim, hit)) {
          hit.t = t;
          hit.u = u;
          hit.v = v;
          hit.Ng = Ng;
          hit.primID = prim;
          hit.geomID = egeom;
          hit.instID = einst;
          hit.entry = eidx;
          found = true;
        }
      }
    }
    if (anyHit && found) return true;
    // internal children still in reach: the nearest is visited next, the
    // others are pushed farthest first
    uint32_t inner = 0;
    for (uint32_t m = mask; m; m &= m - 1) {
      const int i = __ffs(m) - 1;
      if ((n.meta(i) & 0x80u) && pick8(dist, i) <= hit.t) inner |= 1u << i;
    }
    while (inner) {
      int i = __ffs(inner) - 1;
      float di = pick8(dist, i);
      for (uint32_t r = inner & (inner - 1); r; r &= r - 1) {
        const int j = __ffs(r) - 1;
        const float dj = pick8(dist, j);
        if (dj > di) {
          i = j;
          di = dj;
        }
      }
      inner &= ~(1u << i);
      const uint32_t child = n.childBase() + (n.meta(i) & 7u);
      if (!inner) {
        node = child;
        have = true;
      } else {
        st.push(TAG_BLAS | child, di, sc.status);
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
template <bool STATS = false>
B200_D bool traceRay(const Scene &sc, const Ray &ray, HitRec &hit, bool anyHit, bool active = true,
                     TraceStats *ts = nullptr) {
  if (STATS && active) ts->rays++;
  const unsigned group = __activemask();
  Traverser tv;
  tv.init(sc, ray, anyHit);
  bool done = !active || !tv.have;
  for (int guard = 0; guard < (1 << 18); guard++) {
    if (!__any_sync(group, !done)) break;
    if (!done) done = tv.step<STATS>(sc, ts);
  }
  hit = tv.hit;
  return tv.found;
}

// Closest hit (ANY = false) or any hit (ANY = true).
template <bool ANY, bool STATS = false>
B200_D bool traceScene(const Scene &sc, const Ray &ray, HitRec &hit, TraceStats *ts = nullptr) {
  return traceRay<STATS>(sc, ray, hit, ANY, true, ts);
}

}  // namespace b200
