// Oracle (test infrastructure only): BVH build and ray queries; see scene.h.
#include "scene.h"

#include <algorithm>
#include <cfloat>
#include <cmath>

namespace orc {

namespace {

inline Box emptyBox() { return {v3(FLT_MAX), v3(-FLT_MAX)}; }
inline void grow(Box &b, const Box &o) {
  b.lo = vmin(b.lo, o.lo);
  b.hi = vmax(b.hi, o.hi);
}
inline float area(const Box &b) {
  const V3 d = b.hi - b.lo;
  if (d.x < 0) return 0.f;
  return 2.f * (d.x * d.y + d.y * d.z + d.z * d.x);
}
inline V3 center(const Box &b) { return 0.5f * (b.lo + b.hi); }

// Robust slab test (Ize 2013): far distance scaled by 1 + 2*gamma(3).
inline bool hitBox(const Box &b, V3 org, V3 rdir, float tnear, float tfar) {
  float t0 = tnear, t1 = tfar;
  for (int k = 0; k < 3; k++) {
    const float o = get(org, k), r = get(rdir, k);
    float tn = (get(b.lo, k) - o) * r;
    float tf = (get(b.hi, k) - o) * r;
    if (tn > tf) std::swap(tn, tf);
    tf *= 1.0000003576f;
    // NaN (0 * inf) keeps the slab open
    t0 = tn > t0 ? tn : t0;
    t1 = tf < t1 ? tf : t1;
  }
  return t0 <= t1;
}

struct TriPre {
  int kx, ky, kz;
  float Sx, Sy, Sz;
};

inline TriPre pretri(V3 d) {
  TriPre p;
  const V3 a = vabs(d);
  p.kz = 0;
  if (a.y > get(a, p.kz)) p.kz = 1;
  if (a.z > get(a, p.kz)) p.kz = 2;
  p.kx = p.kz == 2 ? 0 : p.kz + 1;
  p.ky = p.kx == 2 ? 0 : p.kx + 1;
  if (get(d, p.kz) < 0.f) std::swap(p.kx, p.ky);
  p.Sx = get(d, p.kx) / get(d, p.kz);
  p.Sy = get(d, p.ky) / get(d, p.kz);
  p.Sz = 1.f / get(d, p.kz);
  return p;
}

// Watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2013).
// u, v follow the convention P = (1-u-v) v0 + u v1 + v v2.
inline bool triTest(const TriPre &p, V3 org, float tnear, float tfar, V3 v0, V3 v1, V3 v2, float &t,
                    float &u, float &v) {
  const V3 A = v0 - org, B = v1 - org, C = v2 - org;
  const float Akz = get(A, p.kz), Bkz = get(B, p.kz), Ckz = get(C, p.kz);
  const float Ax = get(A, p.kx) - p.Sx * Akz;
  const float Ay = get(A, p.ky) - p.Sy * Akz;
  const float Bx = get(B, p.kx) - p.Sx * Bkz;
  const float By = get(B, p.ky) - p.Sy * Bkz;
  const float Cx = get(C, p.kx) - p.Sx * Ckz;
  const float Cy = get(C, p.ky) - p.Sy * Ckz;
  float U = Cx * By - Cy * Bx;
  float V = Ax * Cy - Ay * Cx;
  float W = Bx * Ay - By * Ax;
  if (U == 0.f || V == 0.f || W == 0.f) {
    U = float(double(Cx) * double(By) - double(Cy) * double(Bx));
    V = float(double(Ax) * double(Cy) - double(Ay) * double(Cx));
    W = float(double(Bx) * double(Ay) - double(By) * double(Ax));
  }
  if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
  const float det = U + V + W;
  if (det == 0.f) return false;
  const float Az = p.Sz * Akz, Bz = p.Sz * Bkz, Cz = p.Sz * Ckz;
  const float T = U * Az + V * Bz + W * Cz;
  t = T / det;
  if (!(t >= tnear && t <= tfar)) return false;
  u = V / det;
  v = W / det;
  return true;
}

// Ray/sphere test in the geometric form of Haines et al. (RTG 2019, ch. 7).
inline bool sphTest(V3 org, V3 d, float tnear, float tfar, V4 s, float &t, V3 &Ng) {
  const float rd2 = 1.f / dot(d, d);
  const V3 c0 = v3(s.x, s.y, s.z) - org;
  const float projC0 = dot(c0, d) * rd2;
  const V3 perp = c0 - projC0 * d;
  const float l2 = dot(perp, perp);
  const float r2 = s.w * s.w;
  if (!(l2 <= r2)) return false;
  const float td = std::sqrt((r2 - l2) * rd2);
  const float tf = projC0 - td, tb = projC0 + td;
  if (tf >= tnear && tf <= tfar)
    t = tf;
  else if (tb >= tnear && tb <= tfar)
    t = tb;
  else
    return false;
  Ng = t * d - c0;
  return true;
}

// Embree 4.3.3's point primitives (the reference's OSP_DISC and
// OSP_ORIENTED_DISC, geometry/Spheres.cpp:21-22): a ray-facing disc is hit at
// the centre's projection onto the ray when the ray passes within the radius
// (Ng = -d); an oriented disc where the ray meets its plane inside the radius
// (Ng = its normal).
inline bool discTest(V3 org, V3 d, float tnear, float tfar, V4 s, float &t, V3 &Ng) {
  const float rd2 = 1.f / dot(d, d);
  const V3 c0 = v3(s.x, s.y, s.z) - org;
  const float projC0 = dot(c0, d) * rd2;
  if (!(projC0 >= tnear && projC0 <= tfar)) return false;
  const V3 perp = c0 - projC0 * d;
  if (!(dot(perp, perp) <= s.w * s.w)) return false;
  t = projC0;
  Ng = -d;
  return true;
}
inline bool orientedDiscTest(V3 org, V3 d, float tnear, float tfar, V4 s, V3 n, float &t, V3 &Ng) {
  const float div = dot(d, n);
  if (div == 0.f) return false;
  const V3 c = v3(s.x, s.y, s.z);
  const float tt = dot(c - org, n) / div;
  if (!(tt >= tnear && tt <= tfar)) return false;
  const V3 q = (org + d * tt) - c;
  if (!(dot(q, q) < s.w * s.w)) return false;
  t = tt;
  Ng = n;
  return true;
}
// Planes_intersect_kernel (geometry/Planes.ispc:40-78) with intersectPlane /
// intersectBox (common/Intersect.ih:195-237) and filterIntersectionSingle's
// tnear < t <= tfar (common/FilterIntersect.ih)
inline bool planeTest(V3 org, V3 d, float tnear, float tfar, V4 c, const Box *bounds, float &t, V3 &Ng) {
  const V3 n = v3(c.x, c.y, c.z);
  const float DdN = dot(d, n);
  if (DdN == 0.f) return false;
  const float tt = (c.w - dot(org, n)) / DdN;
  if (!(tt > tnear && tt <= tfar)) return false;
  if (bounds) {
    auto rs = [](float x) { return 1.f / (std::fabs(x) < 1e-18f ? std::copysign(1e-18f, x) : x); };
    const V3 r = v3(rs(d.x), rs(d.y), rs(d.z));
    const V3 m0 = (bounds->lo - org) * r, m1 = (bounds->hi - org) * r;
    const float en = reduce_max(vmin(m0, m1)), ex = reduce_min(vmax(m0, m1));
    if (!(en < ex) || tt < en || tt > ex) return false;
  }
  t = tt;
  Ng = n;
  return true;
}

inline bool better(float t, uint32_t inst, uint32_t geom, uint32_t prim, const Hit &h) {
  if (t != h.t) return t < h.t;
  if (inst != h.instID) return inst < h.instID;
  if (geom != h.geomID) return geom < h.geomID;
  return prim < h.primID;
}

}  // namespace

Box Geometry::primBox(uint32_t p) const {
  if (type == 2) return boxes[p];
  if (type == 0) {
    const V3 a = verts[index[3 * p]], b = verts[index[3 * p + 1]], c = verts[index[3 * p + 2]];
    return {vmin(a, vmin(b, c)), vmax(a, vmax(b, c))};
  }
  if (type == 3) {  // Planes_bounds (geometry/Planes.ispc:17-33)
    const float M = 1e18f;
    if (!planeBounded) return {v3(-M), v3(M)};
    return {vmax(planeBounds[p].lo, v3(-M)), vmin(planeBounds[p].hi, v3(M))};
  }
  const V4 s = spheres[p];
  return {v3(s.x - s.w, s.y - s.w, s.z - s.w), v3(s.x + s.w, s.y + s.w, s.z + s.w)};
}

// Binned SAH (16 bins per axis), leaves of at most 4 primitives.
void Geometry::build() {
  const uint32_t n = nprims();
  prims.resize(n);
  std::vector<Box> boxes(n);
  std::vector<V3> cent(n);
  for (uint32_t i = 0; i < n; i++) {
    prims[i] = i;
    boxes[i] = primBox(i);
    cent[i] = center(boxes[i]);
  }
  nodes.clear();
  nodes.reserve(2 * n + 1);
  struct Task {
    uint32_t node, first, count;
  };
  std::vector<Task> stack;
  nodes.push_back({emptyBox(), -1, 0, n});
  stack.push_back({0, 0, n});
  constexpr int NB = 16;
  while (!stack.empty()) {
    const Task tk = stack.back();
    stack.pop_back();
    Box nb = emptyBox(), cb = emptyBox();
    for (uint32_t i = tk.first; i < tk.first + tk.count; i++) {
      grow(nb, boxes[prims[i]]);
      grow(cb, {cent[prims[i]], cent[prims[i]]});
    }
    Node &node = nodes[tk.node];
    node.box = nb;
    node.first = tk.first;
    node.count = tk.count;
    node.left = -1;
    if (tk.count <= 4) continue;
    float bestCost = FLT_MAX;
    int bestAxis = -1, bestSplit = -1;
    for (int ax = 0; ax < 3; ax++) {
      const float lo = get(cb.lo, ax), ext = get(cb.hi, ax) - lo;
      if (ext <= 0.f) continue;
      Box bb[NB];
      uint32_t bc[NB] = {};
      for (int b = 0; b < NB; b++) bb[b] = emptyBox();
      for (uint32_t i = tk.first; i < tk.first + tk.count; i++) {
        int b = int((get(cent[prims[i]], ax) - lo) / ext * NB);
        b = std::min(std::max(b, 0), NB - 1);
        bc[b]++;
        grow(bb[b], boxes[prims[i]]);
      }
      float rArea[NB];
      uint32_t rCnt[NB];
      Box acc = emptyBox();
      uint32_t cnt = 0;
      for (int b = NB - 1; b > 0; b--) {
        grow(acc, bb[b]);
        cnt += bc[b];
        rArea[b] = area(acc);
        rCnt[b] = cnt;
      }
      acc = emptyBox();
      cnt = 0;
      for (int b = 0; b < NB - 1; b++) {
        grow(acc, bb[b]);
        cnt += bc[b];
        if (cnt == 0 || rCnt[b + 1] == 0) continue;
        const float cost = area(acc) * cnt + rArea[b + 1] * rCnt[b + 1];
        if (cost < bestCost) {
          bestCost = cost;
          bestAxis = ax;
          bestSplit = b;
        }
      }
    }
    uint32_t mid;
    if (bestAxis < 0) {
      mid = tk.first + tk.count / 2;  // all centroids equal: median split
    } else {
      const float lo = get(cb.lo, bestAxis), ext = get(cb.hi, bestAxis) - lo;
      auto it = std::partition(prims.begin() + tk.first, prims.begin() + tk.first + tk.count,
                               [&](uint32_t p) {
                                 int b = int((get(cent[p], bestAxis) - lo) / ext * NB);
                                 b = std::min(std::max(b, 0), NB - 1);
                                 return b <= bestSplit;
                               });
      mid = uint32_t(it - prims.begin());
      if (mid == tk.first || mid == tk.first + tk.count) mid = tk.first + tk.count / 2;
    }
    const uint32_t l = uint32_t(nodes.size());
    nodes[tk.node].left = int32_t(l);
    nodes.push_back({emptyBox(), -1, 0, 0});
    nodes.push_back({emptyBox(), -1, 0, 0});
    stack.push_back({l, tk.first, mid - tk.first});
    stack.push_back({l + 1, mid, tk.first + tk.count - mid});
  }
}

thread_local float rayTime = 0.f;

namespace {
A3 fromRowMajor12(const float *X) {
  A3 a;
  a.l.vx = {X[0], X[4], X[8]};
  a.l.vy = {X[1], X[5], X[9]};
  a.l.vz = {X[2], X[6], X[10]};
  a.p = {X[3], X[7], X[11]};
  return a;
}
}  // namespace

A3 InstanceEntry::xfmAt(float time) const {
  const int n = int(motion.size() / 12);
  float f = t1 > t0 ? (time - t0) / (t1 - t0) * float(n - 1) : 0.f;
  f = std::fmin(std::fmax(f, 0.f), float(n - 1));
  const int fi = int(std::floor(f)), i = fi < n - 2 ? fi : n - 2;
  const float u = f - float(i), w = 1.f - u;
  float X[12];
  for (int k = 0; k < 12; k++) X[k] = w * motion[12 * i + k] + u * motion[12 * (i + 1) + k];
  return fromRowMajor12(X);
}

void Scene::commit() {
  for (auto &g : geoms) g.build();
  for (auto &e : entries) {
    const Box b = geoms[e.geom].nodes.empty() ? Box{v3(0), v3(0)} : geoms[e.geom].nodes[0].box;
    const int nkeys = int(e.motion.size() / 12);
    if (e.identity && nkeys < 2) {
      e.worldBox = b;
      continue;
    }
    Box wb = emptyBox();
    for (int k = 0; k < (nkeys >= 2 ? nkeys : 1); k++) {  // the union over the keys
      const A3 X = nkeys >= 2 ? fromRowMajor12(&e.motion[12 * k]) : e.xfm;
      for (int c = 0; c < 8; c++) {
        const V3 p = {c & 1 ? b.hi.x : b.lo.x, c & 2 ? b.hi.y : b.lo.y, c & 4 ? b.hi.z : b.lo.z};
        const V3 q = xfmPoint(X, p);
        grow(wb, {q, q});
      }
    }
    // pad by a relative ulp margin for the transform's rounding
    const V3 pad = 1e-6f * (vabs(wb.lo) + vabs(wb.hi)) + v3(1e-30f);
    wb.lo = wb.lo - pad;
    wb.hi = wb.hi + pad;
    e.worldBox = wb;
  }
  tlas = Geometry();
  tlas.type = 2;
  for (const auto &e : entries) tlas.boxes.push_back(e.worldBox);
  tlas.build();
}

namespace {

template <bool ANY>
bool traverseBLAS(const Geometry &g, V3 org, V3 dir, float tnear, Hit &hit, uint32_t instID,
                  uint32_t geomID) {
  if (g.nodes.empty()) return false;
  const V3 rdir = {1.f / dir.x, 1.f / dir.y, 1.f / dir.z};
  const TriPre pre = pretri(dir);
  uint32_t stack[128];
  int sp = 0;
  stack[sp++] = 0;
  bool found = false;
  while (sp) {
    const Geometry::Node &n = g.nodes[stack[--sp]];
    if (!hitBox(n.box, org, rdir, tnear, hit.t)) continue;
    if (n.left >= 0) {
      stack[sp++] = uint32_t(n.left);
      stack[sp++] = uint32_t(n.left + 1);
      continue;
    }
    for (uint32_t i = n.first; i < n.first + n.count; i++) {
      const uint32_t p = g.prims[i];
      float t, u = 0.f, v = 0.f;
      V3 Ng;
      bool h;
      if (g.type == 0) {
        const V3 v0 = g.verts[g.index[3 * p]], v1 = g.verts[g.index[3 * p + 1]],
                 v2 = g.verts[g.index[3 * p + 2]];
        h = triTest(pre, org, tnear, hit.t, v0, v1, v2, t, u, v);
        if (h) Ng = cross(v1 - v0, v2 - v0);
      } else if (g.type == 3) {
        h = planeTest(org, dir, tnear, hit.t, g.planes[p], g.planeBounded ? &g.planeBounds[p] : nullptr, t, Ng);
      } else if (g.sphereKind == 1) {
        h = discTest(org, dir, tnear, hit.t, g.spheres[p], t, Ng);
      } else if (g.sphereKind == 2) {
        h = orientedDiscTest(org, dir, tnear, hit.t, g.spheres[p], g.discNormals[p], t, Ng);
      } else {
        h = sphTest(org, dir, tnear, hit.t, g.spheres[p], t, Ng);
      }
      if (!h) continue;
      if (ANY) return true;
      const uint32_t prim = g.type == 0 ? p / g.primDiv : p;  // quads, boxes: the application primitive
      // a quad's second triangle (v2, v3, v1) reports the quad's (u, v) = 1 - its own (Embree's quad hits)
      if (g.type == 0 && g.primDiv == 2 && !g.boxFaces && (p & 1u)) {
        u = 1.f - u;
        v = 1.f - v;
      }
      if (better(t, instID, geomID, prim, hit)) {
        hit.t = t;
        hit.u = u;
        hit.v = v;
        hit.Ng = Ng;
        hit.primID = prim;
        hit.geomID = geomID;
        hit.instID = instID;
        found = true;
      }
    }
  }
  return found;
}

template <bool ANY>
bool traverse(const Scene &s, const Ray &ray, Hit &hit) {
  hit.t = ray.tfar;
  hit.primID = hit.geomID = hit.instID = INVALID_ID;
  hit.entry = INVALID_ID;
  const V3 rdir = {1.f / ray.dir.x, 1.f / ray.dir.y, 1.f / ray.dir.z};
  bool found = false;
  if (s.tlas.nodes.empty()) return false;
  uint32_t stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    const Geometry::Node &n = s.tlas.nodes[stack[--sp]];
    if (!hitBox(n.box, ray.org, rdir, ray.tnear, hit.t)) continue;
    if (n.left >= 0) {
      stack[sp++] = uint32_t(n.left);
      stack[sp++] = uint32_t(n.left + 1);
      continue;
    }
    for (uint32_t k = n.first; k < n.first + n.count; k++) {
      const uint32_t ei = s.tlas.prims[k];
      const InstanceEntry &e = s.entries[ei];
      if (!hitBox(e.worldBox, ray.org, rdir, ray.tnear, hit.t)) continue;
      V3 o = ray.org, d = ray.dir;
      if (e.motion.size() >= 24) {
        const A3 r = rcpAffine(e.xfmAt(rayTime));
        o = xfmPoint(r, ray.org);
        d = xfmVector(r.l, ray.dir);
      } else if (!e.identity) {
        o = xfmPoint(e.rcp, ray.org);
        d = xfmVector(e.rcp.l, ray.dir);
      }
      if (traverseBLAS<ANY>(s.geoms[e.geom], o, d, ray.tnear, hit, e.instID, e.geomID)) {
        if (ANY) return true;
        hit.entry = ei;
        found = true;
      }
    }
  }
  return found;
}

}  // namespace

bool Scene::intersect(const Ray &ray, Hit &hit) const { return traverse<false>(*this, ray, hit); }

bool Scene::occluded(const Ray &ray) const {
  Hit h;
  return traverse<true>(*this, ray, h);
}

}  // namespace orc
