// Device-side vector math, ray/hit records and exact-rounding helpers shared
// by the b200 kernels.  Arithmetic that must agree bit-for-bit with a scalar
// IEEE evaluation (camera rays, intersection, postIntersect) uses the _rn
// intrinsics so nvcc cannot contract it into FMAs.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define B200_HD __host__ __device__ __forceinline__
#define B200_D __device__ __forceinline__

namespace b200 {

constexpr uint32_t INVALID_ID = 0xffffffffu;
constexpr float ULP_EPSILON = 0x1.0fp-21f;  // common/DifferentialGeometry.ih ulpEpsilon

struct V3 {
  float x, y, z;
};

B200_HD V3 mk(float x, float y, float z) { return {x, y, z}; }
B200_HD V3 splat(float a) { return {a, a, a}; }

#ifdef __CUDA_ARCH__
B200_D float fmul(float a, float b) { return __fmul_rn(a, b); }
B200_D float fadd(float a, float b) { return __fadd_rn(a, b); }
B200_D float fsub(float a, float b) { return __fsub_rn(a, b); }
B200_D float fdiv(float a, float b) { return __fdiv_rn(a, b); }
B200_D float fsqrt(float a) { return __fsqrt_rn(a); }
#else
inline float fmul(float a, float b) { return a * b; }
inline float fadd(float a, float b) { return a + b; }
inline float fsub(float a, float b) { return a - b; }
inline float fdiv(float a, float b) { return a / b; }
inline float fsqrt(float a) { return sqrtf(a); }
#endif

// exact (non-contracted) vector ops
B200_HD V3 add(V3 a, V3 b) { return {fadd(a.x, b.x), fadd(a.y, b.y), fadd(a.z, b.z)}; }
B200_HD V3 sub(V3 a, V3 b) { return {fsub(a.x, b.x), fsub(a.y, b.y), fsub(a.z, b.z)}; }
B200_HD V3 mul(float s, V3 a) { return {fmul(s, a.x), fmul(s, a.y), fmul(s, a.z)}; }
B200_HD V3 mul(V3 a, float s) { return {fmul(a.x, s), fmul(a.y, s), fmul(a.z, s)}; }
B200_HD V3 vdiv(V3 a, float s) { return {fdiv(a.x, s), fdiv(a.y, s), fdiv(a.z, s)}; }
B200_HD V3 neg(V3 a) { return {-a.x, -a.y, -a.z}; }
B200_HD float dot(V3 a, V3 b) { return fadd(fadd(fmul(a.x, b.x), fmul(a.y, b.y)), fmul(a.z, b.z)); }
B200_HD V3 cross(V3 a, V3 b) {
  return {fsub(fmul(a.y, b.z), fmul(a.z, b.y)), fsub(fmul(a.z, b.x), fmul(a.x, b.z)),
          fsub(fmul(a.x, b.y), fmul(a.y, b.x))};
}
B200_HD V3 normalize(V3 a) {
  const float r = fdiv(1.f, fsqrt(dot(a, a)));
  return mul(a, r);
}
B200_HD V3 vabs(V3 a) { return {fabsf(a.x), fabsf(a.y), fabsf(a.z)}; }
B200_HD V3 vmin(V3 a, V3 b) { return {fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)}; }
B200_HD V3 vmax(V3 a, V3 b) { return {fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)}; }
B200_HD float reduce_max(V3 a) { return fmaxf(fmaxf(a.x, a.y), a.z); }
B200_HD float comp(V3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }

// fast (contractible) ops for shading code that is compared statistically
B200_HD V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
B200_HD V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
B200_HD V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
B200_HD V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
B200_HD V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
B200_HD V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
B200_HD float fdot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
B200_HD V3 fcross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
B200_HD V3 fnormalize(V3 a) { return a * rsqrtf(fdot(a, a)); }

// Affine transform: rows of a 3x4 matrix (p' = L p + t), row-major.
struct Xfm {
  float m[12];
};
// xfmVector in rkcommon column form: vx*v.x + vy*v.y + vz*v.z, evaluated
// per component as ((c0*x + c1*y) + c2*z) without contraction.
B200_HD V3 xfmVector(const Xfm &a, V3 v) {
  return {fadd(fadd(fmul(a.m[0], v.x), fmul(a.m[1], v.y)), fmul(a.m[2], v.z)),
          fadd(fadd(fmul(a.m[4], v.x), fmul(a.m[5], v.y)), fmul(a.m[6], v.z)),
          fadd(fadd(fmul(a.m[8], v.x), fmul(a.m[9], v.y)), fmul(a.m[10], v.z))};
}
B200_HD V3 xfmPoint(const Xfm &a, V3 v) {
  const V3 l = xfmVector(a, v);
  return {fadd(l.x, a.m[3]), fadd(l.y, a.m[7]), fadd(l.z, a.m[11])};
}
// transpose(L) * v
B200_HD V3 xfmVectorT(const Xfm &a, V3 v) {
  return {fadd(fadd(fmul(a.m[0], v.x), fmul(a.m[4], v.y)), fmul(a.m[8], v.z)),
          fadd(fadd(fmul(a.m[1], v.x), fmul(a.m[5], v.y)), fmul(a.m[9], v.z)),
          fadd(fadd(fmul(a.m[2], v.x), fmul(a.m[6], v.y)), fmul(a.m[10], v.z))};
}

// rkcommon rcp(AffineSpace3f): the adjoint over the determinant in float,
// p' = -(L' p)
B200_HD Xfm rcpXfm(const Xfm &X) {
  const V3 vx = mk(X.m[0], X.m[4], X.m[8]), vy = mk(X.m[1], X.m[5], X.m[9]), vz = mk(X.m[2], X.m[6], X.m[10]);
  const V3 a = cross(vy, vz), b = cross(vz, vx), c = cross(vx, vy);
  const float det = dot(vx, a);
  const V3 ix = vdiv(mk(a.x, b.x, c.x), det), iy = vdiv(mk(a.y, b.y, c.y), det), iz = vdiv(mk(a.z, b.z, c.z), det);
  const V3 p = mk(X.m[3], X.m[7], X.m[11]);
  const V3 ip = add(add(mul(ix, p.x), mul(iy, p.y)), mul(iz, p.z));
  return Xfm{{ix.x, iy.x, iz.x, -ip.x, ix.y, iy.y, iz.y, -ip.y, ix.z, iy.z, iz.z, -ip.z}};
}

// A key-framed instance transform at `time` (Embree's motion-blurred
// instance behind MotionTransform, common/MotionTransform.cpp:10-66: n keys
// evenly spaced over [t0, t1], the two keys around the time blended
// component-wise as (1 - f) a + f b; times outside [t0, t1] take the end
// keys).  keys: n row-major 3x4 matrices.
B200_HD Xfm motionXfm(const float *keys, int n, float t0, float t1, float time) {
  float f = t1 > t0 ? fmul(fdiv(fsub(time, t0), fsub(t1, t0)), float(n - 1)) : 0.f;
  f = fminf(fmaxf(f, 0.f), float(n - 1));
  const int fi = int(floorf(f)), i = fi < n - 2 ? fi : n - 2;
  const float u = fsub(f, float(i));
  const float w = fsub(1.f, u);
  Xfm X;
  for (int k = 0; k < 12; k++) X.m[k] = fadd(fmul(w, keys[12 * i + k]), fmul(u, keys[12 * (i + 1) + k]));
  return X;
}

struct Ray {
  V3 org;
  float tnear;
  V3 dir;
  float tfar;
};

struct Hit {
  float t, u, v;
  V3 Ng;  // unnormalised, object space
  uint32_t primID, geomID, instID;
};

// 80-byte quantised 8-wide BVH node.  Child i's box on axis k is
// [p_k + qlo[k][i] * 2^(e_k-127), p_k + qhi[k][i] * 2^(e_k-127)], rounded
// outward at build time so the decoded box always contains the exact one.
// meta[i]: 0 empty; 0x80|j internal child node childBase+j; otherwise a leaf
// of (meta>>5) primitives starting at primBase + (meta & 31).
struct __align__(16) Node8 {
  float px, py, pz;
  uint8_t ex, ey, ez, imask;
  uint32_t childBase, primBase;
  uint8_t meta[8];
  uint8_t qlo[3][8];
  uint8_t qhi[3][8];
};
static_assert(sizeof(Node8) == 80, "Node8 must be 80 bytes");

// Spheres::commit "type" (geometry/Spheres.cpp:21-22,54: OSP_SPHERE, OSP_DISC,
// OSP_ORIENTED_DISC) and Planes (geometry/Planes.ispc) are the user-primitive types
enum GeomType : uint32_t {
  GEOM_TRIANGLES = 0,
  GEOM_SPHERES = 1,
  GEOM_DISCS = 2,
  GEOM_ORIENTED_DISCS = 3,
  GEOM_PLANES = 4
};
// float4s per BLAS slot of each user-primitive type: spheres and discs
// (centre, radius); oriented discs + (normal, 0); planes (a, b, c, d),
// (lower, bounded flag), (upper, 0)
B200_HD int primStride(uint32_t type) {
  return type == GEOM_ORIENTED_DISCS ? 2 : (type == GEOM_PLANES ? 3 : 1);
}

// One (instance, geometric model) pair of the world: the unit the TLAS is
// built over.  BLAS arrays are shared between entries of the same geometry.
// How a triangle BLAS maps to the application's primitives: plain triangles;
// quads (each two BLAS triangles, primID = triangle / 2, index 4 per quad);
// boxes (each twelve BLAS triangles, primID = triangle / 12, no index).
constexpr uint32_t MESH_TRIANGLES = 0, MESH_QUADS = 1, MESH_BOXES = 2;

struct Entry {
  const Node8 *nodes;        // BLAS nodes (root at 0)
  const float4 *prims;       // triangles: 3 float4 (v0+primID bits, v1, v2); spheres: 1 float4
  const uint32_t *primIDs;   // spheres only: primID per leaf slot
  const float *verts;        // original vertex array (xyz per vertex) for postIntersect
  const uint32_t *index;     // original index array (3 per triangle; 4 per quad for MESH_QUADS)
  const float4 *spheres;     // original sphere array
  uint32_t type, instID, geomID, identity;
  Xfm xfm, rcp;
  float epsScale;            // max |diag(xfm.l)|
  uint32_t materialID;       // per-entry material slot (renderers)
  uint32_t meshKind;         // triangles: MESH_TRIANGLES, MESH_QUADS or MESH_BOXES
  uint32_t pad;
  // per-vertex attributes of a triangle mesh (null: absent)
  const float *normals;      // 3 per vertex
  const float *colors;       // 4 per vertex
  const float *texcoords;    // 2 per vertex
  // motion blur: motionCount >= 2 row-major 3x4 keys over [motionT0,
  // motionT1] (motionXfm); xfm / rcp then unused
  const float *motionKeys;
  int motionCount;
  float motionT0, motionT1;
  int motionPad;
};

}  // namespace b200
