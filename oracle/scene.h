// Oracle (test infrastructure only): two-level scene, CPU binned-SAH BVH and
// ray queries standing in for the reference's Embree calls.
//   modules/cpu/common/World.ih:29-52   traceGeometryRay -> rtcIntersectV
//   modules/cpu/common/World.ih:311-380 isOccluded -> rtcOccludedV
//   modules/cpu/common/Group.cpp:17-31,69-143, World.cpp:16-35,70-188  (BLAS/TLAS)
// Embree 4.3.3 (not vendored) is the reference's intersector.  The oracle
// uses the published watertight ray/triangle test (Woop, Benthin, Wald 2013)
// and the geometric ray/sphere test of Haines et al. (Ray Tracing Gems, 2019,
// ch. 7), which is also the form of Embree's sphere intersector.  Closest-hit
// ties at equal t are broken by the smallest (instID, geomID, primID), so the
// result does not depend on traversal order.
#pragma once
#include <cstdint>
#include <vector>

#include "vecmath.h"

namespace orc {

constexpr uint32_t INVALID_ID = 0xffffffffu;

struct Ray {
  V3 org;
  float tnear;
  V3 dir;
  float tfar;
};

struct Hit {
  float t, u, v;
  V3 Ng;  // unnormalised geometric normal in object space
  uint32_t primID, geomID, instID;
  uint32_t entry;  // index of the (instance, model) entry hit
};

struct Box {
  V3 lo, hi;
};

struct Geometry {
  int type;  // 0 triangles, 1 spheres / discs, 2 boxes (instance level), 3 planes
  std::vector<Box> boxes;
  std::vector<V3> verts;
  std::vector<uint32_t> index;  // 3 per triangle
  std::vector<uint32_t> quadIndex;  // quad meshes: 4 per quad; triangle p is half of quad p / 2
  uint32_t primDiv = 1;  // triangles per application primitive (quads 2, boxes 12): primID = p / primDiv
  bool boxFaces = false;  // box geometry as face triangles (no geometry epsilon)
  std::vector<V4> spheres;      // center, radius
  int sphereKind = 0;           // OSP_SPHERE 0, OSP_DISC 1, OSP_ORIENTED_DISC 2
  std::vector<V3> discNormals;  // oriented discs
  std::vector<V4> planes;       // a, b, c, d: the plane a x + b y + c z = d
  std::vector<Box> planeBounds; // per plane, when planeBounded
  bool planeBounded = false;
  // per-vertex attributes of a triangle mesh (empty: absent)
  std::vector<V3> normals;
  std::vector<V4> colors;
  std::vector<V2> texcoords;
  // BVH2 (binned SAH)
  struct Node {
    Box box;
    int32_t left;   // >=0 internal: left child index (right = left+1); <0 leaf
    uint32_t first, count;
  };
  std::vector<Node> nodes;
  std::vector<uint32_t> prims;
  uint32_t nprims() const {
    return type == 0 ? uint32_t(index.size() / 3)
                     : (type == 1 ? uint32_t(spheres.size()) : (type == 3 ? uint32_t(planes.size()) : uint32_t(boxes.size())));
  }
  Box primBox(uint32_t p) const;
  void build();
};

struct InstanceEntry {
  int geom;          // index into Scene::geoms
  uint32_t instID;   // world instance index
  uint32_t geomID;   // model index within the instance's group
  bool identity;
  int material = -1;  // renderer material slot of the geometric model
  A3 xfm, rcp;
  Box worldBox;
  // motion blur: >= 2 row-major 3x4 keys evenly spaced over [t0, t1]
  std::vector<float> motion;
  float t0 = 0.f, t1 = 1.f;
  // the transform at `time`: the two keys around it blended component-wise,
  // (1 - f) A + f B, times outside [t0, t1] taking the end keys (Embree's
  // key-framed instance, restated)
  A3 xfmAt(float time) const;
};

// rkcommon rcp(AffineSpace3f)
A3 rcpAffine(const A3 &a);

// The ray time of the calling thread's current camera sample (motion blur):
// every query and postIntersect of that sample (camera, extension, shadow
// and AO rays) is taken at it.  Set by the renderers per sample; 0 otherwise.
extern thread_local float rayTime;

struct Scene {
  std::vector<Geometry> geoms;
  std::vector<InstanceEntry> entries;
  Geometry tlas;  // type 2: BVH over the entries' world boxes
  void commit();
  // closest hit; returns false on miss
  bool intersect(const Ray &ray, Hit &hit) const;
  bool occluded(const Ray &ray) const;
};

}  // namespace orc
