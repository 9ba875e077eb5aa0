// GPU BVH build interface (see bvh.cu).
#pragma once
#include "common.cuh"

namespace b200 {

struct WideBVH {
  Node8 *nodes = nullptr;       // root at index 0
  uint32_t *leafPrim = nullptr; // original primitive index per leaf slot
  int nnodes = 0, nprims = 0;
  float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};  // bounds of all primitives
};

struct BLAS {
  WideBVH bvh;
  float4 *prims = nullptr;      // triangles: 3 float4 per slot; spheres: 1 float4
  uint32_t *primIDs = nullptr;  // spheres: primID per slot
};

// sah: top-down 3-axis binned SAH (high quality, the reference's default
// build quality); false: the plain LBVH hierarchy (fastest build, the
// reference's dynamicScene)
cudaError_t buildWide(const float4 *lo, const float4 *hi, int n, cudaStream_t st, WideBVH &out, bool sah = true);
// primDiv: BLAS triangles per application primitive (primID = triangle /
// primDiv): 1 triangles, 2 quads, 12 boxes
cudaError_t buildTriangleBLAS(const float *d_verts, const uint32_t *d_index, int ntris, cudaStream_t st, BLAS &out,
                              bool sah = true, int primDiv = 1);
cudaError_t buildSphereBLAS(const float4 *d_sph, int n, cudaStream_t st, BLAS &out, bool sah = true);
// discs, oriented discs and planes: primStride(type) float4 per primitive
cudaError_t buildUserBLAS(uint32_t type, const float4 *d_data, int n, cudaStream_t st, BLAS &out, bool sah = true);
void freeBLAS(BLAS &b, cudaStream_t st);

}  // namespace b200
