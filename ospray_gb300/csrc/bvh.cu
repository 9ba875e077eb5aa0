// GPU acceleration-structure build: Morton-ordered primitives split either by
// a top-down 3-axis binned SAH (default) or by the Karras 2012 LBVH hierarchy
// (dynamic scenes), collapsed into the 80-byte quantised 8-wide node format
// of common.cuh.  Replaces the Embree BLAS/TLAS builds the reference issues from
// Mesh::commit / Spheres::commit / Group::commit / World::commit
// (modules/cpu/geometry/Mesh.cpp:140-167, geometry/Spheres.cpp:63-97,
// common/Group.cpp:17-31,69-143, common/World.cpp:16-35,70-188).
#include <cub/cub.cuh>

#include "bvh.h"

namespace b200 {

namespace {

constexpr int LEAF_MAX = 3;
constexpr uint32_t LEAF_BIT = 0x80000000u;

__device__ __forceinline__ uint32_t floatFlip(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float floatUnflip(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__global__ void k_tri_bounds(const float *verts, const uint32_t *index, int n, float4 *lo, float4 *hi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t a = index[3 * i], b = index[3 * i + 1], c = index[3 * i + 2];
  const float3 A = {verts[3 * a], verts[3 * a + 1], verts[3 * a + 2]};
  const float3 B = {verts[3 * b], verts[3 * b + 1], verts[3 * b + 2]};
  const float3 C = {verts[3 * c], verts[3 * c + 1], verts[3 * c + 2]};
  lo[i] = make_float4(fminf(A.x, fminf(B.x, C.x)), fminf(A.y, fminf(B.y, C.y)), fminf(A.z, fminf(B.z, C.z)), 0.f);
  hi[i] = make_float4(fmaxf(A.x, fmaxf(B.x, C.x)), fmaxf(A.y, fmaxf(B.y, C.y)), fmaxf(A.z, fmaxf(B.z, C.z)), 0.f);
}

__global__ void k_sph_bounds(const float4 *s, int n, float4 *lo, float4 *hi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 v = s[i];
  lo[i] = make_float4(v.x - v.w, v.y - v.w, v.z - v.w, 0.f);
  hi[i] = make_float4(v.x + v.w, v.y + v.w, v.z + v.w, 0.f);
}

// user primitives (discs, oriented discs: the sphere's box; planes: their
// box clipped to +-1e18, or +-1e18 without one, Planes_bounds
// geometry/Planes.ispc:17-33); data: `stride` float4 per primitive
__global__ void k_user_bounds(const float4 *data, int stride, int n, uint32_t type, float4 *lo, float4 *hi) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 *p = data + size_t(i) * stride;
  if (type == GEOM_PLANES) {
    constexpr float M = 1e18f;
    const float4 a = p[1], b = p[2];
    const bool bounded = a.w != 0.f;
    lo[i] = bounded ? make_float4(fmaxf(a.x, -M), fmaxf(a.y, -M), fmaxf(a.z, -M), 0.f) : make_float4(-M, -M, -M, 0.f);
    hi[i] = bounded ? make_float4(fminf(b.x, M), fminf(b.y, M), fminf(b.z, M), 0.f) : make_float4(M, M, M, 0.f);
    return;
  }
  const float4 v = p[0];
  lo[i] = make_float4(v.x - v.w, v.y - v.w, v.z - v.w, 0.f);
  hi[i] = make_float4(v.x + v.w, v.y + v.w, v.z + v.w, 0.f);
}

// centroid bounds (and overall bounds) via flipped-float atomics; acc[0..5]
// centroid min/max, acc[6..11] box min/max
__global__ void k_bounds(const float4 *lo, const float4 *hi, int n, uint32_t *acc) {
  float cmin[3] = {INFINITY, INFINITY, INFINITY}, cmax[3] = {-INFINITY, -INFINITY, -INFINITY};
  float bmin[3] = {INFINITY, INFINITY, INFINITY}, bmax[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 a = lo[i], b = hi[i];
    const float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
    const float l[3] = {a.x, a.y, a.z}, h[3] = {b.x, b.y, b.z};
    for (int k = 0; k < 3; k++) {
      cmin[k] = fminf(cmin[k], c[k]);
      cmax[k] = fmaxf(cmax[k], c[k]);
      bmin[k] = fminf(bmin[k], l[k]);
      bmax[k] = fmaxf(bmax[k], h[k]);
    }
  }
  for (int k = 0; k < 3; k++) {
    for (int o = 16; o; o >>= 1) {
      cmin[k] = fminf(cmin[k], __shfl_xor_sync(0xffffffffu, cmin[k], o));
      cmax[k] = fmaxf(cmax[k], __shfl_xor_sync(0xffffffffu, cmax[k], o));
      bmin[k] = fminf(bmin[k], __shfl_xor_sync(0xffffffffu, bmin[k], o));
      bmax[k] = fmaxf(bmax[k], __shfl_xor_sync(0xffffffffu, bmax[k], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
    for (int k = 0; k < 3; k++) {
      atomicMin(&acc[k], floatFlip(cmin[k]));
      atomicMax(&acc[3 + k], floatFlip(cmax[k]));
      atomicMin(&acc[6 + k], floatFlip(bmin[k]));
      atomicMax(&acc[9 + k], floatFlip(bmax[k]));
    }
  }
}

__device__ __forceinline__ uint32_t expand10(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

__global__ void k_morton(const float4 *lo, const float4 *hi, int n, const uint32_t *acc, uint32_t *keys,
                         uint32_t *vals) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 a = lo[i], b = hi[i];
  const float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
  uint32_t q[3];
  for (int k = 0; k < 3; k++) {
    const float mn = floatUnflip(acc[k]), mx = floatUnflip(acc[3 + k]);
    const float ext = mx - mn;
    float f = ext > 0.f ? (c[k] - mn) / ext : 0.5f;
    f = fminf(fmaxf(f * 1024.f, 0.f), 1023.f);
    q[k] = uint32_t(f);
  }
  keys[i] = (expand10(q[0]) << 2) | (expand10(q[1]) << 1) | expand10(q[2]);
  vals[i] = uint32_t(i);
}

__device__ __forceinline__ int delta(const uint32_t *keys, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  const uint32_t a = keys[i], b = keys[j];
  if (a == b) return 32 + __clz(uint32_t(i) ^ uint32_t(j));
  return __clz(a ^ b);
}

// Karras 2012: internal node i of n-1
__global__ void k_karras(const uint32_t *keys, int n, uint32_t *left, uint32_t *right, uint32_t *first,
                         uint32_t *parentInt, uint32_t *parentLeaf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = delta(keys, n, i, i - d);
  int lmax = 2;
  while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = delta(keys, n, i, j);
  int s = 0;
  int divisor = 2;
  int t = (l + divisor - 1) / divisor;
  while (t >= 1) {
    if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    if (t == 1) break;
    divisor <<= 1;
    t = (l + divisor - 1) / divisor;
  }
  const int gamma = i + s * d + (d < 0 ? -1 : 0);
  const int lo = min(i, j), hi = max(i, j);
  uint32_t L, R;
  if (lo == gamma) {
    L = LEAF_BIT | uint32_t(gamma);
    parentLeaf[gamma] = uint32_t(i);
  } else {
    L = uint32_t(gamma);
    parentInt[gamma] = uint32_t(i);
  }
  if (hi == gamma + 1) {
    R = LEAF_BIT | uint32_t(gamma + 1);
    parentLeaf[gamma + 1] = uint32_t(i);
  } else {
    R = uint32_t(gamma + 1);
    parentInt[gamma + 1] = uint32_t(i);
  }
  left[i] = L;
  right[i] = R;
  first[i] = uint32_t(lo);
  if (i == 0) parentInt[0] = 0xffffffffu;
}

__device__ __forceinline__ void loadBox(uint32_t ref, const float4 *blo, const float4 *bhi, const float4 *plo,
                                        const float4 *phi, const uint32_t *sorted, float4 &lo, float4 &hi) {
  if (ref & LEAF_BIT) {
    const uint32_t p = sorted[ref & ~LEAF_BIT];
    lo = plo[p];
    hi = phi[p];
  } else {
    lo = __ldcg(blo + ref);
    hi = __ldcg(bhi + ref);
  }
}

// bottom-up boxes; w of the internal box lo holds the primitive count (as bits)
__global__ void k_bottom_up(int n, const uint32_t *left, const uint32_t *right, const uint32_t *parentInt,
                            const uint32_t *parentLeaf, const uint32_t *sorted, const float4 *plo, const float4 *phi,
                            float4 *blo, float4 *bhi, uint32_t *flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t p = parentLeaf[i];
  for (int guard = 0; p != 0xffffffffu && guard < n; guard++) {
    __threadfence();
    if (atomicAdd(&flags[p], 1u) == 0) return;
    __threadfence();
    float4 l0, h0, l1, h1;
    const uint32_t L = left[p], R = right[p];
    loadBox(L, blo, bhi, plo, phi, sorted, l0, h0);
    loadBox(R, blo, bhi, plo, phi, sorted, l1, h1);
    const uint32_t c0 = (L & LEAF_BIT) ? 1u : __float_as_uint(l0.w), c1 = (R & LEAF_BIT) ? 1u : __float_as_uint(l1.w);
    __stcg(blo + p, make_float4(fminf(l0.x, l1.x), fminf(l0.y, l1.y), fminf(l0.z, l1.z), __uint_as_float(c0 + c1)));
    __stcg(bhi + p, make_float4(fmaxf(h0.x, h1.x), fmaxf(h0.y, h1.y), fmaxf(h0.z, h1.z), 0.f));
    p = parentInt[p];
  }
}

// ---------------------------------------------------------------- binned-SAH build
// Top-down binned SAH (Wald 2007, "On fast construction of SAH-based bounding
// volume hierarchies"): a node over the primitive range [first, first+count)
// bins the primitives' centroids into SAH_BINS equal-width bins per axis of
// the range's centroid bounds, takes the axis/boundary with the lowest
// A_L*N_L + A_R*N_R, and partitions the range stably in place.  The Morton
// order is the starting order, so sub-ranges keep spatial locality.  One block
// per node and one launch per tree level; the output is the Karras layout
// (left/right/first, boxes with the count in lo.w) that the 8-wide collapse
// reads, down to single-primitive leaves.
constexpr int SAH_BINS = 16;
constexpr int SAH_MAX_THREADS = 256;

struct SahTask {
  uint32_t first, count;  // primitive range in the index array
  uint32_t node;          // internal node to fill
  uint32_t pad;
  float4 clo, chi;        // centroid bounds of the range
};

// centroid and bin with explicit rounding, so the binning pass and the
// partition pass compute identical bins
__device__ __forceinline__ float3 centroidOf(const float4 *plo, const float4 *phi, uint32_t p) {
  const float4 a = plo[p], b = phi[p];
  return make_float3(__fmul_rn(0.5f, __fadd_rn(a.x, b.x)), __fmul_rn(0.5f, __fadd_rn(a.y, b.y)),
                     __fmul_rn(0.5f, __fadd_rn(a.z, b.z)));
}
__device__ __forceinline__ int sahBin(float c, float lo, float scale) {
  const float f = __fmul_rn(__fsub_rn(c, lo), scale);
  return f >= float(SAH_BINS - 1) ? SAH_BINS - 1 : (f > 0.f ? int(f) : 0);
}
__device__ __forceinline__ float comp(float3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
__device__ __forceinline__ float comp(float4 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

__device__ __forceinline__ float halfArea3(const float l[3], const float h[3]) {
  const float dx = h[0] - l[0], dy = h[1] - l[1], dz = h[2] - l[2];
  return dx * dy + dy * dz + dz * dx;
}

__global__ void k_sah_root(const uint32_t *acc, int n, SahTask *tasks) {
  SahTask t;
  t.first = 0;
  t.count = uint32_t(n);
  t.node = 0;
  t.pad = 0;
  t.clo = make_float4(floatUnflip(acc[0]), floatUnflip(acc[1]), floatUnflip(acc[2]), 0.f);
  t.chi = make_float4(floatUnflip(acc[3]), floatUnflip(acc[4]), floatUnflip(acc[5]), 0.f);
  tasks[0] = t;
}

// counters[0]: next internal node, counters[1]: tasks of the next level
__global__ void __launch_bounds__(SAH_MAX_THREADS) k_sah_level(const SahTask *tasks, SahTask *next, uint32_t *idx,
                                                              uint32_t *tmp, const float4 *plo, const float4 *phi,
                                                              uint32_t *counters, uint32_t *left, uint32_t *right,
                                                              uint32_t *first, float4 *blo, float4 *bhi) {
  __shared__ uint32_t sCnt[3][SAH_BINS];
  __shared__ uint32_t sLo[3][SAH_BINS][3], sHi[3][SAH_BINS][3];  // flipped floats
  __shared__ uint32_t sCb[2][6];                                  // children's centroid bounds, flipped
  __shared__ float sCost[SAH_MAX_THREADS / 32];
  __shared__ int sArg[SAH_MAX_THREADS / 32];
  __shared__ uint32_t sWarp[SAH_MAX_THREADS / 32];
  __shared__ int sBest;
  __shared__ uint32_t sNL;
  const SahTask t = tasks[blockIdx.x];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const uint32_t end = t.first + t.count;
  for (int i = tid; i < 3 * SAH_BINS; i += blockDim.x) {
    (&sCnt[0][0])[i] = 0;
    for (int k = 0; k < 3; k++) {
      (&sLo[0][0][0])[3 * i + k] = 0xffffffffu;
      (&sHi[0][0][0])[3 * i + k] = 0u;
    }
  }
  if (tid < 12) (&sCb[0][0])[tid] = (tid % 6) < 3 ? 0xffffffffu : 0u;
  float clo[3], scale[3];
  for (int k = 0; k < 3; k++) {
    clo[k] = comp(t.clo, k);
    const float ext = __fsub_rn(comp(t.chi, k), clo[k]);
    scale[k] = ext > 0.f ? __fdiv_rn(float(SAH_BINS), ext) : 0.f;
  }
  __syncthreads();
  // bin centroids; per bin the count and the box of its primitives
  for (uint32_t s = t.first + tid; s < end; s += blockDim.x) {
    const uint32_t p = idx[s];
    const float4 a = plo[p], b = phi[p];
    const float3 c = centroidOf(plo, phi, p);
    for (int k = 0; k < 3; k++) {
      const int bin = sahBin(comp(c, k), clo[k], scale[k]);
      atomicAdd(&sCnt[k][bin], 1u);
      atomicMin(&sLo[k][bin][0], floatFlip(a.x));
      atomicMin(&sLo[k][bin][1], floatFlip(a.y));
      atomicMin(&sLo[k][bin][2], floatFlip(a.z));
      atomicMax(&sHi[k][bin][0], floatFlip(b.x));
      atomicMax(&sHi[k][bin][1], floatFlip(b.y));
      atomicMax(&sHi[k][bin][2], floatFlip(b.z));
    }
  }
  __syncthreads();
  // candidate splits: axis k after bin j, one thread each
  constexpr int NCAND = 3 * (SAH_BINS - 1);
  float cost = INFINITY;
  if (tid < NCAND) {
    const int k = tid / (SAH_BINS - 1), j = tid % (SAH_BINS - 1);
    float ll[3] = {INFINITY, INFINITY, INFINITY}, lh[3] = {-INFINITY, -INFINITY, -INFINITY};
    float rl[3] = {INFINITY, INFINITY, INFINITY}, rh[3] = {-INFINITY, -INFINITY, -INFINITY};
    uint32_t nl = 0, nr = 0;
    for (int b = 0; b < SAH_BINS; b++) {
      const uint32_t cnt = sCnt[k][b];
      if (!cnt) continue;
      float *L = b <= j ? ll : rl, *H = b <= j ? lh : rh;
      for (int q = 0; q < 3; q++) {
        L[q] = fminf(L[q], floatUnflip(sLo[k][b][q]));
        H[q] = fmaxf(H[q], floatUnflip(sHi[k][b][q]));
      }
      (b <= j ? nl : nr) += cnt;
    }
    if (nl && nr) cost = halfArea3(ll, lh) * float(nl) + halfArea3(rl, rh) * float(nr);
  }
  // block argmin, lowest candidate index on ties
  int arg = tid;
  for (int o = 16; o; o >>= 1) {
    const float oc = __shfl_xor_sync(0xffffffffu, cost, o);
    const int oa = __shfl_xor_sync(0xffffffffu, arg, o);
    if (oc < cost || (oc == cost && oa < arg)) {
      cost = oc;
      arg = oa;
    }
  }
  if (lane == 0) {
    sCost[warp] = cost;
    sArg[warp] = arg;
  }
  __syncthreads();
  if (tid == 0) {
    float bc = sCost[0];
    int ba = sArg[0];
    for (int w = 1; w < nwarps; w++)
      if (sCost[w] < bc) {
        bc = sCost[w];
        ba = sArg[w];
      }
    sBest = bc < INFINITY ? ba : -1;
  }
  __syncthreads();
  const int best = sBest;
  uint32_t nL = t.count / 2;  // identical centroids: split the range in the middle
  if (best >= 0) {
    const int bk = best / (SAH_BINS - 1), bj = best % (SAH_BINS - 1);
    nL = 0;
    for (int b = 0; b <= bj; b++) nL += sCnt[bk][b];
    // stable partition into tmp: left part at [first, first+nL), right after
    uint32_t doneL = 0, doneR = 0;
    for (uint32_t c0 = t.first; c0 < end; c0 += blockDim.x) {
      const uint32_t s = c0 + tid;
      const bool valid = s < end;
      const uint32_t p = valid ? idx[s] : 0u;
      bool goL = false;
      float3 c = make_float3(0.f, 0.f, 0.f);
      if (valid) {
        c = centroidOf(plo, phi, p);
        goL = sahBin(comp(c, bk), clo[bk], scale[bk]) <= bj;
      }
      const uint32_t bal = __ballot_sync(0xffffffffu, goL);
      if (lane == 0) sWarp[warp] = __popc(bal);
      __syncthreads();
      uint32_t offL = 0, totL = 0;
      for (int w = 0; w < nwarps; w++) {
        const uint32_t v = sWarp[w];
        if (w < warp) offL += v;
        totL += v;
      }
      const uint32_t inChunk = min(uint32_t(blockDim.x), end - c0);
      if (valid) {
        const uint32_t rankL = offL + __popc(bal & ((1u << lane) - 1u));
        const uint32_t rankR = uint32_t(tid) - rankL;
        const uint32_t dst = goL ? t.first + doneL + rankL : t.first + nL + doneR + rankR;
        if (dst < end) tmp[dst] = p;
        uint32_t *cb = sCb[goL ? 0 : 1];
        atomicMin(&cb[0], floatFlip(c.x));
        atomicMin(&cb[1], floatFlip(c.y));
        atomicMin(&cb[2], floatFlip(c.z));
        atomicMax(&cb[3], floatFlip(c.x));
        atomicMax(&cb[4], floatFlip(c.y));
        atomicMax(&cb[5], floatFlip(c.z));
      }
      doneL += totL;
      doneR += inChunk - totL;
      __syncthreads();
    }
    if (tid == 0) sNL = doneL;
    __syncthreads();
    for (uint32_t s = t.first + tid; s < end; s += blockDim.x) idx[s] = tmp[s];
    nL = sNL;
  }
  if (tid == 0) {
    // node box: the union of all bins of one axis
    float l[3] = {INFINITY, INFINITY, INFINITY}, h[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int b = 0; b < SAH_BINS; b++)
      for (int q = 0; q < 3; q++) {
        l[q] = fminf(l[q], floatUnflip(sLo[0][b][q]));
        h[q] = fmaxf(h[q], floatUnflip(sHi[0][b][q]));
      }
    first[t.node] = t.first;
    blo[t.node] = make_float4(l[0], l[1], l[2], __uint_as_float(t.count));
    bhi[t.node] = make_float4(h[0], h[1], h[2], 0.f);
    if (nL == 0 || nL >= t.count) nL = t.count / 2;  // never taken: the partition matches the bins
    const uint32_t cf[2] = {t.first, t.first + nL}, cc[2] = {nL, t.count - nL};
    uint32_t ref[2];
    for (int k = 0; k < 2; k++) {
      if (cc[k] == 1) {
        ref[k] = LEAF_BIT | cf[k];
      } else {
        ref[k] = atomicAdd(&counters[0], 1u);
        SahTask ct;
        ct.first = cf[k];
        ct.count = cc[k];
        ct.node = ref[k];
        ct.pad = 0;
        if (best >= 0) {
          ct.clo = make_float4(floatUnflip(sCb[k][0]), floatUnflip(sCb[k][1]), floatUnflip(sCb[k][2]), 0.f);
          ct.chi = make_float4(floatUnflip(sCb[k][3]), floatUnflip(sCb[k][4]), floatUnflip(sCb[k][5]), 0.f);
        } else {
          ct.clo = t.clo;
          ct.chi = t.chi;
        }
        next[atomicAdd(&counters[1], 1u)] = ct;
      }
    }
    left[t.node] = ref[0];
    right[t.node] = ref[1];
  }
}

struct Task {
  uint32_t ref;   // binary node reference (internal index or LEAF_BIT|sorted index)
  uint32_t wide;  // wide node index to write
};

// Outward-rounded 8-bit bounds of [l, h] on the grid p + q * scale; false if
// they do not fit in 0..255.  Correction loops are bounded.
__device__ __forceinline__ bool quantAxis(float l, float h, float p, float scale, uint8_t &qlo, uint8_t &qhi) {
  float ql = floorf((l - p) / scale);
  for (int i = 0; i < 4 && ql > 0.f && p + ql * scale > l; i++) ql -= 1.f;
  float qh = ceilf((h - p) / scale);
  for (int i = 0; i < 4 && p + qh * scale < h; i++) qh += 1.f;
  const bool ok = ql >= 0.f && qh <= 255.f && p + ql * scale <= l && p + qh * scale >= h;
  qlo = uint8_t(fminf(fmaxf(ql, 0.f), 255.f));
  qhi = uint8_t(fminf(fmaxf(qh, 0.f), 255.f));
  return ok;
}

__device__ __forceinline__ float boxArea(float4 lo, float4 hi) {
  const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
  return dx * dy + dy * dz + dz * dx;
}

__global__ void k_collapse(const Task *tasks, int ntasks, Task *next, uint32_t *counters, const uint32_t *left,
                           const uint32_t *right, const uint32_t *first, const uint32_t *sorted, const float4 *plo,
                           const float4 *phi, const float4 *blo, const float4 *bhi, Node8 *nodes, uint32_t *leafPrim) {
  const int ti = blockIdx.x * blockDim.x + threadIdx.x;
  if (ti >= ntasks) return;
  const Task task = tasks[ti];
  uint32_t ch[8];
  int nc = 0;
  if (task.ref & LEAF_BIT) {
    ch[nc++] = task.ref;
  } else {
    ch[nc++] = left[task.ref];
    ch[nc++] = right[task.ref];
    while (nc < 8) {
      int best = -1;
      float bestA = -1.f;
      for (int c = 0; c < nc; c++) {
        if (ch[c] & LEAF_BIT) continue;
        const float a = boxArea(blo[ch[c]], bhi[ch[c]]);
        if (a > bestA) {
          bestA = a;
          best = c;
        }
      }
      if (best < 0) break;
      const uint32_t r = ch[best];
      ch[best] = left[r];
      ch[nc++] = right[r];
    }
  }
  float4 clo[8], chi[8];
  uint32_t ccnt[8], cfst[8];
  for (int c = 0; c < nc; c++) {
    if (ch[c] & LEAF_BIT) {
      const uint32_t s = ch[c] & ~LEAF_BIT;
      clo[c] = plo[sorted[s]];
      chi[c] = phi[sorted[s]];
      ccnt[c] = 1;
      cfst[c] = s;
    } else {
      clo[c] = blo[ch[c]];
      chi[c] = bhi[ch[c]];
      ccnt[c] = __float_as_uint(clo[c].w);
      cfst[c] = first[ch[c]];
    }
  }
  // node box and quantisation grid
  float nlo[3] = {INFINITY, INFINITY, INFINITY}, nhi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int c = 0; c < nc; c++) {
    nlo[0] = fminf(nlo[0], clo[c].x);
    nlo[1] = fminf(nlo[1], clo[c].y);
    nlo[2] = fminf(nlo[2], clo[c].z);
    nhi[0] = fmaxf(nhi[0], chi[c].x);
    nhi[1] = fmaxf(nhi[1], chi[c].y);
    nhi[2] = fmaxf(nhi[2], chi[c].z);
  }
  // Octant slot order (Ylitie, Karras, Laine, HPG 2017, sec. 3.2): slot s
  // takes the child lying farthest back along the direction of octant s
  // (bit k set: negative along axis k), assigned greedily by lowest cost
  // dot(child centre - node centre, d_s).  A ray of octant o then visits the
  // slots in the order s ^ o = 0, 1, 2, ..., roughly near to far.
  int bySlot[8];
  {
    float cost[8][8];
    for (int c = 0; c < nc; c++) {
      const float dx = 0.5f * (clo[c].x + chi[c].x) - 0.5f * (nlo[0] + nhi[0]);
      const float dy = 0.5f * (clo[c].y + chi[c].y) - 0.5f * (nlo[1] + nhi[1]);
      const float dz = 0.5f * (clo[c].z + chi[c].z) - 0.5f * (nlo[2] + nhi[2]);
      for (int s = 0; s < 8; s++) cost[c][s] = ((s & 1) ? -dx : dx) + ((s & 2) ? -dy : dy) + ((s & 4) ? -dz : dz);
    }
    for (int s = 0; s < 8; s++) bySlot[s] = -1;
    uint32_t freeC = (1u << nc) - 1u, freeS = 0xffu;
    for (int it = 0; it < nc; it++) {
      int bc = -1, bs = -1;
      float bcost = INFINITY;
      for (int c = 0; c < nc; c++) {
        if (!(freeC >> c & 1u)) continue;
        for (int s = 0; s < 8; s++) {
          if (!(freeS >> s & 1u)) continue;
          if (bc < 0 || cost[c][s] < bcost) {
            bcost = cost[c][s];
            bc = c;
            bs = s;
          }
        }
      }
      bySlot[bs] = bc;
      freeC &= ~(1u << bc);
      freeS &= ~(1u << bs);
    }
  }
  // children in slot order
  float4 lo[8], hi[8];
  uint32_t cnt[8], fst[8], ref[8];
  bool used[8], isInt[8];
  int nInt = 0, nPrim = 0;
  for (int s = 0; s < 8; s++) {
    const int c = bySlot[s];
    used[s] = c >= 0;
    isInt[s] = false;
    if (!used[s]) continue;
    lo[s] = clo[c];
    hi[s] = chi[c];
    cnt[s] = ccnt[c];
    fst[s] = cfst[c];
    ref[s] = ch[c];
    isInt[s] = cnt[s] > LEAF_MAX;
    if (isInt[s])
      nInt++;
    else
      nPrim += int(cnt[s]);
  }
  const uint32_t childBase = nInt ? atomicAdd(&counters[0], uint32_t(nInt)) : 0u;
  const uint32_t primBase = nPrim ? atomicAdd(&counters[1], uint32_t(nPrim)) : 0u;
  const uint32_t taskBase = nInt ? atomicAdd(&counters[2], uint32_t(nInt)) : 0u;
  Node8 node;
  node.px = nlo[0];
  node.py = nlo[1];
  node.pz = nlo[2];
  node.childBase = childBase;
  node.primBase = primBase;
  node.imask = 0;
  uint8_t e8[3];
  for (int k = 0; k < 3; k++) {
    const float ext = nhi[k] - nlo[k];
    // the grid step is never below the ulp of the node's coordinates, so each
    // quantisation step moves the decoded bound by at least one ulp
    const float mag = fmaxf(fabsf(nlo[k]), fabsf(nhi[k]));
    const int emin = mag > 0.f ? max(ilogbf(mag) - 23, -126) : -126;
    int e = ext > 0.f ? int(ceilf(log2f(ext / 255.f))) : -126;
    e = max(max(e, emin), -126);
    uint8_t ql[8], qh[8];
    for (int it = 0; it < 32; it++, e++) {
      if (e > 127) {
        e = 127;
      }
      const float scale = __uint_as_float(uint32_t(e + 127) << 23);
      bool ok = true;
      for (int s = 0; s < 8; s++) {
        if (!used[s]) continue;
        const float l = k == 0 ? lo[s].x : (k == 1 ? lo[s].y : lo[s].z);
        const float h = k == 0 ? hi[s].x : (k == 1 ? hi[s].y : hi[s].z);
        ok = ok && quantAxis(l, h, nlo[k], scale, ql[s], qh[s]);
      }
      if (ok || e >= 127) break;
    }
    e8[k] = uint8_t(e + 127);
    for (int s = 0; s < 8; s++) {
      node.qlo[k][s] = used[s] ? ql[s] : uint8_t(255);
      node.qhi[k][s] = used[s] ? qh[s] : uint8_t(0);
    }
  }
  node.ex = e8[0];
  node.ey = e8[1];
  node.ez = e8[2];
  // internal children are stored in slot order, so child slot s is node
  // childBase + popc(imask & ((1 << s) - 1)); leaf primitives likewise
  int ii = 0, po = 0;
  for (int s = 0; s < 8; s++) {
    if (!used[s]) {
      node.meta[s] = 0;
      continue;
    }
    if (isInt[s]) {
      node.meta[s] = uint8_t(0x80 | ii);
      node.imask |= uint8_t(1u << s);
      next[taskBase + ii] = {ref[s], childBase + uint32_t(ii)};
      ii++;
    } else {
      node.meta[s] = uint8_t((cnt[s] << 5) | uint32_t(po));
      for (uint32_t j = 0; j < cnt[s]; j++) leafPrim[primBase + po + j] = sorted[fst[s] + j];
      po += int(cnt[s]);
    }
  }
  nodes[task.wide] = node;
}

// triangle p belongs to primitive p / primDiv (quads 2, boxes 12), its primID
__global__ void k_gather_tris(const uint32_t *leafPrim, int n, const float *verts, const uint32_t *index,
                              float4 *prims, uint32_t primDiv) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint32_t p = leafPrim[s];
  const uint32_t a = index[3 * p], b = index[3 * p + 1], c = index[3 * p + 2];
  prims[3 * s + 0] = make_float4(verts[3 * a], verts[3 * a + 1], verts[3 * a + 2], __uint_as_float(p / primDiv));
  prims[3 * s + 1] = make_float4(verts[3 * b], verts[3 * b + 1], verts[3 * b + 2], 0.f);
  prims[3 * s + 2] = make_float4(verts[3 * c], verts[3 * c + 1], verts[3 * c + 2], 0.f);
}

__global__ void k_gather_sph(const uint32_t *leafPrim, int n, const float4 *sph, float4 *prims, uint32_t *ids) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint32_t p = leafPrim[s];
  prims[s] = sph[p];
  ids[s] = p;
}

__global__ void k_gather_user(const uint32_t *leafPrim, int n, const float4 *data, int stride, float4 *prims,
                              uint32_t *ids) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint32_t p = leafPrim[s];
  for (int k = 0; k < stride; k++) prims[size_t(s) * stride + k] = data[size_t(p) * stride + k];
  ids[s] = p;
}

inline int blocks(int n, int b) { return (n + b - 1) / b; }

}  // namespace

// Builds the wide BVH over n primitive boxes (device arrays lo/hi, float4).
cudaError_t buildWide(const float4 *lo, const float4 *hi, int n, cudaStream_t st, WideBVH &out, bool sah) {
  out = WideBVH{};
  out.nprims = n;
  if (n <= 0) return cudaSuccess;
  cudaError_t err;
  const int ni = n > 1 ? n - 1 : 1;
  uint32_t *acc, *keys, *vals, *keys2, *vals2, *left, *right, *first, *parentInt, *parentLeaf, *flags, *counters;
  float4 *blo, *bhi;
  Task *qa, *qb;
  SahTask *ra, *rb;
  // one scratch allocation, carved into 16-byte aligned pieces; the sizing
  // pass (base == null) and the carving pass use the same sequence
  char *base = nullptr;
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    char *p = base + off;
    off += (bytes + 15) & ~size_t(15);
    return p;
  };
  auto layout = [&]() {
    off = 0;
    acc = (uint32_t *)carve(16 * 4);
    keys = (uint32_t *)carve(4 * size_t(n));
    vals = (uint32_t *)carve(4 * size_t(n));
    keys2 = (uint32_t *)carve(4 * size_t(n));
    vals2 = (uint32_t *)carve(4 * size_t(n));
    left = (uint32_t *)carve(4 * size_t(ni));
    right = (uint32_t *)carve(4 * size_t(ni));
    first = (uint32_t *)carve(4 * size_t(ni));
    parentInt = (uint32_t *)carve(4 * size_t(ni));
    flags = (uint32_t *)carve(4 * size_t(ni));
    parentLeaf = (uint32_t *)carve(4 * size_t(n));
    counters = (uint32_t *)carve(4 * 4);
    blo = (float4 *)carve(sizeof(float4) * size_t(ni));
    bhi = (float4 *)carve(sizeof(float4) * size_t(ni));
    qa = (Task *)carve(sizeof(Task) * size_t(n + 1));
    qb = (Task *)carve(sizeof(Task) * size_t(n + 1));
    // a level holds at most n/2 tasks (each covers two or more primitives)
    const size_t ns = sah ? size_t(n) / 2 + 1 : 0;
    ra = (SahTask *)carve(sizeof(SahTask) * ns);
    rb = (SahTask *)carve(sizeof(SahTask) * ns);
  };
  layout();  // sizing pass with base == null
  if ((err = cudaMallocAsync(&base, off, st))) return err;
  layout();

  if ((err = cudaMallocAsync(&out.nodes, sizeof(Node8) * size_t(n + 1), st))) return err;
  if ((err = cudaMallocAsync(&out.leafPrim, sizeof(uint32_t) * size_t(n), st))) return err;

  const uint32_t accInit[12] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0, 0, 0,
                                0xffffffffu, 0xffffffffu, 0xffffffffu, 0, 0, 0};
  cudaMemcpyAsync(acc, accInit, sizeof(accInit), cudaMemcpyHostToDevice, st);
  k_bounds<<<std::min(blocks(n, 256), 1024), 256, 0, st>>>(lo, hi, n, acc);
  k_morton<<<blocks(n, 256), 256, 0, st>>>(lo, hi, n, acc, keys, vals);
  size_t tmpBytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmpBytes, keys, keys2, vals, vals2, n, 0, 30, st);
  void *tmp = nullptr;
  if ((err = cudaMallocAsync(&tmp, tmpBytes, st))) return err;
  cub::DeviceRadixSort::SortPairs(tmp, tmpBytes, keys, keys2, vals, vals2, n, 0, 30, st);
  cudaFreeAsync(tmp, st);
  const uint32_t *sorted = vals2;
  Task root = {n > 1 ? 0u : LEAF_BIT, 0u};
  uint32_t *hcnt = nullptr;
  cudaMallocHost(&hcnt, 16);
  if (n > 1 && !sah) {
    cudaMemsetAsync(flags, 0, 4 * size_t(ni), st);
    k_karras<<<blocks(n - 1, 256), 256, 0, st>>>(keys2, n, left, right, first, parentInt, parentLeaf);
    k_bottom_up<<<blocks(n, 256), 256, 0, st>>>(n, left, right, parentInt, parentLeaf, sorted, lo, hi, blo, bhi,
                                                 flags);
  } else if (n > 1) {
    // top-down binned SAH from the Morton order, one level per launch; the
    // index array (sorted) is partitioned in place, keys serve as scratch
    k_sah_root<<<1, 1, 0, st>>>(acc, n, ra);
    uint32_t *idx = vals2;
    const uint32_t cinitSah[2] = {1, 0};
    cudaMemcpyAsync(counters, cinitSah, sizeof(cinitSah), cudaMemcpyHostToDevice, st);
    int nt = 1;
    for (int level = 0; nt > 0; level++) {
      if (level > n + 64) {
        err = cudaErrorUnknown;
        break;
      }
      cudaMemsetAsync(counters + 1, 0, 4, st);
      // few large ranges near the root: wide blocks; many small ones: narrow
      const int threads = nt <= 4 * 152 ? SAH_MAX_THREADS : 64;
      k_sah_level<<<nt, threads, 0, st>>>(ra, rb, idx, keys, lo, hi, counters, left, right, first, blo, bhi);
      cudaMemcpyAsync(hcnt, counters, 8, cudaMemcpyDeviceToHost, st);
      if ((err = cudaStreamSynchronize(st))) break;
      nt = int(hcnt[1]);
      std::swap(ra, rb);
    }
  }
  if (err != cudaSuccess) {
    cudaFreeHost(hcnt);
    cudaFreeAsync(base, st);
    return err;
  }
  const uint32_t cinit[4] = {1, 0, 0, 0};
  cudaMemcpyAsync(qa, &root, sizeof(Task), cudaMemcpyHostToDevice, st);
  int ntasks = 1;
  cudaMemcpyAsync(counters, cinit, sizeof(cinit), cudaMemcpyHostToDevice, st);
  // every level consumes at least one binary level, so 2n+64 levels bound it
  for (int level = 0; ntasks > 0; level++) {
    if (level > 2 * n + 64) {
      err = cudaErrorUnknown;
      break;
    }
    cudaMemsetAsync(counters + 2, 0, 4, st);
    k_collapse<<<blocks(ntasks, 128), 128, 0, st>>>(qa, ntasks, qb, counters, left, right, first, sorted, lo, hi, blo,
                                                    bhi, out.nodes, out.leafPrim);
    cudaMemcpyAsync(hcnt, counters, 16, cudaMemcpyDeviceToHost, st);
    if ((err = cudaStreamSynchronize(st))) break;
    ntasks = int(hcnt[2]);
    std::swap(qa, qb);
  }
  out.nnodes = int(hcnt[0]);
  uint32_t accHost[12];
  cudaMemcpyAsync(accHost, acc, sizeof(accHost), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  cudaFreeHost(hcnt);
  for (int k = 0; k < 3; k++) {
    auto unflip = [](uint32_t u) {
      const uint32_t v = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
      float f;
      memcpy(&f, &v, 4);
      return f;
    };
    out.lo[k] = unflip(accHost[6 + k]);
    out.hi[k] = unflip(accHost[9 + k]);
  }
  cudaFreeAsync(base, st);
  if (err != cudaSuccess) return err;
  return cudaGetLastError();
}

cudaError_t buildTriangleBLAS(const float *d_verts, const uint32_t *d_index, int ntris, cudaStream_t st, BLAS &out,
                              bool sah, int primDiv) {
  out = BLAS{};
  if (ntris <= 0) return cudaSuccess;
  float4 *lo, *hi;
  cudaError_t err;
  if ((err = cudaMallocAsync(&lo, sizeof(float4) * ntris, st))) return err;
  if ((err = cudaMallocAsync(&hi, sizeof(float4) * ntris, st))) return err;
  k_tri_bounds<<<blocks(ntris, 256), 256, 0, st>>>(d_verts, d_index, ntris, lo, hi);
  if ((err = buildWide(lo, hi, ntris, st, out.bvh, sah))) return err;
  if ((err = cudaMallocAsync(&out.prims, sizeof(float4) * 3 * size_t(ntris), st))) return err;
  k_gather_tris<<<blocks(ntris, 256), 256, 0, st>>>(out.bvh.leafPrim, ntris, d_verts, d_index, out.prims,
                                                    uint32_t(primDiv));
  cudaFreeAsync(lo, st);
  cudaFreeAsync(hi, st);
  return cudaStreamSynchronize(st);
}

cudaError_t buildSphereBLAS(const float4 *d_sph, int n, cudaStream_t st, BLAS &out, bool sah) {
  out = BLAS{};
  if (n <= 0) return cudaSuccess;
  float4 *lo, *hi;
  cudaError_t err;
  if ((err = cudaMallocAsync(&lo, sizeof(float4) * n, st))) return err;
  if ((err = cudaMallocAsync(&hi, sizeof(float4) * n, st))) return err;
  k_sph_bounds<<<blocks(n, 256), 256, 0, st>>>(d_sph, n, lo, hi);
  if ((err = buildWide(lo, hi, n, st, out.bvh, sah))) return err;
  if ((err = cudaMallocAsync(&out.prims, sizeof(float4) * size_t(n), st))) return err;
  if ((err = cudaMallocAsync(&out.primIDs, sizeof(uint32_t) * size_t(n), st))) return err;
  k_gather_sph<<<blocks(n, 256), 256, 0, st>>>(out.bvh.leafPrim, n, d_sph, out.prims, out.primIDs);
  cudaFreeAsync(lo, st);
  cudaFreeAsync(hi, st);
  return cudaStreamSynchronize(st);
}

cudaError_t buildUserBLAS(uint32_t type, const float4 *d_data, int n, cudaStream_t st, BLAS &out, bool sah) {
  out = BLAS{};
  if (n <= 0) return cudaSuccess;
  const int stride = primStride(type);
  float4 *lo, *hi;
  cudaError_t err;
  if ((err = cudaMallocAsync(&lo, sizeof(float4) * n, st))) return err;
  if ((err = cudaMallocAsync(&hi, sizeof(float4) * n, st))) return err;
  k_user_bounds<<<blocks(n, 256), 256, 0, st>>>(d_data, stride, n, type, lo, hi);
  if ((err = buildWide(lo, hi, n, st, out.bvh, sah))) return err;
  if ((err = cudaMallocAsync(&out.prims, sizeof(float4) * size_t(n) * stride, st))) return err;
  if ((err = cudaMallocAsync(&out.primIDs, sizeof(uint32_t) * size_t(n), st))) return err;
  k_gather_user<<<blocks(n, 256), 256, 0, st>>>(out.bvh.leafPrim, n, d_data, stride, out.prims, out.primIDs);
  cudaFreeAsync(lo, st);
  cudaFreeAsync(hi, st);
  return cudaStreamSynchronize(st);
}

void freeBLAS(BLAS &b, cudaStream_t st) {
  if (b.bvh.nodes) cudaFreeAsync(b.bvh.nodes, st);
  if (b.bvh.leafPrim) cudaFreeAsync(b.bvh.leafPrim, st);
  if (b.prims) cudaFreeAsync(b.prims, st);
  if (b.primIDs) cudaFreeAsync(b.primIDs, st);
  b = BLAS{};
}

}  // namespace b200
