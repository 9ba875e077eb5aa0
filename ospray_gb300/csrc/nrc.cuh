// Neural radiance cache: a multiresolution hash-grid encoding of the hit
// position plus direction / normal / roughness / albedo inputs, and a fully
// fused 64-wide MLP (4 hidden layers, ReLU, no biases beyond a constant-1
// input) whose layers run on the tensor cores in BF16 with FP32 accumulation.
//
// Published methods restated here (no source of either is used):
//   Mueller, Rousselle, Novak, Keller 2021, "Real-time Neural Radiance
//     Caching for Path Tracing" (cache queries at path vertices, training on
//     path-suffix radiance, relative L2 loss with a stop-gradient denominator);
//   Mueller, Evans, Schied, Keller 2022, "Instant Neural Graphics Primitives
//     with a Multiresolution Hash Encoding" (L levels of geometrically growing
//     resolution, spatial hash with primes 1, 2654435761, 805459861 where the
//     dense grid would not fit, trilinear interpolation of F features).
//
// The MLP runs on the 5th-generation tensor cores (tcgen05.mma, BF16 operands
// in shared memory, FP32 accumulators in tensor memory; nrc.cu), 128 samples
// per CTA tile; the weight gradients, reductions over the tile's samples,
// use the warp-level mma.sync below.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "common.cuh"

namespace b200 {
namespace nrc {

constexpr int LEVELS = 16;           // hash-grid levels
constexpr int FEAT = 2;              // features per level (FP16)
constexpr int LOG2_T = 19;           // entries per level = 2^19
constexpr uint32_t TSIZE = 1u << LOG2_T;
constexpr int BASE_RES = 16;         // coarsest grid resolution
constexpr float MAX_RES = 2048.f;    // finest grid resolution
constexpr int WIDTH = 64;            // encoding width = hidden width
constexpr int HIDDEN = 4;            // hidden layers
constexpr int OUT_PAD = 16;          // output layer width (3 used)
constexpr int NUM_W = HIDDEN * WIDTH * WIDTH + WIDTH * OUT_PAD;  // 17,408 weights
constexpr long long NUM_T = (long long)LEVELS * TSIZE * FEAT;    // 16,777,216 table features

// encoding column layout
constexpr int COL_SH = LEVELS * FEAT;  // 32: 16 SH coefficients of the direction
constexpr int COL_N = COL_SH + 16;     // 48: normal
constexpr int COL_R = COL_N + 3;       // 51: roughness
constexpr int COL_A = COL_R + 1;       // 52: albedo
constexpr int COL_ONE = COL_A + 3;     // 55: constant 1

// one query / training sample: 16 floats
//   [0..2] position, [3..5] direction (unit, away from the surface),
//   [6..8] shading normal, [9] roughness, [10..12] albedo, [13..15] target
//   radiance (training) or unused
constexpr int REC = 16;

struct GridD {
  float lo[3];
  float invExtent;  // 1 / largest side of the box: positions map into [0,1]^3
  float levelScale[LEVELS];  // N_l - 1 with N_l = BASE_RES * b^l
  uint32_t levelDense[LEVELS];  // dense side length if (N_l+1)^3 <= T, else 0 (hashed)
};

// the table slot of grid vertex (x, y, z) of a level
B200_D uint32_t gridIndex(const GridD &g, int level, uint32_t x, uint32_t y, uint32_t z) {
  const uint32_t side = g.levelDense[level];
  if (side) return x + side * (y + side * z);
  return (x * 1u ^ y * 2654435761u ^ z * 805459861u) & (TSIZE - 1u);
}

// cell and trilinear weights of a position at a level
struct Cell {
  uint32_t x, y, z;
  float fx, fy, fz;
};

B200_D Cell gridCell(const GridD &g, int level, const float p[3]) {
  Cell c;
  float q[3];
  for (int k = 0; k < 3; k++) {  // rounded per operation, so a CPU float32 restatement finds the same cell
    const float u = fminf(fmaxf(__fmul_rn(__fsub_rn(p[k], g.lo[k]), g.invExtent), 0.f), 1.f);
    q[k] = __fadd_rn(__fmul_rn(u, g.levelScale[level]), 0.5f);
  }
  const float x0 = floorf(q[0]), y0 = floorf(q[1]), z0 = floorf(q[2]);
  c.x = uint32_t(x0);
  c.y = uint32_t(y0);
  c.z = uint32_t(z0);
  c.fx = q[0] - x0;
  c.fy = q[1] - y0;
  c.fz = q[2] - z0;
  return c;
}

// real spherical harmonics up to degree 3 (16 coefficients) of a unit vector
B200_D void shEncode(float x, float y, float z, float *o) {
  const float xx = x * x, yy = y * y, zz = z * z;
  o[0] = 0.28209479177387814f;
  o[1] = -0.48860251190291987f * y;
  o[2] = 0.48860251190291987f * z;
  o[3] = -0.48860251190291987f * x;
  o[4] = 1.0925484305920792f * x * y;
  o[5] = -1.0925484305920792f * y * z;
  o[6] = 0.94617469575755997f * zz - 0.31539156525251999f;
  o[7] = -1.0925484305920792f * x * z;
  o[8] = 0.54627421529603959f * (xx - yy);
  o[9] = 0.59004358992664352f * y * (-3.f * xx + yy);
  o[10] = 2.8906114426405538f * x * y * z;
  o[11] = 0.45704579946446572f * y * (1.f - 5.f * zz);
  o[12] = 0.3731763325901154f * z * (5.f * zz - 3.f);
  o[13] = 0.45704579946446572f * x * (1.f - 5.f * zz);
  o[14] = 1.4453057213202769f * z * (xx - yy);
  o[15] = 0.59004358992664352f * x * (-xx + 3.f * yy);
}

// ---------------------------------------------------------------- mma
B200_D uint32_t packBF16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&v);
}

B200_D void mma16816(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

}  // namespace nrc
}  // namespace b200
