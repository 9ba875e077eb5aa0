// Neural radiance cache: fused inference / training kernels, Adam, and the
// b200_nrc_* C ABI.  See nrc.cuh for the model and the published methods.
#include <cmath>
#include <cstring>
#include <vector>

#include <algorithm>

#include "api_internal.h"
#include "nrc.cuh"

namespace b200 {
namespace nrc {

struct Params {
  GridD grid;
  const __half2 *table;     // [LEVELS][TSIZE] features
  const __nv_bfloat16 *w;   // per layer row-major [in][out]
  const __nv_bfloat16 *wt;  // per layer row-major [out][in]
};

constexpr int LAYER_OUT_OFF = HIDDEN * WIDTH * WIDTH;  // offset of the output layer (64 x 16)
constexpr int W_ROWS = NUM_W / WIDTH;                 // rows of 64 in the [out][in] weights
constexpr int WARPS = 4;                              // warps per block of the fused kernels
constexpr int XS = WIDTH;                             // row stride of the training kernel's activation tiles
// The inference kernel pads its shared-memory rows (weights and the input
// tile) to 72 BF16 (144 B): rows 64 wide (128 B) put the 8 rows an m16n8k16
// fragment load reads into one bank (8-way conflicts); 144-byte rows shift
// each row by 4 banks.
constexpr int XI = WIDTH + 8;                         // inference: row stride of weights and input tile

namespace {

// ---------------------------------------------------------------- encoding
// One warp encodes its 16 samples: lanes 0-15 the hash grid of sample `lane`,
// lanes 16-31 the other inputs of sample `lane - 16`.
B200_D void encodeTile(const Params &P, const float *rec, bool valid, __nv_bfloat16 *X, int ldx, int lane) {
  const int s = lane & 15;
  const float *r = rec + s * REC;
  __nv_bfloat16 *row = X + s * ldx;
  if (lane < 16) {
    for (int l = 0; l < LEVELS; l++) {
      float f0 = 0.f, f1 = 0.f;
      if (valid) {
        const Cell c = gridCell(P.grid, l, r);
        const __half2 *T = P.table + size_t(l) * TSIZE;
        for (int k = 0; k < 8; k++) {
          const uint32_t dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
          const float w = (dx ? c.fx : 1.f - c.fx) * (dy ? c.fy : 1.f - c.fy) * (dz ? c.fz : 1.f - c.fz);
          const float2 v = __half22float2(T[gridIndex(P.grid, l, c.x + dx, c.y + dy, c.z + dz)]);
          f0 += w * v.x;
          f1 += w * v.y;
        }
      }
      *reinterpret_cast<uint32_t *>(row + 2 * l) = packBF16(f0, f1);
    }
  } else {
    float o[32];
    for (int k = 0; k < 32; k++) o[k] = 0.f;
    if (valid) {
      shEncode(r[3], r[4], r[5], o);
      o[COL_N - COL_SH + 0] = r[6];
      o[COL_N - COL_SH + 1] = r[7];
      o[COL_N - COL_SH + 2] = r[8];
      o[COL_R - COL_SH] = r[9];
      o[COL_A - COL_SH + 0] = r[10];
      o[COL_A - COL_SH + 1] = r[11];
      o[COL_A - COL_SH + 2] = r[12];
      o[COL_ONE - COL_SH] = 1.f;
    }
    for (int k = 0; k < 32; k += 2) *reinterpret_cast<uint32_t *>(row + COL_SH + k) = packBF16(o[k], o[k + 1]);
  }
}

// ---------------------------------------------------------------- forward
// Runs the hidden layers on the A operand a[4][4] (replaced by the last
// hidden activation); with `store`, writes every hidden activation H_1..H_4
// (BF16, after ReLU) to H + (l * 16 * XS).  LDW: the row stride of wt.
template <int LDW>
B200_D void hiddenLayers(const Params &P, const __nv_bfloat16 *wt, uint32_t a[4][4], __nv_bfloat16 *H, bool store,
                         int lane) {
  const int g = lane >> 2, t = lane & 3;
  for (int l = 0; l < HIDDEN; l++) {
    float c[8][4];
    for (int j = 0; j < 8; j++) {
      c[j][0] = c[j][1] = c[j][2] = c[j][3] = 0.f;
      for (int kk = 0; kk < 4; kk++) {
        uint32_t b0, b1;
        loadBT(wt + l * WIDTH * LDW, LDW, kk, j, lane, b0, b1);
        mma16816(c[j], a[kk], b0, b1);
      }
    }
    for (int kk = 0; kk < 4; kk++) {
      a[kk][0] = packBF16(fmaxf(c[2 * kk][0], 0.f), fmaxf(c[2 * kk][1], 0.f));
      a[kk][1] = packBF16(fmaxf(c[2 * kk][2], 0.f), fmaxf(c[2 * kk][3], 0.f));
      a[kk][2] = packBF16(fmaxf(c[2 * kk + 1][0], 0.f), fmaxf(c[2 * kk + 1][1], 0.f));
      a[kk][3] = packBF16(fmaxf(c[2 * kk + 1][2], 0.f), fmaxf(c[2 * kk + 1][3], 0.f));
      if (store) {
        __nv_bfloat16 *Hl = H + l * 16 * XS;
        *reinterpret_cast<uint32_t *>(Hl + g * XS + 16 * kk + 2 * t) = a[kk][0];
        *reinterpret_cast<uint32_t *>(Hl + (g + 8) * XS + 16 * kk + 2 * t) = a[kk][1];
        *reinterpret_cast<uint32_t *>(Hl + g * XS + 16 * kk + 8 + 2 * t) = a[kk][2];
        *reinterpret_cast<uint32_t *>(Hl + (g + 8) * XS + 16 * kk + 8 + 2 * t) = a[kk][3];
      }
    }
  }
}

// output layer: o[j] accumulators of n-tile j (columns 8j..8j+7; 0..2 used)
template <int LDW>
B200_D void outputLayer(const __nv_bfloat16 *wt, const uint32_t a[4][4], float o[2][4], int lane) {
  for (int j = 0; j < 2; j++) {
    o[j][0] = o[j][1] = o[j][2] = o[j][3] = 0.f;
    for (int kk = 0; kk < 4; kk++) {
      uint32_t b0, b1;
      loadBT(wt + HIDDEN * WIDTH * LDW, LDW, kk, j, lane, b0, b1);
      mma16816(o[j], a[kk], b0, b1);
    }
  }
}

// n = min(*dn, nmax) when dn is given (a count produced on the device)
B200_D long long deviceCount(long long nmax, const uint32_t *dn, long long offset) {
  if (!dn) return nmax;
  const long long c = (long long)*(volatile const uint32_t *)dn - offset;
  return c < 0 ? 0 : (c < nmax ? c : nmax);
}

__global__ void __launch_bounds__(WARPS * 32) k_nrc_infer(Params P, const float *__restrict__ q, long long nmax,
                                                          const uint32_t *dn, float *__restrict__ out) {
  const long long n = deviceCount(nmax, dn, 0);
  extern __shared__ __align__(16) unsigned char smem[];
  __nv_bfloat16 *wt = reinterpret_cast<__nv_bfloat16 *>(smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *rec = reinterpret_cast<float *>(smem + W_ROWS * XI * 2) + warp * 16 * REC;
  __nv_bfloat16 *X = reinterpret_cast<__nv_bfloat16 *>(smem + W_ROWS * XI * 2 + WARPS * 16 * REC * 4) + warp * 16 * XI;
  // the [out][in] weights, rows of 64 padded to XI
  for (int i = threadIdx.x; i < NUM_W / 2; i += blockDim.x) {
    const int row = (2 * i) / WIDTH, col = (2 * i) % WIDTH;
    reinterpret_cast<uint32_t *>(wt)[(row * XI + col) / 2] = reinterpret_cast<const uint32_t *>(P.wt)[i];
  }
  __syncthreads();
  const long long tiles = (n + 15) / 16;
  for (long long tile = blockIdx.x * (long long)WARPS + warp; tile < tiles; tile += (long long)gridDim.x * WARPS) {
    const long long base = tile * 16;
    for (int k = lane; k < 16 * REC; k += 32) {
      const long long i = base + k / REC;
      rec[k] = i < n ? q[i * REC + k % REC] : 0.f;
    }
    __syncwarp();
    encodeTile(P, rec, base + (lane & 15) < n, X, XI, lane);
    __syncwarp();
    uint32_t a[4][4];
    for (int kk = 0; kk < 4; kk++) loadA(X, XI, kk, lane, a[kk]);
    hiddenLayers<XI>(P, wt, a, nullptr, false, lane);
    float o[2][4];
    outputLayer<XI>(wt, a, o, lane);
    const int g = lane >> 2, t = lane & 3;
    for (int h = 0; h < 2; h++) {
      const long long i = base + g + 8 * h;
      if (i >= n) continue;
      for (int e = 0; e < 2; e++) {
        const int col = 2 * t + e;
        if (col < 3) out[i * 3 + col] = o[0][2 * h + e];
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------- backward
B200_D uint32_t pack2(const __nv_bfloat16 *p0, const __nv_bfloat16 *p1) {
  return uint32_t(*reinterpret_cast<const uint16_t *>(p0)) | (uint32_t(*reinterpret_cast<const uint16_t *>(p1)) << 16);
}

// dW[in][out] += Act^T x dZ over the tile's 16 samples (K = samples):
// Act 16 x 64, dZ 16 x (8 * ntiles) with row stride ldz; dW row stride ldz
B200_D void weightGrad(const __nv_bfloat16 *Act, const __nv_bfloat16 *dZ, int ntiles, int ldz, float *dW, int lane) {
  const int g = lane >> 2, t = lane & 3;
  for (int mi = 0; mi < 4; mi++) {
    uint32_t a[4];
    const int m0 = 16 * mi + g;
    a[0] = pack2(Act + (2 * t) * XS + m0, Act + (2 * t + 1) * XS + m0);
    a[1] = pack2(Act + (2 * t) * XS + m0 + 8, Act + (2 * t + 1) * XS + m0 + 8);
    a[2] = pack2(Act + (2 * t + 8) * XS + m0, Act + (2 * t + 9) * XS + m0);
    a[3] = pack2(Act + (2 * t + 8) * XS + m0 + 8, Act + (2 * t + 9) * XS + m0 + 8);
    for (int j = 0; j < ntiles; j++) {
      const int n0 = 8 * j + g;
      const uint32_t b0 = pack2(dZ + (2 * t) * ldz + n0, dZ + (2 * t + 1) * ldz + n0);
      const uint32_t b1 = pack2(dZ + (2 * t + 8) * ldz + n0, dZ + (2 * t + 9) * ldz + n0);
      float c[4] = {0.f, 0.f, 0.f, 0.f};
      mma16816(c, a, b0, b1);
      const int col = 8 * j + 2 * t;
      atomicAdd(dW + m0 * ldz + col, c[0]);
      atomicAdd(dW + m0 * ldz + col + 1, c[1]);
      atomicAdd(dW + (m0 + 8) * ldz + col, c[2]);
      atomicAdd(dW + (m0 + 8) * ldz + col + 1, c[3]);
    }
  }
}

// the table gradient of one sample and level: d(features) spread over the cell
B200_D void scatterGrid(const Params &P, const float *r, int level, float d0, float d1, float *tgrad) {
  const Cell c = gridCell(P.grid, level, r);
  float *G = tgrad + size_t(level) * TSIZE * FEAT;
  for (int k = 0; k < 8; k++) {
    const uint32_t dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
    const float w = (dx ? c.fx : 1.f - c.fx) * (dy ? c.fy : 1.f - c.fy) * (dz ? c.fz : 1.f - c.fz);
    const uint32_t idx = gridIndex(P.grid, level, c.x + dx, c.y + dy, c.z + dz);
    atomicAdd(G + size_t(idx) * 2, w * d0);
    atomicAdd(G + size_t(idx) * 2 + 1, w * d1);
  }
}

// Forward + backward of the relative L2 loss (Mueller et al. 2021):
//   L = 1/(3N) sum_s sum_c (o - y)^2 / (sg(o)^2 + 0.01)
// Gradients are summed into wgrad (17,408) and tgrad (table, FP32); the loss
// sum into *loss.
__global__ void __launch_bounds__(WARPS * 32) k_nrc_train(Params P, const float *__restrict__ samples, long long nmax,
                                                          const uint32_t *dn, long long offset, float *wgrad,
                                                          float *tgrad, float *loss) {
  const long long n = deviceCount(nmax, dn, offset);
  const float invN3 = n > 0 ? 1.f / (3.f * float(n)) : 0.f;
  extern __shared__ __align__(16) unsigned char smem[];
  __nv_bfloat16 *w = reinterpret_cast<__nv_bfloat16 *>(smem);
  __nv_bfloat16 *wt = w + NUM_W;
  float *dWs = reinterpret_cast<float *>(wt + NUM_W);
  unsigned char *per = reinterpret_cast<unsigned char *>(dWs + NUM_W);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // per warp: records (16 x 16 floats), X + H1..H4 (5 x 16 x 64), dZ (16 x 64), dOut (16 x 16)
  constexpr int PER_WARP = 16 * REC * 4 + 5 * 16 * XS * 2 + 16 * XS * 2 + 16 * 16 * 2;
  float *rec = reinterpret_cast<float *>(per + warp * PER_WARP);
  __nv_bfloat16 *X = reinterpret_cast<__nv_bfloat16 *>(rec + 16 * REC);
  __nv_bfloat16 *H = X + 16 * XS;  // H1..H4
  __nv_bfloat16 *dZ = H + 4 * 16 * XS;
  __nv_bfloat16 *dO = dZ + 16 * XS;
  for (int i = threadIdx.x; i < NUM_W / 2; i += blockDim.x) {
    reinterpret_cast<uint32_t *>(w)[i] = reinterpret_cast<const uint32_t *>(P.w)[i];
    reinterpret_cast<uint32_t *>(wt)[i] = reinterpret_cast<const uint32_t *>(P.wt)[i];
  }
  for (int i = threadIdx.x; i < NUM_W; i += blockDim.x) dWs[i] = 0.f;
  __syncthreads();
  const int g = lane >> 2, t = lane & 3;
  float lossSum = 0.f;
  const long long tiles = (n + 15) / 16;
  for (long long tile = blockIdx.x * (long long)WARPS + warp; tile < tiles; tile += (long long)gridDim.x * WARPS) {
    const long long base = tile * 16;
    for (int k = lane; k < 16 * REC; k += 32) {
      const long long i = base + k / REC;
      rec[k] = i < n ? samples[i * REC + k % REC] : 0.f;
    }
    __syncwarp();
    encodeTile(P, rec, base + (lane & 15) < n, X, XS, lane);
    __syncwarp();
    uint32_t a[4][4];
    for (int kk = 0; kk < 4; kk++) loadA(X, XS, kk, lane, a[kk]);
    hiddenLayers<WIDTH>(P, wt, a, H, true, lane);
    float o[2][4];
    outputLayer<WIDTH>(wt, a, o, lane);
    // loss gradient (columns 0..2 of n-tile 0), staged as dOut 16 x 16
    float d[4];
    for (int q = 0; q < 4; q++) {
      const int row = g + 8 * (q >> 1), col = 2 * t + (q & 1);
      d[q] = 0.f;
      if (col < 3 && base + row < n) {
        const float y = rec[row * REC + 13 + col], ov = o[0][q];
        const float den = ov * ov + 0.01f;
        const float diff = ov - y;
        lossSum += diff * diff / den;
        d[q] = 2.f * diff / den * invN3;
      }
    }
    *reinterpret_cast<uint32_t *>(dO + g * 16 + 2 * t) = packBF16(d[0], d[1]);
    *reinterpret_cast<uint32_t *>(dO + (g + 8) * 16 + 2 * t) = packBF16(d[2], d[3]);
    *reinterpret_cast<uint32_t *>(dO + g * 16 + 8 + 2 * t) = 0u;
    *reinterpret_cast<uint32_t *>(dO + (g + 8) * 16 + 8 + 2 * t) = 0u;
    __syncwarp();
    // output layer: dW4 += H4^T dOut, dH4 = dOut W4^T
    weightGrad(H + 3 * 16 * XS, dO, 2, OUT_PAD, dWs + LAYER_OUT_OFF, lane);
    uint32_t ad[4];
    ad[0] = packBF16(d[0], d[1]);
    ad[1] = packBF16(d[2], d[3]);
    ad[2] = 0u;
    ad[3] = 0u;
    float c[8][4];
    for (int j = 0; j < 8; j++) {
      c[j][0] = c[j][1] = c[j][2] = c[j][3] = 0.f;
      uint32_t b0, b1;
      loadBT(w + LAYER_OUT_OFF, OUT_PAD, 0, j, lane, b0, b1);
      mma16816(c[j], ad, b0, b1);
    }
    for (int l = HIDDEN - 1; l >= 0; l--) {
      // c = dH_{l+1}; through the ReLU into dZ_l (stored and as the A operand)
      const __nv_bfloat16 *Hl = H + l * 16 * XS;  // H_{l+1}
      uint32_t az[4][4];
      for (int j = 0; j < 8; j++) {
        const int col = 8 * j + 2 * t;
        const __nv_bfloat16 *h0 = Hl + g * XS + col, *h1 = Hl + (g + 8) * XS + col;
        const float v0 = __bfloat162float(h0[0]) > 0.f ? c[j][0] : 0.f;
        const float v1 = __bfloat162float(h0[1]) > 0.f ? c[j][1] : 0.f;
        const float v2 = __bfloat162float(h1[0]) > 0.f ? c[j][2] : 0.f;
        const float v3 = __bfloat162float(h1[1]) > 0.f ? c[j][3] : 0.f;
        const uint32_t p01 = packBF16(v0, v1), p23 = packBF16(v2, v3);
        *reinterpret_cast<uint32_t *>(dZ + g * XS + col) = p01;
        *reinterpret_cast<uint32_t *>(dZ + (g + 8) * XS + col) = p23;
        az[j >> 1][(j & 1) * 2 + 0] = p01;
        az[j >> 1][(j & 1) * 2 + 1] = p23;
      }
      __syncwarp();
      const __nv_bfloat16 *Al = l == 0 ? X : H + (l - 1) * 16 * XS;
      weightGrad(Al, dZ, 8, WIDTH, dWs + l * WIDTH * WIDTH, lane);
      // dA_l = dZ_l W_l^T
      for (int j = 0; j < 8; j++) {
        c[j][0] = c[j][1] = c[j][2] = c[j][3] = 0.f;
        for (int kk = 0; kk < 4; kk++) {
          uint32_t b0, b1;
          loadBT(w + l * WIDTH * WIDTH, WIDTH, kk, j, lane, b0, b1);
          mma16816(c[j], az[kk], b0, b1);
        }
      }
      __syncwarp();
    }
    // c = dX: the hash-grid columns 0..31 (n-tiles 0..3): level 4j + t
    for (int j = 0; j < 4; j++)
      for (int h = 0; h < 2; h++) {
        const int row = g + 8 * h;
        if (base + row < n) scatterGrid(P, rec + row * REC, 4 * j + t, c[j][2 * h], c[j][2 * h + 1], tgrad);
      }
    __syncwarp();
  }
  // warp loss sums, then the block's weight gradients into the global sum
  for (int off = 16; off; off >>= 1) lossSum += __shfl_xor_sync(0xffffffffu, lossSum, off);
  if (lane == 0) atomicAdd(loss, lossSum * invN3);
  __syncthreads();
  for (int i = threadIdx.x; i < NUM_W; i += blockDim.x)
    if (dWs[i] != 0.f) atomicAdd(wgrad + i, dWs[i]);
}

constexpr size_t kInferSmem = size_t(W_ROWS) * XI * 2 + WARPS * 16 * REC * 4 + WARPS * 16 * XI * 2;
constexpr size_t kTrainSmem = size_t(NUM_W) * 2 * 2 + size_t(NUM_W) * 4 +
                              WARPS * (16 * REC * 4 + 5 * 16 * XS * 2 + 16 * XS * 2 + 16 * 16 * 2);
static_assert(kTrainSmem <= 227 * 1024, "training kernel shared memory");

// ---------------------------------------------------------------- Adam and parameter copies
// skipped when the step's device-side sample count (dn - offset) is zero
__global__ void k_adam(float *__restrict__ p, float *__restrict__ m, float *__restrict__ v,
                       const float *__restrict__ g, long long n, float lr, float b1, float b2, float eps, float bc1,
                       float bc2, const uint32_t *dn, long long offset) {
  if (dn && deviceCount(1, dn, offset) == 0) return;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  }
}

// master FP32 weights -> BF16 [in][out] and [out][in] copies
__global__ void k_weights_to_bf16(const float *__restrict__ wm, __nv_bfloat16 *w, __nv_bfloat16 *wt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NUM_W) return;
  const __nv_bfloat16 b = __float2bfloat16_rn(wm[i]);
  w[i] = b;
  int in, out, base, nout;
  if (i < LAYER_OUT_OFF) {
    base = (i / (WIDTH * WIDTH)) * WIDTH * WIDTH;
    nout = WIDTH;
  } else {
    base = LAYER_OUT_OFF;
    nout = OUT_PAD;
  }
  in = (i - base) / nout;
  out = (i - base) % nout;
  wt[base + out * WIDTH + in] = b;
}

__global__ void k_table_to_half(const float *__restrict__ tm, __half2 *t, long long pairs) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < pairs; i += (long long)gridDim.x * blockDim.x)
    t[i] = __floats2half2_rn(tm[2 * i], tm[2 * i + 1]);
}

B200_D float hashUniform(uint32_t seed, uint32_t i) {
  uint32_t h = i * 747796405u + seed * 2891336453u + 1u;
  h = ((h >> ((h >> 28) + 4u)) ^ h) * 277803737u;
  h = (h >> 22) ^ h;
  return (h >> 8) * (1.f / 16777216.f);
}

__global__ void k_nrc_init(float *wm, float *tm, long long nt, uint32_t seed) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nt; i += (long long)gridDim.x * blockDim.x) {
    tm[i] = (hashUniform(seed, uint32_t(i)) * 2.f - 1.f) * 1e-4f;
    if (i < NUM_W) {
      const int fanOut = i < LAYER_OUT_OFF ? WIDTH : OUT_PAD;
      const float lim = sqrtf(6.f / float(WIDTH + fanOut));
      wm[i] = (hashUniform(seed ^ 0x9e3779b9u, uint32_t(i)) * 2.f - 1.f) * lim;
    }
  }
}

}  // namespace

// ---------------------------------------------------------------- host object
struct NrcObj {
  DeviceObj *dev;
  GridD grid = {};
  float lr = 1e-2f, beta1 = 0.9f, beta2 = 0.99f, eps = 1e-8f;
  int step = 0;
  __half2 *table = nullptr;
  float *tMaster = nullptr, *tGrad = nullptr, *tM = nullptr, *tV = nullptr;
  __nv_bfloat16 *w = nullptr, *wt = nullptr;
  float *wMaster = nullptr, *wGrad = nullptr, *wM = nullptr, *wV = nullptr;
  float *dLoss = nullptr;
  bool attrsSet = false;

  NrcObj(DeviceObj *d, const float lo[3], const float hi[3], float learningRate, uint32_t seed) : dev(d) {
    dev->retain();
    float ext = 0.f;
    for (int k = 0; k < 3; k++) {
      grid.lo[k] = lo[k];
      ext = std::fmax(ext, hi[k] - lo[k]);
    }
    if (!(ext > 0.f)) throw Error(B200_INVALID_ARGUMENT, "radiance cache: empty bounding box");
    grid.invExtent = 1.f / ext;
    const double b = std::exp(std::log(double(MAX_RES) / BASE_RES) / (LEVELS - 1));
    for (int l = 0; l < LEVELS; l++) {
      const double N = BASE_RES * std::pow(b, l);
      grid.levelScale[l] = float(N - 1.0);
      const double side = std::ceil(N) + 1.0;
      grid.levelDense[l] = side * side * side <= double(TSIZE) ? uint32_t(side) : 0u;
    }
    lr = learningRate;
    auto alloc = [&](void **p, size_t bytes) { check(cudaMalloc(p, bytes), "radiance cache allocation"); };
    alloc((void **)&table, NUM_T / 2 * sizeof(__half2));
    for (float **p : {&tMaster, &tGrad, &tM, &tV}) alloc((void **)p, NUM_T * 4);
    alloc((void **)&w, NUM_W * 2);
    alloc((void **)&wt, NUM_W * 2);
    for (float **p : {&wMaster, &wGrad, &wM, &wV}) alloc((void **)p, NUM_W * 4);
    alloc((void **)&dLoss, 4);
    cudaStream_t st = dev->stream;
    check(cudaMemsetAsync(tM, 0, NUM_T * 4, st), "clear");
    check(cudaMemsetAsync(tV, 0, NUM_T * 4, st), "clear");
    check(cudaMemsetAsync(wM, 0, NUM_W * 4, st), "clear");
    check(cudaMemsetAsync(wV, 0, NUM_W * 4, st), "clear");
    k_nrc_init<<<1024, 256, 0, st>>>(wMaster, tMaster, NUM_T, seed);
    refresh(st);
    check(cudaGetLastError(), "radiance cache init");
  }
  ~NrcObj() {
    cudaSetDevice(dev->dev);
    cudaStreamSynchronize(dev->stream);
    for (void *p : {(void *)table, (void *)tMaster, (void *)tGrad, (void *)tM, (void *)tV, (void *)w, (void *)wt,
                    (void *)wMaster, (void *)wGrad, (void *)wM, (void *)wV, (void *)dLoss, (void *)queries,
                    (void *)qout, (void *)trainVerts, (void *)samples, (void *)qpath, (void *)fcounters})
      if (p) cudaFree(p);
    dev->release();
  }
  void refresh(cudaStream_t st) {
    k_weights_to_bf16<<<(NUM_W + 255) / 256, 256, 0, st>>>(wMaster, w, wt);
    k_table_to_half<<<1024, 256, 0, st>>>(tMaster, table, NUM_T / 2);
  }
  Params params() const { return Params{grid, table, w, wt}; }

  // ---- per-frame buffers of the cache-terminated path tracer
  float *queries = nullptr, *qout = nullptr, *trainVerts = nullptr, *samples = nullptr;
  uint32_t *qpath = nullptr, *fcounters = nullptr;
  long long qcap = 0, vcap = 0;
  void frameBuffers(long long npaths, long long nverts) {
    auto grow = [&](void **p, size_t bytes) {
      if (*p) cudaFree(*p);
      *p = nullptr;
      check(cudaMalloc(p, bytes), "radiance cache frame buffers");
    };
    if (npaths > qcap || nverts > vcap) check(cudaStreamSynchronize(dev->stream), "sync");
    if (npaths > qcap) {
      grow((void **)&queries, size_t(npaths) * REC * 4);
      grow((void **)&qout, size_t(npaths) * 3 * 4);
      grow((void **)&qpath, size_t(npaths) * 4);
      qcap = npaths;
    }
    if (nverts > vcap) {
      grow((void **)&trainVerts, size_t(nverts) * 20 * 4);
      grow((void **)&samples, size_t(nverts) * REC * 4);
      vcap = nverts;
    }
    if (!fcounters) check(cudaMalloc(&fcounters, 16), "radiance cache counters");
  }
  static void inferHook(void *self, cudaStream_t st) {
    NrcObj *o = static_cast<NrcObj *>(self);
    o->infer(o->queries, o->qcap, o->qout, st, o->fcounters);
  }
  void setAttrs() {
    if (attrsSet) return;
    check(cudaFuncSetAttribute(k_nrc_train, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTrainSmem)), "smem");
    check(cudaFuncSetAttribute(k_nrc_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kInferSmem)), "smem");
    attrsSet = true;
  }
  // n queries, or min(*dn, n) when dn (a device count) is given
  void infer(const float *q, long long n, float *out, cudaStream_t st, const uint32_t *dn = nullptr) {
    if (n <= 0) return;
    setAttrs();
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev->dev);
    const long long tiles = (n + 15) / 16;
    const long long blocks = std::min<long long>((tiles + WARPS - 1) / WARPS, (long long)sms * 4);
    k_nrc_infer<<<unsigned(blocks), WARPS * 32, kInferSmem, st>>>(params(), q, n, dn, out);
    check(cudaGetLastError(), "radiance cache inference");
  }
  // gradients of the loss over n samples into wGrad / tGrad (cleared first)
  void gradients(const float *s, long long n, cudaStream_t st, const uint32_t *dn = nullptr, long long offset = 0) {
    setAttrs();
    check(cudaMemsetAsync(tGrad, 0, NUM_T * 4, st), "clear");
    check(cudaMemsetAsync(wGrad, 0, NUM_W * 4, st), "clear");
    check(cudaMemsetAsync(dLoss, 0, 4, st), "clear");
    if (n <= 0) return;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev->dev);
    const long long tiles = (n + 15) / 16;
    const long long blocks = std::min<long long>((tiles + WARPS - 1) / WARPS, (long long)sms);
    k_nrc_train<<<unsigned(blocks), WARPS * 32, kTrainSmem, st>>>(params(), s + offset * REC, n, dn, offset, wGrad,
                                                                   tGrad, dLoss);
    check(cudaGetLastError(), "radiance cache training");
  }
  // one Adam step on n samples (with dn: on min(*dn - offset, n) samples
  // from s + offset records, skipped when that is zero)
  void train(const float *s, long long n, cudaStream_t st, const uint32_t *dn = nullptr, long long offset = 0) {
    gradients(s, n, st, dn, offset);
    if (n <= 0) return;
    step++;
    const float bc1 = 1.f - std::pow(beta1, float(step)), bc2 = 1.f - std::pow(beta2, float(step));
    k_adam<<<2048, 256, 0, st>>>(tMaster, tM, tV, tGrad, NUM_T, lr, beta1, beta2, eps, bc1, bc2, dn, offset);
    k_adam<<<(NUM_W + 255) / 256, 256, 0, st>>>(wMaster, wM, wV, wGrad, NUM_W, lr, beta1, beta2, eps, bc1, bc2, dn,
                                                offset);
    refresh(st);
    check(cudaGetLastError(), "radiance cache Adam step");
  }
};

}  // namespace nrc
}  // namespace b200

using namespace b200;
using b200::nrc::NrcObj;

namespace {
template <class F>
int nrcGuard(DeviceObj *dev, F f) {
  try {
    check(cudaSetDevice(dev->dev), "cudaSetDevice");
    f();
    return B200_NO_ERROR;
  } catch (const Error &e) {
    dev->lastError = e.what();
    return e.code;
  } catch (const std::exception &e) {
    dev->lastError = e.what();
    return B200_UNKNOWN_ERROR;
  }
}
}  // namespace

extern "C" {

int b200_nrc_create(b200_device d, const b200_nrc_desc *desc, b200_nrc *out) {
  if (!d || !desc || !out) return B200_INVALID_ARGUMENT;
  DeviceObj *dev = reinterpret_cast<DeviceObj *>(d);
  return nrcGuard(dev, [&]() {
    *out = reinterpret_cast<b200_nrc>(new NrcObj(dev, desc->boundsLo, desc->boundsHi, desc->learningRate, desc->seed));
  });
}

int b200_nrc_release(b200_nrc h) {
  if (!h) return B200_INVALID_ARGUMENT;
  delete reinterpret_cast<NrcObj *>(h);
  return B200_NO_ERROR;
}

int b200_nrc_infer(b200_nrc h, const float *queries, int64_t n, float *out, void *stream) {
  if (!h || (n > 0 && (!queries || !out))) return B200_INVALID_ARGUMENT;
  NrcObj *o = reinterpret_cast<NrcObj *>(h);
  return nrcGuard(o->dev, [&]() { o->infer(queries, n, out, stream ? (cudaStream_t)stream : o->dev->stream); });
}

int b200_nrc_train(b200_nrc h, const float *samples, int64_t n, float *loss, void *stream) {
  if (!h || (n > 0 && !samples)) return B200_INVALID_ARGUMENT;
  NrcObj *o = reinterpret_cast<NrcObj *>(h);
  return nrcGuard(o->dev, [&]() {
    cudaStream_t st = stream ? (cudaStream_t)stream : o->dev->stream;
    o->train(samples, n, st);
    if (loss) check(cudaMemcpyAsync(loss, o->dLoss, 4, cudaMemcpyDeviceToDevice, st), "loss");
  });
}

int b200_nrc_gradients(b200_nrc h, const float *samples, int64_t n, float *wgrad, float *tgrad, float *loss,
                       void *stream) {
  if (!h || (n > 0 && !samples)) return B200_INVALID_ARGUMENT;
  NrcObj *o = reinterpret_cast<NrcObj *>(h);
  return nrcGuard(o->dev, [&]() {
    cudaStream_t st = stream ? (cudaStream_t)stream : o->dev->stream;
    o->gradients(samples, n, st);
    if (wgrad) check(cudaMemcpyAsync(wgrad, o->wGrad, nrc::NUM_W * 4, cudaMemcpyDeviceToDevice, st), "copy");
    if (tgrad) check(cudaMemcpyAsync(tgrad, o->tGrad, nrc::NUM_T * 4, cudaMemcpyDeviceToDevice, st), "copy");
    if (loss) check(cudaMemcpyAsync(loss, o->dLoss, 4, cudaMemcpyDeviceToDevice, st), "copy");
  });
}

int b200_nrc_get_params(b200_nrc h, float *weights, float *table) {
  if (!h) return B200_INVALID_ARGUMENT;
  NrcObj *o = reinterpret_cast<NrcObj *>(h);
  return nrcGuard(o->dev, [&]() {
    check(cudaStreamSynchronize(o->dev->stream), "sync");
    if (weights) check(cudaMemcpy(weights, o->wMaster, nrc::NUM_W * 4, cudaMemcpyDeviceToHost), "read weights");
    if (table) check(cudaMemcpy(table, o->tMaster, nrc::NUM_T * 4, cudaMemcpyDeviceToHost), "read table");
  });
}

int b200_nrc_set_params(b200_nrc h, const float *weights, const float *table) {
  if (!h) return B200_INVALID_ARGUMENT;
  NrcObj *o = reinterpret_cast<NrcObj *>(h);
  return nrcGuard(o->dev, [&]() {
    check(cudaStreamSynchronize(o->dev->stream), "sync");
    if (weights) check(cudaMemcpy(o->wMaster, weights, nrc::NUM_W * 4, cudaMemcpyHostToDevice), "write weights");
    if (table) check(cudaMemcpy(o->tMaster, table, nrc::NUM_T * 4, cudaMemcpyHostToDevice), "write table");
    o->refresh(o->dev->stream);
    check(cudaStreamSynchronize(o->dev->stream), "sync");
  });
}

void b200_nrc_frame_defaults(b200_nrc_frame *f) {
  if (!f) return;
  f->trainPaths = 16384;
  f->trainSteps = 4;
  f->trainBatch = 16384;
  f->train = 1;
  f->useCache = 1;
  f->epochs = 1;
}

int b200_render_pt_nrc(b200_scene s, const b200_camera_desc *camera, const b200_pt_params *p,
                       const b200_material *materials, int nmaterials, b200_frame f, b200_nrc h,
                       const b200_nrc_frame *nfp, void *stream) {
  if (!s || !camera || !p || !f || !h) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  FrameObj *fb = reinterpret_cast<FrameObj *>(f);
  NrcObj *o = reinterpret_cast<NrcObj *>(h);
  b200_nrc_frame np;
  b200_nrc_frame_defaults(&np);
  if (nfp) np = *nfp;
  return nrcGuard(sc->dev, [&]() {
    if (!sc->committed) throw Error(B200_INVALID_OPERATION, "scene not committed");
    if (o->dev != sc->dev) throw Error(B200_INVALID_ARGUMENT, "the cache belongs to another device");
    if (!(p->pixelSamples >= 1 && p->maxPathLength >= 0 && p->pixelFilter >= B200_PF_POINT &&
          p->pixelFilter <= B200_PF_BLACKMAN_HARRIS && nmaterials >= 0 && (nmaterials == 0 || materials)))
      throw Error(B200_INVALID_ARGUMENT, "bad path tracer parameters");
    if (np.trainPaths < 0 || np.trainSteps < 0 || np.trainBatch < 1 || np.epochs < 0)
      throw Error(B200_INVALID_ARGUMENT, "bad radiance cache frame parameters");
    cudaStream_t st = stream ? (cudaStream_t)stream : sc->dev->stream;
    uploadMaterials(sc, materials, nmaterials);
    const PtParamsD d = makePtParams(*p, sc->nLights, nmaterials);
    DeviceObj *dev = sc->dev;
    const long long npaths = (long long)fb->W * fb->H * p->pixelSamples;
    ensurePtWorkspace(dev, ptWorkspaceBytes(npaths));
    const uint32_t slots = uint32_t(std::min<long long>(np.trainPaths, npaths));
    const uint32_t maxLen1 = uint32_t(p->maxPathLength + 1);
    o->frameBuffers(npaths, std::max<long long>(1, (long long)slots * maxLen1));
    NrcFrameD nf;
    nf.queries = o->queries;
    nf.qpath = o->qpath;
    nf.qout = o->qout;
    nf.counters = o->fcounters;
    nf.trainVerts = o->trainVerts;
    nf.samples = o->samples;
    nf.maxLen1 = maxLen1;
    nf.trainSlots = slots;
    nf.trainStride = slots ? uint32_t(std::max<long long>(1, npaths / slots)) : 1u;
    // a different subset of paths trains every frame
    uint32_t hsh = uint32_t(fb->frameID) * 2654435761u + 0x9e3779b9u;
    hsh ^= hsh >> 15;
    nf.trainOffset = hsh % nf.trainStride;
    nf.sampleCap = uint32_t(o->vcap);
    nf.useCache = np.useCache ? 1u : 0u;
    fb->beginFrame(p->pixelSamples, st);
    check(launchRenderPT(dev->tables, sc->view(), makeCamera(*camera), dev->filter(p->pixelFilter), d,
                         sc->dMaterials, sc->dLights, sc->dLightCdf, dev->albedoTables(), fb->view(), false, dev->ptWs,
                         dev->ptWsBytes, st, &nf, &NrcObj::inferHook, o),
          "path tracer launch");
    fb->frameID++;
    framePostProcess(fb, st);
    if (np.train)
      for (int e = 0; e < np.epochs; e++)
        for (int k = 0; k < np.trainSteps; k++)
          o->train(o->samples, np.trainBatch, st, o->fcounters + 1, (long long)k * np.trainBatch);
  });
}

int b200_nrc_grid(b200_nrc h, float *lo_invext4, float *scales16, uint32_t *dense16) {
  if (!h) return B200_INVALID_ARGUMENT;
  const NrcObj *o = reinterpret_cast<NrcObj *>(h);
  if (lo_invext4) {
    std::memcpy(lo_invext4, o->grid.lo, 12);
    lo_invext4[3] = o->grid.invExtent;
  }
  if (scales16) std::memcpy(scales16, o->grid.levelScale, sizeof(o->grid.levelScale));
  if (dense16) std::memcpy(dense16, o->grid.levelDense, sizeof(o->grid.levelDense));
  return B200_NO_ERROR;
}

}  // extern "C"
