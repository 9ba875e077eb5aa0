// Neural radiance cache: fused inference / training kernels, Adam, and the
// b200_nrc_* C ABI.  See nrc.cuh for the model and the published methods.
#include <cmath>
#include <cstring>
#include <vector>

#include <algorithm>

#include "api_internal.h"
#include "nrc.cuh"
#include "tcgen05.cuh"

namespace b200 {
namespace nrc {

struct Params {
  GridD grid;
  const __half2 *table;     // [LEVELS][TSIZE] features
  const __nv_bfloat16 *w;   // per layer row-major [in][out]
  const __nv_bfloat16 *wt;  // per layer row-major [out][in]
};

constexpr int LAYER_OUT_OFF = HIDDEN * WIDTH * WIDTH;  // offset of the output layer (64 x 16)

namespace {

// n = min(*dn, nmax) when dn is given (a count produced on the device)
B200_D long long deviceCount(long long nmax, const uint32_t *dn, long long offset) {
  if (!dn) return nmax;
  const long long c = (long long)*(volatile const uint32_t *)dn - offset;
  return c < 0 ? 0 : (c < nmax ? c : nmax);
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

// ---------------------------------------------------------------- tensor-core check
// One 128 x N x 64 BF16 GEMM through the tcgen05 path (operands staged in the
// K-major shared-memory layout, accumulator in TMEM, read back by the four
// warps' lane quadrants): the building block of the MLP kernels, checkable
// against a host matrix product.
__global__ void __launch_bounds__(128) k_tc_check(const float *A, const float *B, int N, float *D, uint32_t *status) {
  __shared__ __align__(128) unsigned char sA[128 * 64 * 2];
  __shared__ __align__(128) unsigned char sB[64 * 64 * 2];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmemBase;
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int i = tid; i < 128 * 64; i += 128)
    *reinterpret_cast<__nv_bfloat16 *>(sA + tc::kmajorOffset(i / 64, i % 64, 64)) = __float2bfloat16_rn(A[i]);
  for (int i = tid; i < N * 64; i += 128)
    *reinterpret_cast<__nv_bfloat16 *>(sB + tc::kmajorOffset(i / 64, i % 64, 64)) = __float2bfloat16_rn(B[i]);
  if (warp == 0) tc::tmemAlloc(&tmemBase, 64);
  if (tid == 0) tc::mbarInit(&bar, 1);
  tc::fenceProxyAsync();
  tc::fenceBeforeSync();
  __syncthreads();
  tc::fenceAfterSync();
  const uint32_t tmem = tmemBase;
  if (tid == 0) {
    tc::gemmIssue(tmem, tc::smemAddr(sA), 64, tc::smemAddr(sB), 64, 64, tc::idescBF16(128, N));
    tc::commit(&bar);
  }
  const bool ok = __syncthreads_and(tc::mbarWait(&bar, 0)) != 0;
  tc::fenceAfterSync();
  if (ok) {
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tc::tmemLoad16(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0), v);
      for (int k = 0; k < 16; k++) D[size_t(tid) * N + c0 + k] = v[k];
    }
  } else if (tid == 0) {
    atomicOr(status, 1u);
  }
  tc::fenceBeforeSync();
  __syncthreads();
  if (warp == 0) tc::tmemDealloc(tmem, 64);
}

// ---------------------------------------------------------------- tcgen05 kernels
// The same model on the 5th-generation tensor cores.  A CTA of 128 threads
// (4 warps) owns tiles of 128 samples: thread t encodes sample t into row t
// of the BF16 input tile in shared memory (K-major no-swizzle layout, see
// tcgen05.cuh); one thread issues each layer's GEMM (128 x N x 64 as four
// K = 16 tcgen05.mma) with the FP32 accumulator in tensor memory; every
// thread reads its row back with tcgen05.ld (warp w owns TMEM lanes
// 32w..32w+31 = rows of its threads), applies the ReLU and writes the next
// layer's BF16 input row.  Training also runs the backward data path
// (dA_l = dZ_l W_l^T) on the tensor cores; the weight gradients
// dW_l = A_l^T dZ_l (K = the 128 samples) are reduced per warp with
// mma.sync and added to the global gradient once per tile.
constexpr int TC_M = 128;                          // samples per tile
constexpr uint32_t TC_LAYER_BYTES = 64 * 64 * 2;   // one 64 x 64 BF16 operand
constexpr uint32_t TC_OUT_BYTES = OUT_PAD * 64 * 2;
constexpr uint32_t TC_TILE_BYTES = TC_M * 64 * 2;  // 128 x 64 activation tile
constexpr uint32_t TC_W_BYTES = HIDDEN * TC_LAYER_BYTES + TC_OUT_BYTES;
constexpr uint32_t TC_TMEM_COLS = 64;

// stages the weights as tcgen05 B operands (N x K K-major): `wt` [out][in] as
// forward operands (N = out, K = in), `w` [in][out] as backward ones (N = in,
// K = out; the output layer's K is 16)
B200_D void stageWeights(const Params &P, unsigned char *sWt, unsigned char *sW) {
  for (int i = threadIdx.x; i < NUM_W; i += blockDim.x) {
    const int l = i / (WIDTH * WIDTH), r = i % (WIDTH * WIDTH);
    if (l < HIDDEN) {
      const int o = r / WIDTH, in = r % WIDTH;  // wt: [out][in]
      *reinterpret_cast<__nv_bfloat16 *>(sWt + l * TC_LAYER_BYTES + tc::kmajorOffset(o, in, 64)) = P.wt[i];
      if (sW) {  // w: [in][out] -> operand rows = in, K = out
        const int in2 = r / WIDTH, o2 = r % WIDTH;
        *reinterpret_cast<__nv_bfloat16 *>(sW + l * TC_LAYER_BYTES + tc::kmajorOffset(in2, o2, 64)) = P.w[i];
      }
    } else {
      const int j = i - LAYER_OUT_OFF;
      const int o = j / WIDTH, in = j % WIDTH;  // wt output layer: [16 out][64 in]
      *reinterpret_cast<__nv_bfloat16 *>(sWt + HIDDEN * TC_LAYER_BYTES + tc::kmajorOffset(o, in, 64)) = P.wt[i];
      if (sW) {  // w output layer: [64 in][16 out] -> rows = in, K = 16
        const int in2 = j / OUT_PAD, o2 = j % OUT_PAD;
        *reinterpret_cast<__nv_bfloat16 *>(sW + HIDDEN * TC_LAYER_BYTES + tc::kmajorOffset(in2, o2, OUT_PAD)) =
            P.w[i];
      }
    }
  }
}

// the 64 encoded inputs of one sample (record r), FP32
B200_D void encodeRow(const Params &P, const float *r, float *x) {
  for (int l = 0; l < LEVELS; l++) {
    const Cell c = gridCell(P.grid, l, r);
    const __half2 *T = P.table + size_t(l) * TSIZE;
    float f0 = 0.f, f1 = 0.f;
    for (int k = 0; k < 8; k++) {
      const uint32_t dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
      const float w = (dx ? c.fx : 1.f - c.fx) * (dy ? c.fy : 1.f - c.fy) * (dz ? c.fz : 1.f - c.fz);
      const float2 v = __half22float2(T[gridIndex(P.grid, l, c.x + dx, c.y + dy, c.z + dz)]);
      f0 += w * v.x;
      f1 += w * v.y;
    }
    x[2 * l] = f0;
    x[2 * l + 1] = f1;
  }
  shEncode(r[3], r[4], r[5], x + COL_SH);
  for (int k = COL_N; k < WIDTH; k++) x[k] = 0.f;
  x[COL_N + 0] = r[6];
  x[COL_N + 1] = r[7];
  x[COL_N + 2] = r[8];
  x[COL_R] = r[9];
  x[COL_A + 0] = r[10];
  x[COL_A + 1] = r[11];
  x[COL_A + 2] = r[12];
  x[COL_ONE] = 1.f;
}

// row `row` of a K-wide BF16 operand tile from FP32 values (optionally ReLU'd)
template <int K>
B200_D void storeRow(unsigned char *tile, int row, const float *v, bool relu) {
#pragma unroll
  for (int c = 0; c < K; c += 8) {
    uint4 q;
    uint32_t *w = reinterpret_cast<uint32_t *>(&q);
#pragma unroll
    for (int e = 0; e < 4; e++) {
      float a = v[c + 2 * e], b = v[c + 2 * e + 1];
      if (relu) {
        a = fmaxf(a, 0.f);
        b = fmaxf(b, 0.f);
      }
      w[e] = packBF16(a, b);
    }
    *reinterpret_cast<uint4 *>(tile + tc::kmajorOffset(row, c, K)) = q;
  }
}

// this thread's accumulator row: `n` FP32 columns from column c0
B200_D void loadRow(uint32_t tmem, int warp, int c0, int n, float *v) {
  for (int c = 0; c < n; c += 16) tc::tmemLoad16(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0 + c), v + c);
}

// one GEMM on the tensor cores: thread 0 issues, everyone waits (the
// operands written by the threads are made visible to the async proxy first).
// false if the MMA did not complete in time (reported via *status).
B200_D bool tcGemm(uint32_t tmem, const unsigned char *a, int aK, const unsigned char *b, int bK, int K, int N,
                   uint64_t *bar, uint32_t &phase, uint32_t *status) {
  tc::fenceProxyAsync();
  tc::fenceBeforeSync();
  __syncthreads();
  tc::fenceAfterSync();
  if (threadIdx.x == 0) {
    tc::gemmIssue(tmem, tc::smemAddr(a), aK, tc::smemAddr(b), bK, K, tc::idescBF16(TC_M, N));
    tc::commit(bar);
  }
  const bool ok = __syncthreads_and(tc::mbarWait(bar, phase)) != 0;
  phase ^= 1u;
  tc::fenceAfterSync();
  if (!ok && threadIdx.x == 0) atomicOr(status, 1u);
  return ok;
}

__global__ void __launch_bounds__(TC_M) k_nrc_infer_tc(Params P, const float *__restrict__ q, long long nmax,
                                                       const uint32_t *dn, float *__restrict__ out, uint32_t *status) {
  const long long n = deviceCount(nmax, dn, 0);
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char *sWt = smem;                 // forward B operands
  unsigned char *sX = smem + TC_W_BYTES;     // the activation tile
  uint64_t *bar = reinterpret_cast<uint64_t *>(sX + TC_TILE_BYTES);
  uint32_t *tmemSlot = reinterpret_cast<uint32_t *>(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5;
  stageWeights(P, sWt, nullptr);
  if (warp == 0) tc::tmemAlloc(tmemSlot, TC_TMEM_COLS);
  if (tid == 0) tc::mbarInit(bar, 1);
  tc::fenceBeforeSync();
  __syncthreads();
  tc::fenceAfterSync();
  const uint32_t tmem = *tmemSlot;
  uint32_t phase = 0;
  const long long tiles = (n + TC_M - 1) / TC_M;
  bool ok = true;
  for (long long tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
    const long long i = tile * TC_M + tid;
    float x[WIDTH];
    if (i < n) {
      float r[REC];
      for (int k = 0; k < REC; k += 4) *reinterpret_cast<float4 *>(r + k) = *reinterpret_cast<const float4 *>(q + i * REC + k);
      encodeRow(P, r, x);
    } else {
      for (int k = 0; k < WIDTH; k++) x[k] = 0.f;
    }
    storeRow<WIDTH>(sX, tid, x, false);
    for (int l = 0; l < HIDDEN && ok; l++) {
      ok = tcGemm(tmem, sX, WIDTH, sWt + l * TC_LAYER_BYTES, WIDTH, WIDTH, WIDTH, bar, phase, status);
      if (!ok) break;
      loadRow(tmem, warp, 0, WIDTH, x);
      tc::fenceBeforeSync();
      storeRow<WIDTH>(sX, tid, x, true);  // the MMA that read sX has completed
    }
    if (!ok) break;
    ok = tcGemm(tmem, sX, WIDTH, sWt + HIDDEN * TC_LAYER_BYTES, WIDTH, WIDTH, OUT_PAD, bar, phase, status);
    if (!ok) break;
    float o[16];
    loadRow(tmem, warp, 0, 16, o);
    tc::fenceBeforeSync();
    if (i < n)
      for (int c = 0; c < 3; c++) out[i * 3 + c] = o[c];
  }
  tc::fenceBeforeSync();
  __syncthreads();
  if (warp == 0) tc::tmemDealloc(tmem, TC_TMEM_COLS);
}

// mma.sync fragment reads from K-major tiles: A[m][k] = Act[sample k][feature m]
// (two samples per register), B[k][n] = G[sample k][column n]
B200_D uint32_t tilePair(const unsigned char *tile, int K, int s0, int c) {
  const uint16_t lo = *reinterpret_cast<const uint16_t *>(tile + tc::kmajorOffset(s0, c, K));
  const uint16_t hi = *reinterpret_cast<const uint16_t *>(tile + tc::kmajorOffset(s0 + 1, c, K));
  return uint32_t(lo) | (uint32_t(hi) << 16);
}

// dW[in][out] += Act^T G over the tile's 128 samples; warp w owns the input
// rows 16w..16w+15 and all `nOut` output columns; one global add per weight
template <int NOUT>
B200_D void weightGradTile(const unsigned char *act, const unsigned char *G, float *dW, int warp, int lane) {
  const int g = lane >> 2, t = lane & 3;
  float c[NOUT / 8][4];
#pragma unroll
  for (int j = 0; j < NOUT / 8; j++) c[j][0] = c[j][1] = c[j][2] = c[j][3] = 0.f;
  const int m0 = 16 * warp + g;
  for (int kk = 0; kk < TC_M / 16; kk++) {
    const int s = 16 * kk + 2 * t;
    uint32_t a[4];
    a[0] = tilePair(act, WIDTH, s, m0);
    a[1] = tilePair(act, WIDTH, s, m0 + 8);
    a[2] = tilePair(act, WIDTH, s + 8, m0);
    a[3] = tilePair(act, WIDTH, s + 8, m0 + 8);
#pragma unroll
    for (int j = 0; j < NOUT / 8; j++) {
      const uint32_t b0 = tilePair(G, NOUT, s, 8 * j + g), b1 = tilePair(G, NOUT, s + 8, 8 * j + g);
      mma16816(c[j], a, b0, b1);
    }
  }
#pragma unroll
  for (int j = 0; j < NOUT / 8; j++) {
    const int col = 8 * j + 2 * t;
    atomicAdd(dW + m0 * NOUT + col, c[j][0]);
    atomicAdd(dW + m0 * NOUT + col + 1, c[j][1]);
    atomicAdd(dW + (m0 + 8) * NOUT + col, c[j][2]);
    atomicAdd(dW + (m0 + 8) * NOUT + col + 1, c[j][3]);
  }
}

__global__ void __launch_bounds__(TC_M) k_nrc_train_tc(Params P, const float *__restrict__ samples, long long nmax,
                                                       const uint32_t *dn, long long offset, float *wgrad,
                                                       float *tgrad, float *loss, uint32_t *status) {
  const long long n = deviceCount(nmax, dn, offset);
  const float invN3 = n > 0 ? 1.f / (3.f * float(n)) : 0.f;
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char *sWt = smem;                        // forward B operands
  unsigned char *sW = sWt + TC_W_BYTES;             // backward B operands
  unsigned char *sA = sW + TC_W_BYTES;              // X, H1..H4 (5 tiles)
  unsigned char *sZ = sA + 5 * TC_TILE_BYTES;       // dZ tile
  unsigned char *sO = sZ + TC_TILE_BYTES;           // dOut tile (128 x 16)
  uint64_t *bar = reinterpret_cast<uint64_t *>(sO + TC_M * OUT_PAD * 2);
  uint32_t *tmemSlot = reinterpret_cast<uint32_t *>(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  stageWeights(P, sWt, sW);
  if (warp == 0) tc::tmemAlloc(tmemSlot, TC_TMEM_COLS);
  if (tid == 0) tc::mbarInit(bar, 1);
  tc::fenceBeforeSync();
  __syncthreads();
  tc::fenceAfterSync();
  const uint32_t tmem = *tmemSlot;
  uint32_t phase = 0;
  float lossSum = 0.f;
  const long long tiles = (n + TC_M - 1) / TC_M;
  bool ok = true;
  for (long long tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
    const long long i = tile * TC_M + tid;
    const bool valid = i < n;
    float r[REC];
    float v[WIDTH];
    if (valid) {
      for (int k = 0; k < REC; k += 4)
        *reinterpret_cast<float4 *>(r + k) = *reinterpret_cast<const float4 *>(samples + (offset + i) * REC + k);
      encodeRow(P, r, v);
    } else {
      for (int k = 0; k < REC; k++) r[k] = 0.f;
      for (int k = 0; k < WIDTH; k++) v[k] = 0.f;
    }
    __syncthreads();  // the previous tile's readers of the tiles are done
    storeRow<WIDTH>(sA, tid, v, false);
    // forward: H_{l+1} = ReLU(A_l W_l)
    for (int l = 0; l < HIDDEN && ok; l++) {
      ok = tcGemm(tmem, sA + l * TC_TILE_BYTES, WIDTH, sWt + l * TC_LAYER_BYTES, WIDTH, WIDTH, WIDTH, bar, phase,
                  status);
      if (!ok) break;
      loadRow(tmem, warp, 0, WIDTH, v);
      tc::fenceBeforeSync();
      storeRow<WIDTH>(sA + (l + 1) * TC_TILE_BYTES, tid, v, true);
    }
    if (!ok) break;
    ok = tcGemm(tmem, sA + HIDDEN * TC_TILE_BYTES, WIDTH, sWt + HIDDEN * TC_LAYER_BYTES, WIDTH, WIDTH, OUT_PAD, bar,
                phase, status);
    if (!ok) break;
    // relative L2 loss and its gradient (columns 0..2), staged as dOut
    float o[16], d[16];
    loadRow(tmem, warp, 0, 16, o);
    tc::fenceBeforeSync();
    for (int c = 0; c < 16; c++) d[c] = 0.f;
    if (valid)
      for (int c = 0; c < 3; c++) {
        const float y = r[13 + c], ov = o[c];
        const float den = ov * ov + 0.01f;
        const float diff = ov - y;
        lossSum += diff * diff / den;
        d[c] = 2.f * diff / den * invN3;
      }
    storeRow<OUT_PAD>(sO, tid, d, false);
    // dH4 = dOut W_out^T (K = 16) on the tensor cores; dW_out by the warps
    ok = tcGemm(tmem, sO, OUT_PAD, sW + HIDDEN * TC_LAYER_BYTES, OUT_PAD, OUT_PAD, WIDTH, bar, phase, status);
    if (!ok) break;
    weightGradTile<OUT_PAD>(sA + HIDDEN * TC_TILE_BYTES, sO, wgrad + LAYER_OUT_OFF, warp, lane);
    for (int l = HIDDEN - 1; l >= 0 && ok; l--) {
      // dZ_l = dH_{l+1} through the ReLU of H_{l+1}
      loadRow(tmem, warp, 0, WIDTH, v);
      tc::fenceBeforeSync();
      const unsigned char *H = sA + (l + 1) * TC_TILE_BYTES;
      for (int c = 0; c < WIDTH; c++)
        if (!(__bfloat162float(*reinterpret_cast<const __nv_bfloat16 *>(H + tc::kmajorOffset(tid, c, WIDTH))) > 0.f))
          v[c] = 0.f;
      __syncthreads();  // every warp's reads of the previous dZ are done
      storeRow<WIDTH>(sZ, tid, v, false);
      // dA_l = dZ_l W_l^T on the tensor cores; dW_l = A_l^T dZ_l by the warps
      ok = tcGemm(tmem, sZ, WIDTH, sW + l * TC_LAYER_BYTES, WIDTH, WIDTH, WIDTH, bar, phase, status);
      if (!ok) break;
      weightGradTile<WIDTH>(sA + l * TC_TILE_BYTES, sZ, wgrad + l * WIDTH * WIDTH, warp, lane);
    }
    if (!ok) break;
    // dX: the hash-grid columns 0..31 -> the table gradient
    loadRow(tmem, warp, 0, 32, v);
    tc::fenceBeforeSync();
    if (valid)
      for (int lv = 0; lv < LEVELS; lv++) scatterGrid(P, r, lv, v[2 * lv], v[2 * lv + 1], tgrad);
  }
  for (int off = 16; off; off >>= 1) lossSum += __shfl_xor_sync(0xffffffffu, lossSum, off);
  if (lane == 0) atomicAdd(loss, lossSum * invN3);
  tc::fenceBeforeSync();
  __syncthreads();
  if (warp == 0) tc::tmemDealloc(tmem, TC_TMEM_COLS);
}

constexpr size_t kInferTcSmem = TC_W_BYTES + TC_TILE_BYTES + 16;
constexpr size_t kTrainTcSmem = 2 * TC_W_BYTES + 6 * TC_TILE_BYTES + TC_M * OUT_PAD * 2 + 16;
static_assert(kTrainTcSmem <= 227 * 1024, "tcgen05 training kernel shared memory");



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
  uint32_t *dStatus = nullptr;  // bit 0: a tensor-core MMA did not complete in time
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
    alloc((void **)&dStatus, 4);
    cudaStream_t st = dev->stream;
    check(cudaMemsetAsync(dStatus, 0, 4, st), "clear");
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
                    (void *)wMaster, (void *)wGrad, (void *)wM, (void *)wV, (void *)dLoss, (void *)dStatus,
                    (void *)queries,
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
    check(cudaFuncSetAttribute(k_nrc_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTrainTcSmem)),
          "smem");
    check(cudaFuncSetAttribute(k_nrc_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kInferTcSmem)),
          "smem");
    attrsSet = true;
  }
  // raises if a kernel of this cache reported an MMA that did not complete
  // (synchronous; called where the API waits anyway)
  void checkStatus() {
    uint32_t h = 0;
    check(cudaMemcpy(&h, dStatus, 4, cudaMemcpyDeviceToHost), "radiance cache status");
    if (h) throw Error(B200_UNKNOWN_ERROR, "radiance cache: a tensor-core MMA did not complete");
  }
  // n queries, or min(*dn, n) when dn (a device count) is given
  void infer(const float *q, long long n, float *out, cudaStream_t st, const uint32_t *dn = nullptr) {
    if (n <= 0) return;
    setAttrs();
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev->dev);
    const long long tiles = (n + TC_M - 1) / TC_M;
    const long long blocks = std::min<long long>(tiles, (long long)sms * 4);
    k_nrc_infer_tc<<<unsigned(blocks), TC_M, kInferTcSmem, st>>>(params(), q, n, dn, out, dStatus);
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
    const long long tiles = (n + TC_M - 1) / TC_M;
    const long long blocks = std::min<long long>(tiles, (long long)sms);
    k_nrc_train_tc<<<unsigned(blocks), TC_M, kTrainTcSmem, st>>>(params(), s, n, dn, offset, wGrad, tGrad, dLoss,
                                                                   dStatus);
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
  // (also reports a tensor-core MMA that did not complete in an earlier call)
  if (!h) return B200_INVALID_ARGUMENT;
  NrcObj *o = reinterpret_cast<NrcObj *>(h);
  return nrcGuard(o->dev, [&]() {
    check(cudaStreamSynchronize(o->dev->stream), "sync");
    o->checkStatus();
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
    if (sc->hasMotion())
      throw Error(B200_INVALID_ARGUMENT, "radiance cache: scenes with motion-blurred instances are rendered by b200_render_pt");
    if (o->dev != sc->dev) throw Error(B200_INVALID_ARGUMENT, "the cache belongs to another device");
    if (!(p->pixelSamples >= 1 && p->maxPathLength >= 0 && p->pixelFilter >= B200_PF_POINT &&
          p->pixelFilter <= B200_PF_BLACKMAN_HARRIS && nmaterials >= 0 && (nmaterials == 0 || materials)))
      throw Error(B200_INVALID_ARGUMENT, "bad path tracer parameters");
    if (np.trainPaths < 0 || np.trainSteps < 0 || np.trainBatch < 1 || np.epochs < 0)
      throw Error(B200_INVALID_ARGUMENT, "bad radiance cache frame parameters");
    cudaStream_t st = stream ? (cudaStream_t)stream : sc->dev->stream;
    uploadMaterials(sc, materials, nmaterials);
    const PtParamsD d = makePtParams(*p, sc, materials, nmaterials, sc->transparentMaterials);
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

extern "C" int b200_tensor_core_check(b200_device d, const float *a, const float *b, int n, float *out) {
  using namespace b200;
  if (!d || !a || !b || !out) return B200_INVALID_ARGUMENT;
  DeviceObj *dev = reinterpret_cast<DeviceObj *>(d);
  if (n != 16 && n != 32 && n != 64) {
    dev->lastError = "b200_tensor_core_check: n must be 16, 32 or 64";
    return B200_INVALID_ARGUMENT;
  }
  float *dA = nullptr, *dB = nullptr, *dD = nullptr;
  uint32_t *dS = nullptr;
  auto cleanup = [&]() {
    for (void *p : {(void *)dA, (void *)dB, (void *)dD, (void *)dS})
      if (p) cudaFree(p);
  };
  try {
    check(cudaSetDevice(dev->dev), "cudaSetDevice");
    check(cudaMalloc(&dA, 128 * 64 * 4), "alloc");
    check(cudaMalloc(&dB, size_t(n) * 64 * 4), "alloc");
    check(cudaMalloc(&dD, size_t(128) * n * 4), "alloc");
    check(cudaMalloc(&dS, 4), "alloc");
    check(cudaMemset(dS, 0, 4), "clear");
    check(cudaMemcpy(dA, a, 128 * 64 * 4, cudaMemcpyHostToDevice), "upload");
    check(cudaMemcpy(dB, b, size_t(n) * 64 * 4, cudaMemcpyHostToDevice), "upload");
    nrc::k_tc_check<<<1, 128, 0, dev->stream>>>(dA, dB, n, dD, dS);
    check(cudaGetLastError(), "tensor-core check launch");
    check(cudaStreamSynchronize(dev->stream), "tensor-core check");
    uint32_t st = 0;
    check(cudaMemcpy(&st, dS, 4, cudaMemcpyDeviceToHost), "status");
    check(cudaMemcpy(out, dD, size_t(128) * n * 4, cudaMemcpyDeviceToHost), "download");
    cleanup();
    if (st) {
      dev->lastError = "b200_tensor_core_check: the MMA did not complete";
      return B200_UNKNOWN_ERROR;
    }
    return B200_NO_ERROR;
  } catch (const Error &e) {
    cleanup();
    dev->lastError = e.what();
    return e.code;
  }
}
