// Framebuffer post-processing: the tonemapper frame operation and the final
// colour conversion, fused into one pass over the accumulated RGBA32F colour.
//
// The reference runs them as a chain of kernels per frame
// (LocalFrameBuffer::postProcess, modules/cpu/fb/LocalFB.cpp:459-477): every
// user frame operation writes a post-processed colour buffer, then
// ColorConversion_kernel (fb/frame_ops/ColorConversion.ispc:11-36) writes
// the buffer that ospMapFrameBuffer returns.  Here one kernel reads each
// pixel once (16 B) and writes only the mapped result (4 B for RGBA8/SRGBA,
// 16 B for RGBA32F); it is HBM-bound.
#include <cmath>
#include <vector>

#include "api_internal.h"

namespace b200 {
namespace {

__global__ void k_frame_post(const float4 *__restrict__ color, long long n, int format, int tonemap, ToneMapD tm,
                             void *__restrict__ out) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride)
    postPixel(color, i, format, tonemap, tm, out);
}

}  // namespace

// ToneMapper::commit (fb/frame_ops/ToneMapper.cpp:16-51): clamps the user
// parameters and solves the curve's b and c so that midIn maps to midOut and
// hdrMax to 1 (the same expression, evaluated in the same order, so the
// coefficients are the reference's to the bit).
ToneMapD makeToneMap(const b200_tonemapper &u) {
  ToneMapD t;
  t.exposure = u.exposure;
  t.a = std::fmax(u.contrast, 0.0001f);
  t.d = std::fmin(std::fmax(u.shoulder, 0.0001f), 1.f);
  const float m = std::fmin(std::fmax(u.midIn, 0.0001f), 1.f);
  const float n = std::fmin(std::fmax(u.midOut, 0.0001f), 1.f);
  const float w = std::fmax(u.hdrMax, 1.f);
  const float a = t.a, d = t.d;
  const float mad = powf(m, a * d), ma = powf(m, a), wa = powf(w, a), wad = powf(w, a * d);
  const float num = mad * n * wa - ma * wad;
  const float den = mad * n - n * wad;
  t.b = -((powf(m, -a * d) * (-ma + (n * num) / den)) / n);
  t.c = std::fmax(num / den, 0.f);
  t.aces = u.acesColor ? 1 : 0;
  return t;
}

namespace {
// Variance_kernel (fb/frame_ops/Variance.ispc:11-49): per 8x8 task, the mean
// over its pixels (with den2 = r + g + b + 1 - a > 0) of the L1 difference
// between the accumulated colour and the odd-frame accumulation, over
// sqrt(den2), times 64
__global__ void k_task_variance(const float4 *__restrict__ color, const float4 *__restrict__ var, int W, int H,
                                int tx, int ty, float *__restrict__ err) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= tx * ty) return;
  const int x0 = (t % tx) * FrameObj::TASK, y0 = (t / tx) * FrameObj::TASK;
  float v = 0.f;
  int cnt = 0;
  for (int y = y0; y < min(y0 + FrameObj::TASK, H); y++)
    for (int x = x0; x < min(x0 + FrameObj::TASK, W); x++) {
      const float4 c = color[size_t(y) * W + x], s = var[size_t(y) * W + x];
      const float den2 = c.x + c.y + c.z + (1.f - c.w);
      if (den2 > 0.f) {
        cnt++;
        v += (fabsf(c.x - s.x) + fabsf(c.y - s.y) + fabsf(c.z - s.z) + fabsf(c.w - s.w)) / sqrtf(den2);
      }
    }
  if (cnt) v /= float(cnt);
  err[t] = v * 64.f;
}
// LocalFrameBuffer::getRenderTaskIDs (fb/LocalFB.cpp:238-260): a task is
// rendered when its error exceeds the threshold
__global__ void k_task_select(const float *__restrict__ err, int n, float threshold, uint8_t *__restrict__ active) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) active[t] = err[t] > threshold ? 1 : 0;
}
}  // namespace

void FrameObj::beginFrame(int spp, cudaStream_t st) {
  // FrameBuffer::beginFrame: the coin flip on every even frame
  const bool even = (frameID & 1) == 0;
  if (even) pickOdd = (mtGen() & 1u) != 0;
  accumVariance = variance != nullptr && even != pickOdd;
  // FrameBuffer::minimumAdaptiveFrames: max(2, 16 / spp)
  const int minFrames = std::max(2, 16 / std::max(1, spp));
  adaptive = errorThreshold > 0.f && taskErr && taskErrValid && frameID >= minFrames;
  if (adaptive) {
    const int nt = tasksX() * tasksY();
    k_task_select<<<(nt + 255) / 256, 256, 0, st>>>(taskErr, nt, errorThreshold, taskActive);
    check(cudaGetLastError(), "task selection");
  }
}

void framePostProcess(FrameObj *fb, cudaStream_t st, bool variance) {
  // the variance estimate follows every odd frame (LocalFrameBuffer::postProcess)
  if (variance && fb->taskErr && fb->frameID >= 2 && ((fb->frameID - 1) & 1)) {
    const int nt = fb->tasksX() * fb->tasksY();
    k_task_variance<<<(nt + 127) / 128, 128, 0, st>>>(fb->color, fb->variance, fb->W, fb->H, fb->tasksX(),
                                                       fb->tasksY(), fb->taskErr);
    check(cudaGetLastError(), "variance estimate");
    fb->taskErrValid = true;
  }
  if (fb->format == B200_FB_NONE) return;
  const long long n = (long long)fb->W * fb->H;
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, fb->dev->dev);
  const long long blocks = std::min<long long>((n + 255) / 256, (long long)sms * 8);
  k_frame_post<<<unsigned(blocks), 256, 0, st>>>(fb->color, n, fb->format, fb->toneMapOn ? 1 : 0, fb->toneMap,
                                                 fb->mapped);
  check(cudaGetLastError(), "frame post-process");
}

}  // namespace b200

// ---------------------------------------------------------------- relMSE
namespace b200 {
namespace {
// sum over pixels of the mean over rgb of (x - r)^2 / (r^2 + 0.01); with a
// reference depth channel, only over the pixels whose reference depth is
// finite (their first hit is geometry), counted in sum[1]
__global__ void k_relmse(const float4 *__restrict__ x, const float4 *__restrict__ r, const float *__restrict__ rdepth,
                         long long n, double *sum) {
  double acc = 0.0, cnt = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (rdepth && !isfinite(rdepth[i])) continue;
    const float4 a = x[i], b = r[i];
    const float e = ((a.x - b.x) * (a.x - b.x) / (b.x * b.x + 0.01f) + (a.y - b.y) * (a.y - b.y) / (b.y * b.y + 0.01f) +
                     (a.z - b.z) * (a.z - b.z) / (b.z * b.z + 0.01f)) *
                    (1.f / 3.f);
    acc += double(e);
    cnt += 1.0;
  }
  for (int off = 16; off; off >>= 1) {
    acc += __shfl_xor_sync(0xffffffffu, acc, off);
    cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(sum, acc);
    atomicAdd(sum + 1, cnt);
  }
}

int relmse(b200_frame f, b200_frame ref, bool hitsOnly, double *out, int64_t *npix) {
  if (!f || !ref || !out) return B200_INVALID_ARGUMENT;
  FrameObj *a = reinterpret_cast<FrameObj *>(f), *b = reinterpret_cast<FrameObj *>(ref);
  if (a->W != b->W || a->H != b->H || a->dev != b->dev) return B200_INVALID_ARGUMENT;
  if (hitsOnly && !b->depth) {
    a->dev->lastError = "relMSE over hit pixels: the reference framebuffer has no DEPTH channel";
    return B200_INVALID_ARGUMENT;
  }
  try {
    check(cudaSetDevice(a->dev->dev), "cudaSetDevice");
    cudaStream_t st = a->dev->stream;
    double *d = nullptr;
    check(cudaMallocAsync(&d, 2 * sizeof(double), st), "alloc");
    check(cudaMemsetAsync(d, 0, 2 * sizeof(double), st), "clear");
    const long long n = (long long)a->W * a->H;
    k_relmse<<<unsigned(std::min<long long>((n + 255) / 256, 152 * 8)), 256, 0, st>>>(
        a->color, b->color, hitsOnly ? b->depth : nullptr, n, d);
    double h[2] = {0.0, 0.0};
    check(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, st), "read");
    check(cudaFreeAsync(d, st), "free");
    check(cudaStreamSynchronize(st), "sync");
    *out = h[1] > 0.0 ? h[0] / h[1] : 0.0;
    if (npix) *npix = int64_t(h[1]);
    return B200_NO_ERROR;
  } catch (const Error &e) {
    a->dev->lastError = e.what();
    return e.code;
  }
}
}  // namespace
}  // namespace b200

extern "C" int b200_frame_relmse(b200_frame f, b200_frame ref, double *out) {
  return b200::relmse(f, ref, false, out, nullptr);
}

extern "C" int b200_frame_relmse_hits(b200_frame f, b200_frame ref, double *out, int64_t *npix) {
  return b200::relmse(f, ref, true, out, npix);
}

// LiveVarianceFrameOp::getAvgError (fb/frame_ops/Variance.cpp:32-46): the mean
// error of the tasks at or above the threshold, or the largest error when
// none is; inf before any estimate (FrameBuffer::getVariance)
extern "C" int b200_frame_variance(b200_frame f, float threshold, float *out) {
  using namespace b200;
  if (!f || !out) return B200_INVALID_ARGUMENT;
  FrameObj *fb = reinterpret_cast<FrameObj *>(f);
  if (!fb->taskErr || !fb->taskErrValid) {
    *out = INFINITY;
    return B200_NO_ERROR;
  }
  try {
    check(cudaSetDevice(fb->dev->dev), "cudaSetDevice");
    std::vector<float> e(size_t(fb->tasksX()) * fb->tasksY());
    check(cudaMemcpyAsync(e.data(), fb->taskErr, e.size() * 4, cudaMemcpyDeviceToHost, fb->dev->stream), "read");
    check(cudaStreamSynchronize(fb->dev->stream), "sync");
    float mx = 0.f, sum = 0.f;
    int active = 0;
    for (float v : e) {
      mx = std::fmax(mx, v);
      if (v >= threshold) {
        sum += v;
        active++;
      }
    }
    *out = active ? sum / float(active) : mx;
    return B200_NO_ERROR;
  } catch (const Error &e) {
    fb->dev->lastError = e.what();
    return e.code;
  }
}
