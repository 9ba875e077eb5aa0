// Launch interface between the host-side C-ABI (api.cu) and the kernels.
#pragma once
#include "render_common.cuh"

namespace b200 {

struct AOParamsD {
  int spp, aoSamples;
  float aoRadius, aoIntensity;
  float bg[4];
};

cudaError_t launchTrace(const Scene &sc, const float4 *rays, long long n, int occlusion, float *outF, uint32_t *outI,
                        cudaStream_t st);
cudaError_t launchRenderAO(const SamplerTables *T, const Scene &sc, const CameraD &cam, const PixelFilterD &pf, const AOParamsD &p,
                           const FrameD &fb, bool stats, cudaStream_t st);

}  // namespace b200
