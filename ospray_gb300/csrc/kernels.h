// Launch interface between the host-side C-ABI (api.cu) and the kernels.
#pragma once
#include "pt_bsdf.cuh"
#include "render_common.cuh"

namespace b200 {

enum LightType : int { LIGHT_QUAD = 0, LIGHT_AMBIENT = 1 };

// light in world space; quad: nnormal = normalize(edge2 x edge1), ppdf = 1/area
struct LightD {
  int type, visible;
  V3 position, edge1, edge2, nnormal, radiance;
  float ppdf;
};

struct PtParamsD {
  int spp, maxPathLength, roulettePathLength, maxScatteringEvents;
  int nFirst, nIndirect, numLights, numMaterials;
  float minContribution, maxContribution;
  float bg[4];
};

cudaError_t computeAlbedoTables(AlbedoTablesD *T, cudaStream_t st);
cudaError_t launchRenderPT(const SamplerTables *T, const Scene &sc, const CameraD &cam, const PixelFilterD &pf,
                           const PtParamsD &p, const MaterialD *mats, const LightD *lights, const float *lightCdf,
                           const AlbedoTablesD *AT, const FrameD &fb, bool stats, unsigned int *work,
                           cudaStream_t st);

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
