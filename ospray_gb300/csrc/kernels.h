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

// structured-regular volume (x fastest) with its transfer function and
// macrocell emptiness grid (16^3-voxel cells)
struct VolumeD {
  const float *data;
  int nx, ny, nz;
  V3 origin, spacing;
  int cx, cy, cz;
  const uint8_t *cellEmpty;
  const float3 *tfColor;
  const float *tfOpacity;
  int ncolor, nopacity;
  float vlo, vhi, densityScale;
};

struct ScivisParamsD {
  int spp;
  float samplingRate;
  float bg[4];
};

cudaError_t buildMacrocells(VolumeD &v, uint8_t *empty, cudaStream_t st);
cudaError_t launchRenderScivisVolume(const SamplerTables *T, const Scene &sc, const VolumeD &vol, const CameraD &cam,
                                     const PixelFilterD &pf, const ScivisParamsD &p, const FrameD &fb, bool stats,
                                     cudaStream_t st);

cudaError_t computeAlbedoTables(AlbedoTablesD *T, cudaStream_t st);
cudaError_t launchRenderPT(const SamplerTables *T, const Scene &sc, const CameraD &cam, const PixelFilterD &pf,
                           const PtParamsD &p, const MaterialD *mats, const LightD *lights, const float *lightCdf,
                           const AlbedoTablesD *AT, const FrameD &fb, bool stats, void *workspace,
                           size_t wsBytes, cudaStream_t st);
// bytes of path-tracer workspace for a frame of npaths = W * H * spp paths
size_t ptWorkspaceBytes(long long npaths);

struct AOParamsD {
  int spp, aoSamples;
  float aoRadius, aoIntensity;
  float bg[4];
};

// Renderer_pick: one camera ray at screen (sx, sy), closest hit; out[0] hit,
// out[1..3] world position bits, out[4..6] instID, geomID, primID.
cudaError_t launchPick(const Scene &sc, const CameraD &cam, float sx, float sy, uint32_t *out, cudaStream_t st);
cudaError_t launchTrace(const Scene &sc, const float4 *rays, long long n, int occlusion, float *outF, uint32_t *outI,
                        cudaStream_t st);
cudaError_t launchRenderAO(const SamplerTables *T, const Scene &sc, const CameraD &cam, const PixelFilterD &pf, const AOParamsD &p,
                           const FrameD &fb, bool stats, cudaStream_t st);

}  // namespace b200
