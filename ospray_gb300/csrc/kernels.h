// Launch interface between the host-side C-ABI (api.cu) and the kernels.
#pragma once
#include <vector>

#include "frame_post.cuh"
#include "pt_bsdf.cuh"
#include "render_common.cuh"

namespace b200 {

// Device time of the hot kernels, measured live: while a device's timer is
// enabled, the renderers record a pair of CUDA events on the launch stream
// around each launch of the kinds below; read() sums their elapsed times.
enum KernelKind : int { KK_TRACE_CLOSEST = 0, KK_TRACE_SHADOW = 1, KK_SHADE = 2, KK_AO = 3, KK_SCIVIS = 4, KK_COUNT = 5 };

struct KernelTimer {
  struct Rec {
    int kind;
    cudaEvent_t a, b;
  };
  std::vector<cudaEvent_t> pool;
  std::vector<Rec> recs;
  cudaEvent_t open = nullptr;
  double ms[KK_COUNT] = {};
  long long launches[KK_COUNT] = {};
  cudaEvent_t get() {
    if (pool.empty()) {
      cudaEvent_t e = nullptr;
      cudaEventCreate(&e);
      return e;
    }
    cudaEvent_t e = pool.back();
    pool.pop_back();
    return e;
  }
  void begin(cudaStream_t st) {
    open = get();
    cudaEventRecord(open, st);
  }
  void end(int kind, cudaStream_t st) {
    cudaEvent_t b = get();
    cudaEventRecord(b, st);
    recs.push_back({kind, open, b});
    open = nullptr;
  }
  // folds the recorded pairs into ms/launches (waits for the last one)
  void collect() {
    for (const Rec &r : recs) {
      float t = 0.f;
      cudaEventSynchronize(r.b);
      if (cudaEventElapsedTime(&t, r.a, r.b) == cudaSuccess) {
        ms[r.kind] += t;
        launches[r.kind]++;
      }
      pool.push_back(r.a);
      pool.push_back(r.b);
    }
    recs.clear();
  }
  ~KernelTimer() {
    for (const Rec &r : recs) {
      cudaEventDestroy(r.a);
      cudaEventDestroy(r.b);
    }
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
  }
};

// scoped begin/end around one launch (no-op without a timer)
struct KernelScope {
  KernelTimer *t;
  int kind;
  cudaStream_t st;
  KernelScope(KernelTimer *t_, int k, cudaStream_t s) : t(t_), kind(k), st(s) {
    if (t) t->begin(st);
  }
  ~KernelScope() {
    if (t) t->end(kind, st);
  }
};

enum LightType : int { LIGHT_QUAD = 0, LIGHT_AMBIENT = 1, LIGHT_DISTANT = 2, LIGHT_SPHERE = 3, LIGHT_SPOT = 4 };

// light in world space; quad: nnormal = normalize(edge2 x edge1), ppdf = 1/area
// quad: position, edge1/2, nnormal, ppdf; distant: dir (towards the light),
// cosAngle, conePdf, radiance = irradiance; sphere: position, radius,
// radiance (of the surface), intensity (radiative intensity of a point light);
// spot: position, dir (it points to), edge1/edge2 = c0/c90 (ring frame),
// cosAngle = cosAngleMax, conePdf = cosAngleScale, ppdf = ring area pdf,
// radius / innerRadius, radiance, intensity
struct LightD {
  int type, visible;
  V3 position, edge1, edge2, nnormal, radiance;
  float ppdf;
  V3 dir, intensity;
  float cosAngle, conePdf, radius, innerRadius;
};

struct PtParamsD {
  int spp, maxPathLength, roulettePathLength, maxScatteringEvents;
  int nFirst, nIndirect, numLights, numMaterials;
  float minContribution, maxContribution;
  float bg[4];
  int transparentShadows;  // some material lets shadow rays through: shadow rays loop over closest hits
  int allMaterials;        // some material is not opaque principled: the shading kernel with every material type
  const TextureD *backplate;  // the renderer's backplate (null: bg)
  float mipBiasFactor;        // 2^mipMapBias
  const TextureD *maxDepth;   // the renderer's maxDepth texture (null: no limit)
};

// structured-regular volume with its transfer function and macrocell
// emptiness grid (16^3-voxel cells).  The voxels are stored in 8^3-voxel
// bricks (2 KB, x fastest inside a brick, bricks x fastest), so the 8 taps
// of a trilinear sample and the next samples along a ray share cache lines
// and DRAM pages; voxel (i, j, k) is at data[ax(i) + ay(j) + az(k)] (brickAddr).
struct VolumeD {
  const float *data;
  int nx, ny, nz;
  int bx, by, bz;  // bricks per axis
  V3 origin, spacing;
  int cx, cy, cz;
  const uint8_t *cellEmpty;
  const float3 *tfColor;
  const float *tfOpacity;
  int ncolor, nopacity;
  float vlo, vhi, densityScale;
  float gradientShadingScale;  // VolumetricModel "gradientShadingScale" (0: off)
  int identity;                // no instance transform; else rays go to volume space by rcp
  Xfm rcp;
};

struct ScivisParamsD {
  int spp;
  float samplingRate;
  float bg[4];
  const TextureD *backplate, *maxDepth;  // renderer maps (null: bg / no limit)
  float mipBiasFactor;
};

// SciVis surfaces: per renderer material slot the OBJ parameters that
// evalMaterial reads (render/scivis/surfaces.ih:44-84); isObj 0 = any other
// material type, shaded with the SciVis defaults (white, opaque).
struct ScivisMatD {
  int isObj;
  float kd[3], ks[3], ns, d, tf[3];
  const TextureD *kdMap;  // obj map_kd (null: none)
};

// SciVis surface shading inputs: lights in SciVisData order (the ambient,
// visible-only lights first, render/scivis/SciVisData.cpp:15-105), the summed
// ambient radiance (aoColorPi = aoColor * pi) and the renderer parameters
// (render/scivis/SciVis.cpp:29-36, render/Renderer.cpp:43).
struct ScivisSurfD {
  const ScivisMatD *mats;
  int nmats;
  const LightD *lights;
  int nlights, numVisibleOnly;
  V3 aoColor;
  int shadows, visibleLights, aoSamples;
  float aoRadius, minContribution;
  int hasVolume;
  int hasSurfaces;    // 0: a volume-only world (no ray is traced against surfaces)
  int opaqueShadows;  // every material opaque and no volume: shadow and AO rays as any-hit queries
  int attrs;          // vertex attributes or an obj map_kd: the kernel with DG_COLOR / DG_TEXCOORD and ray cones
};

constexpr int VOL_BRICK = 8;
// bytes of the bricked copy of an nx x ny x nz volume
size_t brickedVolumeBytes(int nx, int ny, int nz);
// linear (x fastest) -> bricked layout of v (v.data is the bricked output)
cudaError_t brickVolume(const VolumeD &v, const float *linear, float *bricked, cudaStream_t st);
cudaError_t buildMacrocells(VolumeD &v, uint8_t *empty, cudaStream_t st);
cudaError_t launchRenderScivisVolume(const SamplerTables *T, const Scene &sc, const VolumeD &vol, const CameraD &cam,
                                     const PixelFilterD &pf, const ScivisParamsD &p, const FrameD &fb, bool stats,
                                     cudaStream_t st, KernelTimer *kt = nullptr);
cudaError_t launchRenderScivisSurfaces(const SamplerTables *T, const Scene &sc, const VolumeD &vol, const CameraD &cam,
                                       const PixelFilterD &pf, const ScivisParamsD &p, const ScivisSurfD &S,
                                       const FrameD &fb, bool stats, cudaStream_t st, KernelTimer *kt = nullptr);

// Path tracing with the neural radiance cache: per frame, paths whose index
// p satisfies (p + trainOffset) % trainStride == 0 are training paths (slot
// (p + trainOffset) / trainStride < trainSlots); they are traced in full and
// record every vertex (20 floats: the 13 cache inputs, throughput, the
// contribution so far, the path index).  Every other path, at its first
// vertex after a diffuse bounce, appends a cache query (16 floats: inputs and
// throughput; qpath = its index) and ends; after each bounce the queries are
// answered (qout, by the caller's inference callback) and throughput x
// radiance is added to the paths.  After the frame the training vertices
// become training samples (inputs + suffix radiance (C_end - C_i) / T_i).
struct NrcFrameD {
  float *queries;
  uint32_t *qpath;
  float *qout;
  uint32_t *counters;  // [0] queries of the current bounce, [1] training samples
  float *trainVerts;   // trainSlots x maxLen1 x 20
  float *samples;      // sampleCap x 16
  uint32_t maxLen1, trainStride, trainOffset, trainSlots, sampleCap;
  uint32_t useCache;  // 0: no path ends in the cache (training-data frames)
};

cudaError_t computeAlbedoTables(AlbedoTablesD *T, cudaStream_t st);
cudaError_t launchRenderPT(const SamplerTables *T, const Scene &sc, const CameraD &cam, const PixelFilterD &pf,
                           const PtParamsD &p, const MaterialD *mats, const LightD *lights, const float *lightCdf,
                           const AlbedoTablesD *AT, const FrameD &fb, bool stats, void *workspace,
                           size_t wsBytes, cudaStream_t st, const NrcFrameD *nrc = nullptr,
                           void (*nrcInfer)(void *ctx, cudaStream_t st) = nullptr, void *nrcCtx = nullptr,
                           KernelTimer *kt = nullptr, float *rayTimes = nullptr);
// bytes of path-tracer workspace for a frame of npaths = W * H * spp paths
size_t ptWorkspaceBytes(long long npaths);

struct AOParamsD {
  int spp, aoSamples;
  float aoRadius, aoIntensity;
  float bg[4];
  float volumeSamplingRate;
  const TextureD *backplate, *maxDepth;  // renderer maps (null: bg / no limit)
  float mipBiasFactor;
  const ScivisMatD *mats;  // surface colour / opacity materials (getSurfaceColor); null: white, opaque
  int nmats;
};

// ---- batches: many render requests in one wavefront
enum BatchKind : int { BATCH_PT = 0, BATCH_AO = 1 };

// one request as the host describes it
struct BatchReqH {
  int kind;
  Scene sc;
  CameraD cam;
  PixelFilterD pf;
  PtParamsD pt;  // BATCH_PT
  AOParamsD ao;  // BATCH_AO (aoSamples up to 2 go through the shadow queue, more are traced in place)
  const MaterialD *mats;
  const LightD *lights;
  const float *lightCdf;
  FrameD fb;
  // the frame's post-processing (framePostProcess): mapped format, tonemapper, mapped buffer
  int postFormat, postTonemap;
  ToneMapD postTm;
  void *postOut;
};

// B200_SHADE_PARTITION: the path tracers split the queues of bounces >= 1
// into diffuse-based hits, other hits and misses before shading
// (k_partition; 1,051 vs 910 Mrays/s on the 1080p bench, 996 with misses
// and other hits in one part).  The camera rays' queue is left in pixel
// order, which is already coherent (partitioning it too gave 977 with two
// parts).
#ifndef B200_SHADE_PARTITION
#define B200_SHADE_PARTITION 1
#endif

// launch shape of the batched wavefront (what the autotuner picks)
struct BatchTuning {
  long long wavePaths;  // path slots per wave (workspace size)
  int traceBlocksPerSM;  // persistent trace grid = SMs x this
  int shadeBlocksPerSM;
};

// One wave: a contiguous run of whole pixels of consecutive requests.
struct BatchWave {
  int segOffset, nseg;  // its segments in the segment table
  long long npaths, npix;
  int maxBounces;       // max path length over its requests (AO: 0)
  int completeFirst, completeEnd;  // requests whose last pixel is in this wave
};

// Splits the requests' paths (pixel-major, spp per pixel) into waves of at
// most wavePaths paths and builds the device tables (requests + segments) in
// `tables` (host bytes, uploaded by the caller before the waves run).
// byte offsets of the tables after the request table, and the wave count
struct BatchLayout {
  size_t segs, waves, post;
  int nwaves;
};
void planBatch(const SamplerTables *T, const AlbedoTablesD *AT, const BatchReqH *reqs, int n, long long wavePaths,
               std::vector<unsigned char> &tables, std::vector<BatchWave> &waves, BatchLayout &layout);
// Enqueues one wave: generate, bounces (closest trace, shade, shadow trace),
// finalize into each request's framebuffer.  dtables = device copy of tables.
cudaError_t launchBatchWave(const void *dtables, size_t segTableOffset, const BatchWave &w, const BatchTuning &tune,
                            void *workspace, size_t wsBytes, unsigned long long *rayCount, cudaStream_t st);
// Enqueues the whole batch frame as ONE cooperative persistent launch: the
// waves' stages (generate, per bounce closest trace / shade / shadow trace,
// finalize) run in order inside the kernel, separated by grid-wide barriers;
// completed requests are post-processed and stamped inside it (stamps[n] =
// start).  `barrier` is 4 words the call clears; barrier[2] != 0 after the
// launch means a barrier wait ran longer than timeoutNs (every block then
// left the kernel; the frame is incomplete).
cudaError_t launchBatchPersistent(const void *dtables, const BatchLayout &layout, int nreqs, const BatchTuning &tune,
                                  void *workspace, size_t wsBytes, unsigned long long *rayCount,
                                  unsigned long long *stamps, uint32_t *barrier, unsigned long long timeoutNs,
                                  cudaStream_t st);
// resident blocks per SM of the persistent batch kernel (its grid = SMs x this)
int batchPersistentBlocksPerSM();
// writes the global timer into stamps[first..end) (request completion times)
cudaError_t launchStamp(unsigned long long *stamps, int first, int end, cudaStream_t st);

// Renderer_pick: one camera ray at screen (sx, sy), closest hit; out[0] hit,
// out[1..3] world position bits, out[4..6] instID, geomID, primID.
cudaError_t launchPick(const Scene &sc, const CameraD &cam, float sx, float sy, uint32_t *out, cudaStream_t st);
cudaError_t launchTrace(const Scene &sc, const float4 *rays, long long n, int occlusion, float *outF, uint32_t *outI,
                        cudaStream_t st);
cudaError_t launchRenderAO(const SamplerTables *T, const Scene &sc, const CameraD &cam, const PixelFilterD &pf, const AOParamsD &p,
                           const FrameD &fb, bool stats, cudaStream_t st, KernelTimer *kt = nullptr, const VolumeD *vol = nullptr,
                           bool surf = false);

}  // namespace b200
