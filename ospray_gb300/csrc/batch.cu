// Batched rendering (b200_batch_*): many requests in one wavefront, run
// either as a sequence of wavefront kernels per wave (launched directly or
// captured as a CUDA graph) or as one cooperative persistent launch that
// runs every wave's stages itself (captured as a one-kernel graph), with an
// autotuner over the wavefront's launch shape.
//
// The host keeps the requests as (scene, frame, camera, parameters); each
// render rebuilds the small device tables (requests, segments, waves,
// post-processing; frame IDs advance) and uploads them before launching.
// The launch sequence itself depends only on the wave plan, the tuning, the
// mode and the frames' post-processing, so it is captured once and replayed
// until one of those changes.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "api_internal.h"

namespace b200 {

struct BatchObj {
  struct Req {
    int kind;
    SceneObj *scene;
    FrameObj *fb;
    b200_camera_desc cam;
    int pixelFilter;
    PtParamsD pt;
    AOParamsD ao;
    MaterialD *dMats = nullptr;
  };
  DeviceObj *dev;
  std::vector<Req> reqs;
  BatchTuning tune = {int64_t(1) << 23, 4, 2};
  void *ws = nullptr;
  size_t wsBytes = 0;
  void *dtables = nullptr;
  size_t tablesCap = 0;
  void *htables = nullptr;  // pinned staging copy of the table
  size_t htablesCap = 0;
  unsigned long long *dStamps = nullptr, *dRays = nullptr;
  uint32_t *dBarrier = nullptr;  // the persistent kernel's grid barrier (4 words)
  int stampsCap = 0;
  std::vector<BatchWave> waves;
  BatchLayout layout = {};
  int mode = B200_BATCH_GRAPH;  // of the last render (the autotuner tunes for it)
  unsigned long long barrierTimeoutNs = 4000000000ull;  // the persistent kernel's bounded barrier wait
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<float> graphKey;  // what the captured graph depends on

  explicit BatchObj(DeviceObj *d) : dev(d) { dev->retain(); }
  ~BatchObj() {
    cudaSetDevice(dev->dev);
    cudaStreamSynchronize(dev->stream);
    dropGraph();
    for (Req &r : reqs)
      if (r.dMats) cudaFree(r.dMats);
    if (ws) cudaFree(ws);
    if (dtables) cudaFree(dtables);
    if (htables) cudaFreeHost(htables);
    if (dStamps) cudaFree(dStamps);
    if (dRays) cudaFree(dRays);
    if (dBarrier) cudaFree(dBarrier);
    dev->release();
  }
  void dropGraph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    graphKey.clear();
  }

  std::vector<BatchReqH> describe() const {
    std::vector<BatchReqH> h(reqs.size());
    for (size_t i = 0; i < reqs.size(); i++) {
      const Req &r = reqs[i];
      BatchReqH &d = h[i];
      d = BatchReqH{};
      d.kind = r.kind;
      d.sc = r.scene->view();
      d.cam = makeCamera(r.cam);
      d.pf = dev->filter(r.pixelFilter);
      d.pt = r.pt;
      d.ao = r.ao;
      d.mats = r.dMats;
      d.lights = r.scene->dLights;
      d.lightCdf = r.scene->dLightCdf;
      d.fb = r.fb->view();
      d.fb.accumVariance = 0;     // batched frames keep no variance estimate
      d.fb.taskActive = nullptr;  // and render every task
      d.postFormat = r.fb->format;
      d.postTonemap = r.fb->toneMapOn ? 1 : 0;
      d.postTm = r.fb->toneMap;
      d.postOut = r.fb->mapped;
    }
    return h;
  }

  // everything the captured kernel sequence depends on, besides the table
  std::vector<float> key() const {
    std::vector<float> k = {float(mode), float(tune.wavePaths), float(tune.traceBlocksPerSM),
                            float(tune.shadeBlocksPerSM), float(reqs.size()), float(barrierTimeoutNs)};
    for (const Req &r : reqs) {
      const FrameObj *f = r.fb;
      k.insert(k.end(), {float(r.kind), float(f->W), float(f->H), float(f->format), f->toneMapOn ? 1.f : 0.f,
                         f->toneMap.exposure, f->toneMap.a, f->toneMap.b, f->toneMap.c, f->toneMap.d,
                         float(f->toneMap.aces), float(r.kind == BATCH_PT ? r.pt.spp : r.ao.spp),
                         float(r.kind == BATCH_PT ? r.pt.maxPathLength : 0)});
    }
    return k;
  }

  // plans the waves, sizes the buffers and uploads the request table
  void prepare(cudaStream_t st) {
    std::vector<unsigned char> tables;
    const std::vector<BatchReqH> h = describe();
    planBatch(dev->tables, dev->albedoTables(), h.data(), int(h.size()), tune.wavePaths, tables, waves, layout);
    const size_t need = ptWorkspaceBytes(tune.wavePaths);
    if (need > wsBytes || tables.size() > tablesCap || int(reqs.size()) + 1 > stampsCap) {
      check(cudaStreamSynchronize(st), "sync");
      dropGraph();
    }
    if (need > wsBytes) {
      if (ws) cudaFree(ws);
      ws = nullptr;
      wsBytes = 0;
      check(cudaMalloc(&ws, need), "batch workspace");
      wsBytes = need;
    }
    if (tables.size() > tablesCap) {
      if (dtables) cudaFree(dtables);
      dtables = nullptr;
      check(cudaMalloc(&dtables, tables.size()), "batch tables");
      tablesCap = tables.size();
    }
    if (tables.size() > htablesCap) {
      check(cudaStreamSynchronize(st), "sync");
      if (htables) cudaFreeHost(htables);
      htables = nullptr;
      check(cudaMallocHost(&htables, tables.size()), "batch staging");
      htablesCap = tables.size();
    }
    if (int(reqs.size()) + 1 > stampsCap) {
      if (dStamps) cudaFree(dStamps);
      if (!dRays) check(cudaMalloc(&dRays, sizeof(unsigned long long)), "batch ray counter");
      check(cudaMalloc(&dStamps, sizeof(unsigned long long) * (reqs.size() + 1)), "batch stamps");
      stampsCap = int(reqs.size()) + 1;
    }
    if (!dBarrier) {
      check(cudaMalloc(&dBarrier, 4 * sizeof(uint32_t)), "batch barrier");
      check(cudaMemset(dBarrier, 0, 4 * sizeof(uint32_t)), "clear batch barrier");
    }
    // the staging buffer may still feed the previous render's copy
    check(cudaStreamSynchronize(st), "sync");
    checkBarrier();
    std::memcpy(htables, tables.data(), tables.size());
    check(cudaMemcpyAsync(dtables, htables, tables.size(), cudaMemcpyHostToDevice, st), "upload batch table");
  }

  // after the stream has drained: did a barrier wait of the persistent
  // kernel time out?  (It then left the frame incomplete.)
  void checkBarrier() {
    if (!dBarrier) return;
    uint32_t w[4] = {0, 0, 0, 0};
    check(cudaMemcpy(w, dBarrier, sizeof(w), cudaMemcpyDeviceToHost), "read batch barrier");
    if (w[2]) {
      check(cudaMemset(dBarrier, 0, sizeof(w)), "clear batch barrier");
      throw Error(B200_UNKNOWN_ERROR, "batch: a grid barrier of the persistent kernel timed out; the frame is incomplete");
    }
  }

  // the whole frame of every request: the capturable launch sequence
  void enqueue(cudaStream_t st) {
    const int n = int(reqs.size());
    check(cudaMemsetAsync(dRays, 0, sizeof(unsigned long long), st), "clear ray counter");
    if (mode == B200_BATCH_PERSISTENT) {
      check(launchBatchPersistent(dtables, layout, n, tune, ws, wsBytes, dRays, dStamps, dBarrier, barrierTimeoutNs,
                                  st),
            "persistent batch kernel");
      return;
    }
    check(launchStamp(dStamps, n, n + 1, st), "stamp");
    for (const BatchWave &w : waves) {
      check(launchBatchWave(dtables, layout.segs, w, tune, ws, wsBytes, dRays, st), "batch wave");
      for (int r = w.completeFirst; r >= 0 && r < w.completeEnd; r++) framePostProcess(reqs[r].fb, st, false);
      if (w.completeFirst >= 0) check(launchStamp(dStamps, w.completeFirst, w.completeEnd, st), "stamp");
    }
  }

  void render(int m) {
    if (reqs.empty()) throw Error(B200_INVALID_OPERATION, "empty batch");
    if (m < B200_BATCH_KERNELS || m > B200_BATCH_PERSISTENT) throw Error(B200_INVALID_ARGUMENT, "bad batch mode");
    cudaStream_t st = dev->stream;
    mode = m;
    prepare(st);
    if (m != B200_BATCH_KERNELS) {
      const std::vector<float> k = key();
      if (!exec || k != graphKey) {
        dropGraph();
        check(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
        try {
          enqueue(st);
        } catch (...) {
          cudaGraph_t g = nullptr;
          cudaStreamEndCapture(st, &g);
          if (g) cudaGraphDestroy(g);
          throw;
        }
        check(cudaStreamEndCapture(st, &graph), "end capture");
        check(cudaGraphInstantiate(&exec, graph, 0), "instantiate graph");
        graphKey = k;
      }
      check(cudaGraphLaunch(exec, st), "graph launch");
    } else {
      enqueue(st);
    }
    for (Req &r : reqs) r.fb->frameID++;
  }
};

namespace {
template <class F>
int batchGuard(BatchObj *b, F f) {
  try {
    check(cudaSetDevice(b->dev->dev), "cudaSetDevice");
    f();
    return B200_NO_ERROR;
  } catch (const Error &e) {
    b->dev->lastError = e.what();
    return e.code;
  } catch (const std::exception &e) {
    b->dev->lastError = e.what();
    return B200_UNKNOWN_ERROR;
  }
}

void requireArg(bool c, const char *msg) {
  if (!c) throw Error(B200_INVALID_ARGUMENT, msg);
}
}  // namespace

}  // namespace b200

using namespace b200;

extern "C" {

int b200_batch_create(b200_device d, b200_batch *out) {
  if (!d || !out) return B200_INVALID_ARGUMENT;
  *out = reinterpret_cast<b200_batch>(new BatchObj(reinterpret_cast<DeviceObj *>(d)));
  return B200_NO_ERROR;
}

int b200_batch_release(b200_batch h) {
  if (!h) return B200_INVALID_ARGUMENT;
  delete reinterpret_cast<BatchObj *>(h);
  return B200_NO_ERROR;
}

int b200_batch_add_ao(b200_batch h, b200_scene s, const b200_camera_desc *camera, const b200_ao_params *p,
                      b200_frame f) {
  if (!h || !s || !camera || !p || !f) return B200_INVALID_ARGUMENT;
  BatchObj *b = reinterpret_cast<BatchObj *>(h);
  return batchGuard(b, [&]() {
    SceneObj *sc = reinterpret_cast<SceneObj *>(s);
    FrameObj *fb = reinterpret_cast<FrameObj *>(f);
    requireArg(sc->dev == b->dev && fb->dev == b->dev, "scene and framebuffer must belong to the batch's device");
    requireArg(sc->committed, "scene not committed");
    requireArg(!sc->hasMotion(), "batch: scenes with motion-blurred instances are rendered by the single-request calls");
    requireArg(p->pixelSamples >= 1 && p->aoSamples >= 0, "bad AO parameters");
    requireArg(p->pixelFilter >= B200_PF_POINT && p->pixelFilter <= B200_PF_BLACKMAN_HARRIS, "bad pixel filter");
    // the batched AO shading is the white, opaque surface case
    requireArg(p->nmaterials == 0 && !p->backplate && !p->maxDepth && !sc->hasAttributes,
               "batch: AO with materials, vertex attributes, backplate or maxDepth is rendered by b200_render_ao only");
    BatchObj::Req r;
    r.kind = BATCH_AO;
    r.scene = sc;
    r.fb = fb;
    r.cam = *camera;
    r.pixelFilter = p->pixelFilter;
    r.pt = PtParamsD{};
    r.ao = makeAOParams(*p);
    b->reqs.push_back(r);
  });
}

int b200_batch_add_pt(b200_batch h, b200_scene s, const b200_camera_desc *camera, const b200_pt_params *p,
                      const b200_material *materials, int nmaterials, b200_frame f) {
  if (!h || !s || !camera || !p || !f) return B200_INVALID_ARGUMENT;
  BatchObj *b = reinterpret_cast<BatchObj *>(h);
  return batchGuard(b, [&]() {
    SceneObj *sc = reinterpret_cast<SceneObj *>(s);
    FrameObj *fb = reinterpret_cast<FrameObj *>(f);
    requireArg(sc->dev == b->dev && fb->dev == b->dev, "scene and framebuffer must belong to the batch's device");
    requireArg(sc->committed, "scene not committed");
    requireArg(!sc->hasMotion(), "batch: scenes with motion-blurred instances are rendered by the single-request calls");
    requireArg(p->pixelSamples >= 1 && p->maxPathLength >= 0, "bad path tracer parameters");
    requireArg(p->pixelFilter >= B200_PF_POINT && p->pixelFilter <= B200_PF_BLACKMAN_HARRIS, "bad pixel filter");
    requireArg(nmaterials >= 0 && (nmaterials == 0 || materials), "bad material array");
    BatchObj::Req r;
    r.kind = BATCH_PT;
    r.scene = sc;
    r.fb = fb;
    r.cam = *camera;
    r.pixelFilter = p->pixelFilter;
    // the batched wavefront traces shadow rays as any-hit queries only and
    // keeps no ray cones (texture level selection) in its path records
    requireArg(!anyTransparent(materials, nmaterials),
               "batch: materials that let shadow rays through (opacity < 1, obj tf / d, glass) are rendered by "
               "b200_render_pt only");
    for (int i = 0; i < nmaterials; i++)
      requireArg(!materials[i].baseColorMap, "batch: textured materials are rendered by b200_render_pt only");
    requireArg(!p->backplate && !p->maxDepth, "batch: backplate and maxDepth textures are rendered by b200_render_pt only");
    r.pt = makePtParams(*p, sc, materials, nmaterials, false);
    requireArg(!r.pt.transparentShadows,
               "batch: vertex colours with alpha < 1 under obj materials are rendered by b200_render_pt only");
    r.pt.allMaterials = 1;
    r.ao = AOParamsD{};
    if (nmaterials) {
      std::vector<MaterialD> m(nmaterials);
      for (int i = 0; i < nmaterials; i++) m[i] = toMaterialD(materials[i]);
      check(cudaMalloc(&r.dMats, sizeof(MaterialD) * nmaterials), "batch materials");
      check(cudaMemcpy(r.dMats, m.data(), sizeof(MaterialD) * nmaterials, cudaMemcpyHostToDevice),
            "upload batch materials");
    }
    b->reqs.push_back(r);
  });
}

int b200_batch_get_tuning(b200_batch h, b200_batch_tuning *out) {
  if (!h || !out) return B200_INVALID_ARGUMENT;
  const BatchObj *b = reinterpret_cast<BatchObj *>(h);
  out->wavePaths = b->tune.wavePaths;
  out->traceBlocksPerSM = b->tune.traceBlocksPerSM;
  out->shadeBlocksPerSM = b->tune.shadeBlocksPerSM;
  return B200_NO_ERROR;
}

int b200_batch_set_tuning(b200_batch h, const b200_batch_tuning *t) {
  if (!h || !t) return B200_INVALID_ARGUMENT;
  BatchObj *b = reinterpret_cast<BatchObj *>(h);
  return batchGuard(b, [&]() {
    requireArg(t->wavePaths >= 1024 && t->wavePaths <= (int64_t(1) << 28), "wavePaths out of range");
    requireArg(t->traceBlocksPerSM >= 1 && t->traceBlocksPerSM <= 16, "traceBlocksPerSM out of range");
    requireArg(t->shadeBlocksPerSM >= 1 && t->shadeBlocksPerSM <= 16, "shadeBlocksPerSM out of range");
    b->tune = {t->wavePaths, t->traceBlocksPerSM, t->shadeBlocksPerSM};
  });
}

int b200_batch_autotune(b200_batch h, int candidates, b200_batch_tuning *best) {
  if (!h) return B200_INVALID_ARGUMENT;
  BatchObj *b = reinterpret_cast<BatchObj *>(h);
  return batchGuard(b, [&]() {
    requireArg(!b->reqs.empty(), "empty batch");
    long long total = 0;
    int maxSpp = 1;
    for (const auto &r : b->reqs) {
      const int spp = r.kind == BATCH_PT ? r.pt.spp : r.ao.spp;
      total += (long long)r.fb->W * r.fb->H * spp;
      maxSpp = std::max(maxSpp, spp);
    }
    // candidate wave sizes from 2M path slots up to the whole batch (or 16M)
    std::vector<long long> sizes;
    for (long long w = 1 << 21; w < (1 << 24) && w < total; w *= 2) sizes.push_back(w);
    sizes.push_back(std::max<long long>(std::min<long long>(total, 1 << 24), maxSpp));
    // the persistent kernel's residency is fixed (all co-resident blocks):
    // only the wave size varies for it
    const int tuneMode = b->mode == B200_BATCH_PERSISTENT ? B200_BATCH_PERSISTENT : B200_BATCH_KERNELS;
    std::vector<BatchTuning> cands;
    for (long long w : sizes)
      if (tuneMode == B200_BATCH_PERSISTENT)
        cands.push_back({w, b->tune.traceBlocksPerSM, b->tune.shadeBlocksPerSM});
      else
        for (int tb : {2, 3, 4, 5})
          for (int sb : {1, 2}) cands.push_back({w, tb, sb});
    if (candidates > 0 && size_t(candidates) < cands.size()) {
      // an even spread over the set
      std::vector<BatchTuning> pick;
      for (int i = 0; i < candidates; i++) pick.push_back(cands[size_t(i) * cands.size() / candidates]);
      cands = pick;
    }
    cudaStream_t st = b->dev->stream;
    cudaEvent_t e0, e1;
    check(cudaEventCreate(&e0), "event");
    check(cudaEventCreate(&e1), "event");
    float bestMs = 1e30f;
    BatchTuning bestT = b->tune;
    std::vector<int> frameIDs;
    for (const auto &r : b->reqs) frameIDs.push_back(r.fb->frameID);
    try {
      for (const BatchTuning &t : cands) {
        b->tune = t;
        b->render(tuneMode);  // warm-up (workspace, caches)
        check(cudaEventRecord(e0, st), "event");
        b->render(tuneMode);
        check(cudaEventRecord(e1, st), "event");
        check(cudaEventSynchronize(e1), "event");
        float ms = 0.f;
        check(cudaEventElapsedTime(&ms, e0, e1), "event");
        if (ms < bestMs) {
          bestMs = ms;
          bestT = t;
        }
      }
    } catch (...) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->tune = bestT;
    b->dropGraph();
    for (auto &r : b->reqs) r.fb->frameID = 0;
    if (best) {
      best->wavePaths = bestT.wavePaths;
      best->traceBlocksPerSM = bestT.traceBlocksPerSM;
      best->shadeBlocksPerSM = bestT.shadeBlocksPerSM;
    }
  });
}

int b200_batch_set_barrier_timeout(b200_batch h, uint64_t ns) {
  if (!h) return B200_INVALID_ARGUMENT;
  reinterpret_cast<BatchObj *>(h)->barrierTimeoutNs = ns ? ns : 4000000000ull;
  return B200_NO_ERROR;
}

int b200_batch_render(b200_batch h, int mode) {
  if (!h) return B200_INVALID_ARGUMENT;
  BatchObj *b = reinterpret_cast<BatchObj *>(h);
  return batchGuard(b, [&]() { b->render(mode); });
}

int b200_batch_info(b200_batch h, int64_t *info) {
  if (!h || !info) return B200_INVALID_ARGUMENT;
  const BatchObj *b = reinterpret_cast<BatchObj *>(h);
  int64_t kernels = 1, paths = 0;  // the start stamp
  for (const BatchWave &w : b->waves) paths += w.npaths;
  if (b->mode == B200_BATCH_PERSISTENT) kernels = 1;  // everything in one launch
  else for (const BatchWave &w : b->waves) {
    kernels += 1 + 4 * int64_t(w.maxBounces + 1) + 1 + 1;  // generate, bounces, ray tail, finalize
    if (B200_SHADE_PARTITION) kernels += w.maxBounces;     // the queue partitions
    if (w.completeFirst >= 0) {
      kernels += 1;  // stamp
      for (int r = w.completeFirst; r < w.completeEnd; r++) kernels += b->reqs[r].fb->format != B200_FB_NONE;
    }
  }
  info[0] = int64_t(b->waves.size());
  info[1] = kernels;
  info[2] = paths;
  info[3] = int64_t(b->reqs.size());
  return B200_NO_ERROR;
}

int b200_batch_timings(b200_batch h, double *ms, int n, uint64_t *rays) {
  if (!h) return B200_INVALID_ARGUMENT;
  BatchObj *b = reinterpret_cast<BatchObj *>(h);
  return batchGuard(b, [&]() {
    requireArg(b->dStamps != nullptr, "batch not rendered");
    check(cudaStreamSynchronize(b->dev->stream), "sync");
    b->checkBarrier();
    const int nr = int(b->reqs.size());
    std::vector<unsigned long long> t(nr + 1);
    check(cudaMemcpy(t.data(), b->dStamps, sizeof(unsigned long long) * (nr + 1), cudaMemcpyDeviceToHost),
          "read stamps");
    if (ms)
      for (int i = 0; i < std::min(n, nr); i++) ms[i] = double(t[i] - t[nr]) * 1e-6;
    if (rays) {
      unsigned long long r = 0;
      check(cudaMemcpy(&r, b->dRays, sizeof(r), cudaMemcpyDeviceToHost), "read ray count");
      *rays = r;
    }
  });
}

}  // extern "C"
