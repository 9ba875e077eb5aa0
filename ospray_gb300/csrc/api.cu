// Host side of the b200 C ABI (include/b200.h): device, world, framebuffer
// and renderer objects that own device memory and launch the kernels.
// Every entry point catches its own failures and returns an OSPError code,
// like the reference's API wrappers (ospray/api/API.cpp:28-66).
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/b200.h"
#include "api_internal.h"

namespace b200 {

void check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw Error(e == cudaErrorMemoryAllocation ? B200_OUT_OF_MEMORY : B200_UNKNOWN_ERROR,
                                    std::string(what) + ": " + cudaGetErrorString(e));
}

namespace {

// Halton digit permutations (Faure) and bit-reversed Joe-Kuo Sobol matrices;
// the constructions behind modules/cpu/math/halton.inl and sobol.inl.
void buildTables(SamplerTables &t) {
  auto perm = [](uint32_t base, int nd, const uint32_t *sigma, uint32_t *out) {
    uint32_t n = 1;
    for (int k = 0; k < nd; k++) n *= base;
    for (uint32_t i = 0; i < n; i++) {
      uint32_t v = 0, x = i;
      for (int k = 0; k < nd; k++, x /= base) v = v * base + sigma[x % base];
      out[i] = v;
    }
  };
  static const uint32_t f3[3] = {0, 1, 2}, f5[5] = {0, 3, 2, 1, 4}, f7[7] = {0, 2, 5, 3, 1, 4, 6};
  perm(3, 5, f3, t.perm3);
  perm(5, 3, f5, t.perm5);
  perm(7, 3, f7, t.perm7);
  struct Dim {
    int s;
    uint32_t a, m[3];
  };
  static const Dim dims[4] = {{1, 0, {1, 0, 0}}, {2, 1, {1, 3, 0}}, {3, 1, {1, 3, 1}}, {3, 2, {1, 1, 1}}};
  for (int d = 0; d < 4; d++) {
    uint64_t m[33];
    const int s = dims[d].s;
    for (int k = 1; k <= s; k++) m[k] = dims[d].m[k - 1];
    for (int k = s + 1; k <= 32; k++) {
      uint64_t v = m[k - s] ^ (m[k - s] << s);
      for (int j = 1; j < s; j++)
        if ((dims[d].a >> (s - 1 - j)) & 1u) v ^= m[k - j] << j;
      m[k] = v;
    }
    for (int i = 0; i < 32; i++) {
      uint32_t x = uint32_t(m[i + 1] << (31 - i)), r = 0;
      for (int b = 0; b < 32; b++) r |= ((x >> b) & 1u) << (31 - b);
      t.sobolRev[4 * i + d] = r;
    }
  }
}

// LUT importance table of a pixel filter (pf/LUTPixelFilter.ispc:60-144 with
// Distribution1D_create / Distribution2D_init)
void buildFilterLUT(int type, float &width, int &lutW, std::vector<float> &cx, std::vector<float> &cy) {
  width = type == B200_PF_MITCHELL ? 4.f : 3.f;
  lutW = int(std::ceil(width)) * 5;
  cx.assign(size_t(lutW) * lutW, 0.f);
  cy.assign(lutW, 0.f);
  auto create1D = [](int n, float *cdf) {
    float sum = cdf[0];
    for (int i = 1; i < n; i++) cdf[i] = sum += cdf[i];
    const float rcpSum = 1.f / sum;
    for (int i = 0; i < n; i++) cdf[i] = cdf[i] >= sum ? 0x1.000002p+0f : cdf[i] * rcpSum;
    return sum;
  };
  for (int y = 0; y < lutW; y++) {
    const float fy = (y + 0.5f) * (1.f / float(lutW));
    for (int x = 0; x < lutW; x++) {
      const float fx = (x + 0.5f) * (1.f / float(lutW));
      const float px = (fx - 0.5f) * width, py = (fy - 0.5f) * width;
      float e = 0.f;
      if (type == B200_PF_GAUSS) {
        const float sigma = (0.5f * width) / 3.f;
        e = std::exp(-0.5f * ((px * px + py * py) / (sigma * sigma)));
      } else if (type == B200_PF_MITCHELL) {
        const float B = 1.f / 3.f, C = 1.f / 3.f;
        const float tx = px / width * 4.f, ty = py / width * 4.f;
        const float f = std::sqrt(tx * tx + ty * ty), f2 = f * f, f3 = f2 * f;
        if (f < 1.f)
          e = (1.f / 6.f) * ((12.f - 9.f * B - 6.f * C) * f3 + (-18.f + 12.f * B + 6.f * C) * f2 + (6.f - 2.f * B));
        else if (f < 2.f)
          e = (1.f / 6.f) *
              ((-B - 6.f * C) * f3 + (6.f * B + 30.f * C) * f2 + (-12.f * B - 48.f * C) * f + (8.f * B + 24.f * C));
      } else {
        const float f = std::sqrt(px * px + py * py) + width / 2.f;
        const float w = 1.f / width;
        const float pi2 = float(2.0 * M_PI);
        e = 0.35875f - 0.48829f * std::cos(pi2 * f * w) + 0.14128f * std::cos(2.f * pi2 * f * w) -
            0.01168f * std::cos(3.f * pi2 * f * w);
      }
      cx[size_t(y) * lutW + x] = e > 0.f ? e : 0.f;
    }
    cy[y] = create1D(lutW, &cx[size_t(y) * lutW]);
  }
  create1D(lutW, cy.data());
}

}  // namespace

DeviceObj::DeviceObj(int cudaDev) : dev(cudaDev) {
  check(cudaSetDevice(dev), "cudaSetDevice");
  check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
  SamplerTables t;
  buildTables(t);
  check(cudaMalloc(&tables, sizeof(SamplerTables)), "cudaMalloc tables");
  check(cudaMalloc(&work, 64), "cudaMalloc work counter");
  check(cudaMalloc(&pickBuf, 32), "cudaMalloc pick result");
  check(cudaMemcpy(tables, &t, sizeof(t), cudaMemcpyHostToDevice), "upload tables");
  for (int type = B200_PF_GAUSS; type <= B200_PF_BLACKMAN_HARRIS; type++) {
    std::vector<float> cx, cy;
    float w;
    int lw;
    buildFilterLUT(type, w, lw, cx, cy);
    FilterLUT &L = luts[type];
    L.width = w;
    L.lutW = lw;
    check(cudaMalloc(&L.cdf_x, cx.size() * 4), "cudaMalloc lut");
    check(cudaMalloc(&L.cdf_y, cy.size() * 4), "cudaMalloc lut");
    check(cudaMemcpy(L.cdf_x, cx.data(), cx.size() * 4, cudaMemcpyHostToDevice), "upload lut");
    check(cudaMemcpy(L.cdf_y, cy.data(), cy.size() * 4, cudaMemcpyHostToDevice), "upload lut");
  }
}

const AlbedoTablesD *DeviceObj::albedoTables() {
  if (!albedo) {
    check(cudaMalloc(&albedo, sizeof(AlbedoTablesD)), "cudaMalloc albedo tables");
    check(computeAlbedoTables(albedo, stream), "albedo tables");
  }
  return albedo;
}

DeviceObj::~DeviceObj() {
  cudaSetDevice(dev);
  cudaStreamSynchronize(stream);
  cudaFree(tables);
  cudaFree(work);
  cudaFree(pickBuf);
  if (albedo) cudaFree(albedo);
  if (ptWs) cudaFree(ptWs);
  if (ptTimes) cudaFree(ptTimes);
  delete timer;
  for (auto &L : luts) {
    cudaFree(L.cdf_x);
    cudaFree(L.cdf_y);
  }
  cudaStreamDestroy(stream);
}

PixelFilterD DeviceObj::filter(int type) const {
  PixelFilterD pf = {};
  pf.type = type <= B200_PF_BOX ? type : 2;
  if (type == B200_PF_POINT) pf.width = 0.f;
  if (type == B200_PF_BOX) pf.width = 1.f;
  if (type >= B200_PF_GAUSS && type <= B200_PF_BLACKMAN_HARRIS) {
    pf.width = luts[type].width;
    pf.lutW = luts[type].lutW;
    pf.cdf_x = luts[type].cdf_x;
    pf.cdf_y = luts[type].cdf_y;
  }
  return pf;
}

// A material as the shading kernels read it, with each type's commit-time
// normalisation: OBJ scales kd + ks + tf down to 1 (OBJ::commit,
// render/materials/OBJ.cpp:45-53); glass keeps the inside and outside media
// as (ior, log(attenuation colour) / attenuation distance) (Glass::commit,
// Glass.cpp:27-50); thin glass keeps 1 / eta and log(colour) x thickness /
// distance (ThinGlass::commit, ThinGlass.cpp:27-45).
MaterialD toMaterialD(const b200_material &m) {
  MaterialD d;
  std::memset(&d, 0, sizeof(d));
  d.kind = uint32_t(m.type);
  d.opacity = 1.f;
  d.iorIn = d.iorOut = 1.f;
  const float eps = 1e-6f;
  switch (m.type) {
    case B200_MATERIAL_PRINCIPLED:
      d.r = m.baseColor[0];
      d.g = m.baseColor[1];
      d.b = m.baseColor[2];
      d.roughness = m.roughness;
      d.metallic = m.metallic;
      d.opacity = m.opacity;
      d.ns = m.specular;
      d.eta = m.ior;
      d.tf[0] = m.diffuse;
      for (int c = 0; c < 3; c++) d.ks[c] = m.edgeColor[c];
      d.pad0 = m.specularMetallic ? 1.f : 0.f;
      if (1.f - m.opacity > eps) d.flags |= MATF_TRANSPARENT;
      break;
    case B200_MATERIAL_OBJ: {
      float kd[3], ks[3], tf[3], total = 0.f;
      for (int c = 0; c < 3; c++) {
        kd[c] = m.baseColor[c];
        ks[c] = m.ks[c];
        tf[c] = m.tf[c];
        total = std::max(total, kd[c] + ks[c] + tf[c]);
      }
      if (total > 1.f)
        for (int c = 0; c < 3; c++) {
          kd[c] /= total;
          ks[c] /= total;
          tf[c] /= total;
        }
      d.r = kd[0];
      d.g = kd[1];
      d.b = kd[2];
      for (int c = 0; c < 3; c++) {
        d.ks[c] = ks[c];
        d.tf[c] = tf[c];
      }
      d.ns = m.ns;
      d.opacity = m.opacity;
      for (int c = 0; c < 3; c++)
        if (tf[c] * m.opacity + (1.f - m.opacity) > 0.f) d.flags |= MATF_TRANSPARENT;
      break;
    }
    case B200_MATERIAL_METAL:
      d.roughness = m.roughness;
      for (int c = 0; c < 3; c++) {
        d.ceta[c] = m.eta[c];
        d.ck[c] = m.k[c];
      }
      break;
    case B200_MATERIAL_GLASS:
      d.iorIn = m.eta[0];
      d.iorOut = m.eta[1];
      for (int c = 0; c < 3; c++) d.att[c] = std::log(m.attenuationColor[c]) / std::max(m.attenuationDistance, eps);
      d.flags |= MATF_TRANSPARENT;
      break;
    case B200_MATERIAL_THINGLASS: {
      d.eta = 1.f / m.eta[0];
      const float scale = m.thickness * (1.f / std::max(m.attenuationDistance, eps));
      for (int c = 0; c < 3; c++) d.att[c] = std::log(m.attenuationColor[c]) * scale;
      d.flags |= MATF_TRANSPARENT;
      break;
    }
    default:
      throw Error(B200_INVALID_ARGUMENT, "unknown material type " + std::to_string(m.type));
  }
  if (m.baseColorMap && (m.type == B200_MATERIAL_PRINCIPLED || m.type == B200_MATERIAL_OBJ)) {
    d.map = textureDevice(m.baseColorMap);
    if (textureHasAlpha(m.baseColorMap)) d.flags |= MATF_MAP_ALPHA | MATF_TRANSPARENT;
  }
  return d;
}

bool anyTransparent(const b200_material *materials, int n) {
  for (int i = 0; i < n; i++)
    if (toMaterialD(materials[i]).flags & MATF_TRANSPARENT) return true;
  return false;
}

// a principled material the principled-only shading kernel does not carry:
// specular, ior, diffuse or edgeColor other than 1, or a smooth conductor
// (roughness 0 with metallic > 0; a smooth dielectric coating at ior 1 and
// Lambert equal that kernel's microfacet forms)
static bool principledNeedsFull(const b200_material &m) {
  return m.specular != 1.f || m.ior != 1.f || m.diffuse != 1.f || m.edgeColor[0] != 1.f || m.edgeColor[1] != 1.f ||
         m.edgeColor[2] != 1.f || (m.roughness < 1e-6f && m.metallic > 1e-6f);
}

// a material list that needs the shading kernel with every material type:
// a type other than principled, a principled material beyond the defaults
// above, a colour map, or a material shadow rays pass through
bool anyNonPrincipled(const b200_material *materials, int n) {
  for (int i = 0; i < n; i++)
    if (materials[i].type != B200_MATERIAL_PRINCIPLED || materials[i].baseColorMap ||
        principledNeedsFull(materials[i]) || (toMaterialD(materials[i]).flags & MATF_TRANSPARENT))
      return true;
  return false;
}

std::vector<ScivisMatD> toScivisMats(const b200_scivis_material *materials, int n) {
  std::vector<ScivisMatD> h(n);
  for (int i = 0; i < n; i++) {
    const b200_scivis_material &m = materials[i];
    ScivisMatD &d = h[i];
    std::memset(&d, 0, sizeof(d));
    d.isObj = m.isObj != 0;
    for (int k = 0; k < 3; k++) {
      d.kd[k] = m.kd[k];
      d.ks[k] = m.ks[k];
      d.tf[k] = m.tf[k];
    }
    d.ns = m.ns;
    d.d = m.d;
    d.kdMap = m.isObj ? textureDevice(m.kdMap) : nullptr;
  }
  return h;
}

// the renderer's material list on the device, uploaded when it changed
// (compared as device records: a texture made again at a reused host address
// still has a new device descriptor)
void uploadMaterials(SceneObj *sc, const b200_material *materials, int nmaterials) {
  std::vector<MaterialD> h(nmaterials);
  bool transparent = false;
  for (int i = 0; i < nmaterials; i++) {
    h[i] = toMaterialD(materials[i]);
    transparent = transparent || (h[i].flags & MATF_TRANSPARENT);
  }
  const bool same = int(sc->lastMaterials.size()) == nmaterials &&
                    (nmaterials == 0 ||
                     std::memcmp(sc->lastMaterials.data(), h.data(), sizeof(MaterialD) * nmaterials) == 0);
  if (!same) {
    if (nmaterials > sc->capMaterials) {
      if (sc->dMaterials) cudaFree(sc->dMaterials);
      check(cudaMalloc(&sc->dMaterials, sizeof(MaterialD) * nmaterials), "alloc materials");
      sc->capMaterials = nmaterials;
    }
    if (nmaterials)
      check(cudaMemcpy(sc->dMaterials, h.data(), sizeof(MaterialD) * nmaterials, cudaMemcpyHostToDevice),
            "upload materials");
    sc->lastMaterials = h;
    sc->transparentMaterials = transparent;
  }
  sc->nMaterials = nmaterials;
}

// the path workspace: grown on demand, kept for later frames
void ensurePtWorkspace(DeviceObj *dev, size_t need) {
  if (need <= dev->ptWsBytes) return;
  if (dev->ptWs) {
    check(cudaStreamSynchronize(dev->stream), "sync");
    cudaFree(dev->ptWs);
    dev->ptWs = nullptr;
    dev->ptWsBytes = 0;
  }
  check(cudaMalloc(&dev->ptWs, need), "path tracer workspace");
  dev->ptWsBytes = need;
}

// the per-path ray times of a frame of n paths (motion blur)
float *ensurePtTimes(DeviceObj *dev, long long n) {
  if (size_t(n) > dev->ptTimesCap) {
    check(cudaStreamSynchronize(dev->stream), "sync");
    if (dev->ptTimes) cudaFree(dev->ptTimes);
    dev->ptTimes = nullptr;
    dev->ptTimesCap = 0;
    check(cudaMalloc(&dev->ptTimes, sizeof(float) * size_t(n)), "path times");
    dev->ptTimesCap = size_t(n);
  }
  return dev->ptTimes;
}

// PathTracer::commit (render/pathtracer/PathTracer.cpp:29-51): light sample
// counts (lightSamples < 0: all lights at the first bounce; one after it
// when limitIndirectLightSamples), the backplate and mipMapBias
// (Renderer::commit render/Renderer.cpp:41-91).  Shadow rays loop over
// closest hits when a material lets them through (`transparentMaterials`) or
// vertex colours with alpha < 1 meet an obj material (its d scales by the
// colour's alpha); the shading kernel with every material type runs for
// other types than opaque principled, colour maps or vertex attributes.
PtParamsD makePtParams(const b200_pt_params &p, const SceneObj *sc, const b200_material *materials, int nmaterials,
                       bool transparentMaterials) {
  const int nl = sc->nLights;
  bool anyObj = false;
  for (int i = 0; i < nmaterials; i++) anyObj = anyObj || materials[i].type == B200_MATERIAL_OBJ;
  PtParamsD d;
  d.transparentShadows = transparentMaterials || (sc->colorAlpha && anyObj) ? 1 : 0;
  d.allMaterials = anyNonPrincipled(materials, nmaterials) || sc->hasAttributes ? 1 : 0;
  d.spp = p.pixelSamples;
  d.maxPathLength = p.maxPathLength;
  d.roulettePathLength = p.roulettePathLength;
  d.maxScatteringEvents = p.maxScatteringEvents;
  d.nFirst = p.lightSamples >= 0 && nl > 0 ? p.lightSamples : std::min(1024, nl);
  d.nIndirect = p.limitIndirectLightSamples && d.nFirst >= 1 ? 1 : d.nFirst;
  if (nl == 0) d.nFirst = d.nIndirect = 0;
  d.numLights = nl;
  d.numMaterials = nmaterials;
  d.minContribution = p.minContribution;
  d.maxContribution = p.maxContribution;
  for (int k = 0; k < 4; k++) d.bg[k] = p.backgroundColor[k];
  d.backplate = textureDevice(p.backplate);
  d.mipBiasFactor = std::pow(2.f, p.mipMapBias);
  d.maxDepth = textureDevice(p.maxDepth);
  return d;
}

AOParamsD makeAOParams(const b200_ao_params &p) {
  AOParamsD d;
  d.spp = p.pixelSamples;
  d.aoSamples = p.aoSamples;
  d.aoRadius = p.aoDistance;
  d.aoIntensity = p.aoIntensity;
  d.volumeSamplingRate = p.volumeSamplingRate > 0.f ? p.volumeSamplingRate : 1.f;
  for (int k = 0; k < 4; k++) d.bg[k] = p.backgroundColor[k];
  d.backplate = textureDevice(p.backplate);
  d.maxDepth = textureDevice(p.maxDepth);
  d.mipBiasFactor = std::pow(2.f, p.mipMapBias);
  d.mats = nullptr;  // set by the caller once the materials are on the device
  d.nmats = 0;
  return d;
}

// PerspectiveCamera::commit without stereo, aperture or motion blur
// Camera::commit's shutter (camera/Camera.cpp:44-52,100-119)
static void setShutter(const b200_camera_desc &c, CameraD &cam) {
  auto cl = [](float v) { return std::fmin(std::fmax(v, 0.f), 1.f); };
  float lo = cl(c.shutter[0]), hi = cl(c.shutter[1]);
  if (lo > hi) lo = hi;
  const int type = c.shutterType;
  const float dur = std::fmin(std::fmax(c.rollingShutterDuration, 0.f), hi - lo);
  cam.needTime = type == 0 ? hi - lo != 0.f : dur != 0.f;
  if (type != 0) {  // rolling: upper reduced by the duration; left / down run backwards
    hi -= dur;
    if (type == 2 || type == 3) std::swap(lo, hi);
  }
  cam.shutterLo = lo;
  cam.shutterHi = hi;
  cam.rollingDuration = dur;
  cam.shutterMode = type == 0 ? 0 : (type == 1 || type == 2 ? 1 : 2);
}

static CameraD makeCameraFrame(const b200_camera_desc &c);

CameraD makeCamera(const b200_camera_desc &c) {
  CameraD cam = makeCameraFrame(c);
  setShutter(c, cam);
  // the sub-image (Camera::commit camera/Camera.cpp:42-43,108-109); all
  // zero: the whole image
  const bool whole = c.imageStart[0] == 0.f && c.imageStart[1] == 0.f && c.imageEnd[0] == 0.f && c.imageEnd[1] == 0.f;
  cam.subLoX = whole ? 0.f : c.imageStart[0];
  cam.subLoY = whole ? 0.f : c.imageStart[1];
  cam.subHiX = whole ? 1.f : c.imageEnd[0];
  cam.subHiY = whole ? 1.f : c.imageEnd[1];
  const int sm = cam.type == 1 ? 0 : c.stereoMode;  // the orthographic camera has no stereo
  cam.split = sm == 3 ? 1 : sm == 4 ? 2 : 0;
  cam.coneScale = std::fabs(cam.subHiY - cam.subLoY) * (sm == 4 ? 2.f : 1.f);
  if (cam.type == 2) {  // PanoramicCamera::commit (camera/PanoramicCamera.cpp:45-52)
    const float h = 0.5f * c.interpupillaryDistance;
    cam.ipdOffset = mk(sm == 4 ? -h : h, 0.f, 0.f);
    cam.monoEye = sm == 1 ? -1.f : sm == 2 ? 1.f : 0.f;
  }
  return cam;
}

static CameraD makeCameraFrame(const b200_camera_desc &c) {
  const V3 pos = mk(c.position[0], c.position[1], c.position[2]);
  const V3 dir = mk(c.direction[0], c.direction[1], c.direction[2]);
  const V3 up = mk(c.up[0], c.up[1], c.up[2]);
  if (c.type == B200_CAMERA_ORTHOGRAPHIC) {  // OrthographicCamera::commit
    const float h = c.height;
    const V3 d = normalize(dir);
    V3 du = normalize(cross(d, up));
    const V3 dv = mul(cross(du, d), h);
    du = mul(du, h * c.aspect);
    CameraD cam = {};
    cam.type = 1;
    cam.dir_00 = d;
    cam.du_size = du;
    cam.dv_up = dv;
    cam.org = sub(sub(pos, mul(0.5f, du)), mul(0.5f, dv));
    cam.nearClip = c.nearClip > 0.f ? c.nearClip : 0.f;
    return cam;
  }
  if (c.type == B200_CAMERA_PANORAMIC) {  // PanoramicCamera::commit
    const V3 vz = mul(normalize(dir), -1.f);
    const V3 vx = normalize(cross(up, vz));
    CameraD cam = {};
    cam.type = 2;
    cam.du_size = vx;
    cam.dv_up = cross(vz, vx);
    cam.dir_00 = vz;
    cam.org = pos;
    cam.nearClip = c.nearClip > 0.f ? c.nearClip : 0.f;
    return cam;
  }
  const float deg2rad = float(1.745329251994329576923690768489e-2);
  // stereo (PerspectiveCamera.cpp:37-91): side by side halves the aspect,
  // top / bottom doubles it; left / right move the origin by half the
  // interpupillary distance along the film's x axis, the split modes keep
  // the offset (negated for top / bottom: the left eye at the top)
  const float aspect = c.stereoMode == 3 ? c.aspect * 0.5f : c.stereoMode == 4 ? c.aspect * 2.f : c.aspect;
  const float ipy = 2.f * std::tan(deg2rad * (0.5f * c.fovy));
  const float ipx = ipy * aspect;
  V3 d00 = normalize(dir);
  V3 du = normalize(cross(d00, up));
  V3 dv = c.architectural ? normalize(up) : cross(du, d00);  // architectural: the film parallel to up
  V3 ipd = mul(0.5f * c.interpupillaryDistance, du);
  V3 org = pos;
  if (c.stereoMode == 1) org = sub(org, ipd);
  if (c.stereoMode == 2) org = add(org, ipd);
  if (c.stereoMode == 4) ipd = mul(-1.f, ipd);
  du = mul(du, ipx);
  dv = mul(dv, ipy);
  d00 = sub(sub(d00, mul(0.5f, du)), mul(0.5f, dv));
  CameraD cam = {};
  // depth of field: the lens radius over the image plane, the frame
  // prescaled to the focal plane
  cam.scaledAperture = c.apertureRadius != 0.f ? c.apertureRadius / (ipx * c.focusDistance) : 0.f;
  if (cam.scaledAperture > 0.f) {
    du = mul(du, c.focusDistance);
    dv = mul(dv, c.focusDistance);
    d00 = mul(d00, c.focusDistance);
  }
  cam.aspect = aspect;
  cam.imgPlaneY = ipy;
  cam.org = org;
  cam.ipdOffset = ipd;
  cam.dir_00 = d00;
  cam.du_size = du;
  cam.dv_up = dv;
  cam.nearClip = c.nearClip > 0.f ? c.nearClip : 0.f;
  cam.type = 0;
  return cam;
}

// rkcommon rcp(AffineSpace3f) (rcpXfm) on a row-major 3x4 array
static void rcpAffine(const float *X, float *R) {
  Xfm x;
  std::memcpy(x.m, X, sizeof(x.m));
  const Xfm r = rcpXfm(x);
  std::memcpy(R, r.m, sizeof(r.m));
}

SceneObj::SceneObj(DeviceObj *d) : dev(d) {
  dev->retain();
  check(cudaMalloc(&status, 16), "cudaMalloc status");
  check(cudaMalloc(&counters, 64), "cudaMalloc counters");
  check(cudaMemset(counters, 0, 64), "memset counters");
  check(cudaMemset(status, 0, 16), "memset status");
}

SceneObj::~SceneObj() {
  cudaStream_t st = dev->stream;
  for (auto &g : geoms) {
    freeBLAS(g.blas, st);
    if (g.dverts) cudaFreeAsync(g.dverts, st);
    if (g.dindex) cudaFreeAsync(g.dindex, st);
    if (g.dquad) cudaFreeAsync(g.dquad, st);
    if (g.dsph) cudaFreeAsync(g.dsph, st);
    if (g.duser) cudaFreeAsync(g.duser, st);
    for (float *p : {g.dnormals, g.dcolors, g.dtexcoords})
      if (p) cudaFreeAsync(p, st);
  }
  if (tlas.nodes) cudaFreeAsync(tlas.nodes, st);
  if (tlas.leafPrim) cudaFreeAsync(tlas.leafPrim, st);
  if (dEntries) cudaFreeAsync(dEntries, st);
  if (dMotion) cudaFreeAsync(dMotion, st);
  cudaStreamSynchronize(st);
  if (dLights) cudaFree(dLights);
  if (dScivisLights) cudaFree(dScivisLights);
  if (dScivisMats) cudaFree(dScivisMats);
  if (dAoMats) cudaFree(dAoMats);
  if (dLightCdf) cudaFree(dLightCdf);
  if (dMaterials) cudaFree(dMaterials);
  for (void *p : {(void *)dVolData, (void *)dTfOpacity, (void *)dTfColor, (void *)dCellEmpty})
    if (p) cudaFree(p);
  cudaFree(status);
  cudaFree(counters);
  dev->release();
}

void SceneObj::commit() {
  cudaStream_t st = dev->stream;
  for (auto &g : geoms) {
    if (g.built) continue;
    if (g.type == GEOM_TRIANGLES)
      check(buildTriangleBLAS(g.dverts, g.dindex, int(g.nprims), st, g.blas, !dynamic,
                              g.meshKind == MESH_QUADS ? 2 : (g.meshKind == MESH_BOXES ? 12 : 1)),
            "BLAS build");
    else if (g.type == GEOM_SPHERES)
      check(buildSphereBLAS(g.dsph, int(g.nprims), st, g.blas, !dynamic), "BLAS build");
    else
      check(buildUserBLAS(uint32_t(g.type), g.duser ? g.duser : g.dsph, int(g.nprims), st, g.blas, !dynamic),
            "BLAS build");
    g.built = true;
  }
  // entries and their world boxes
  hasAttributes = colorAlpha = false;
  std::vector<Entry> he(entries.size());
  std::vector<float> keys;             // the motion-blurred entries' keys, one array
  std::vector<size_t> keyOff(entries.size(), 0);
  std::vector<float4> lo(entries.size()), hi(entries.size());
  float wlo[3] = {INFINITY, INFINITY, INFINITY}, whi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (size_t i = 0; i < entries.size(); i++) {
    const EntryH &e = entries[i];
    const GeomObj &g = geoms[e.geom];
    Entry &d = he[i];
    std::memset(&d, 0, sizeof(d));
    d.nodes = g.blas.bvh.nodes;
    d.prims = g.blas.prims;
    d.primIDs = g.blas.primIDs;
    d.verts = g.dverts;
    d.index = g.dquad ? g.dquad : g.dindex;
    d.meshKind = g.meshKind;
    d.spheres = g.dsph;
    d.normals = g.dnormals;
    d.colors = g.dcolors;
    d.texcoords = g.dtexcoords;
    hasAttributes = hasAttributes || g.dnormals || g.dcolors || g.dtexcoords;
    colorAlpha = colorAlpha || g.colorAlpha;
    d.type = uint32_t(g.type);
    d.instID = e.instID;
    d.geomID = e.geomID;
    d.identity = e.identity ? 1u : 0u;
    std::memcpy(d.xfm.m, e.xfm, sizeof(e.xfm));
    rcpAffine(e.xfm, d.rcp.m);
    d.epsScale = std::fmax(std::fabs(e.xfm[0]), std::fmax(std::fabs(e.xfm[5]), std::fabs(e.xfm[10])));
    d.materialID = uint32_t(e.material);
    const int nkeys = int(e.motion.size() / 12);
    if (nkeys >= 2) {
      keyOff[i] = keys.size();
      keys.insert(keys.end(), e.motion.begin(), e.motion.end());
      d.identity = 0u;
      d.motionCount = nkeys;
      d.motionT0 = e.t0;
      d.motionT1 = e.t1;
    }
    const float *blo = g.blas.bvh.lo, *bhi = g.blas.bvh.hi;
    float l[3] = {INFINITY, INFINITY, INFINITY}, h[3] = {-INFINITY, -INFINITY, -INFINITY};
    if (g.nprims == 0) {
      l[0] = l[1] = l[2] = h[0] = h[1] = h[2] = 0.f;
    } else if (e.identity && nkeys < 2) {
      for (int k = 0; k < 3; k++) {
        l[k] = blo[k];
        h[k] = bhi[k];
      }
    } else {
      // the box under each key (a blend of two keys maps every point to a
      // blend of its images, inside the union)
      for (int kk = 0; kk < std::max(nkeys, 1); kk++) {
        const float *X = nkeys >= 2 ? e.motion.data() + 12 * kk : e.xfm;
        for (int c = 0; c < 8; c++) {
          const float p[3] = {c & 1 ? bhi[0] : blo[0], c & 2 ? bhi[1] : blo[1], c & 4 ? bhi[2] : blo[2]};
          for (int r = 0; r < 3; r++) {
            const float v = ((X[4 * r] * p[0] + X[4 * r + 1] * p[1]) + X[4 * r + 2] * p[2]) + X[4 * r + 3];
            l[r] = std::fmin(l[r], v);
            h[r] = std::fmax(h[r], v);
          }
        }
      }
      for (int k = 0; k < 3; k++) {
        const float pad = 1e-6f * (std::fabs(l[k]) + std::fabs(h[k])) + 1e-30f;
        l[k] -= pad;
        h[k] += pad;
      }
    }
    lo[i] = make_float4(l[0], l[1], l[2], 0.f);
    hi[i] = make_float4(h[0], h[1], h[2], 0.f);
    for (int k = 0; k < 3; k++) {
      wlo[k] = std::fmin(wlo[k], l[k]);
      whi[k] = std::fmax(whi[k], h[k]);
    }
  }
  for (int k = 0; k < 3; k++) {
    bounds[k] = wlo[k];
    bounds[3 + k] = whi[k];
  }
  if (tlas.nodes) cudaFreeAsync(tlas.nodes, st);
  if (tlas.leafPrim) cudaFreeAsync(tlas.leafPrim, st);
  if (dEntries) cudaFreeAsync(dEntries, st);
  if (dMotion) cudaFreeAsync(dMotion, st);
  tlas = WideBVH{};
  dEntries = nullptr;
  dMotion = nullptr;
  if (!keys.empty()) {
    check(cudaMallocAsync(&dMotion, sizeof(float) * keys.size(), st), "alloc motion keys");
    check(cudaMemcpyAsync(dMotion, keys.data(), sizeof(float) * keys.size(), cudaMemcpyHostToDevice, st),
          "upload motion keys");
    check(cudaStreamSynchronize(st), "sync");  // the host key array goes out of scope
    for (size_t i = 0; i < entries.size(); i++)
      if (he[i].motionCount >= 2) he[i].motionKeys = dMotion + keyOff[i];
  }
  if (!entries.empty()) {
    float4 *dlo, *dhi;
    const size_t n = entries.size();
    check(cudaMallocAsync(&dEntries, sizeof(Entry) * n, st), "alloc entries");
    check(cudaMemcpyAsync(dEntries, he.data(), sizeof(Entry) * n, cudaMemcpyHostToDevice, st), "upload entries");
    check(cudaMallocAsync(&dlo, sizeof(float4) * n, st), "alloc");
    check(cudaMallocAsync(&dhi, sizeof(float4) * n, st), "alloc");
    check(cudaMemcpyAsync(dlo, lo.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, st), "upload");
    check(cudaMemcpyAsync(dhi, hi.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, st), "upload");
    check(buildWide(dlo, dhi, int(n), st, tlas, !dynamic), "TLAS build");
    cudaFreeAsync(dlo, st);
    cudaFreeAsync(dhi, st);
  }
  check(cudaStreamSynchronize(st), "commit");
  committed = true;
}

Scene SceneObj::view() const {
  Scene s;
  s.tlas = tlas.nodes;
  s.tlasLeaf = tlas.leafPrim;
  s.entries = dEntries;
  s.nentries = int(entries.size());
  s.ntlas = entries.empty() ? 0 : tlas.nnodes;
  s.hasUser = 0;
  for (const EntryH &e : entries)
    if ((geoms[e.geom].type != GEOM_TRIANGLES && geoms[e.geom].type != GEOM_SPHERES) || e.motion.size() > 12)
      s.hasUser = 1;
  s.time = 0.f;
  s.status = status;
  s.counters = counters;
  return s;
}

FrameObj::FrameObj(DeviceObj *d, int w, int h, int fmt, uint32_t ch) : dev(d), W(w), H(h), format(fmt), channels(ch) {
  dev->retain();
  const size_t n = size_t(w) * h;
  auto alloc = [&](void **p, size_t bytes) {
    check(cudaMalloc(p, bytes), "cudaMalloc framebuffer");
    check(cudaMemset(*p, 0, bytes), "cudaMemset framebuffer");
  };
  alloc((void **)&color, n * sizeof(float4));
  if (ch & B200_FB_DEPTH) alloc((void **)&depth, n * 4);
  if (ch & B200_FB_VARIANCE) {
    alloc((void **)&variance, n * sizeof(float4));
    alloc((void **)&taskErr, size_t(tasksX()) * tasksY() * 4);
    alloc((void **)&taskActive, size_t(tasksX()) * tasksY());
  }
  if (ch & B200_FB_NORMAL) alloc((void **)&normal, n * sizeof(float3));
  if (ch & B200_FB_ALBEDO) alloc((void **)&albedo, n * sizeof(float3));
  if (ch & (B200_FB_NORMAL | B200_FB_ALBEDO)) alloc((void **)&aux, n * 6 * sizeof(float));
  if (ch & B200_FB_ID_PRIMITIVE) alloc((void **)&primID, n * 4);
  if (ch & B200_FB_ID_OBJECT) alloc((void **)&geomID, n * 4);
  if (ch & B200_FB_ID_INSTANCE) alloc((void **)&instID, n * 4);
  if (fmt != B200_FB_NONE) alloc(&mapped, n * (fmt == B200_FB_RGBA32F ? 16 : 4));
}

FrameObj::~FrameObj() {
  cudaStreamSynchronize(dev->stream);
  for (auto &m : hostMaps) cudaFreeHost(m.second.first);
  if (taskErr) cudaFree(taskErr);
  if (taskActive) cudaFree(taskActive);
  if (aux) cudaFree(aux);
  for (void *p : {(void *)color, (void *)depth, (void *)variance, (void *)normal, (void *)albedo, (void *)primID,
                  (void *)geomID, (void *)instID, mapped})
    if (p) cudaFree(p);
  dev->release();
}

FrameD FrameObj::view() const {
  FrameD f = {};
  f.color = color;
  f.depth = depth;
  f.primID = primID;
  f.geomID = geomID;
  f.instID = instID;
  f.variance = variance;
  f.normal = normal;
  f.albedo = albedo;
  f.aux = aux;
  f.W = W;
  f.H = H;
  f.frameID = frameID;
  f.accumVariance = accumVariance ? 1 : 0;
  f.taskActive = adaptive ? taskActive : nullptr;
  f.tasksX = tasksX();
  return f;
}

void *FrameObj::channel(uint32_t c) const {
  switch (c) {
    case B200_FB_COLOR: return mapped ? mapped : (void *)color;
    case B200_FB_ACCUM: return color;
    case B200_FB_DEPTH: return depth;
    case B200_FB_VARIANCE: return variance;
    case B200_FB_NORMAL: return normal;
    case B200_FB_ALBEDO: return albedo;
    case B200_FB_ID_PRIMITIVE: return primID;
    case B200_FB_ID_OBJECT: return geomID;
    case B200_FB_ID_INSTANCE: return instID;
    default: return nullptr;
  }
}

size_t FrameObj::channelBytes(uint32_t c) const {
  const size_t n = size_t(W) * H;
  switch (c) {
    case B200_FB_COLOR: return n * (format == B200_FB_RGBA8 || format == B200_FB_SRGBA ? 4 : 16);
    case B200_FB_ACCUM:
    case B200_FB_VARIANCE: return n * 16;
    case B200_FB_NORMAL:
    case B200_FB_ALBEDO: return n * 12;
    default: return n * 4;
  }
}

}  // namespace b200

using namespace b200;

namespace {
thread_local std::string g_noDeviceError;

template <class F>
int guarded(DeviceObj *dev, F f) {
  try {
    if (dev) check(cudaSetDevice(dev->dev), "cudaSetDevice");
    f();
    return B200_NO_ERROR;
  } catch (const Error &e) {
    (dev ? dev->lastError : g_noDeviceError) = e.what();
    return e.code;
  } catch (const std::bad_alloc &) {
    (dev ? dev->lastError : g_noDeviceError) = "host out of memory";
    return B200_OUT_OF_MEMORY;
  } catch (const std::exception &e) {
    (dev ? dev->lastError : g_noDeviceError) = e.what();
    return B200_UNKNOWN_ERROR;
  }
}

inline void require(bool c, const char *msg) {
  if (!c) throw Error(B200_INVALID_ARGUMENT, msg);
}
}  // namespace

extern "C" {

int b200_device_create(int cuda_device, b200_device *out) {
  if (!out) return B200_INVALID_ARGUMENT;
  return guarded(nullptr, [&]() {
    int n = 0;
    check(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
    require(cuda_device >= 0 && cuda_device < n, "no such CUDA device");
    *out = reinterpret_cast<b200_device>(new DeviceObj(cuda_device));
  });
}

int b200_device_release(b200_device d) {
  if (!d) return B200_INVALID_ARGUMENT;
  reinterpret_cast<DeviceObj *>(d)->release();
  return B200_NO_ERROR;
}

const char *b200_device_last_error(b200_device d) {
  return d ? reinterpret_cast<DeviceObj *>(d)->lastError.c_str() : g_noDeviceError.c_str();
}

void *b200_device_stream(b200_device d) { return d ? (void *)reinterpret_cast<DeviceObj *>(d)->stream : nullptr; }

int b200_device_sync(b200_device d) {
  if (!d) return B200_INVALID_ARGUMENT;
  DeviceObj *dev = reinterpret_cast<DeviceObj *>(d);
  return guarded(dev, [&]() { check(cudaStreamSynchronize(dev->stream), "sync"); });
}

int b200_kernel_timing(b200_device d, int enable) {
  if (!d) return B200_INVALID_ARGUMENT;
  DeviceObj *dev = reinterpret_cast<DeviceObj *>(d);
  return guarded(dev, [&]() {
    if (enable && !dev->timer) dev->timer = new KernelTimer();
    if (!enable && dev->timer) {
      check(cudaStreamSynchronize(dev->stream), "sync");
      delete dev->timer;
      dev->timer = nullptr;
    }
  });
}

int b200_kernel_timing_read(b200_device d, double *ms, int64_t *launches, int n, int reset) {
  if (!d || n < 0 || (n > 0 && (!ms || !launches))) return B200_INVALID_ARGUMENT;
  DeviceObj *dev = reinterpret_cast<DeviceObj *>(d);
  return guarded(dev, [&]() {
    if (!dev->timer) throw Error(B200_INVALID_OPERATION, "kernel timing is not enabled");
    dev->timer->collect();
    for (int k = 0; k < n; k++) {
      ms[k] = k < KK_COUNT ? dev->timer->ms[k] : 0.0;
      launches[k] = k < KK_COUNT ? dev->timer->launches[k] : 0;
    }
    if (reset)
      for (int k = 0; k < KK_COUNT; k++) {
        dev->timer->ms[k] = 0.0;
        dev->timer->launches[k] = 0;
      }
  });
}

int b200_scene_create(b200_device d, b200_scene *out) {
  if (!d || !out) return B200_INVALID_ARGUMENT;
  DeviceObj *dev = reinterpret_cast<DeviceObj *>(d);
  return guarded(dev, [&]() { *out = reinterpret_cast<b200_scene>(new SceneObj(dev)); });
}

int b200_scene_release(b200_scene s) {
  if (!s) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  cudaSetDevice(sc->dev->dev);
  delete sc;  // may drop the last reference to its device
  return B200_NO_ERROR;
}

int b200_scene_add_mesh(b200_scene s, const float *vertex, int64_t nverts, const uint32_t *index, int64_t ntris,
                        int *geom_out) {
  if (!s) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  return guarded(sc->dev, [&]() {
    require(nverts >= 0 && ntris >= 0 && (nverts == 0 || vertex) && (ntris == 0 || index), "bad mesh arrays");
    require(ntris < (int64_t(1) << 31) && nverts < (int64_t(1) << 31), "mesh too large");
    for (int64_t i = 0; i < 3 * ntris; i++) require(index[i] < uint64_t(nverts), "mesh index out of range");
    GeomObj g;
    g.type = GEOM_TRIANGLES;
    g.nprims = ntris;
    g.nverts = nverts;
    cudaStream_t st = sc->dev->stream;
    check(cudaMallocAsync(&g.dverts, sizeof(float) * 3 * size_t(nverts > 0 ? nverts : 1), st), "alloc vertices");
    check(cudaMallocAsync(&g.dindex, sizeof(uint32_t) * 3 * size_t(ntris > 0 ? ntris : 1), st), "alloc index");
    if (nverts) check(cudaMemcpyAsync(g.dverts, vertex, 12 * size_t(nverts), cudaMemcpyHostToDevice, st), "upload");
    if (ntris) check(cudaMemcpyAsync(g.dindex, index, 12 * size_t(ntris), cudaMemcpyHostToDevice, st), "upload");
    check(cudaStreamSynchronize(st), "upload mesh");
    sc->geoms.push_back(g);
    if (geom_out) *geom_out = int(sc->geoms.size() - 1);
  });
}

int b200_scene_set_mesh_attributes(b200_scene s, int geom, const float *normal, const float *color,
                                   const float *texcoord) {
  if (!s) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  return guarded(sc->dev, [&]() {
    require(geom >= 0 && geom < int(sc->geoms.size()), "bad geometry index");
    GeomObj &g = sc->geoms[geom];
    require(g.type == GEOM_TRIANGLES && g.meshKind == MESH_TRIANGLES,
            "vertex attributes: triangle meshes only (quad meshes, boxes and spheres take none)");
    require(!g.built, "vertex attributes: set them before the scene's commit");
    cudaStream_t st = sc->dev->stream;
    auto upload = [&](float *&dst, const float *src, int comps) {
      if (dst) cudaFreeAsync(dst, st);
      dst = nullptr;
      if (!src || g.nverts == 0) return;
      check(cudaMallocAsync(&dst, sizeof(float) * comps * size_t(g.nverts), st), "alloc vertex attributes");
      check(cudaMemcpyAsync(dst, src, sizeof(float) * comps * size_t(g.nverts), cudaMemcpyHostToDevice, st),
            "upload vertex attributes");
    };
    upload(g.dnormals, normal, 3);
    upload(g.dcolors, color, 4);
    g.colorAlpha = false;
    for (int64_t i = 0; color && i < g.nverts; i++) g.colorAlpha = g.colorAlpha || color[4 * i + 3] != 1.f;
    upload(g.dtexcoords, texcoord, 2);
    check(cudaStreamSynchronize(st), "upload vertex attributes");
    sc->committed = false;
  });
}

// A quad (v0, v1, v2, v3) is the triangle pair (v0, v1, v3), (v2, v3, v1),
// Embree's quad decomposition; both carry the quad's primID.
int b200_scene_add_quad_mesh(b200_scene s, const float *vertex, int64_t nverts, const uint32_t *index,
                             int64_t nquads, int *geom_out) {
  if (!s) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  return guarded(sc->dev, [&]() {
    require(nverts >= 0 && nquads >= 0 && (nverts == 0 || vertex) && (nquads == 0 || index), "bad mesh arrays");
    require(nquads < (int64_t(1) << 30) && nverts < (int64_t(1) << 31), "mesh too large");
    for (int64_t i = 0; i < 4 * nquads; i++) require(index[i] < uint64_t(nverts), "mesh index out of range");
    std::vector<uint32_t> tri(size_t(6 * nquads));
    for (int64_t q = 0; q < nquads; q++) {
      const uint32_t *v = index + 4 * q;
      uint32_t *t = tri.data() + 6 * q;
      t[0] = v[0], t[1] = v[1], t[2] = v[3];
      t[3] = v[2], t[4] = v[3], t[5] = v[1];
    }
    GeomObj g;
    g.type = GEOM_TRIANGLES;
    g.meshKind = MESH_QUADS;
    g.nprims = 2 * nquads;
    cudaStream_t st = sc->dev->stream;
    check(cudaMallocAsync(&g.dverts, sizeof(float) * 3 * size_t(nverts > 0 ? nverts : 1), st), "alloc vertices");
    check(cudaMallocAsync(&g.dindex, sizeof(uint32_t) * 6 * size_t(nquads > 0 ? nquads : 1), st), "alloc index");
    check(cudaMallocAsync(&g.dquad, sizeof(uint32_t) * 4 * size_t(nquads > 0 ? nquads : 1), st), "alloc index");
    if (nverts) check(cudaMemcpyAsync(g.dverts, vertex, 12 * size_t(nverts), cudaMemcpyHostToDevice, st), "upload");
    if (nquads) {
      check(cudaMemcpyAsync(g.dindex, tri.data(), 24 * size_t(nquads), cudaMemcpyHostToDevice, st), "upload");
      check(cudaMemcpyAsync(g.dquad, index, 16 * size_t(nquads), cudaMemcpyHostToDevice, st), "upload");
    }
    check(cudaStreamSynchronize(st), "upload mesh");
    sc->geoms.push_back(g);
    if (geom_out) *geom_out = int(sc->geoms.size() - 1);
  });
}

// Boxes::commit (geometry/Boxes.cpp:33-46): each box3f becomes its 8
// corners and 12 triangles (two per face) carrying the box's primID; a ray
// hits the first face in [tnear, tfar], the exit face when it starts inside,
// as intersectBox + filterIntersectionBoth (common/Intersect.ih:195-223).
int b200_scene_add_boxes(b200_scene s, const float *boxes, int64_t n, int *geom_out) {
  if (!s) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  return guarded(sc->dev, [&]() {
    require(n >= 0 && (n == 0 || boxes) && n < (int64_t(1) << 26), "bad box array");
    std::vector<float> v(size_t(24 * n));
    std::vector<uint32_t> tri(size_t(36 * n));
    // faces as corner quads; corner c = (x: c & 1, y: c >> 1 & 1, z: c >> 2)
    static const int F[6][4] = {{0, 4, 6, 2}, {1, 3, 7, 5}, {0, 1, 5, 4}, {2, 6, 7, 3}, {0, 2, 3, 1}, {4, 5, 7, 6}};
    for (int64_t b = 0; b < n; b++) {
      const float *lo = boxes + 6 * b, *hi = lo + 3;
      for (int c = 0; c < 8; c++) {
        v[size_t(24 * b + 3 * c + 0)] = (c & 1) ? hi[0] : lo[0];
        v[size_t(24 * b + 3 * c + 1)] = (c & 2) ? hi[1] : lo[1];
        v[size_t(24 * b + 3 * c + 2)] = (c & 4) ? hi[2] : lo[2];
      }
      for (int f = 0; f < 6; f++) {
        uint32_t *t = tri.data() + 36 * b + 6 * f;
        const uint32_t o = uint32_t(8 * b);
        t[0] = o + F[f][0], t[1] = o + F[f][1], t[2] = o + F[f][2];
        t[3] = o + F[f][0], t[4] = o + F[f][2], t[5] = o + F[f][3];
      }
    }
    GeomObj g;
    g.type = GEOM_TRIANGLES;
    g.meshKind = MESH_BOXES;
    g.nprims = 12 * n;
    cudaStream_t st = sc->dev->stream;
    check(cudaMallocAsync(&g.dverts, sizeof(float) * 24 * size_t(n > 0 ? n : 1), st), "alloc vertices");
    check(cudaMallocAsync(&g.dindex, sizeof(uint32_t) * 36 * size_t(n > 0 ? n : 1), st), "alloc index");
    if (n) {
      check(cudaMemcpyAsync(g.dverts, v.data(), 96 * size_t(n), cudaMemcpyHostToDevice, st), "upload");
      check(cudaMemcpyAsync(g.dindex, tri.data(), 144 * size_t(n), cudaMemcpyHostToDevice, st), "upload");
    }
    check(cudaStreamSynchronize(st), "upload boxes");
    sc->geoms.push_back(g);
    if (geom_out) *geom_out = int(sc->geoms.size() - 1);
  });
}

int b200_scene_add_spheres(b200_scene s, const float *spheres, int64_t n, int *geom_out) {
  if (!s) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  return guarded(sc->dev, [&]() {
    require(n >= 0 && (n == 0 || spheres) && n < (int64_t(1) << 31), "bad sphere array");
    GeomObj g;
    g.type = GEOM_SPHERES;
    g.nprims = n;
    cudaStream_t st = sc->dev->stream;
    check(cudaMallocAsync(&g.dsph, sizeof(float4) * size_t(n > 0 ? n : 1), st), "alloc spheres");
    if (n) check(cudaMemcpyAsync(g.dsph, spheres, 16 * size_t(n), cudaMemcpyHostToDevice, st), "upload");
    check(cudaStreamSynchronize(st), "upload spheres");
    sc->geoms.push_back(g);
    if (geom_out) *geom_out = int(sc->geoms.size() - 1);
  });
}

int b200_scene_add_discs(b200_scene s, const float *discs, int64_t n, const float *normals, int *geom_out) {
  if (!s) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  return guarded(sc->dev, [&]() {
    require(n >= 0 && (n == 0 || discs) && n < (int64_t(1) << 31), "bad disc array");
    GeomObj g;
    g.type = normals ? GEOM_ORIENTED_DISCS : GEOM_DISCS;
    g.nprims = n;
    cudaStream_t st = sc->dev->stream;
    const size_t m = size_t(n > 0 ? n : 1);
    check(cudaMallocAsync(&g.dsph, sizeof(float4) * m, st), "alloc discs");
    if (n) check(cudaMemcpyAsync(g.dsph, discs, 16 * size_t(n), cudaMemcpyHostToDevice, st), "upload");
    if (normals) {  // interleaved (centre, radius), (normal, 0)
      std::vector<float4> h(2 * size_t(n));
      for (int64_t i = 0; i < n; i++) {
        h[2 * i] = make_float4(discs[4 * i], discs[4 * i + 1], discs[4 * i + 2], discs[4 * i + 3]);
        h[2 * i + 1] = make_float4(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2], 0.f);
      }
      check(cudaMallocAsync(&g.duser, sizeof(float4) * 2 * m, st), "alloc discs");
      if (n) check(cudaMemcpyAsync(g.duser, h.data(), 32 * size_t(n), cudaMemcpyHostToDevice, st), "upload");
    }
    check(cudaStreamSynchronize(st), "upload discs");
    sc->geoms.push_back(g);
    if (geom_out) *geom_out = int(sc->geoms.size() - 1);
  });
}

int b200_scene_add_planes(b200_scene s, const float *coeffs, int64_t n, const float *bounds, int *geom_out) {
  if (!s) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  return guarded(sc->dev, [&]() {
    require(n >= 0 && (n == 0 || coeffs) && n < (int64_t(1) << 31), "bad plane array");
    GeomObj g;
    g.type = GEOM_PLANES;
    g.nprims = n;
    std::vector<float4> h(3 * size_t(n));
    for (int64_t i = 0; i < n; i++) {
      const float *c = coeffs + 4 * i;
      h[3 * i] = make_float4(c[0], c[1], c[2], c[3]);
      if (bounds) {
        const float *b = bounds + 6 * i;
        h[3 * i + 1] = make_float4(b[0], b[1], b[2], 1.f);
        h[3 * i + 2] = make_float4(b[3], b[4], b[5], 0.f);
      } else {
        h[3 * i + 1] = h[3 * i + 2] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    cudaStream_t st = sc->dev->stream;
    check(cudaMallocAsync(&g.duser, sizeof(float4) * 3 * size_t(n > 0 ? n : 1), st), "alloc planes");
    if (n) check(cudaMemcpyAsync(g.duser, h.data(), 48 * size_t(n), cudaMemcpyHostToDevice, st), "upload");
    check(cudaStreamSynchronize(st), "upload planes");
    sc->geoms.push_back(g);
    if (geom_out) *geom_out = int(sc->geoms.size() - 1);
  });
}

int b200_scene_add_instance(b200_scene s, int geom, uint32_t inst_id, uint32_t geom_id, const float *xfm,
                            int material_id) {
  if (!s) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  return guarded(sc->dev, [&]() {
    require(geom >= 0 && size_t(geom) < sc->geoms.size(), "no such geometry");
    EntryH e;
    e.geom = geom;
    e.instID = inst_id;
    e.geomID = geom_id;
    e.identity = xfm == nullptr;
    static const float I[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    std::memcpy(e.xfm, xfm ? xfm : I, sizeof(e.xfm));
    e.material = material_id;
    sc->entries.push_back(e);
    sc->committed = false;
  });
}

int b200_scene_add_instance_motion(b200_scene s, int geom, uint32_t inst_id, uint32_t geom_id, const float *xfms,
                                   int nkeys, float t0, float t1, int material_id) {
  if (!s) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  return guarded(sc->dev, [&]() {
    require(geom >= 0 && size_t(geom) < sc->geoms.size(), "no such geometry");
    require(xfms && nkeys >= 2, "motion blur needs at least two transforms");
    require(std::isfinite(t0) && std::isfinite(t1), "time range is not finite");
    for (int k = 0; k < 12 * nkeys; k++) require(std::isfinite(xfms[k]), "motion transform is not finite");
    EntryH e;
    e.geom = geom;
    e.instID = inst_id;
    e.geomID = geom_id;
    e.identity = false;
    std::memcpy(e.xfm, xfms, sizeof(e.xfm));
    e.material = material_id;
    e.motion.assign(xfms, xfms + 12 * size_t(nkeys));
    e.t0 = t0;
    e.t1 = t1 < t0 ? t0 : t1;  // MotionTransform::readParams: upper raised to lower
    sc->entries.push_back(e);
    sc->committed = false;
  });
}

int b200_scene_set_dynamic(b200_scene s, int dynamic) {
  if (!s) return B200_INVALID_ARGUMENT;
  reinterpret_cast<SceneObj *>(s)->dynamic = dynamic != 0;
  return B200_NO_ERROR;
}

int b200_scene_commit(b200_scene s) {
  if (!s) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  return guarded(sc->dev, [&]() { sc->commit(); });
}

int b200_scene_bounds(b200_scene s, float *box6) {
  if (!s || !box6) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  if (!sc->committed) return B200_INVALID_OPERATION;
  std::memcpy(box6, sc->bounds, sizeof(sc->bounds));
  return B200_NO_ERROR;
}

int b200_scene_stats(b200_scene s, int64_t *st) {
  if (!s || !st) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  st[0] = st[1] = 0;
  for (auto &g : sc->geoms) {
    st[0] += g.blas.bvh.nnodes;
    st[1] += g.nprims;
  }
  st[2] = sc->tlas.nnodes;
  return B200_NO_ERROR;
}

int b200_trace(b200_scene s, const float *rays, int64_t n, int occlusion, float *hit_f, uint32_t *hit_id,
               void *stream) {
  if (!s) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  return guarded(sc->dev, [&]() {
    if (!sc->committed) throw Error(B200_INVALID_OPERATION, "scene not committed");
    require(n >= 0 && (n == 0 || (rays && hit_f && (occlusion || hit_id))), "bad ray arrays");
    require((reinterpret_cast<uintptr_t>(rays) & 15) == 0, "rays must be 16-byte aligned");
    cudaStream_t st = stream ? (cudaStream_t)stream : sc->dev->stream;
    check(launchTrace(sc->view(), reinterpret_cast<const float4 *>(rays), n, occlusion, hit_f, hit_id, st),
          "trace launch");
  });
}

int b200_frame_create(b200_device d, int w, int h, int format, uint32_t channels, b200_frame *out) {
  if (!d || !out) return B200_INVALID_ARGUMENT;
  DeviceObj *dev = reinterpret_cast<DeviceObj *>(d);
  return guarded(dev, [&]() {
    require(w > 0 && h > 0 && int64_t(w) * h < (int64_t(1) << 31), "bad framebuffer size");
    require(format >= B200_FB_NONE && format <= B200_FB_RGBA32F, "unknown framebuffer format");
    *out = reinterpret_cast<b200_frame>(new FrameObj(dev, w, h, format, channels));
  });
}

size_t b200_frame_channel_bytes(b200_frame f, uint32_t c) {
  if (!f) return 0;
  FrameObj *fb = reinterpret_cast<FrameObj *>(f);
  return fb->channel(c) ? fb->channelBytes(c) : 0;
}

void b200_tonemapper_defaults(b200_tonemapper *tm) {
  if (!tm) return;
  tm->exposure = 1.f;
  tm->contrast = 1.6773f;
  tm->shoulder = 0.9714f;
  tm->midIn = 0.18f;
  tm->midOut = 0.18f;
  tm->hdrMax = 11.0785f;
  tm->acesColor = 1;
}

void b200_material_defaults(b200_material *m, int type) {
  if (!m) return;
  std::memset(m, 0, sizeof(*m));
  m->type = type;
  m->opacity = 1.f;
  m->attenuationColor[0] = m->attenuationColor[1] = m->attenuationColor[2] = 1.f;
  m->attenuationDistance = 1.f;
  m->thickness = 1.f;
  m->specular = m->ior = m->diffuse = 1.f;
  m->edgeColor[0] = m->edgeColor[1] = m->edgeColor[2] = 1.f;
  m->specularMetallic = 1;
  switch (type) {
    case B200_MATERIAL_PRINCIPLED:  // Principled::commit, render/materials/Principled.cpp:37-79
    case B200_MATERIAL_OBJ:         // OBJMaterial::commit, OBJ.cpp:28-38
      m->baseColor[0] = m->baseColor[1] = m->baseColor[2] = 0.8f;
      m->ns = 10.f;
      break;
    case B200_MATERIAL_METAL:  // Metal::commit, Metal.cpp:27-31: aluminium (math/spectrum.h RGB_AL_ETA / RGB_AL_K)
      m->eta[0] = 1.47f;
      m->eta[1] = 0.984f;
      m->eta[2] = 0.602f;
      m->k[0] = 7.64f;
      m->k[1] = 6.55f;
      m->k[2] = 5.36f;
      m->roughness = 0.1f;
      break;
    case B200_MATERIAL_GLASS:  // Glass::commit, Glass.cpp:27-38
      m->eta[0] = 1.5f;
      m->eta[1] = 1.f;
      break;
    case B200_MATERIAL_THINGLASS:  // ThinGlass::commit, ThinGlass.cpp:27-33
      m->eta[0] = 1.5f;
      break;
    default:
      break;
  }
}

int b200_frame_set_tonemapper(b200_frame f, const b200_tonemapper *tm) {
  if (!f) return B200_INVALID_ARGUMENT;
  FrameObj *fb = reinterpret_cast<FrameObj *>(f);
  return guarded(fb->dev, [&]() {
    fb->toneMapOn = tm != nullptr;
    if (tm) fb->toneMap = makeToneMap(*tm);
  });
}

int b200_frame_release(b200_frame f) {
  if (!f) return B200_INVALID_ARGUMENT;
  FrameObj *fb = reinterpret_cast<FrameObj *>(f);
  cudaSetDevice(fb->dev->dev);
  delete fb;  // may drop the last reference to its device
  return B200_NO_ERROR;
}

int b200_frame_reset(b200_frame f) {
  if (!f) return B200_INVALID_ARGUMENT;
  FrameObj *fb = reinterpret_cast<FrameObj *>(f);
  fb->frameID = 0;
  fb->taskErrValid = false;
  fb->mtGen.seed(43u);  // FrameBuffer::clear: the coin flips start over
  fb->pickOdd = false;
  return B200_NO_ERROR;
}

int b200_frame_set_variance_threshold(b200_frame f, float threshold) {
  if (!f) return B200_INVALID_ARGUMENT;
  FrameObj *fb = reinterpret_cast<FrameObj *>(f);
  if (!std::isfinite(threshold)) {
    fb->dev->lastError = "varianceThreshold is not finite";
    return B200_INVALID_ARGUMENT;
  }
  fb->errorThreshold = threshold;
  return B200_NO_ERROR;
}

int b200_frame_id(b200_frame f) { return f ? reinterpret_cast<FrameObj *>(f)->frameID : -1; }

void *b200_frame_channel(b200_frame f, uint32_t c) { return f ? reinterpret_cast<FrameObj *>(f)->channel(c) : nullptr; }

int b200_frame_read(b200_frame f, uint32_t c, void *dst, size_t bytes) {
  if (!f || !dst) return B200_INVALID_ARGUMENT;
  FrameObj *fb = reinterpret_cast<FrameObj *>(f);
  return guarded(fb->dev, [&]() {
    void *src = fb->channel(c);
    require(src != nullptr, "channel not present");
    require(bytes >= fb->channelBytes(c), "destination too small");
    check(cudaMemcpyAsync(dst, src, fb->channelBytes(c), cudaMemcpyDeviceToHost, fb->dev->stream), "read");
    check(cudaStreamSynchronize(fb->dev->stream), "read");
  });
}

int b200_frame_map(b200_frame f, uint32_t c, const void **out) {
  if (!f || !out) return B200_INVALID_ARGUMENT;
  FrameObj *fb = reinterpret_cast<FrameObj *>(f);
  return guarded(fb->dev, [&]() {
    void *src = fb->channel(c);
    require(src != nullptr, "channel not present");
    const size_t bytes = fb->channelBytes(c);
    std::pair<void *, size_t> *buf = nullptr;
    for (auto &m : fb->hostMaps)
      if (m.first == c) buf = &m.second;
    if (!buf) {
      fb->hostMaps.push_back({c, {nullptr, 0}});
      buf = &fb->hostMaps.back().second;
    }
    if (buf->second < bytes) {
      if (buf->first) cudaFreeHost(buf->first);
      buf->first = nullptr;
      buf->second = 0;
      check(cudaMallocHost(&buf->first, bytes), "pinned map buffer");
      buf->second = bytes;
    }
    check(cudaMemcpyAsync(buf->first, src, bytes, cudaMemcpyDeviceToHost, fb->dev->stream), "map");
    check(cudaStreamSynchronize(fb->dev->stream), "map");
    *out = buf->first;
  });
}

int b200_render_ao(b200_scene s, const b200_camera_desc *camera, const b200_ao_params *p, b200_frame f, void *stream) {
  if (!s || !camera || !p || !f) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  FrameObj *fb = reinterpret_cast<FrameObj *>(f);
  return guarded(sc->dev, [&]() {
    if (!sc->committed) throw Error(B200_INVALID_OPERATION, "scene not committed");
    require(p->pixelSamples >= 1 && p->aoSamples >= 0, "bad AO parameters");
    require(p->pixelFilter >= B200_PF_POINT && p->pixelFilter <= B200_PF_BLACKMAN_HARRIS, "bad pixel filter");
    require(p->nmaterials >= 0 && (p->nmaterials == 0 || p->materials), "bad material array");
    AOParamsD d = makeAOParams(*p);
    cudaStream_t st = stream ? (cudaStream_t)stream : sc->dev->stream;
    if (p->nmaterials > 0) {  // the surface-colour materials, uploaded when they changed
      const std::vector<ScivisMatD> h = toScivisMats(p->materials, p->nmaterials);
      const bool same = sc->lastAoMats.size() == h.size() &&
                        std::memcmp(sc->lastAoMats.data(), h.data(), sizeof(ScivisMatD) * h.size()) == 0;
      if (!same) {
        if (p->nmaterials > sc->capAoMats) {
          check(cudaStreamSynchronize(st), "sync");
          if (sc->dAoMats) cudaFree(sc->dAoMats);
          sc->dAoMats = nullptr;
          check(cudaMalloc(&sc->dAoMats, sizeof(ScivisMatD) * h.size()), "alloc materials");
          sc->capAoMats = p->nmaterials;
        }
        check(cudaMemcpy(sc->dAoMats, h.data(), sizeof(ScivisMatD) * h.size(), cudaMemcpyHostToDevice),
              "upload materials");
        sc->lastAoMats = h;
      }
      d.mats = sc->dAoMats;
      d.nmats = p->nmaterials;
    }
    fb->beginFrame(p->pixelSamples, st);
    check(launchRenderAO(sc->dev->tables, sc->view(), makeCamera(*camera), sc->dev->filter(p->pixelFilter), d,
                         fb->view(), p->collectStats != 0, st, sc->dev->timer, sc->hasVolume ? &sc->vol : nullptr,
                         d.nmats > 0 || sc->hasAttributes),
          "AO launch");
    fb->frameID++;
    framePostProcess(fb, st);
  });
}

int b200_scene_set_lights(b200_scene s, const b200_light *lights, int n) {
  if (!s) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  return guarded(sc->dev, [&]() {
    require(n >= 0 && (n == 0 || lights), "bad light array");
    std::vector<LightD> h(n);
    for (int i = 0; i < n; i++) {
      const b200_light &L = lights[i];
      require(L.type == B200_LIGHT_QUAD || L.type == B200_LIGHT_AMBIENT || L.type == B200_LIGHT_DISTANT ||
                  L.type == B200_LIGHT_SPHERE || L.type == B200_LIGHT_SPOT,
              "unsupported light type");
      LightD &d = h[i];
      std::memset(&d, 0, sizeof(d));
      d.type = L.type;
      d.visible = L.visible;
      d.radiance = mk(L.color[0] * L.intensity, L.color[1] * L.intensity, L.color[2] * L.intensity);
      if (L.type == B200_LIGHT_QUAD) {
        d.position = mk(L.position[0], L.position[1], L.position[2]);
        d.edge1 = mk(L.edge1[0], L.edge1[1], L.edge1[2]);
        d.edge2 = mk(L.edge2[0], L.edge2[1], L.edge2[2]);
        const V3 nd = cross(d.edge2, d.edge1);
        d.ppdf = 1.f / std::sqrt(dot(nd, nd));
        require(std::isfinite(d.ppdf), "degenerate quad light");
        d.nnormal = mul(nd, d.ppdf);
      } else if (L.type == B200_LIGHT_DISTANT) {
        // DirectionalLight::commit: towards the light, cone of half the angular diameter
        const V3 dir = mk(L.direction[0], L.direction[1], L.direction[2]);
        const float len = std::sqrt(dot(dir, dir));
        require(len > 0.f && std::isfinite(len), "distant light: zero direction");
        d.dir = mul(dir, -1.f / len);
        const float ad = std::fmin(std::fmax(L.angularDiameter, 0.f), 180.f);
        d.cosAngle = std::cos(ad * 0.5f * float(M_PI / 180.0));
        d.conePdf = d.cosAngle < 0.99999988f ? 1.f / (2.f * float(M_PI) * (1.f - d.cosAngle)) : INFINITY;
      } else if (L.type == B200_LIGHT_SPHERE) {
        // PointLight::processIntensityQuantityType (INTENSITY): the radiance of the
        // sphere's visible disk, and the intensity of a point light
        require(L.radius >= 0.f, "sphere light: negative radius");
        d.position = mk(L.position[0], L.position[1], L.position[2]);
        d.radius = L.radius;
        d.intensity = d.radiance;
        d.radiance = L.radius > 0.f ? mul(d.radiance, 1.f / (float(M_PI) * L.radius * L.radius)) : mk(0.f, 0.f, 0.f);
      } else if (L.type == B200_LIGHT_SPOT) {
        // SpotLight::commit / createSh / processIntensityQuantityType (INTENSITY)
        const V3 dir = mk(L.direction[0], L.direction[1], L.direction[2]);
        const float len = std::sqrt(dot(dir, dir));
        require(len > 0.f && std::isfinite(len), "spot light: zero direction");
        d.position = mk(L.position[0], L.position[1], L.position[2]);
        d.dir = mul(dir, 1.f / len);
        const V3 c0 = std::fabs(dir.x) < std::fabs(dir.y) ? mk(0.f, dir.z, dir.y) : mk(dir.z, 0.f, dir.x);
        V3 c90 = cross(c0, d.dir);
        c90 = mul(c90, 1.f / std::sqrt(dot(c90, c90)));
        d.edge1 = cross(d.dir, c90);
        d.edge2 = c90;
        const float opening = std::fmin(std::fmax(L.openingAngle, 0.f), 360.f);
        const float penumbra = std::fmin(std::fmax(L.penumbraAngle, 0.f), 0.5f * opening);
        const float deg = float(M_PI / 180.0);
        d.cosAngle = std::cos(deg * 0.5f * opening);
        d.conePdf = 1.f / (std::cos(deg * (0.5f * opening - penumbra)) - d.cosAngle);
        d.radius = std::fmax(0.f, L.radius);
        d.innerRadius = std::fmin(std::fmax(L.innerRadius, 0.f), 0.999f * d.radius);
        const float ring = float(M_PI) * (d.radius * d.radius - d.innerRadius * d.innerRadius);
        d.ppdf = 1.f / ring;
        d.intensity = d.radiance;
        d.radiance = d.radius > 0.f ? mul(d.radiance, 1.f / ring) : mk(0.f, 0.f, 0.f);
      }
    }
    // uniform light-selection CDF (Distribution1D_create over all-ones)
    std::vector<float> cdf(n, 1.f);
    if (n) {
      float sum = cdf[0];
      for (int i = 1; i < n; i++) cdf[i] = sum += cdf[i];
      const float r = 1.f / sum;
      for (auto &c : cdf) c = c >= sum ? 0x1.000002p+0f : c * r;
    }
    // SciVisData order (render/scivis/SciVisData.cpp:15-58): an ambient light
    // takes slot numVisibleOnly, the light there moves to the end
    std::vector<LightD> sv;
    int visibleOnly = 0;
    V3 aoColor = mk(0.f, 0.f, 0.f);
    for (int i = 0; i < n; i++) {
      if (h[i].type == LIGHT_AMBIENT) {
        if (visibleOnly == int(sv.size())) {
          sv.push_back(h[i]);
        } else {
          sv.push_back(sv[visibleOnly]);
          sv[visibleOnly] = h[i];
        }
        visibleOnly++;
        aoColor = aoColor + h[i].radiance;
      } else {
        sv.push_back(h[i]);
      }
    }
    if (sc->dLights) cudaFree(sc->dLights);
    if (sc->dLightCdf) cudaFree(sc->dLightCdf);
    if (sc->dScivisLights) cudaFree(sc->dScivisLights);
    sc->dLights = nullptr;
    sc->dLightCdf = nullptr;
    sc->dScivisLights = nullptr;
    sc->nLights = n;
    sc->numVisibleOnly = visibleOnly;
    sc->aoColor = aoColor;
    if (n) {
      check(cudaMalloc(&sc->dLights, sizeof(LightD) * n), "alloc lights");
      check(cudaMalloc(&sc->dLightCdf, sizeof(float) * n), "alloc lights");
      check(cudaMalloc(&sc->dScivisLights, sizeof(LightD) * n), "alloc lights");
      check(cudaMemcpy(sc->dLights, h.data(), sizeof(LightD) * n, cudaMemcpyHostToDevice), "upload lights");
      check(cudaMemcpy(sc->dLightCdf, cdf.data(), sizeof(float) * n, cudaMemcpyHostToDevice), "upload lights");
      check(cudaMemcpy(sc->dScivisLights, sv.data(), sizeof(LightD) * n, cudaMemcpyHostToDevice), "upload lights");
    }
  });
}

int b200_render_pt(b200_scene s, const b200_camera_desc *camera, const b200_pt_params *p,
                   const b200_material *materials, int nmaterials, b200_frame f, void *stream) {
  if (!s || !camera || !p || !f) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  FrameObj *fb = reinterpret_cast<FrameObj *>(f);
  return guarded(sc->dev, [&]() {
    if (!sc->committed) throw Error(B200_INVALID_OPERATION, "scene not committed");
    require(p->pixelSamples >= 1 && p->maxPathLength >= 0, "bad path tracer parameters");
    require(p->pixelFilter >= B200_PF_POINT && p->pixelFilter <= B200_PF_BLACKMAN_HARRIS, "bad pixel filter");
    require(nmaterials >= 0 && (nmaterials == 0 || materials), "bad material array");
    cudaStream_t st = stream ? (cudaStream_t)stream : sc->dev->stream;
    uploadMaterials(sc, materials, nmaterials);
    const PtParamsD d =
        makePtParams(*p, sc, materials, nmaterials, sc->transparentMaterials);
    DeviceObj *dev = sc->dev;
    const long long npaths = (long long)fb->W * fb->H * p->pixelSamples;
    ensurePtWorkspace(dev, ptWorkspaceBytes(npaths));
    float *times = sc->hasMotion() ? ensurePtTimes(dev, npaths) : nullptr;
    fb->beginFrame(p->pixelSamples, st);
    check(launchRenderPT(dev->tables, sc->view(), makeCamera(*camera), dev->filter(p->pixelFilter), d,
                         sc->dMaterials, sc->dLights, sc->dLightCdf, dev->albedoTables(), fb->view(),
                         p->collectStats != 0, dev->ptWs, dev->ptWsBytes, st, nullptr, nullptr, nullptr,
                         dev->timer, times),
          "path tracer launch");
    fb->frameID++;
    framePostProcess(fb, st);
  });
}

int b200_scene_set_volume(b200_scene s, const float *data, int nx, int ny, int nz, const float *origin,
                          const float *spacing, const float *color, int ncolor, const float *opacity, int nopacity,
                          const float *valueRange, float densityScale) {
  if (!s) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  return guarded(sc->dev, [&]() {
    require(data && origin && spacing && color && opacity && valueRange, "null volume argument");
    require(nx >= 2 && ny >= 2 && nz >= 2, "volume needs at least 2 vertices per axis");
    require(ncolor >= 1 && nopacity >= 1, "empty transfer function");
    require(spacing[0] > 0.f && spacing[1] > 0.f && spacing[2] > 0.f, "bad grid spacing");
    require(valueRange[1] > valueRange[0], "bad value range");
    for (void *p : {(void *)sc->dVolData, (void *)sc->dTfOpacity, (void *)sc->dTfColor, (void *)sc->dCellEmpty})
      if (p) cudaFree(p);
    sc->dVolData = sc->dTfOpacity = nullptr;
    sc->dTfColor = nullptr;
    sc->dCellEmpty = nullptr;
    sc->hasVolume = false;
    const size_t nvox = size_t(nx) * ny * nz;
    cudaStream_t st = sc->dev->stream;
    struct Staging {
      float *p = nullptr;
      ~Staging() {
        if (p) cudaFree(p);
      }
    } staging;
    check(cudaMalloc(&staging.p, nvox * sizeof(float)), "alloc volume staging");
    float *linear = staging.p;
    check(cudaMalloc(&sc->dVolData, brickedVolumeBytes(nx, ny, nz)), "alloc volume");
    check(cudaMalloc(&sc->dTfColor, ncolor * sizeof(float3)), "alloc transfer function");
    check(cudaMalloc(&sc->dTfOpacity, nopacity * sizeof(float)), "alloc transfer function");
    check(cudaMemcpyAsync(linear, data, nvox * sizeof(float), cudaMemcpyHostToDevice, st), "upload volume");
    check(cudaMemcpyAsync(sc->dTfColor, color, ncolor * sizeof(float3), cudaMemcpyHostToDevice, st), "upload tf");
    check(cudaMemcpyAsync(sc->dTfOpacity, opacity, nopacity * sizeof(float), cudaMemcpyHostToDevice, st),
          "upload tf");
    VolumeD &v = sc->vol;
    v.data = sc->dVolData;
    v.nx = nx;
    v.ny = ny;
    v.nz = nz;
    v.bx = (nx + VOL_BRICK - 1) / VOL_BRICK;
    v.by = (ny + VOL_BRICK - 1) / VOL_BRICK;
    v.bz = (nz + VOL_BRICK - 1) / VOL_BRICK;
    v.origin = mk(origin[0], origin[1], origin[2]);
    v.spacing = mk(spacing[0], spacing[1], spacing[2]);
    v.cx = std::max(1, (nx - 1 + 15) / 16);
    v.cy = std::max(1, (ny - 1 + 15) / 16);
    v.cz = std::max(1, (nz - 1 + 15) / 16);
    v.tfColor = sc->dTfColor;
    v.tfOpacity = sc->dTfOpacity;
    v.ncolor = ncolor;
    v.nopacity = nopacity;
    v.vlo = valueRange[0];
    v.vhi = valueRange[1];
    v.densityScale = densityScale;
    v.gradientShadingScale = sc->gradientShadingScale;
    v.identity = sc->volIdentity ? 1 : 0;
    v.rcp = sc->volRcp;
    check(brickVolume(v, linear, sc->dVolData, st), "brick volume");
    check(cudaStreamSynchronize(st), "brick volume");
    check(cudaMalloc(&sc->dCellEmpty, size_t(v.cx) * v.cy * v.cz), "alloc macrocells");
    check(buildMacrocells(v, sc->dCellEmpty, st), "macrocells");
    v.cellEmpty = sc->dCellEmpty;
    check(cudaStreamSynchronize(st), "volume commit");
    sc->hasVolume = true;
  });
}

int b200_scene_set_volume_transform(b200_scene s, const float *xfm) {
  if (!s) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  return guarded(sc->dev, [&]() {
    sc->volIdentity = xfm == nullptr;
    if (xfm) {
      for (int k = 0; k < 12; k++) require(std::isfinite(xfm[k]), "volume transform is not finite");
      rcpAffine(xfm, sc->volRcp.m);
      for (int k = 0; k < 12; k++) require(std::isfinite(sc->volRcp.m[k]), "volume transform is singular");
    }
    sc->vol.identity = sc->volIdentity ? 1 : 0;
    sc->vol.rcp = sc->volRcp;
  });
}

int b200_scene_set_volume_gradient_shading(b200_scene s, float gradientShadingScale) {
  if (!s) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  return guarded(sc->dev, [&]() {
    require(std::isfinite(gradientShadingScale), "gradientShadingScale is not finite");
    sc->gradientShadingScale = gradientShadingScale;
    sc->vol.gradientShadingScale = gradientShadingScale;
  });
}

int b200_render_scivis(b200_scene s, const b200_camera_desc *camera, const b200_scivis_params *p,
                       const b200_scivis_material *materials, int nmaterials, b200_frame f, void *stream) {
  if (!s || !camera || !p || !f) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  FrameObj *fb = reinterpret_cast<FrameObj *>(f);
  return guarded(sc->dev, [&]() {
    const bool surfaces = sc->committed && sc->tlas.nnodes > 0;
    if (!surfaces && !sc->hasVolume) throw Error(B200_INVALID_OPERATION, "world has no surfaces and no volume");
    require(p->pixelSamples >= 1 && p->volumeSamplingRate > 0.f, "bad scivis parameters");
    require(p->pixelFilter >= B200_PF_POINT && p->pixelFilter <= B200_PF_BLACKMAN_HARRIS, "bad pixel filter");
    require(p->aoSamples >= 0, "bad scivis parameters");
    require(nmaterials >= 0 && (nmaterials == 0 || materials), "bad material array");
    ScivisParamsD d;
    d.spp = p->pixelSamples;
    d.samplingRate = p->volumeSamplingRate;
    for (int k = 0; k < 4; k++) d.bg[k] = p->backgroundColor[k];
    d.backplate = textureDevice(p->backplate);
    d.maxDepth = textureDevice(p->maxDepth);
    d.mipBiasFactor = std::pow(2.f, p->mipMapBias);
    cudaStream_t st = stream ? (cudaStream_t)stream : sc->dev->stream;
    fb->beginFrame(p->pixelSamples, st);
    if (!surfaces && !(sc->vol.gradientShadingScale > 0.f) && !p->backplate && !p->maxDepth) {
      check(launchRenderScivisVolume(sc->dev->tables, sc->view(), sc->vol, makeCamera(*camera),
                                     sc->dev->filter(p->pixelFilter), d, fb->view(), p->collectStats != 0, st,
                                     sc->dev->timer),
            "scivis launch");
    } else {
      // (compared as device records: a texture made again at a reused host
      // address still has a new device descriptor)
      std::vector<ScivisMatD> h = toScivisMats(materials, nmaterials);
      const bool same = int(sc->lastScivisMats.size()) == nmaterials &&
                        (nmaterials == 0 ||
                         std::memcmp(sc->lastScivisMats.data(), h.data(), sizeof(ScivisMatD) * nmaterials) == 0);
      // opaque: no obj material lets light through (d < 1, tf, a map with
      // alpha) and no vertex colour has alpha < 1
      bool opaque = !sc->colorAlpha, mapped = false;
      for (int i = 0; i < nmaterials; i++) {
        const b200_scivis_material &m = materials[i];
        if (m.isObj && !(m.d == 1.f && m.tf[0] * m.d == 0.f && m.tf[1] * m.d == 0.f && m.tf[2] * m.d == 0.f))
          opaque = false;
        if (m.isObj && m.kdMap) {
          mapped = true;
          if (textureHasAlpha(m.kdMap)) opaque = false;
        }
      }
      if (!same) {
        if (nmaterials > sc->capScivisMats) {
          if (sc->dScivisMats) cudaFree(sc->dScivisMats);
          sc->dScivisMats = nullptr;
          check(cudaMalloc(&sc->dScivisMats, sizeof(ScivisMatD) * nmaterials), "alloc materials");
          sc->capScivisMats = nmaterials;
        }
        if (nmaterials)
          check(cudaMemcpy(sc->dScivisMats, h.data(), sizeof(ScivisMatD) * nmaterials, cudaMemcpyHostToDevice),
                "upload materials");
        sc->lastScivisMats = h;
      }
      ScivisSurfD S;
      S.mats = sc->dScivisMats;
      S.nmats = nmaterials;
      S.lights = sc->dScivisLights;
      S.nlights = sc->nLights;
      S.numVisibleOnly = sc->numVisibleOnly;
      S.aoColor = sc->aoColor;
      S.shadows = p->shadows != 0;
      S.visibleLights = p->visibleLights != 0;
      S.aoSamples = p->aoSamples;
      S.aoRadius = p->aoDistance;
      S.minContribution = p->minContribution;
      S.hasVolume = sc->hasVolume;
      S.hasSurfaces = surfaces;
      S.opaqueShadows = opaque && !sc->hasVolume;
      S.attrs = sc->hasAttributes || mapped;
      check(launchRenderScivisSurfaces(sc->dev->tables, sc->view(), sc->vol, makeCamera(*camera),
                                       sc->dev->filter(p->pixelFilter), d, S, fb->view(), p->collectStats != 0, st,
                                       sc->dev->timer),
            "scivis launch");
    }
    fb->frameID++;
    framePostProcess(fb, st);
  });
}

namespace {
struct EventObj {
  DeviceObj *dev;
  cudaEvent_t ev = nullptr;
};
}  // namespace

int b200_event_record(b200_device d, b200_event *out) {
  if (!d || !out) return B200_INVALID_ARGUMENT;
  DeviceObj *dev = reinterpret_cast<DeviceObj *>(d);
  return guarded(dev, [&]() {
    EventObj *e = new EventObj{dev};
    if (cudaEventCreate(&e->ev) != cudaSuccess || cudaEventRecord(e->ev, dev->stream) != cudaSuccess) {
      if (e->ev) cudaEventDestroy(e->ev);
      delete e;
      throw Error(B200_UNKNOWN_ERROR, "cannot record a CUDA event");
    }
    dev->retain();
    *out = reinterpret_cast<b200_event>(e);
  });
}

int b200_event_query(b200_event h) {
  if (!h) return -B200_INVALID_ARGUMENT;
  EventObj *e = reinterpret_cast<EventObj *>(h);
  cudaSetDevice(e->dev->dev);
  const cudaError_t r = cudaEventQuery(e->ev);
  if (r == cudaSuccess) return 1;
  if (r == cudaErrorNotReady) return 0;
  e->dev->lastError = std::string("event query: ") + cudaGetErrorString(r);
  return -B200_UNKNOWN_ERROR;
}

int b200_event_wait(b200_event h) {
  if (!h) return B200_INVALID_ARGUMENT;
  EventObj *e = reinterpret_cast<EventObj *>(h);
  return guarded(e->dev, [&]() { check(cudaEventSynchronize(e->ev), "event wait"); });
}

float b200_event_elapsed_ms(b200_event a, b200_event b) {
  if (!a || !b) return 0.f;
  EventObj *ea = reinterpret_cast<EventObj *>(a), *eb = reinterpret_cast<EventObj *>(b);
  float ms = 0.f;
  cudaSetDevice(ea->dev->dev);
  if (cudaEventElapsedTime(&ms, ea->ev, eb->ev) != cudaSuccess) return 0.f;
  return ms;
}

int b200_event_release(b200_event h) {
  if (!h) return B200_INVALID_ARGUMENT;
  EventObj *e = reinterpret_cast<EventObj *>(h);
  cudaSetDevice(e->dev->dev);
  cudaEventDestroy(e->ev);
  DeviceObj *dev = e->dev;
  delete e;
  dev->release();
  return B200_NO_ERROR;
}

int b200_pick(b200_scene s, const b200_camera_desc *camera, float sx, float sy, b200_pick_result *res) {
  if (!s || !camera || !res) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  return guarded(sc->dev, [&]() {
    require(sc->committed, "scene not committed");
    DeviceObj *dev = sc->dev;
    check(launchPick(sc->view(), makeCamera(*camera), sx, sy, dev->pickBuf, dev->stream), "pick launch");
    uint32_t w[8];
    check(cudaMemcpyAsync(w, dev->pickBuf, sizeof(w), cudaMemcpyDeviceToHost, dev->stream), "pick read");
    check(cudaStreamSynchronize(dev->stream), "pick sync");
    res->hasHit = int(w[0]);
    memcpy(res->worldPosition, w + 1, 12);
    res->instID = w[4];
    res->geomID = w[5];
    res->primID = w[6];
  });
}

int b200_scene_counters(b200_scene s, int64_t *out4, int reset) {
  if (!s || !out4) return B200_INVALID_ARGUMENT;
  SceneObj *sc = reinterpret_cast<SceneObj *>(s);
  return guarded(sc->dev, [&]() {
    unsigned long long c[4];
    check(cudaStreamSynchronize(sc->dev->stream), "sync");
    check(cudaMemcpy(c, sc->counters, sizeof(c), cudaMemcpyDeviceToHost), "read counters");
    for (int k = 0; k < 4; k++) out4[k] = int64_t(c[k]);
    if (reset) check(cudaMemset(sc->counters, 0, sizeof(c)), "reset counters");
  });
}

}  // extern "C"
