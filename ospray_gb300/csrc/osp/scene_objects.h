// Scene-object types of the b200 OSPRay device (the types registered by the
// reference's module_cpu that the GB300 path implements:
// geometry/registration.cpp "mesh", "sphere"; camera "perspective";
// render/registration.cpp "ao", "scivis", "pathtracer", "principled",
// "obj"; lights/registration.cpp "quad", "ambient"; texture/registration
// "texture2d"; volume
// "structuredRegular"; transferFunction "piecewiseLinear";
// fb/registration.cpp "tonemapper").  commit() reads the parameters each
// type understands (names and defaults of the reference's ::commit methods,
// cited per type) into host state; the world commit uploads it.
#pragma once

#include <vector>

#include "objects.h"

namespace b200osp {

class B200Device;

struct SceneObj : Obj {
  using Obj::Obj;
  virtual void commit(B200Device &) {}
};

// Texture2D::commit (texture/Texture2D.cpp:55-135): "data" (2D), "format",
// "filter", "wrapMode"; the MIP chain is generated on the device
struct TextureObj : SceneObj {
  using SceneObj::SceneObj;
  ~TextureObj() override;
  b200_texture tex = nullptr;
  void commit(B200Device &) override;
};

// Mesh::commit (geometry/Mesh.cpp:37-204), Spheres::commit (geometry/Spheres.cpp:46-106)
struct GeometryObj : SceneObj {
  using SceneObj::SceneObj;
  std::vector<float> verts;     // mesh: xyz per vertex
  // mesh: "vertex.normal" (3), "vertex.color" (4; vec3f gets alpha 1) and
  // "vertex.texcoord" (2) per vertex, empty when absent
  std::vector<float> normals, colors, texcoords;
  std::vector<uint32_t> index;  // mesh: 3 per triangle, or 4 per quad when quads
  bool quads = false;           // mesh with a vec4ui "index"
  std::vector<float> spheres;   // sphere: xyzr per sphere
  std::vector<float> boxes;     // box: lower xyz, upper xyz per box
  int sphereType = OSP_SPHERE;  // sphere: "type" (OSP_SPHERE, OSP_DISC, OSP_ORIENTED_DISC)
  std::vector<float> discNormals;  // sphere of OSP_ORIENTED_DISC: "sphere.normal", xyz per disc
  std::vector<float> planes, planeBounds;  // plane: "plane.coefficients" (4), "plane.bounds" (6) or empty
  void commit(B200Device &) override;
  void bounds(float lo[3], float hi[3]) const;
};

// Principled::commit (render/materials/Principled.cpp:37-79) and
// OBJMaterial::commit (render/materials/OBJ.cpp) on the parameters the
// GB300 path tracer evaluates
struct MaterialObj : SceneObj {
  using SceneObj::SceneObj;
  Ref<TextureObj> colorMap;      // principled "map_baseColor" / obj "map_kd"
  b200_material mat = {};        // as the path tracer reads it (baseColorMap: see colorMapHandle)
  b200_texture colorMapHandle() const { return colorMap ? colorMap->tex : nullptr; }
  // the SciVis / AO record with the obj map_kd as of now
  b200_scivis_material scivis() const {
    b200_scivis_material m = sv;
    m.kdMap = sv.isObj ? colorMapHandle() : nullptr;
    return m;
  }
  b200_scivis_material sv = {};  // as the SciVis renderer reads it
  void commit(B200Device &) override;
};

// GeometricModel::commit (geometry/GeometricModel.cpp)
struct GeometricModelObj : SceneObj {
  using SceneObj::SceneObj;
  Ref<GeometryObj> geometry;  // from the "geometry" parameter
  Ref<MaterialObj> material;  // an object material, or
  int materialIndex = -1;           // an index into the renderer's material list
  void commit(B200Device &) override;
};

// StructuredRegular (volume/Volume.cpp:60-222)
struct VolumeObj : SceneObj {
  using SceneObj::SceneObj;
  std::vector<float> voxels;
  int dims[3] = {0, 0, 0};
  float origin[3] = {0, 0, 0}, spacing[3] = {1, 1, 1};
  void commit(B200Device &) override;
};

// LinearTransferFunction::commit (volume/transferFunction/LinearTransferFunction.cpp:22-155)
struct TransferFunctionObj : SceneObj {
  using SceneObj::SceneObj;
  std::vector<float> color, opacity;
  float range[2] = {0.f, 1.f};
  void commit(B200Device &) override;
};

// VolumetricModel::commit (volume/VolumetricModel.cpp:30-82)
struct VolumetricModelObj : SceneObj {
  using SceneObj::SceneObj;
  Ref<VolumeObj> volume;
  Ref<TransferFunctionObj> tf;
  float densityScale = 1.f;
  float gradientShadingScale = 0.f;
  void commit(B200Device &) override;
};

// Group::commit (common/Group.cpp:69-143)
struct GroupObj : SceneObj {
  using SceneObj::SceneObj;
  std::vector<Ref<GeometricModelObj>> models;    // from the "geometry" data parameter
  std::vector<Ref<VolumetricModelObj>> volumes;  // from the "volume" data parameter
  void commit(B200Device &) override;
};

// Instance::commit (common/Instance.cpp)
struct InstanceObj : SceneObj {
  using SceneObj::SceneObj;
  Ref<GroupObj> group;
  float xfm[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};  // row-major 3x4
  bool identity = true;
  std::vector<float> motion;  // "motion.transform" keys, row-major 3x4 each (>= 2: motion blur)
  float time[2] = {0.f, 1.f};  // "time" of the keys
  void commit(B200Device &) override;
};

// QuadLight::commit (lights/QuadLight.cpp:68-108), AmbientLight::commit (lights/AmbientLight.cpp:40-60)
struct LightObj : SceneObj {
  using SceneObj::SceneObj;
  b200_light light = {};
  void commit(B200Device &) override;
};

// World::commit (common/World.cpp:70-188): the b200 scene is built here
struct WorldObj : SceneObj {
  using SceneObj::SceneObj;
  ~WorldObj() override;
  b200_scene scene = nullptr;
  std::vector<Ref<InstanceObj>> instances;      // index = instID of hits
  std::vector<Ref<MaterialObj>> objectMaterials;  // ids 0..K-1; renderer list from K on
  bool hasGeometry = false, hasVolume = false;
  void commit(B200Device &) override;
};

// PerspectiveCamera::commit (camera/PerspectiveCamera.cpp:30-117)
struct CameraObj : SceneObj {
  using SceneObj::SceneObj;
  b200_camera_desc desc = {};
  void commit(B200Device &) override;
};

// Renderer::commit (render/Renderer.cpp:38-92) + AORenderer / PathTracer / SciVis ::commit
struct RendererObj : SceneObj {
  using SceneObj::SceneObj;
  b200_ao_params ao = {};
  b200_pt_params pt = {};
  b200_scivis_params scivis = {};
  std::vector<Ref<MaterialObj>> materials;  // the "material" list
  Ref<TextureObj> backplate;                // "map_backplate"
  Ref<TextureObj> maxDepth;                 // "map_maxDepth"
  float mipMapBias = 0.f;                   // "mipMapBias"
  float varianceThreshold = 0.f;
  void commit(B200Device &) override;
};

// ToneMapper::commit (fb/frame_ops/ToneMapper.cpp:16-51)
struct ImageOpObj : SceneObj {
  using SceneObj::SceneObj;
  b200_tonemapper tm = {};
  void commit(B200Device &) override;
};

// LocalFrameBuffer (fb/LocalFB.cpp)
struct FrameBufferObj : SceneObj {
  FrameBufferObj(B200Device &dev, int w, int h, OSPFrameBufferFormat fmt, uint32_t channels);
  ~FrameBufferObj() override;
  b200_frame fb = nullptr;
  int width, height;
  OSPFrameBufferFormat format;
  uint32_t channels;
  std::map<const void *, std::vector<unsigned char>> mapped;  // heap copies (a channel mapped twice)
  std::map<const void *, uint32_t> pinnedMapped;  // b200_frame_map buffers in use: pointer -> channel
  float errorThreshold = 0.f;  // varianceThreshold of the last renderer
  void commit(B200Device &) override;
};

// an OSPFuture: completion events around one frame on the device stream; it
// holds references on what the frame reads until it is released
struct FutureObj : Obj {
  FutureObj() : Obj(OSP_FUTURE, "frame") {}
  ~FutureObj() override;
  b200_event start = nullptr, end = nullptr;
  std::vector<Obj *> held;
};

}  // namespace b200osp
