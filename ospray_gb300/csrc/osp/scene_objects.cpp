// commit() of the b200 OSPRay device's scene objects.
#include "scene_objects.h"

#include <cmath>
#include <map>

#include "b200_device.h"

namespace b200osp {

namespace {
const float kZero3[3] = {0.f, 0.f, 0.f};
const float kOne3[3] = {1.f, 1.f, 1.f};

template <class T>
std::vector<Ref<T>> objectList(DataObj *d, OSPDataType kind, const char *what) {
  std::vector<Ref<T>> out;
  if (!d) return out;
  if (d->elem != kind) throw Error(OSP_INVALID_ARGUMENT, std::string(what) + ": data array of the wrong object type");
  for (uint64_t i = 0; i < d->count(); i++) {
    Obj *o = d->object(i);
    if (!o) throw Error(OSP_INVALID_ARGUMENT, std::string(what) + ": null element");
    out.push_back(Ref<T>(static_cast<T *>(o)));
  }
  return out;
}

float length3(const float v[3]) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }
}  // namespace

// ---------------------------------------------------------------- textures

TextureObj::~TextureObj() {
  if (tex) b200_texture_release(tex);
}

void TextureObj::commit(B200Device &dev) {
  DataObj *d = getData("data");
  if (!d || d->n[2] > 1)
    throw Error(OSP_INVALID_ARGUMENT, "texture2d must have 2D 'data' array using the first two dimensions");
  const int format = getInt("format", OSP_TEXTURE_FORMAT_INVALID);
  if (format == OSP_TEXTURE_FORMAT_INVALID) throw Error(OSP_INVALID_ARGUMENT, "texture2d: invalid 'format'");
  const int filter = getInt("filter", OSP_TEXTURE_FILTER_LINEAR);
  int wrap[2] = {OSP_TEXTURE_WRAP_REPEAT, OSP_TEXTURE_WRAP_REPEAT};
  const Param *wp = find("wrapMode");
  if (wp && (wp->type == OSP_VEC2UI || wp->type == OSP_VEC2I)) {
    std::memcpy(wrap, wp->bytes.data(), 8);
  } else if (wp) {
    wrap[0] = wrap[1] = getInt("wrapMode", OSP_TEXTURE_WRAP_REPEAT);
  }
  static const int texel[16] = {4, 4, 16, 3, 3, 12, 1, 4, 1, 2, 2, 8, 6, 4, 2, 8};
  if (format < 0 || format > 15)
    throw Error(OSP_INVALID_ARGUMENT, "texture2d: 'format' not supported by the b200 device (half-float formats)");
  if (size_t(texel[format]) != sizeOfType(d->elem))
    throw Error(OSP_INVALID_ARGUMENT, "texture2d: 'format' does not match the type of 'data'");
  const auto bytes = d->compact();
  b200_texture t = nullptr;
  dev.check(b200_texture_create(dev.handle(), int(d->n[0]), int(d->n[1]), format, filter, wrap[0], wrap[1], 1,
                                bytes.data(), &t));
  if (tex) b200_texture_release(tex);
  tex = t;
}

namespace {
// a texture parameter (the object itself, as OSPRay's getParamObject<Texture>)
Ref<TextureObj> textureParam(Obj &o, const char *name) {
  return Ref<TextureObj>(static_cast<TextureObj *>(o.getObject(name, OSP_TEXTURE)));
}
}  // namespace

// ---------------------------------------------------------------- geometry

void GeometryObj::commit(B200Device &dev) {
  verts.clear();
  normals.clear();
  colors.clear();
  texcoords.clear();
  index.clear();
  spheres.clear();
  boxes.clear();
  if (type == "mesh") {
    DataObj *v = getData("vertex.position");
    DataObj *ix = getData("index");
    if (!v || v->elem != OSP_VEC3F) throw Error(OSP_INVALID_ARGUMENT, "mesh: 'vertex.position' must be vec3f data");
    const auto vb = v->compact();
    verts.resize(v->count() * 3);
    std::memcpy(verts.data(), vb.data(), vb.size());
    if (!ix) throw Error(OSP_INVALID_ARGUMENT, "mesh: 'index' data is required");
    // Mesh::commit (geometry/Mesh.cpp:114-145): vec3ui triangles or vec4ui quads
    quads = ix->elem == OSP_VEC4UI || ix->elem == OSP_VEC4I;
    if (!quads && ix->elem != OSP_VEC3UI && ix->elem != OSP_VEC3I)
      throw Error(OSP_INVALID_ARGUMENT, "mesh: 'index' must be vec3ui or vec4ui data");
    const auto ib = ix->compact();
    index.resize(ix->count() * (quads ? 4 : 3));
    std::memcpy(index.data(), ib.data(), ib.size());
    for (uint32_t i : index)
      if (i >= v->count()) throw Error(OSP_INVALID_ARGUMENT, "mesh: index out of range of 'vertex.position'");
    // per-vertex attributes (Mesh::commit geometry/Mesh.cpp:37-113)
    auto attr = [&](const char *name, OSPDataType want, std::vector<float> &dst, int comps) {
      DataObj *a = getData(name);
      if (!a) return;
      const bool rgb = comps == 4 && a->elem == OSP_VEC3F;
      if (a->elem != want && !rgb)
        throw Error(OSP_INVALID_ARGUMENT, std::string("mesh: '") + name + "' has an unsupported element type");
      if (a->count() != v->count())
        throw Error(OSP_INVALID_ARGUMENT, std::string("mesh: '") + name + "' must have one element per vertex");
      const auto b = a->compact();
      dst.resize(a->count() * comps);
      if (rgb) {
        for (uint64_t i = 0; i < a->count(); i++) {
          std::memcpy(&dst[4 * i], b.data() + 12 * i, 12);
          dst[4 * i + 3] = 1.f;
        }
      } else {
        std::memcpy(dst.data(), b.data(), b.size());
      }
    };
    attr("vertex.normal", OSP_VEC3F, normals, 3);
    attr("vertex.color", OSP_VEC4F, colors, 4);
    attr("vertex.texcoord", OSP_VEC2F, texcoords, 2);
    if (quads && (!normals.empty() || !colors.empty() || !texcoords.empty())) {
      dev.warn("mesh: per-vertex attributes of quad meshes are not supported by the b200 device; ignored");
      normals.clear();
      colors.clear();
      texcoords.clear();
    }
  } else if (type == "plane") {
    // Planes::commit (geometry/Planes.cpp): "plane.coefficients" vec4f, optional "plane.bounds" box3f
    DataObj *c = getData("plane.coefficients");
    if (!c || c->elem != OSP_VEC4F) throw Error(OSP_INVALID_ARGUMENT, "plane: 'plane.coefficients' must be vec4f data");
    const auto cb = c->compact();
    planes.resize(c->count() * 4);
    std::memcpy(planes.data(), cb.data(), cb.size());
    planeBounds.clear();
    if (DataObj *b = getData("plane.bounds")) {
      if (b->elem != OSP_BOX3F || b->count() != c->count())
        throw Error(OSP_INVALID_ARGUMENT, "plane: 'plane.bounds' must be box3f data, one per plane");
      const auto bb = b->compact();
      planeBounds.resize(b->count() * 6);
      std::memcpy(planeBounds.data(), bb.data(), bb.size());
    }
  } else if (type == "box") {
    // Boxes::commit (geometry/Boxes.cpp:33-46): "box" data of box3f
    DataObj *b = getData("box");
    if (!b || b->elem != OSP_BOX3F) throw Error(OSP_INVALID_ARGUMENT, "box: 'box' must be box3f data");
    const auto bb = b->compact();
    boxes.resize(b->count() * 6);
    std::memcpy(boxes.data(), bb.data(), bb.size());
  } else {  // sphere
    DataObj *p = getData("sphere.position");
    if (!p || p->elem != OSP_VEC3F) throw Error(OSP_INVALID_ARGUMENT, "sphere: 'sphere.position' must be vec3f data");
    DataObj *r = getData("sphere.radius");
    const float radius = getFloat("radius", 0.01f);
    std::vector<float> radii;
    if (r) {
      radii = r->toFloats();
      if (radii.size() != p->count()) throw Error(OSP_INVALID_ARGUMENT, "sphere: 'sphere.radius' size differs");
    }
    const auto pb = p->compact();
    spheres.resize(p->count() * 4);
    for (uint64_t i = 0; i < p->count(); i++) {
      std::memcpy(&spheres[4 * i], pb.data() + 12 * i, 12);
      spheres[4 * i + 3] = r ? radii[i] : radius;
    }
    // Spheres::commit "type" (geometry/Spheres.cpp:43-54): spheres, ray-facing
    // discs, or discs oriented by "sphere.normal"
    sphereType = getInt("type", OSP_SPHERE);
    if (sphereType != OSP_SPHERE && sphereType != OSP_DISC && sphereType != OSP_ORIENTED_DISC)
      throw Error(OSP_INVALID_ARGUMENT, "sphere: unknown 'type'");
    discNormals.clear();
    if (sphereType == OSP_ORIENTED_DISC) {
      DataObj *nd = getData("sphere.normal");
      if (!nd || nd->elem != OSP_VEC3F || nd->count() != p->count())
        throw Error(OSP_INVALID_ARGUMENT, "sphere: oriented discs need 'sphere.normal' vec3f data, one per disc");
      const auto nb = nd->compact();
      discNormals.resize(nd->count() * 3);
      std::memcpy(discNormals.data(), nb.data(), nb.size());
    }
  }
}

void GeometryObj::bounds(float lo[3], float hi[3]) const {
  for (int k = 0; k < 3; k++) {
    lo[k] = INFINITY;
    hi[k] = -INFINITY;
  }
  if (type == "mesh") {
    for (uint32_t i : index)
      for (int k = 0; k < 3; k++) {
        lo[k] = std::fmin(lo[k], verts[3 * i + k]);
        hi[k] = std::fmax(hi[k], verts[3 * i + k]);
      }
  } else if (type == "plane") {  // Planes_bounds: the boxes clipped to +-1e18, or +-1e18
    for (size_t i = 0; 4 * i < planes.size(); i++)
      for (int k = 0; k < 3; k++) {
        lo[k] = std::fmin(lo[k], planeBounds.empty() ? -1e18f : std::fmax(planeBounds[6 * i + k], -1e18f));
        hi[k] = std::fmax(hi[k], planeBounds.empty() ? 1e18f : std::fmin(planeBounds[6 * i + 3 + k], 1e18f));
      }
  } else if (type == "box") {
    for (size_t i = 0; 6 * i < boxes.size(); i++)
      for (int k = 0; k < 3; k++) {
        lo[k] = std::fmin(lo[k], boxes[6 * i + k]);
        hi[k] = std::fmax(hi[k], boxes[6 * i + 3 + k]);
      }
  } else {
    for (size_t i = 0; 4 * i < spheres.size(); i++)
      for (int k = 0; k < 3; k++) {
        lo[k] = std::fmin(lo[k], spheres[4 * i + k] - spheres[4 * i + 3]);
        hi[k] = std::fmax(hi[k], spheres[4 * i + k] + spheres[4 * i + 3]);
      }
  }
}

// ---------------------------------------------------------------- materials

void MaterialObj::commit(B200Device &dev) {
  sv = {};
  static const float kOne3[3] = {1.f, 1.f, 1.f};
  if (type == "principled") {  // Principled::commit, render/materials/Principled.cpp:37-79
    b200_material_defaults(&mat, B200_MATERIAL_PRINCIPLED);
    const float def[3] = {0.8f, 0.8f, 0.8f};
    getVec3("baseColor", mat.baseColor, def);
    colorMap = textureParam(*this, "map_baseColor");
    mat.roughness = getFloat("roughness", 0.f);
    mat.metallic = getFloat("metallic", 0.f);
    mat.opacity = getFloat("opacity", 1.f);
    mat.specular = getFloat("specular", 1.f);
    mat.ior = getFloat("ior", 1.f);
    mat.diffuse = getFloat("diffuse", 1.f);
    getVec3("edgeColor", mat.edgeColor, kOne3);
    mat.specularMetallic = getBool("specularMetallic", true) ? 1 : 0;
    // parameters of the principled model the GB300 path tracer does not
    // evaluate: accepted at their defaults, reported otherwise
    struct Def {
      const char *name;
      float value;
    };
    static const Def fixed[] = {{"transmission", 0.f}, {"anisotropy", 0.f}, {"coat", 0.f},
                                {"sheen", 0.f},        {"backlight", 0.f},  {"thin", 0.f}};
    for (const Def &d : fixed)
      if (has(d.name) && getFloat(d.name, d.value) != d.value)
        dev.warn(std::string("principled material: '") + d.name + "' other than " + std::to_string(d.value) +
                 " is not supported by the b200 device; using the default");
  } else if (type == "obj") {  // OBJMaterial::commit, render/materials/OBJ.cpp:28-65
    b200_material_defaults(&mat, B200_MATERIAL_OBJ);
    const float def[3] = {0.8f, 0.8f, 0.8f};
    float kd[3], ks[3], tf[3];
    getVec3("kd", kd, def);
    getVec3("ks", ks, kZero3);
    getVec3("tf", tf, kZero3);
    colorMap = textureParam(*this, "map_kd");
    if (!colorMap) colorMap = textureParam(*this, "map_Kd");
    // the path tracer gets the raw parameters (the device scales kd + ks + tf
    // down to 1 itself); SciVis reads the scaled ones
    for (int k = 0; k < 3; k++) {
      mat.baseColor[k] = kd[k];
      mat.ks[k] = ks[k];
      mat.tf[k] = tf[k];
    }
    mat.ns = getFloat("ns", 10.f);
    mat.opacity = getFloat("d", 1.f);
    float total = 0.f;
    for (int k = 0; k < 3; k++) total = std::max(total, kd[k] + ks[k] + tf[k]);
    if (total > 1.f)
      for (int k = 0; k < 3; k++) {
        kd[k] /= total;
        ks[k] /= total;
        tf[k] /= total;
      }
    sv.isObj = 1;
    for (int k = 0; k < 3; k++) {
      sv.kd[k] = kd[k];
      sv.ks[k] = ks[k];
      sv.tf[k] = tf[k];
    }
    sv.ns = mat.ns;
    sv.d = mat.opacity;
  } else if (type == "metal") {  // Metal::commit, render/materials/Metal.cpp:27-70 (RGB eta / k)
    b200_material_defaults(&mat, B200_MATERIAL_METAL);
    const float e0[3] = {mat.eta[0], mat.eta[1], mat.eta[2]}, k0[3] = {mat.k[0], mat.k[1], mat.k[2]};
    getVec3("eta", mat.eta, e0);
    getVec3("k", mat.k, k0);
    mat.roughness = getFloat("roughness", 0.1f);
    if (has("ior")) dev.warn("metal material: spectral 'ior' data is not supported by the b200 device; using eta / k");
  } else if (type == "glass") {  // Glass::commit, render/materials/Glass.cpp:27-50
    b200_material_defaults(&mat, B200_MATERIAL_GLASS);
    mat.eta[0] = getFloat("etaInside", getFloat("eta", 1.5f));
    mat.eta[1] = getFloat("etaOutside", 1.f);
    float c[3];
    getVec3("attenuationColorInside", c, kOne3);
    if (!has("attenuationColorInside")) getVec3("attenuationColor", c, kOne3);
    for (int k = 0; k < 3; k++) mat.attenuationColor[k] = c[k];
    mat.attenuationDistance = getFloat("attenuationDistance", 1.f);
    if (has("attenuationColorOutside"))
      dev.warn("glass material: 'attenuationColorOutside' is not supported by the b200 device; using 1");
  } else {  // thinGlass: ThinGlass::commit, render/materials/ThinGlass.cpp:27-45
    b200_material_defaults(&mat, B200_MATERIAL_THINGLASS);
    mat.eta[0] = getFloat("eta", 1.5f);
    getVec3("attenuationColor", mat.attenuationColor, kOne3);
    mat.attenuationDistance = getFloat("attenuationDistance", 1.f);
    mat.thickness = getFloat("thickness", 1.f);
  }
  if (type != "principled" && type != "obj") colorMap = Ref<TextureObj>();
  mat.baseColorMap = nullptr;  // set from colorMap at each render
}

void GeometricModelObj::commit(B200Device &) {
  geometry = Ref<GeometryObj>(static_cast<GeometryObj *>(getObject("geometry", OSP_GEOMETRY)));
  if (!geometry) throw Error(OSP_INVALID_ARGUMENT, "geometric model without geometry");
  material = Ref<MaterialObj>();
  materialIndex = -1;
  const Param *p = find("material");
  if (p) {
    if (p->obj && p->obj->kind == OSP_MATERIAL) {
      material = Ref<MaterialObj>(static_cast<MaterialObj *>(p->obj));
    } else if (p->obj && p->obj->kind == OSP_DATA) {
      DataObj *d = static_cast<DataObj *>(p->obj);
      if (d->count() != 1)
        throw Error(OSP_INVALID_ARGUMENT, "geometric model: per-primitive materials are not supported by the b200 device");
      if (d->elem == OSP_MATERIAL)
        material = Ref<MaterialObj>(static_cast<MaterialObj *>(d->object(0)));
      else if (d->elem == OSP_UINT || d->elem == OSP_INT)
        std::memcpy(&materialIndex, d->at(0), 4);
      else
        throw Error(OSP_INVALID_ARGUMENT, "geometric model: 'material' data of an unsupported type");
    } else {
      materialIndex = getInt("material", -1);
    }
  }
}

// ---------------------------------------------------------------- volumes

void VolumeObj::commit(B200Device &dev) {
  DataObj *d = getData("data");
  if (!d) throw Error(OSP_INVALID_ARGUMENT, "structuredRegular volume: 'data' is required");
  for (int k = 0; k < 3; k++) dims[k] = int(d->n[k]);
  voxels = d->toFloats();
  getVec3("gridOrigin", origin, kZero3);
  getVec3("gridSpacing", spacing, kOne3);
  if (getBool("cellCentered", false))
    dev.warn("structuredRegular volume: cell-centred grids are sampled vertex-centred by the b200 device");
}

void TransferFunctionObj::commit(B200Device &) {
  DataObj *c = getData("color");
  DataObj *o = getData("opacity");
  if (!c || c->elem != OSP_VEC3F) throw Error(OSP_INVALID_ARGUMENT, "piecewiseLinear: 'color' must be vec3f data");
  if (!o) throw Error(OSP_INVALID_ARGUMENT, "piecewiseLinear: 'opacity' data is required");
  const auto cb = c->compact();
  color.resize(c->count() * 3);
  std::memcpy(color.data(), cb.data(), cb.size());
  opacity = o->toFloats();
  if (!getBox1("value", range) && !getBox1("valueRange", range)) {
    range[0] = 0.f;
    range[1] = 1.f;
  }
}

void VolumetricModelObj::commit(B200Device &dev) {
  volume = Ref<VolumeObj>(static_cast<VolumeObj *>(getObject("volume", OSP_VOLUME)));
  tf = Ref<TransferFunctionObj>(static_cast<TransferFunctionObj *>(getObject("transferFunction", OSP_TRANSFER_FUNCTION)));
  if (!volume || !tf) throw Error(OSP_INVALID_ARGUMENT, "volumetric model needs 'volume' and 'transferFunction'");
  densityScale = getFloat("densityScale", 1.f);
  gradientShadingScale = getFloat("gradientShadingScale", 0.f);
}

// ---------------------------------------------------------------- hierarchy

void GroupObj::commit(B200Device &dev) {
  models = objectList<GeometricModelObj>(getData("geometry"), OSP_GEOMETRIC_MODEL, "group 'geometry'");
  volumes = objectList<VolumetricModelObj>(getData("volume"), OSP_VOLUMETRIC_MODEL, "group 'volume'");
  if (getData("light")) dev.warn("group lights are not supported by the b200 device; put lights on the world");
}

void InstanceObj::commit(B200Device &) {
  group = Ref<GroupObj>(static_cast<GroupObj *>(getObject("group", OSP_GROUP)));
  if (!group) throw Error(OSP_INVALID_ARGUMENT, "instance without a group");
  float a[12];  // OSP_AFFINE3F: l.vx, l.vy, l.vz, p
  identity = true;
  if (getAffine("transform", a) || getAffine("xfm", a)) {
    for (int r = 0; r < 3; r++) {
      xfm[4 * r + 0] = a[0 + r];
      xfm[4 * r + 1] = a[3 + r];
      xfm[4 * r + 2] = a[6 + r];
      xfm[4 * r + 3] = a[9 + r];
    }
    static const float id[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    identity = std::memcmp(xfm, id, sizeof(id)) == 0;
  }
  // MotionTransform::readParams (common/MotionTransform.cpp:10-66): key
  // transforms "motion.transform" over "time" (default [0, 1]); one key is
  // the plain transform.  The quaternion form (motion.scale / rotation /
  // translation) is not supported.
  motion.clear();
  if (DataObj *m = getData("motion.transform")) {
    if (m->elem != OSP_AFFINE3F) throw Error(OSP_INVALID_ARGUMENT, "instance: 'motion.transform' must be affine3f data");
    const auto mb = m->compact();
    const uint64_t nk = m->count();
    std::vector<float> keys(12 * nk);
    for (uint64_t k = 0; k < nk; k++) {
      float a2[12];
      std::memcpy(a2, mb.data() + 48 * k, 48);
      for (int r = 0; r < 3; r++) {
        keys[12 * k + 4 * r + 0] = a2[0 + r];
        keys[12 * k + 4 * r + 1] = a2[3 + r];
        keys[12 * k + 4 * r + 2] = a2[6 + r];
        keys[12 * k + 4 * r + 3] = a2[9 + r];
      }
    }
    if (nk == 1) {
      std::memcpy(xfm, keys.data(), sizeof(xfm));
      static const float id[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
      identity = std::memcmp(xfm, id, sizeof(id)) == 0;
    } else if (nk > 1) {
      motion = keys;
      identity = false;
      time[0] = 0.f;
      time[1] = 1.f;
      getBox1("time", time);
    }
  }
  if (has("motion.scale") || has("motion.rotation") || has("motion.translation") || has("motion.pivot"))
    throw Error(OSP_INVALID_ARGUMENT, "instance: quaternion motion blur is not supported by the b200 device");
}

void LightObj::commit(B200Device &dev) {
  light.visible = getBool("visible", true) ? 1 : 0;
  getVec3("color", light.color, kOne3);
  light.intensity = getFloat("intensity", 1.f);
  if (type == "quad") {
    light.type = B200_LIGHT_QUAD;
    const float e1[3] = {1.f, 0.f, 0.f}, e2[3] = {0.f, 1.f, 0.f};
    getVec3("position", light.position, kZero3);
    getVec3("edge1", light.edge1, e1);
    getVec3("edge2", light.edge2, e2);
    const int q = getInt("intensityQuantity", OSP_INTENSITY_QUANTITY_RADIANCE);
    const float c[3] = {light.edge1[1] * light.edge2[2] - light.edge1[2] * light.edge2[1],
                        light.edge1[2] * light.edge2[0] - light.edge1[0] * light.edge2[2],
                        light.edge1[0] * light.edge2[1] - light.edge1[1] * light.edge2[0]};
    const float area = length3(c);
    if (q == OSP_INTENSITY_QUANTITY_INTENSITY) {
      light.intensity /= area;
    } else if (q == OSP_INTENSITY_QUANTITY_POWER) {
      light.intensity /= float(M_PI) * area;
    } else if (q != OSP_INTENSITY_QUANTITY_RADIANCE) {
      dev.warn("quad light: unsupported 'intensityQuantity' value");
      light.intensity = 0.f;
    }
  } else if (type == "distant") {
    // DirectionalLight::commit / processIntensityQuantityType (lights/DirectionalLight.cpp:77-105)
    light.type = B200_LIGHT_DISTANT;
    const float dz[3] = {0.f, 0.f, 1.f};
    getVec3("direction", light.direction, dz);
    light.angularDiameter = std::fmin(std::fmax(getFloat("angularDiameter", 0.f), 0.f), 180.f);
    const int q = getInt("intensityQuantity", OSP_INTENSITY_QUANTITY_IRRADIANCE);
    if (q == OSP_INTENSITY_QUANTITY_RADIANCE) {
      const float cosAngle = std::cos(light.angularDiameter * 0.5f * float(M_PI / 180.0));
      light.intensity *= 2.f * float(M_PI) * (1.f - cosAngle);
    } else if (q != OSP_INTENSITY_QUANTITY_IRRADIANCE) {
      dev.warn("distant light: unsupported 'intensityQuantity' value");
      light.intensity = 0.f;
    }
  } else if (type == "sphere") {
    // PointLight::commit / processIntensityQuantityType (lights/PointLight.cpp:68-121):
    // the b200 light takes the radiative intensity
    light.type = B200_LIGHT_SPHERE;
    getVec3("position", light.position, kZero3);
    light.radius = getFloat("radius", 0.f);
    const int q = getInt("intensityQuantity", OSP_INTENSITY_QUANTITY_INTENSITY);
    if (q == OSP_INTENSITY_QUANTITY_POWER) {
      light.intensity /= 4.f * float(M_PI);
    } else if (q == OSP_INTENSITY_QUANTITY_RADIANCE && light.radius > 0.f) {
      light.intensity *= float(M_PI) * light.radius * light.radius;  // radiance x visible disk area
    } else if (q != OSP_INTENSITY_QUANTITY_INTENSITY) {
      dev.warn("sphere light: unsupported 'intensityQuantity' value");
      light.intensity = 0.f;
    }
  } else if (type == "spot") {
    // SpotLight::commit / processIntensityQuantityType (lights/SpotLight.cpp:76-140)
    light.type = B200_LIGHT_SPOT;
    const float dz[3] = {0.f, 0.f, 1.f};
    getVec3("position", light.position, kZero3);
    getVec3("direction", light.direction, dz);
    light.openingAngle = getFloat("openingAngle", 180.f);
    light.penumbraAngle = getFloat("penumbraAngle", 5.f);
    light.radius = std::fmax(0.f, getFloat("radius", 0.f));
    light.innerRadius = std::fmin(std::fmax(getFloat("innerRadius", 0.f), 0.f), 0.999f * light.radius);
    const int q = getInt("intensityQuantity", OSP_INTENSITY_QUANTITY_INTENSITY);
    const float opening = std::fmin(std::fmax(light.openingAngle, 0.f), 360.f);
    const float c = std::cos(float(M_PI) * opening * 0.5f / 180.f);
    const float capCosInt = float(M_PI) * (1.f - c * c);
    const float ring = float(M_PI) * (light.radius * light.radius - light.innerRadius * light.innerRadius);
    if (q == OSP_INTENSITY_QUANTITY_POWER) {
      light.intensity /= capCosInt;
    } else if (q == OSP_INTENSITY_QUANTITY_RADIANCE && light.radius > 0.f) {
      light.intensity *= ring;  // radiance x ring area
    } else if (q != OSP_INTENSITY_QUANTITY_INTENSITY) {
      dev.warn("spot light: unsupported 'intensityQuantity' value");
      light.intensity = 0.f;
    }
  } else {  // ambient
    light.type = B200_LIGHT_AMBIENT;
    const int q = getInt("intensityQuantity", OSP_INTENSITY_QUANTITY_RADIANCE);
    if (q == OSP_INTENSITY_QUANTITY_IRRADIANCE) {
      light.intensity /= float(M_PI);
    } else if (q != OSP_INTENSITY_QUANTITY_RADIANCE) {
      dev.warn("ambient light: unsupported 'intensityQuantity' value");
      light.intensity = 0.f;
    }
  }
}

// ---------------------------------------------------------------- world

WorldObj::~WorldObj() {
  if (scene) b200_scene_release(scene);
}

void WorldObj::commit(B200Device &dev) {
  instances = objectList<InstanceObj>(getData("instance"), OSP_INSTANCE, "world 'instance'");
  const std::vector<Ref<LightObj>> lights = objectList<LightObj>(getData("light"), OSP_LIGHT, "world 'light'");

  b200_scene s = nullptr;
  dev.check(b200_scene_create(dev.handle(), &s));
  dev.check(b200_scene_set_dynamic(s, getBool("dynamicScene", false) ? 1 : 0));
  try {
    std::map<GeometryObj *, int> geomIndex;
    std::map<MaterialObj *, int> matIndex;
    objectMaterials.clear();
    for (const auto &inst : instances)
      for (const auto &m : inst->group->models)
        if (m->material && !matIndex.count(m->material.get())) {
          matIndex[m->material.get()] = int(objectMaterials.size());
          objectMaterials.push_back(m->material);
        }
    const int K = int(objectMaterials.size());
    hasGeometry = hasVolume = false;
    for (size_t i = 0; i < instances.size(); i++) {
      InstanceObj *inst = instances[i].get();
      for (size_t j = 0; j < inst->group->models.size(); j++) {
        GeometricModelObj *m = inst->group->models[j].get();
        GeometryObj *g = m->geometry.get();
        auto it = geomIndex.find(g);
        int gi;
        if (it == geomIndex.end()) {
          if (g->type == "mesh" && g->quads)
            dev.check(b200_scene_add_quad_mesh(s, g->verts.data(), int64_t(g->verts.size() / 3), g->index.data(),
                                               int64_t(g->index.size() / 4), &gi));
          else if (g->type == "mesh") {
            dev.check(b200_scene_add_mesh(s, g->verts.data(), int64_t(g->verts.size() / 3), g->index.data(),
                                          int64_t(g->index.size() / 3), &gi));
            if (!g->normals.empty() || !g->colors.empty() || !g->texcoords.empty())
              dev.check(b200_scene_set_mesh_attributes(s, gi, g->normals.empty() ? nullptr : g->normals.data(),
                                                       g->colors.empty() ? nullptr : g->colors.data(),
                                                       g->texcoords.empty() ? nullptr : g->texcoords.data()));
          }
          else if (g->type == "box")
            dev.check(b200_scene_add_boxes(s, g->boxes.data(), int64_t(g->boxes.size() / 6), &gi));
          else if (g->type == "plane")
            dev.check(b200_scene_add_planes(s, g->planes.data(), int64_t(g->planes.size() / 4),
                                            g->planeBounds.empty() ? nullptr : g->planeBounds.data(), &gi));
          else if (g->sphereType != OSP_SPHERE)
            dev.check(b200_scene_add_discs(s, g->spheres.data(), int64_t(g->spheres.size() / 4),
                                           g->sphereType == OSP_ORIENTED_DISC ? g->discNormals.data() : nullptr, &gi));
          else
            dev.check(b200_scene_add_spheres(s, g->spheres.data(), int64_t(g->spheres.size() / 4), &gi));
          geomIndex[g] = gi;
        } else {
          gi = it->second;
        }
        const int mat =
            m->material ? matIndex[m->material.get()] : (m->materialIndex >= 0 ? K + m->materialIndex : -1);
        if (inst->motion.size() >= 24)
          dev.check(b200_scene_add_instance_motion(s, gi, uint32_t(i), uint32_t(j), inst->motion.data(),
                                                   int(inst->motion.size() / 12), inst->time[0], inst->time[1], mat));
        else
          dev.check(
              b200_scene_add_instance(s, gi, uint32_t(i), uint32_t(j), inst->identity ? nullptr : inst->xfm, mat));
        hasGeometry = true;
      }
      for (const auto &vmr : inst->group->volumes) {
        VolumetricModelObj *vm = vmr.get();
        if (hasVolume) {
          dev.warn("world: the b200 device renders one volumetric model per world; further ones are ignored");
          continue;
        }
        VolumeObj *v = vm->volume.get();
        TransferFunctionObj *tf = vm->tf.get();
        dev.check(b200_scene_set_volume(s, v->voxels.data(), v->dims[0], v->dims[1], v->dims[2], v->origin,
                                        v->spacing, tf->color.data(), int(tf->color.size() / 3), tf->opacity.data(),
                                        int(tf->opacity.size()), tf->range, vm->densityScale));
        dev.check(b200_scene_set_volume_gradient_shading(s, vm->gradientShadingScale));
        dev.check(b200_scene_set_volume_transform(s, inst->identity ? nullptr : inst->xfm));
        hasVolume = true;
      }
    }
    std::vector<b200_light> L;
    for (const auto &l : lights) L.push_back(l->light);
    dev.check(b200_scene_set_lights(s, L.data(), int(L.size())));
    dev.check(b200_scene_commit(s));
  } catch (...) {
    b200_scene_release(s);
    throw;
  }
  if (scene) b200_scene_release(scene);
  scene = s;
}

// ---------------------------------------------------------------- camera, renderer, image ops

void CameraObj::commit(B200Device &dev) {
  const float dir[3] = {0.f, 0.f, 1.f}, up[3] = {0.f, 1.f, 0.f};
  getVec3("position", desc.position, kZero3);
  getVec3("direction", desc.direction, dir);
  getVec3("up", desc.up, up);
  desc.fovy = getFloat("fovy", 60.f);
  desc.aspect = getFloat("aspect", 1.f);
  desc.nearClip = getFloat("nearClip", 1e-6f);
  // OrthographicCamera::commit "height"; PanoramicCamera (equirectangular)
  desc.type = type == "orthographic" ? B200_CAMERA_ORTHOGRAPHIC
                                     : (type == "panoramic" ? B200_CAMERA_PANORAMIC : B200_CAMERA_PERSPECTIVE);
  desc.height = getFloat("height", 1.f);
  // Camera::commit (camera/Camera.cpp:44-52): shutter, shutter type, rolling duration
  desc.shutter[0] = desc.shutter[1] = 0.5f;
  getBox1("shutter", desc.shutter);
  desc.shutterType = getInt("shutterType", OSP_SHUTTER_GLOBAL);
  if (desc.shutterType < OSP_SHUTTER_GLOBAL || desc.shutterType > OSP_SHUTTER_ROLLING_UP)
    throw Error(OSP_INVALID_ARGUMENT, "camera: unknown 'shutterType'");
  desc.rollingShutterDuration = getFloat("rollingShutterDuration", 0.f);
  if (getData("motion.transform") || has("motion.scale") || has("motion.rotation") || has("motion.translation"))
    dev.warn("camera: camera motion blur is not supported by the b200 device");
  // PerspectiveCamera::commit (camera/PerspectiveCamera.cpp:30-36): depth of field, architectural
  desc.apertureRadius = getFloat("apertureRadius", 0.f);
  desc.focusDistance = getFloat("focusDistance", 1.f);
  desc.architectural = getBool("architectural", false) ? 1 : 0;
  if (desc.apertureRadius != 0.f && desc.type != B200_CAMERA_PERSPECTIVE)
    dev.warn("camera: depth of field is supported by the perspective camera only");
  // Camera::commit (camera/Camera.cpp:42-43): the sub-image, a vec2f pair
  desc.imageStart[0] = desc.imageStart[1] = 0.f;
  desc.imageEnd[0] = desc.imageEnd[1] = 1.f;
  getBox1("imageStart", desc.imageStart);
  getBox1("imageEnd", desc.imageEnd);
  // PerspectiveCamera::commit / PanoramicCamera::commit: stereo
  desc.stereoMode = getInt("stereoMode", OSP_STEREO_NONE);
  if (desc.stereoMode < OSP_STEREO_NONE || desc.stereoMode > OSP_STEREO_TOP_BOTTOM)
    throw Error(OSP_INVALID_ARGUMENT, "camera: unknown 'stereoMode'");
  desc.interpupillaryDistance = getFloat("interpupillaryDistance", 0.0635f);
  if (desc.stereoMode != OSP_STEREO_NONE && desc.type == B200_CAMERA_ORTHOGRAPHIC)
    dev.warn("camera: the orthographic camera has no stereo mode");
}

void RendererObj::commit(B200Device &) {
  const int spp = std::max(1, getInt("pixelSamples", 1));
  const float bg0[4] = {0.f, 0.f, 0.f, 0.f};
  float bg[4];
  getColor4("backgroundColor", bg, bg0);
  const int pf = getInt("pixelFilter", OSP_PIXELFILTER_GAUSS);
  varianceThreshold = getFloat("varianceThreshold", 0.f);
  const int maxDepth = std::max(0, getInt("maxPathLength", 20));
  const float minContribution = getFloat("minContribution", 0.001f);
  materials = objectList<MaterialObj>(getData("material"), OSP_MATERIAL, "renderer 'material'");
  backplate = textureParam(*this, "map_backplate");
  this->maxDepth = textureParam(*this, "map_maxDepth");
  mipMapBias = getFloat("mipMapBias", 0.f);
  if (type == "ao") {
    ao.pixelSamples = spp;
    ao.aoSamples = getInt("aoSamples", 1);
    ao.aoDistance = getFloat("aoDistance", getFloat("aoRadius", 1e20f));
    ao.aoIntensity = getFloat("aoIntensity", 1.f);
    std::memcpy(ao.backgroundColor, bg, 16);
    ao.pixelFilter = pf;
    ao.collectStats = 0;
    ao.volumeSamplingRate = getFloat("volumeSamplingRate", 1.f);  // AORenderer::commit
  } else if (type == "pathtracer") {
    pt.pixelSamples = spp;
    pt.maxPathLength = maxDepth;
    pt.roulettePathLength = getInt("roulettePathLength", 5);
    pt.maxScatteringEvents = getInt("maxScatteringEvents", 20);
    pt.lightSamples = getInt("lightSamples", -1);
    pt.limitIndirectLightSamples = getBool("limitIndirectLightSamples", true) ? 1 : 0;
    pt.minContribution = minContribution;
    pt.maxContribution = getFloat("maxContribution", INFINITY);
    std::memcpy(pt.backgroundColor, bg, 16);
    pt.pixelFilter = pf;
    pt.collectStats = 0;
    pt.mipMapBias = mipMapBias;
  } else {  // scivis (SciVis::commit, render/scivis/SciVis.cpp:27-36)
    scivis.pixelSamples = spp;
    scivis.volumeSamplingRate = getFloat("volumeSamplingRate", 1.f);
    std::memcpy(scivis.backgroundColor, bg, 16);
    scivis.pixelFilter = pf;
    scivis.collectStats = 0;
    scivis.shadows = getBool("shadows", false) ? 1 : 0;
    scivis.visibleLights = getBool("visibleLights", false) ? 1 : 0;
    scivis.aoSamples = std::max(0, getInt("aoSamples", 0));
    scivis.aoDistance = getFloat("aoDistance", 1e20f);
    scivis.minContribution = minContribution;
  }
}

void ImageOpObj::commit(B200Device &) {
  b200_tonemapper d;
  b200_tonemapper_defaults(&d);
  tm.exposure = getFloat("exposure", d.exposure);
  tm.contrast = getFloat("contrast", d.contrast);
  tm.shoulder = getFloat("shoulder", d.shoulder);
  tm.midIn = getFloat("midIn", d.midIn);
  tm.midOut = getFloat("midOut", d.midOut);
  tm.hdrMax = getFloat("hdrMax", d.hdrMax);
  tm.acesColor = getBool("acesColor", d.acesColor != 0) ? 1 : 0;
}

// ---------------------------------------------------------------- framebuffer

FrameBufferObj::FrameBufferObj(B200Device &dev, int w, int h, OSPFrameBufferFormat fmt, uint32_t ch)
    : SceneObj(OSP_FRAMEBUFFER, "local"), width(w), height(h), format(fmt), channels(ch) {
  uint32_t b200ch = B200_FB_COLOR;  // the colour buffer always exists on the device
  if (ch & OSP_FB_DEPTH) b200ch |= B200_FB_DEPTH;
  if (ch & OSP_FB_ACCUM) b200ch |= B200_FB_ACCUM;
  if (ch & OSP_FB_VARIANCE) b200ch |= B200_FB_VARIANCE;
  if (ch & OSP_FB_NORMAL) b200ch |= B200_FB_NORMAL;
  if (ch & OSP_FB_ALBEDO) b200ch |= B200_FB_ALBEDO;
  if (ch & OSP_FB_ID_PRIMITIVE) b200ch |= B200_FB_ID_PRIMITIVE;
  if (ch & OSP_FB_ID_OBJECT) b200ch |= B200_FB_ID_OBJECT;
  if (ch & OSP_FB_ID_INSTANCE) b200ch |= B200_FB_ID_INSTANCE;
  dev.check(b200_frame_create(dev.handle(), w, h, int(fmt), b200ch, &fb));
}

FrameBufferObj::~FrameBufferObj() {
  if (fb) b200_frame_release(fb);
}

void FrameBufferObj::commit(B200Device &dev) {
  DataObj *ops = getData("imageOperation");
  const b200_tonemapper *tm = nullptr;
  if (ops) {
    if (ops->elem != OSP_IMAGE_OPERATION)
      throw Error(OSP_INVALID_ARGUMENT, "framebuffer 'imageOperation' must be image-operation data");
    if (ops->count() > 1) dev.warn("framebuffer: the b200 device applies one tonemapper; further operations ignored");
    tm = &static_cast<ImageOpObj *>(ops->object(0))->tm;
  }
  dev.check(b200_frame_set_tonemapper(fb, tm));
}

FutureObj::~FutureObj() {
  if (end) {
    b200_event_wait(end);
    b200_event_release(end);
  }
  if (start) b200_event_release(start);
  for (Obj *o : held) o->release();
}

}  // namespace b200osp
