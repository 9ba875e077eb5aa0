// Parameter staging and data arrays of the b200 OSPRay device.
#include "objects.h"

#include <cmath>

namespace b200osp {

bool isObjectType(OSPDataType t) { return t >= OSP_OBJECT && t <= OSP_WORLD; }

// bytes of one element of each OSPDataType (ospray/common/OSPCommon.cpp
// sizeOf): vectors are N scalars, boxes 2 N, linear/affine their matrices
size_t sizeOfType(OSPDataType t) {
  if (isObjectType(t) || t == OSP_DEVICE || t == OSP_VOID_PTR) return sizeof(void *);
  if (t == OSP_BOOL) return 1;
  if (t == OSP_STRING) return sizeof(char *);
  struct Range {
    int base;
    size_t scalar;
  };
  static const Range ranges[] = {{OSP_CHAR, 1},  {OSP_UCHAR, 1}, {OSP_SHORT, 2}, {OSP_USHORT, 2},
                                 {OSP_INT, 4},   {OSP_UINT, 4},  {OSP_LONG, 8},  {OSP_ULONG, 8},
                                 {OSP_HALF, 2},  {OSP_FLOAT, 4}, {OSP_DOUBLE, 8}};
  for (const Range &r : ranges)
    if (int(t) >= r.base && int(t) < r.base + 4) return r.scalar * size_t(int(t) - r.base + 1);
  if (t >= OSP_BOX1I && t <= OSP_BOX4I) return 8 * size_t(int(t) - OSP_BOX1I + 1);
  if (t >= OSP_BOX1F && t <= OSP_BOX4F) return 8 * size_t(int(t) - OSP_BOX1F + 1);
  switch (t) {
    case OSP_LINEAR2F: return 16;
    case OSP_LINEAR3F: return 36;
    case OSP_AFFINE2F: return 24;
    case OSP_AFFINE3F: return 48;
    case OSP_QUATF: return 16;
    default: break;
  }
  throw Error(OSP_INVALID_ARGUMENT, "unknown OSPDataType " + std::to_string(int(t)));
}

const char *kindName(OSPDataType k) {
  switch (k) {
    case OSP_DATA: return "data";
    case OSP_CAMERA: return "camera";
    case OSP_FRAMEBUFFER: return "framebuffer";
    case OSP_FUTURE: return "future";
    case OSP_GEOMETRIC_MODEL: return "geometric model";
    case OSP_GEOMETRY: return "geometry";
    case OSP_GROUP: return "group";
    case OSP_IMAGE_OPERATION: return "image operation";
    case OSP_INSTANCE: return "instance";
    case OSP_LIGHT: return "light";
    case OSP_MATERIAL: return "material";
    case OSP_RENDERER: return "renderer";
    case OSP_TEXTURE: return "texture";
    case OSP_TRANSFER_FUNCTION: return "transfer function";
    case OSP_VOLUME: return "volume";
    case OSP_VOLUMETRIC_MODEL: return "volumetric model";
    case OSP_WORLD: return "world";
    default: return "object";
  }
}

Obj::~Obj() {
  for (auto &kv : params)
    if (kv.second.obj) kv.second.obj->release();
}

void Obj::setParam(const char *name, OSPDataType t, const void *mem) {
  if (t == OSP_UNKNOWN) throw Error(OSP_INVALID_ARGUMENT, std::string("parameter '") + name + "' of type OSP_UNKNOWN");
  Param p;
  p.type = t;
  if (t == OSP_STRING) {
    const char *s = static_cast<const char *>(mem);
    if (s) p.bytes.assign(s, s + strlen(s) + 1);
  } else {
    const size_t n = sizeOfType(t);
    if (!mem) throw Error(OSP_INVALID_ARGUMENT, std::string("null value for parameter '") + name + "'");
    p.bytes.assign(static_cast<const unsigned char *>(mem), static_cast<const unsigned char *>(mem) + n);
    if (isObjectType(t)) {
      std::memcpy(&p.obj, mem, sizeof(Obj *));
      if (p.obj) p.obj->retain();
    }
  }
  auto it = params.find(name);
  if (it != params.end() && it->second.obj) it->second.obj->release();
  params[name] = std::move(p);
}

void Obj::removeParam(const char *name) {
  auto it = params.find(name);
  if (it == params.end()) return;
  if (it->second.obj) it->second.obj->release();
  params.erase(it);
}

std::vector<std::string> Obj::unusedParams() const {
  std::vector<std::string> out;
  for (const auto &kv : params)
    if (!kv.second.used) out.push_back(kv.first);
  return out;
}

void Obj::resetUsed() {
  for (auto &kv : params) kv.second.used = false;
}

const Param *Obj::find(const char *name) {
  auto it = params.find(name);
  if (it == params.end()) return nullptr;
  it->second.used = true;
  return &it->second;
}

namespace {
template <class T>
T load(const Param *p, size_t i = 0) {
  T v;
  std::memcpy(&v, p->bytes.data() + i * sizeof(T), sizeof(T));
  return v;
}
}  // namespace

float Obj::getFloat(const char *name, float def) {
  const Param *p = find(name);
  if (!p) return def;
  switch (p->type) {
    case OSP_FLOAT: return load<float>(p);
    case OSP_DOUBLE: return float(load<double>(p));
    case OSP_INT: return float(load<int32_t>(p));
    case OSP_UINT: return float(load<uint32_t>(p));
    default: return def;
  }
}

int Obj::getInt(const char *name, int def) {
  const Param *p = find(name);
  if (!p) return def;
  switch (p->type) {
    case OSP_INT: return load<int32_t>(p);
    case OSP_UINT: return int(load<uint32_t>(p));
    case OSP_UCHAR: return int(load<uint8_t>(p));
    case OSP_SHORT: return int(load<int16_t>(p));
    case OSP_USHORT: return int(load<uint16_t>(p));
    case OSP_LONG: return int(load<int64_t>(p));
    case OSP_ULONG: return int(load<uint64_t>(p));
    case OSP_BOOL: return load<uint8_t>(p) ? 1 : 0;
    default: return def;
  }
}

bool Obj::getBool(const char *name, bool def) {
  const Param *p = find(name);
  if (!p) return def;
  if (p->type == OSP_BOOL) return load<uint8_t>(p) != 0;
  if (p->type == OSP_INT || p->type == OSP_UINT) return load<int32_t>(p) != 0;
  return def;
}

void Obj::getVec3(const char *name, float out[3], const float def[3]) {
  const Param *p = find(name);
  std::memcpy(out, def, 12);
  if (!p) return;
  if (p->type == OSP_VEC3F || p->type == OSP_VEC4F) {
    for (int k = 0; k < 3; k++) out[k] = load<float>(p, k);
  } else if (p->type == OSP_FLOAT) {
    out[0] = out[1] = out[2] = load<float>(p);
  } else if (p->type == OSP_VEC3I) {
    for (int k = 0; k < 3; k++) out[k] = float(load<int32_t>(p, k));
  }
}

void Obj::getColor4(const char *name, float out[4], const float def[4]) {
  const Param *p = find(name);
  std::memcpy(out, def, 16);
  if (!p) return;
  if (p->type == OSP_VEC4F) {
    for (int k = 0; k < 4; k++) out[k] = load<float>(p, k);
  } else if (p->type == OSP_VEC3F) {
    // a vec3f or float colour is transparent (Renderer::commit, render/Renderer.cpp:62-64)
    for (int k = 0; k < 3; k++) out[k] = load<float>(p, k);
    out[3] = 0.f;
  } else if (p->type == OSP_FLOAT) {
    out[0] = out[1] = out[2] = load<float>(p);
    out[3] = 0.f;
  }
}

bool Obj::getBox1(const char *name, float out[2]) {
  const Param *p = find(name);
  if (!p || (p->type != OSP_BOX1F && p->type != OSP_VEC2F)) return false;
  out[0] = load<float>(p, 0);
  out[1] = load<float>(p, 1);
  return true;
}

bool Obj::getAffine(const char *name, float out12[12]) {
  const Param *p = find(name);
  if (!p || p->type != OSP_AFFINE3F) return false;
  for (int k = 0; k < 12; k++) out12[k] = load<float>(p, k);
  return true;
}

Obj *Obj::getObject(const char *name, OSPDataType kind) {
  const Param *p = find(name);
  if (!p || !p->obj) return nullptr;
  if (p->obj->kind != kind)
    throw Error(OSP_INVALID_ARGUMENT, std::string("parameter '") + name + "' must be a " + kindName(kind) +
                                          ", got a " + kindName(p->obj->kind));
  return p->obj;
}

DataObj *Obj::getData(const char *name) {
  const Param *p = find(name);
  if (!p || !p->obj) return nullptr;
  if (p->obj->kind != OSP_DATA)
    throw Error(OSP_INVALID_ARGUMENT, std::string("parameter '") + name + "' must be an OSPData array");
  return static_cast<DataObj *>(p->obj);
}

// ---------------------------------------------------------------- data

DataObj::DataObj(OSPDataType e, const void *shared, uint64_t n1, int64_t s1, uint64_t n2, int64_t s2, uint64_t n3,
                 int64_t s3, OSPDeleterCallback del, const void *user)
    : Obj(OSP_DATA, "shared"), elem(e), deleter(del), deleterUser(user), sharedPtr(shared) {
  if (!shared) throw Error(OSP_INVALID_ARGUMENT, "ospNewSharedData: null pointer");
  if (n1 == 0 || n2 == 0 || n3 == 0) throw Error(OSP_INVALID_ARGUMENT, "ospNewSharedData: zero items");
  const size_t es = sizeOfType(e);
  n[0] = n1;
  n[1] = n2;
  n[2] = n3;
  stride[0] = s1 ? s1 : int64_t(es);
  stride[1] = s2 ? s2 : stride[0] * int64_t(n1);
  stride[2] = s3 ? s3 : stride[1] * int64_t(n2);
  ptr = static_cast<const unsigned char *>(shared);
  if (isObjectType(e)) {
    // object arrays are copied (the caller may pass a temporary) and retained
    owned = compact();
    ptr = owned.data();
    stride[0] = int64_t(es);
    stride[1] = stride[0] * int64_t(n1);
    stride[2] = stride[1] * int64_t(n2);
    for (uint64_t i = 0; i < count(); i++)
      if (Obj *o = object(i)) o->retain();
  }
}

DataObj::DataObj(OSPDataType e, uint64_t n1, uint64_t n2, uint64_t n3) : Obj(OSP_DATA, "owned"), elem(e) {
  if (n1 == 0 || n2 == 0 || n3 == 0) throw Error(OSP_INVALID_ARGUMENT, "ospNewData: zero items");
  const size_t es = sizeOfType(e);
  n[0] = n1;
  n[1] = n2;
  n[2] = n3;
  owned.assign(es * n1 * n2 * n3, 0);
  ptr = owned.data();
  stride[0] = int64_t(es);
  stride[1] = stride[0] * int64_t(n1);
  stride[2] = stride[1] * int64_t(n2);
}

DataObj::~DataObj() {
  if (isObjectType(elem))
    for (uint64_t i = 0; i < count(); i++)
      if (Obj *o = object(i)) o->release();
  if (deleter) deleter(deleterUser, sharedPtr);
}

std::vector<unsigned char> DataObj::compact() const {
  const size_t es = sizeOfType(elem);
  std::vector<unsigned char> out(es * count());
  size_t o = 0;
  for (uint64_t k = 0; k < n[2]; k++)
    for (uint64_t j = 0; j < n[1]; j++)
      for (uint64_t i = 0; i < n[0]; i++, o += es) std::memcpy(out.data() + o, at(i, j, k), es);
  return out;
}

std::vector<float> DataObj::toFloats() const {
  std::vector<float> out;
  out.reserve(count());
  for (uint64_t k = 0; k < n[2]; k++)
    for (uint64_t j = 0; j < n[1]; j++)
      for (uint64_t i = 0; i < n[0]; i++) {
        const unsigned char *p = at(i, j, k);
        switch (elem) {
          case OSP_FLOAT: {
            float v;
            std::memcpy(&v, p, 4);
            out.push_back(v);
          } break;
          case OSP_DOUBLE: {
            double v;
            std::memcpy(&v, p, 8);
            out.push_back(float(v));
          } break;
          case OSP_UCHAR: out.push_back(float(*p)); break;
          case OSP_SHORT: {
            int16_t v;
            std::memcpy(&v, p, 2);
            out.push_back(float(v));
          } break;
          case OSP_USHORT: {
            uint16_t v;
            std::memcpy(&v, p, 2);
            out.push_back(float(v));
          } break;
          case OSP_INT: {
            int32_t v;
            std::memcpy(&v, p, 4);
            out.push_back(float(v));
          } break;
          case OSP_UINT: {
            uint32_t v;
            std::memcpy(&v, p, 4);
            out.push_back(float(v));
          } break;
          default: throw Error(OSP_INVALID_ARGUMENT, "data array: element type is not a scalar");
        }
      }
  return out;
}

void DataObj::copyFrom(const DataObj &src, uint64_t i1, uint64_t i2, uint64_t i3) {
  if (owned.empty() || ptr != owned.data() || type != "owned")
    throw Error(OSP_INVALID_OPERATION, "ospCopyData: the destination must come from ospNewData");
  if (src.elem != elem) throw Error(OSP_INVALID_ARGUMENT, "ospCopyData: element types differ");
  if (i1 + src.n[0] > n[0] || i2 + src.n[1] > n[1] || i3 + src.n[2] > n[2])
    throw Error(OSP_INVALID_ARGUMENT, "ospCopyData: source does not fit at the destination index");
  const size_t es = sizeOfType(elem);
  for (uint64_t k = 0; k < src.n[2]; k++)
    for (uint64_t j = 0; j < src.n[1]; j++)
      for (uint64_t i = 0; i < src.n[0]; i++) {
        unsigned char *d = owned.data() + (i + i1) * stride[0] + (j + i2) * stride[1] + (k + i3) * stride[2];
        if (isObjectType(elem)) {
          Obj *old, *nu;
          std::memcpy(&old, d, sizeof(old));
          std::memcpy(&nu, src.at(i, j, k), sizeof(nu));
          if (nu) nu->retain();
          if (old) old->release();
        }
        std::memcpy(d, src.at(i, j, k), es);
      }
}

}  // namespace b200osp
