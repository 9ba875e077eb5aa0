// Host objects of the b200 OSPRay device: parameter staging, data arrays and
// the scene-object types the GB300 render path supports.
//
// Parameters are staged and take effect at ospCommit (ospray/common/
// Managed.h:132-148, modules/cpu/ISPCDevice.cpp:474-500): setParam copies
// the value (object values are retained), commit() reads what the object
// type understands, and every parameter no commit looked at is reported once
// as ignored.  Shared data (ospNewSharedData) aliases application memory
// until it is read at the holder's commit, where it is copied (and uploaded
// to the GPU by the world commit); object arrays are copied and their
// elements retained at creation.
#pragma once

#include <atomic>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../../include/b200.h"
#include "device.h"

namespace b200osp {

using ospapi::Error;

size_t sizeOfType(OSPDataType t);
bool isObjectType(OSPDataType t);
const char *kindName(OSPDataType kind);

struct Obj;

struct Param {
  OSPDataType type = OSP_UNKNOWN;
  std::vector<unsigned char> bytes;
  Obj *obj = nullptr;  // retained object value
  bool used = false;
};

struct Obj {
  std::atomic<int> refs{1};
  OSPDataType kind;
  std::string type;
  std::map<std::string, Param> params;
  bool committed = false;

  Obj(OSPDataType k, std::string t) : kind(k), type(std::move(t)) {}
  virtual ~Obj();
  void retain() { refs.fetch_add(1); }
  void release() {
    if (refs.fetch_sub(1) == 1) delete this;
  }

  void setParam(const char *name, OSPDataType t, const void *mem);
  void removeParam(const char *name);
  // the parameters the last commit did not read
  std::vector<std::string> unusedParams() const;
  void resetUsed();

  // typed reads (mark the parameter used); `def` when absent or of another type
  const Param *find(const char *name);
  float getFloat(const char *name, float def);
  int getInt(const char *name, int def);
  bool getBool(const char *name, bool def);
  void getVec3(const char *name, float out[3], const float def[3]);
  // colour given as float, vec3f or vec4f (alpha 1 / given)
  void getColor4(const char *name, float out[4], const float def[4]);
  bool getBox1(const char *name, float out[2]);
  bool getAffine(const char *name, float out12[12]);
  Obj *getObject(const char *name, OSPDataType kind);
  struct DataObj *getData(const char *name);
  bool has(const char *name) const { return params.count(name) != 0; }
};

// a counted reference: what an object keeps from its last commit stays alive
// even if the application changes or releases the parameter afterwards
template <class T>
struct Ref {
  T *p = nullptr;
  Ref() = default;
  Ref(T *x) : p(x) {
    if (p) p->retain();
  }
  Ref(const Ref &o) : Ref(o.p) {}
  Ref &operator=(const Ref &o) {
    if (o.p) o.p->retain();
    if (p) p->release();
    p = o.p;
    return *this;
  }
  ~Ref() {
    if (p) p->release();
  }
  T *operator->() const { return p; }
  T *get() const { return p; }
  explicit operator bool() const { return p != nullptr; }
};

struct DataObj : Obj {
  OSPDataType elem;
  uint64_t n[3] = {1, 1, 1};
  int64_t stride[3] = {0, 0, 0};
  const unsigned char *ptr = nullptr;  // shared memory, or owned.data()
  std::vector<unsigned char> owned;
  OSPDeleterCallback deleter = nullptr;
  const void *deleterUser = nullptr;
  const void *sharedPtr = nullptr;

  DataObj(OSPDataType e, const void *shared, uint64_t n1, int64_t s1, uint64_t n2, int64_t s2, uint64_t n3,
          int64_t s3, OSPDeleterCallback del, const void *user);
  DataObj(OSPDataType e, uint64_t n1, uint64_t n2, uint64_t n3);
  ~DataObj() override;
  uint64_t count() const { return n[0] * n[1] * n[2]; }
  const unsigned char *at(uint64_t i, uint64_t j = 0, uint64_t k = 0) const {
    return ptr + i * stride[0] + j * stride[1] + k * stride[2];
  }
  // compact copy of all elements as bytes (sizeOfType(elem) each)
  std::vector<unsigned char> compact() const;
  // element i of an object array
  Obj *object(uint64_t i) const {
    Obj *o;
    std::memcpy(&o, at(i), sizeof(o));
    return o;
  }
  // all elements converted to float (scalar element types only)
  std::vector<float> toFloats() const;
  void copyFrom(const DataObj &src, uint64_t i1, uint64_t i2, uint64_t i3);
};

}  // namespace b200osp
