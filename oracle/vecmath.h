// Oracle (test infrastructure only): scalar vector math for the CPU
// restatement of the reference render path.  Built with -ffp-contract=off so
// every product is rounded separately, matching the CUDA side's explicit
// non-contracted arithmetic in ray generation and intersection.
#pragma once
#include <cmath>
#include <cstdint>

namespace orc {

struct V3 {
  float x, y, z;
};
struct V2 {
  float x, y;
};
struct V4 {
  float x, y, z, w;
};

inline V3 v3(float a) { return {a, a, a}; }
inline V3 v3(float a, float b, float c) { return {a, b, c}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
// normalize as x * (1/sqrt(x.x)): three correctly rounded steps
inline V3 normalize(V3 a) {
  const float r = 1.f / std::sqrt(dot(a, a));
  return a * r;
}
inline V3 vabs(V3 a) { return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)}; }
inline V3 vmin(V3 a, V3 b) { return {std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)}; }
inline V3 vmax(V3 a, V3 b) { return {std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)}; }
inline float reduce_max(V3 a) { return std::fmax(std::fmax(a.x, a.y), a.z); }
inline float reduce_min(V3 a) { return std::fmin(std::fmin(a.x, a.y), a.z); }
inline float get(V3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
inline float clampf(float x, float lo, float hi) { return std::fmin(std::fmax(x, lo), hi); }
inline float lerpf(float f, float a, float b) { return (1.f - f) * a + f * b; }
inline V3 lerp3(float f, V3 a, V3 b) { return (1.f - f) * a + f * b; }

// column-major 3x3 (vx, vy, vz columns) + translation, as rkcommon affine3f
struct L3 {
  V3 vx, vy, vz;
};
struct A3 {
  L3 l;
  V3 p;
};
inline V3 xfmVector(const L3 &l, V3 v) { return l.vx * v.x + l.vy * v.y + l.vz * v.z; }
inline V3 xfmPoint(const A3 &a, V3 v) { return xfmVector(a.l, v) + a.p; }
inline L3 transposed(const L3 &l) {
  return {{l.vx.x, l.vy.x, l.vz.x}, {l.vx.y, l.vy.y, l.vz.y}, {l.vx.z, l.vy.z, l.vz.z}};
}

// Shading frame around N (rkcommon 1.14.2 math/LinearSpace.ih frame(N)):
// dx from the two candidate perpendiculars, dy = N x dx.
inline L3 frame(V3 N) {
  const V3 dx0 = {0.f, N.z, -N.y};
  const V3 dx1 = {-N.z, 0.f, N.x};
  const V3 dx = normalize(std::fabs(N.x) < std::fabs(N.y) ? dx0 : dx1);
  const V3 dy = normalize(cross(N, dx));
  return {dx, dy, N};
}

}  // namespace orc
