// Seeded synthetic scene generators for the render workloads.
//
// Every generator draws from one splitmix64 stream per seed, in the order
// documented beside each function, so the CUDA renderer, the CPU oracle and
// the benchmark all consume byte-identical inputs.  These are inputs, not part
// of the render path: they replace the reference's scene builders
// (apps/common/ospray_testing/builders/*.cpp) for the named workloads.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <thread>
#include <vector>

namespace {

struct SplitMix64 {
  uint64_t s;
  explicit SplitMix64(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  // uniform in [0,1) with 24 bits of mantissa
  float uniform() { return float(next() >> 40) * (1.0f / 16777216.0f); }
  float uniform(float lo, float hi) { return lo + (hi - lo) * uniform(); }
};

// integer lattice hash -> [0,1); used by value noise
inline float lattice(int32_t x, int32_t y, int32_t z, uint32_t seed) {
  uint64_t h = uint64_t(uint32_t(x)) * 0x9E3779B185EBCA87ull;
  h ^= uint64_t(uint32_t(y)) * 0xC2B2AE3D27D4EB4Full;
  h ^= uint64_t(uint32_t(z)) * 0x165667B19E3779F9ull;
  h ^= uint64_t(seed) * 0xD6E8FEB86659FD93ull;
  h ^= h >> 32;
  h *= 0xD6E8FEB86659FD93ull;
  h ^= h >> 32;
  return float(h >> 40) * (1.0f / 16777216.0f);
}

inline float smooth(float t) { return t * t * (3.f - 2.f * t); }

// trilinear value noise with smoothstep weights, range [0,1)
inline float value_noise(float x, float y, float z, uint32_t seed) {
  const float fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
  const int32_t ix = int32_t(fx), iy = int32_t(fy), iz = int32_t(fz);
  const float tx = smooth(x - fx), ty = smooth(y - fy), tz = smooth(z - fz);
  float c[8];
  for (int k = 0; k < 8; k++)
    c[k] = lattice(ix + (k & 1), iy + ((k >> 1) & 1), iz + ((k >> 2) & 1), seed);
  const float x00 = c[0] + tx * (c[1] - c[0]);
  const float x10 = c[2] + tx * (c[3] - c[2]);
  const float x01 = c[4] + tx * (c[5] - c[4]);
  const float x11 = c[6] + tx * (c[7] - c[6]);
  const float y0 = x00 + ty * (x10 - x00);
  const float y1 = x01 + ty * (x11 - x01);
  return y0 + tz * (y1 - y0);
}

template <class F>
void parallel_rows(int64_t n, F f) {
  unsigned nt = std::thread::hardware_concurrency();
  if (nt == 0) nt = 4;
  if (nt > 64) nt = 64;
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; t++)
    th.emplace_back([=]() {
      for (int64_t i = t; i < n; i += nt) f(i);
    });
  for (auto &x : th) x.join();
}

}  // namespace

extern "C" {

// Height field of n x n vertices over [0,1]^2 (x = i/(n-1), z = j/(n-1)) with
// y = 0.1 * sum_{k=1..4} 2^-k sin(2^k pi (a_k x + b_k z) + phi_k).
// Draw order from splitmix64(seed): for k = 1..4: a_k, b_k, phi_k.
// Two triangles per cell, cells row-major (j outer, i inner), winding
// (v00, v01, v10), (v10, v01, v11) so the geometric normal points to +y.
// verts: n*n*3 floats; index: 2*(n-1)^2*3 uint32.
void b200sg_heightfield(uint64_t seed, int n, float *verts, uint32_t *index) {
  SplitMix64 rng(seed);
  float a[4], b[4], phi[4];
  for (int k = 0; k < 4; k++) {
    a[k] = rng.uniform(-1.f, 1.f);
    b[k] = rng.uniform(-1.f, 1.f);
    phi[k] = rng.uniform(0.f, 6.283185307179586f);
  }
  const double inv = 1.0 / double(n - 1);
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) {
      const double x = i * inv, z = j * inv;
      double y = 0.0;
      for (int k = 0; k < 4; k++) {
        const double f = std::ldexp(1.0, k + 1);
        y += std::ldexp(1.0, -(k + 1)) *
             std::sin(f * M_PI * (a[k] * x + b[k] * z) + phi[k]);
      }
      float *v = verts + 3 * (size_t(j) * n + i);
      v[0] = float(x);
      v[1] = float(0.1 * y);
      v[2] = float(z);
    }
  size_t t = 0;
  for (int j = 0; j + 1 < n; j++)
    for (int i = 0; i + 1 < n; i++) {
      const uint32_t v00 = j * n + i, v10 = v00 + 1, v01 = v00 + n, v11 = v01 + 1;
      uint32_t *p = index + 6 * t;
      p[0] = v00; p[1] = v01; p[2] = v10;
      p[3] = v10; p[4] = v01; p[5] = v11;
      t++;
    }
}

// Spheres with centres U([0,1] x [0,0.3] x [0,1]) and radius U(r0, r1).
// Draw order from splitmix64(seed): per sphere cx, cy, cz, r.
// out: count*4 floats (x, y, z, radius).
void b200sg_spheres(uint64_t seed, int count, float r0, float r1, float *out) {
  SplitMix64 rng(seed);
  for (int s = 0; s < count; s++) {
    out[4 * s + 0] = rng.uniform();
    out[4 * s + 1] = 0.3f * rng.uniform();
    out[4 * s + 2] = rng.uniform();
    out[4 * s + 3] = rng.uniform(r0, r1);
  }
}

// Unit octahedron subdivided `levels` times (8 * 4^levels triangles), pushed
// to the unit sphere and displaced along the normal by
// amp * value_noise(freq * p, seed).  Returns vertex count through *nverts
// when verts is null (sizing call); index holds 8*4^levels*3 uint32.
void b200sg_displaced_sphere(int levels, float amp, float freq, uint32_t seed,
                             float *verts, uint32_t *index, int *nverts) {
  std::vector<float> V = {1, 0, 0, -1, 0, 0, 0, 1, 0, 0, -1, 0, 0, 0, 1, 0, 0, -1};
  std::vector<uint32_t> F = {0, 2, 4, 2, 1, 4, 1, 3, 4, 3, 0, 4,
                             2, 0, 5, 1, 2, 5, 3, 1, 5, 0, 3, 5};
  for (int l = 0; l < levels; l++) {
    std::map<uint64_t, uint32_t> mid;
    auto midpoint = [&](uint32_t a, uint32_t b) {
      const uint64_t key = a < b ? (uint64_t(a) << 32 | b) : (uint64_t(b) << 32 | a);
      auto it = mid.find(key);
      if (it != mid.end()) return it->second;
      const uint32_t id = uint32_t(V.size() / 3);
      float m[3];
      for (int c = 0; c < 3; c++) m[c] = 0.5f * (V[3 * a + c] + V[3 * b + c]);
      const float len = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
      for (int c = 0; c < 3; c++) V.push_back(m[c] / len);
      mid[key] = id;
      return id;
    };
    std::vector<uint32_t> G;
    G.reserve(F.size() * 4);
    for (size_t f = 0; f < F.size(); f += 3) {
      const uint32_t a = F[f], b = F[f + 1], c = F[f + 2];
      const uint32_t ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
      const uint32_t tri[12] = {a, ab, ca, ab, b, bc, ca, bc, c, ab, bc, ca};
      G.insert(G.end(), tri, tri + 12);
    }
    F.swap(G);
  }
  const int nv = int(V.size() / 3);
  if (nverts) *nverts = nv;
  if (!verts) return;
  for (int v = 0; v < nv; v++) {
    const float *p = &V[3 * v];
    const float d = 1.f + amp * value_noise(freq * p[0], freq * p[1], freq * p[2], seed);
    for (int c = 0; c < 3; c++) verts[3 * v + c] = p[c] * d;
  }
  std::memcpy(index, F.data(), F.size() * sizeof(uint32_t));
}

// Instance table for the path-tracer scene: per instance a row-major 3x4
// affine transform (rotation from a uniform random quaternion, uniform scale
// U(s0,s1), translation U([0,box]^3)) and a principled material
// (baseColor U(0,1)^3, roughness U(0.05,1), metallic 1 with probability
// pmetal).  Draw order per instance: q0..q3 (Gaussian pairs via Box-Muller on
// 4 uniforms), scale, tx, ty, tz, r, g, b, roughness, metallic-coin.
// xfm: count*12 floats; mat: count*5 floats (r, g, b, roughness, metallic).
void b200sg_instances(uint64_t seed, int count, float s0, float s1, float box,
                      float pmetal, float *xfm, float *mat) {
  SplitMix64 rng(seed);
  for (int i = 0; i < count; i++) {
    float u[4];
    for (int k = 0; k < 4; k++) u[k] = rng.uniform();
    // Shoemake's uniform random rotation from three uniforms (4th unused)
    const float r1 = std::sqrt(1.f - u[0]), r2 = std::sqrt(u[0]);
    const float t1 = 6.283185307179586f * u[1], t2 = 6.283185307179586f * u[2];
    const float qx = std::sin(t1) * r1, qy = std::cos(t1) * r1;
    const float qz = std::sin(t2) * r2, qw = std::cos(t2) * r2;
    const float s = rng.uniform(s0, s1);
    const float tx = rng.uniform(0.f, box), ty = rng.uniform(0.f, box),
                tz = rng.uniform(0.f, box);
    const float R[9] = {1 - 2 * (qy * qy + qz * qz), 2 * (qx * qy - qz * qw), 2 * (qx * qz + qy * qw),
                        2 * (qx * qy + qz * qw), 1 - 2 * (qx * qx + qz * qz), 2 * (qy * qz - qx * qw),
                        2 * (qx * qz - qy * qw), 2 * (qy * qz + qx * qw), 1 - 2 * (qx * qx + qy * qy)};
    float *X = xfm + 12 * i;
    for (int r = 0; r < 3; r++) {
      for (int c = 0; c < 3; c++) X[4 * r + c] = s * R[3 * r + c];
    }
    X[3] = tx; X[7] = ty; X[11] = tz;
    float *M = mat + 5 * i;
    M[0] = rng.uniform(); M[1] = rng.uniform(); M[2] = rng.uniform();
    M[3] = rng.uniform(0.05f, 1.f);
    M[4] = rng.uniform() < pmetal ? 1.f : 0.f;
  }
}

// Structured-regular volume n^3 (x fastest) of fractal value noise:
// sum_{o<octaves} gain^o * noise(base_freq * lacunarity^o * p), p in [0,1]^3,
// then min-max normalised to [0,1].  Uses all host threads.
void b200sg_fractal_volume(int n, int octaves, float base_freq, uint32_t seed, float *out) {
  const float inv = 1.f / float(n - 1);
  parallel_rows(int64_t(n), [&](int64_t z) {
    for (int y = 0; y < n; y++)
      for (int x = 0; x < n; x++) {
        float f = base_freq, amp = 1.f, v = 0.f;
        for (int o = 0; o < octaves; o++) {
          v += amp * value_noise(f * x * inv, f * y * inv, f * float(z) * inv, seed + o);
          f *= 2.f;
          amp *= 0.5f;
        }
        out[(size_t(z) * n + y) * n + x] = v;
      }
  });
  const size_t N = size_t(n) * n * n;
  float lo = out[0], hi = out[0];
  for (size_t i = 1; i < N; i++) {
    lo = out[i] < lo ? out[i] : lo;
    hi = out[i] > hi ? out[i] : hi;
  }
  const float s = hi > lo ? 1.f / (hi - lo) : 0.f;
  parallel_rows(int64_t(n), [&](int64_t z) {
    float *p = out + size_t(z) * n * n;
    for (size_t i = 0; i < size_t(n) * n; i++) p[i] = (p[i] - lo) * s;
  });
}

// Seeded colour ramp of `count` RGB entries: piecewise-linear between 5
// random control colours drawn from splitmix64(seed) (r, g, b per control).
void b200sg_color_ramp(uint64_t seed, int count, float *rgb) {
  SplitMix64 rng(seed);
  float ctrl[5][3];
  for (int c = 0; c < 5; c++)
    for (int k = 0; k < 3; k++) ctrl[c][k] = rng.uniform();
  for (int i = 0; i < count; i++) {
    const float t = count > 1 ? float(i) / float(count - 1) * 4.f : 0.f;
    int s = int(t);
    if (s > 3) s = 3;
    const float f = t - s;
    for (int k = 0; k < 3; k++) rgb[3 * i + k] = ctrl[s][k] + f * (ctrl[s + 1][k] - ctrl[s][k]);
  }
}

}  // extern "C"
