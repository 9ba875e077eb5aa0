// Oracle (test infrastructure only): CPU restatement of the reference's
// random and quasi-random samplers.
//   modules/cpu/math/random.ih:20-55   MurmurHash3 mix/finalize, tripleHash
//   modules/cpu/math/random.ih:80-95   CranleyPattersonRotation
//   modules/cpu/math/random.ih:116-154 RandomSampler (PCG32)
//   modules/cpu/math/random.ih:159-190 TEA (8 rounds)
//   modules/cpu/math/random.ih:233-266 OwenHash2 / Owen scrambling
//   modules/cpu/math/random.ih:283-394 LDSampler (shuffled, Owen-scrambled Sobol)
//   modules/cpu/math/halton.ih:38-86   Halton / permuted Halton
//   modules/cpu/math/sobol.ih:38-91    Sobol_revSample{2,3,4}
// The reference ships its Halton permutation and Sobol matrix tables as data
// (math/halton.inl, math/sobol.inl).  Here they are regenerated from the
// published constructions they come from: Faure permutations of the digits
// (bases 3: identity, 5: {0,3,2,1,4}, 7: {0,2,5,3,1,4,6}) applied to a
// digit-reversed index, and the Joe-Kuo (2008, new-joe-kuo-6.21201) direction
// numbers for Sobol dimensions 2..5.  A test checks both against the
// reference's tables.
#pragma once
#include <cstdint>

#include "vecmath.h"

namespace orc {

inline uint32_t reverseBits(uint32_t i) {
  i = (i << 16) | (i >> 16);
  i = ((i & 0x00ff00ffu) << 8) | ((i & 0xff00ff00u) >> 8);
  i = ((i & 0x0f0f0f0fu) << 4) | ((i & 0xf0f0f0f0u) >> 4);
  i = ((i & 0x33333333u) << 2) | ((i & 0xccccccccu) >> 2);
  i = ((i & 0x55555555u) << 1) | ((i & 0xaaaaaaaau) >> 1);
  return i;
}

// rkcommon to_float_unorm: top 24 bits scaled into [0,1)
inline float to_float_unorm(uint32_t a) { return float(a >> 8) * (1.0f / 16777216.0f); }

struct Tables {
  uint32_t perm3[243], perm5[125], perm7[343];
  uint32_t sobolRev[4 * 32];
  Tables() {
    static const uint32_t s3[3] = {0, 1, 2}, s5[5] = {0, 3, 2, 1, 4}, s7[7] = {0, 2, 5, 3, 1, 4, 6};
    build_perm(3, 5, s3, perm3);
    build_perm(5, 3, s5, perm5);
    build_perm(7, 3, s7, perm7);
    build_sobol();
  }
  // perm[i] = sum_k sigma(digit_k(i)) * base^(ndigits-1-k): the digit-reversed,
  // Faure-permuted value of i's first `ndigits` base-`base` digits.
  static void build_perm(uint32_t base, int ndigits, const uint32_t *sigma, uint32_t *perm) {
    uint32_t n = 1;
    for (int k = 0; k < ndigits; k++) n *= base;
    for (uint32_t i = 0; i < n; i++) {
      uint32_t v = 0, x = i;
      for (int k = 0; k < ndigits; k++) {
        v = v * base + sigma[x % base];
        x /= base;
      }
      perm[i] = v;
    }
  }
  // Joe-Kuo direction numbers for dimensions 2..5 (s, a, m_1..m_s):
  //   (1, 0, {1}), (2, 1, {1,3}), (3, 1, {1,3,1}), (3, 2, {1,1,1}).
  // sobolRev[4*i + d] = bit-reverse of v_{i+1} = m_{i+1} << (31 - i).
  void build_sobol() {
    const int S[4] = {1, 2, 3, 3};
    const uint32_t A[4] = {0, 1, 1, 2};
    const uint32_t M0[4][3] = {{1, 0, 0}, {1, 3, 0}, {1, 3, 1}, {1, 1, 1}};
    for (int d = 0; d < 4; d++) {
      uint64_t m[33];
      const int s = S[d];
      for (int k = 1; k <= s; k++) m[k] = M0[d][k - 1];
      for (int k = s + 1; k <= 32; k++) {
        uint64_t v = m[k - s] ^ (m[k - s] << s);
        for (int j = 1; j < s; j++)
          if ((A[d] >> (s - 1 - j)) & 1u) v ^= m[k - j] << j;
        m[k] = v;
      }
      for (int i = 0; i < 32; i++)
        sobolRev[4 * i + d] = reverseBits(uint32_t(m[i + 1] << (31 - i)));
    }
  }
};

const Tables &tables();

inline float Halton_sample2(uint32_t index) { return to_float_unorm(reverseBits(index)); }
inline float Halton_sample3(uint32_t index) {
  const uint32_t *p = tables().perm3;
  return float(p[index % 243u] * 14348907u + p[(index / 243u) % 243u] * 59049u +
               p[(index / 59049u) % 243u] * 243u + p[(index / 14348907u) % 243u]) *
         float(1.0 / 3486784401u);
}
inline float PermHalton_sample5(uint32_t index) {
  const uint32_t *p = tables().perm5;
  return float(p[index % 125u] * 1953125u + p[(index / 125u) % 125u] * 15625u +
               p[(index / 15625u) % 125u] * 125u + p[(index / 1953125u) % 125u]) *
         float(1.0 / 244140625u);
}
inline float PermHalton_sample7(uint32_t index) {
  const uint32_t *p = tables().perm7;
  return float(p[index % 343u] * 117649u + p[(index / 343u) % 343u] * 343u +
               p[(index / 117649u) % 343u]) *
         float(1.0 / 40353607u);
}

inline float CranleyPattersonRotation(float x, float dx) {
  x += dx;
  if (x >= 1.f) x -= 1.f;
  return x;
}

inline uint32_t MurmurHash3_mix(uint32_t hash, uint32_t k) {
  k *= 0xcc9e2d51u;
  k = (k << 15) | (k >> 17);
  k *= 0x1b873593u;
  hash ^= k;
  hash = ((hash << 13) | (hash >> 19)) * 5u + 0xe6546b64u;
  return hash;
}
inline uint32_t MurmurHash3_finalize(uint32_t h) {
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  h *= 0xc2b2ae35u;
  h ^= h >> 16;
  return h;
}
inline uint32_t tripleHash(uint32_t x) {
  x ^= x >> 17;
  x *= 0xed5ad4bbu;
  x ^= x >> 11;
  x *= 0xac4c1b51u;
  x ^= x >> 15;
  x *= 0x31848babu;
  x ^= x >> 14;
  return x;
}

struct RandomSampler {
  uint64_t state;
  uint32_t stream;
  uint32_t pcg32() {
    const uint64_t old = state;
    state = old * 6364136223846793005ull + (stream | 1u);
    const uint32_t xs = uint32_t(((old >> 18u) ^ old) >> 27u);
    const uint32_t rot = uint32_t(old >> 59u);
    return (xs >> rot) | (xs << ((-rot) & 31));
  }
  float getFloat() { return to_float_unorm(pcg32()); }
  void init(uint32_t seed, uint32_t strm) {
    state = 0;
    stream = (strm << 1u) | 1u;
    state = MurmurHash3_mix(uint32_t(state), seed);
    state = MurmurHash3_finalize(uint32_t(state));
    pcg32();
    state += seed;
    pcg32();
  }
};

inline void tea8(uint32_t &v0_, uint32_t &v1_) {
  uint32_t v0 = v0_, v1 = v1_, sum = 0;
  for (int i = 0; i < 8; i++) {
    sum += 0x9e3779b9u;
    v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + sum) ^ ((v1 >> 5) + 0xc8013ea4u);
    v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + sum) ^ ((v0 >> 5) + 0x7e95761eu);
  }
  v0_ = v0;
  v1_ = v1;
}

inline uint32_t OwenHash2(uint32_t x, uint32_t seed) {
  x ^= x * 0x3d20adeau;
  x += seed;
  x *= (seed >> 16) | 1u;
  x ^= x * 0x05526c56u;
  x ^= x * 0x53a22864u;
  return x;
}

enum : uint32_t {
  SCRAMBLE0 = 0x9374b0d3u,
  SCRAMBLE1 = 0x1ec38426u,
  SCRAMBLE2 = 0xdb81c29cu,
  SCRAMBLE3 = 0x5628372bu,
  SCRAMBLE4 = 0xbcb745bdu
};

struct LDSampler {
  uint32_t revIndex, scramble, baseIndexLight, idxMask, idxMaskLight;
  void init(uint32_t seed, uint32_t sampleIndex, uint32_t sampleOffsetLight = 0, uint32_t bits = 16,
            uint32_t bitsLight = 16) {
    revIndex = reverseBits(sampleIndex);
    scramble = seed;
    baseIndexLight = sampleOffsetLight;
    idxMask = bits > 31 ? ~0u : ~(~0u >> bits);
    idxMaskLight = bitsLight > 31 ? ~0u : ~(~0u >> bitsLight);
  }
  static float scr(uint32_t sample, uint32_t s) { return to_float_unorm(reverseBits(OwenHash2(sample, s))); }
  static void revSample(uint32_t revIdx, uint32_t out[4]) {
    const uint32_t *M = tables().sobolRev;
    out[0] = out[1] = out[2] = out[3] = 0;
    for (uint32_t i = 0; revIdx; revIdx <<= 1, i += 4)
      if (revIdx & 0x80000000u) {
        out[0] ^= M[i];
        out[1] ^= M[i + 1];
        out[2] ^= M[i + 2];
        out[3] ^= M[i + 3];
      }
  }
  void nextGroup() { scramble = tripleHash(scramble); }
  V2 get3LightSamples(uint32_t idx, bool split, float &ss) const {
    uint32_t r = split ? reverseBits(baseIndexLight + idx) : revIndex;
    r = OwenHash2(r, scramble);
    r &= split ? idxMaskLight : idxMask;
    uint32_t s[4];
    revSample(r, s);
    V2 res;
    res.x = scr(reverseBits(r), scramble ^ SCRAMBLE0);
    res.y = scr(s[0], scramble ^ SCRAMBLE1);
    ss = scr(s[1], scramble ^ SCRAMBLE2);
    return res;
  }
  V2 getNext4Samples(float &ss, uint32_t &u) {
    nextGroup();
    const uint32_t r = OwenHash2(revIndex, scramble) & idxMask;
    uint32_t s[4];
    revSample(r, s);
    V2 res;
    res.x = scr(reverseBits(r), scramble ^ SCRAMBLE0);
    res.y = scr(s[0], scramble ^ SCRAMBLE1);
    ss = scr(s[1], scramble ^ SCRAMBLE2);
    u = s[2];
    return res;
  }
  float finalizeDim3(uint32_t revRes) const { return scr(revRes, scramble ^ SCRAMBLE3); }
  V2 getNext5Samples(uint32_t ss[3]) {
    nextGroup();
    const uint32_t r = OwenHash2(revIndex, scramble) & idxMask;
    uint32_t s[4];
    revSample(r, s);
    V2 res;
    res.x = scr(reverseBits(r), scramble ^ SCRAMBLE0);
    res.y = scr(s[0], scramble ^ SCRAMBLE1);
    ss[0] = s[1];
    ss[1] = s[2];
    ss[2] = s[3];
    return res;
  }
  V2 finalizeDim23(const uint32_t rr[3]) const {
    return {scr(rr[0], scramble ^ SCRAMBLE2), scr(rr[1], scramble ^ SCRAMBLE3)};
  }
  float finalizeDim4(const uint32_t rr[3]) const { return scr(rr[2], scramble ^ SCRAMBLE4); }
};

}  // namespace orc
