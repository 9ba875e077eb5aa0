// Device samplers with the reference's exact integer arithmetic:
//   modules/cpu/math/random.ih  (MurmurHash3, tripleHash, PCG32 RandomSampler,
//                               TEA, OwenHash2, LDSampler), math/halton.ih,
//   math/sobol.ih (revSample).
// The Halton digit permutations (Faure permutations, digit-reversed) and the
// bit-reversed Sobol matrices (Joe-Kuo 2008 direction numbers, dims 2..5) are
// generated on the host at device creation (tables.cpp) and live in global
// memory (lanes index them divergently, which constant memory serialises).
#pragma once
#include "common.cuh"

namespace b200 {

struct SamplerTables {
  uint32_t perm3[243], perm5[125], perm7[343];
  uint32_t sobolRev[128];
};

B200_D uint32_t reverseBits(uint32_t x) { return __brev(x); }
B200_D float to_float_unorm(uint32_t a) { return float(a >> 8) * (1.0f / 16777216.0f); }

B200_D float Halton_sample2(uint32_t index) { return to_float_unorm(__brev(index)); }
B200_D float Halton_sample3(const SamplerTables *T, uint32_t index) {
  const uint32_t *p = T->perm3;
  return float(__ldg(p + index % 243u) * 14348907u + __ldg(p + (index / 243u) % 243u) * 59049u +
               __ldg(p + (index / 59049u) % 243u) * 243u + __ldg(p + (index / 14348907u) % 243u)) *
         float(1.0 / 3486784401u);
}
B200_D float PermHalton_sample5(const SamplerTables *T, uint32_t index) {
  const uint32_t *p = T->perm5;
  return float(__ldg(p + index % 125u) * 1953125u + __ldg(p + (index / 125u) % 125u) * 15625u + __ldg(p + (index / 15625u) % 125u) * 125u +
               __ldg(p + (index / 1953125u) % 125u)) *
         float(1.0 / 244140625u);
}
B200_D float PermHalton_sample7(const SamplerTables *T, uint32_t index) {
  const uint32_t *p = T->perm7;
  return float(__ldg(p + index % 343u) * 117649u + __ldg(p + (index / 343u) % 343u) * 343u + __ldg(p + (index / 117649u) % 343u)) *
         float(1.0 / 40353607u);
}

B200_D float cpRotate(float x, float dx) {
  x = fadd(x, dx);
  if (x >= 1.f) x = fsub(x, 1.f);
  return x;
}

B200_D uint32_t murmurMix(uint32_t hash, uint32_t k) {
  k *= 0xcc9e2d51u;
  k = (k << 15) | (k >> 17);
  k *= 0x1b873593u;
  hash ^= k;
  return ((hash << 13) | (hash >> 19)) * 5u + 0xe6546b64u;
}
B200_D uint32_t murmurFinalize(uint32_t h) {
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  h *= 0xc2b2ae35u;
  h ^= h >> 16;
  return h;
}
B200_D uint32_t tripleHash(uint32_t x) {
  x ^= x >> 17;
  x *= 0xed5ad4bbu;
  x ^= x >> 11;
  x *= 0xac4c1b51u;
  x ^= x >> 15;
  x *= 0x31848babu;
  x ^= x >> 14;
  return x;
}

struct PCG {
  uint64_t state;
  uint32_t stream;
  B200_D uint32_t next() {
    const uint64_t old = state;
    state = old * 6364136223846793005ull + (stream | 1u);
    const uint32_t xs = uint32_t(((old >> 18u) ^ old) >> 27u);
    const uint32_t rot = uint32_t(old >> 59u);
    return (xs >> rot) | (xs << ((-rot) & 31));
  }
  B200_D float getFloat() { return to_float_unorm(next()); }
  B200_D void init(uint32_t seed, uint32_t strm) {
    stream = (strm << 1u) | 1u;
    state = murmurFinalize(murmurMix(0u, seed));
    next();
    state += seed;
    next();
  }
};

B200_D void tea8(uint32_t &v0_, uint32_t &v1_) {
  uint32_t v0 = v0_, v1 = v1_, sum = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    sum += 0x9e3779b9u;
    v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + sum) ^ ((v1 >> 5) + 0xc8013ea4u);
    v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + sum) ^ ((v0 >> 5) + 0x7e95761eu);
  }
  v0_ = v0;
  v1_ = v1;
}

B200_D uint32_t owenHash2(uint32_t x, uint32_t seed) {
  x ^= x * 0x3d20adeau;
  x += seed;
  x *= (seed >> 16) | 1u;
  x ^= x * 0x05526c56u;
  x ^= x * 0x53a22864u;
  return x;
}

constexpr uint32_t SCRAMBLE0 = 0x9374b0d3u, SCRAMBLE1 = 0x1ec38426u, SCRAMBLE2 = 0xdb81c29cu,
                   SCRAMBLE3 = 0x5628372bu, SCRAMBLE4 = 0xbcb745bdu;

struct LDSampler {
  uint32_t revIndex, scramble, baseIndexLight, idxMask, idxMaskLight;
  const uint32_t *sobol;  // SamplerTables::sobolRev
  B200_D void init(const SamplerTables *T, uint32_t seed, uint32_t sampleIndex, uint32_t sampleOffsetLight = 0, uint32_t bits = 16,
                   uint32_t bitsLight = 16) {
    sobol = T->sobolRev;
    revIndex = __brev(sampleIndex);
    scramble = seed;
    baseIndexLight = sampleOffsetLight;
    idxMask = bits > 31 ? ~0u : ~(~0u >> bits);
    idxMaskLight = bitsLight > 31 ? ~0u : ~(~0u >> bitsLight);
  }
  static B200_D float scr(uint32_t sample, uint32_t s) { return to_float_unorm(__brev(owenHash2(sample, s))); }
  B200_D void revSample(uint32_t r, uint32_t out[4]) const {
    out[0] = out[1] = out[2] = out[3] = 0;
    for (uint32_t i = 0; r; r <<= 1, i += 4)
      if (r & 0x80000000u) {
        out[0] ^= __ldg(sobol + i);
        out[1] ^= __ldg(sobol + i + 1);
        out[2] ^= __ldg(sobol + i + 2);
        out[3] ^= __ldg(sobol + i + 3);
      }
  }
  B200_D void nextGroup() { scramble = tripleHash(scramble); }
  B200_D float2 get3LightSamples(uint32_t idx, bool split, float &ss) const {
    uint32_t r = split ? __brev(baseIndexLight + idx) : revIndex;
    r = owenHash2(r, scramble);
    r &= split ? idxMaskLight : idxMask;
    uint32_t s[4];
    revSample(r, s);
    ss = scr(s[1], scramble ^ SCRAMBLE2);
    return make_float2(scr(__brev(r), scramble ^ SCRAMBLE0), scr(s[0], scramble ^ SCRAMBLE1));
  }
  B200_D float2 getNext4Samples(float &ss, uint32_t &u) {
    nextGroup();
    const uint32_t r = owenHash2(revIndex, scramble) & idxMask;
    uint32_t s[4];
    revSample(r, s);
    ss = scr(s[1], scramble ^ SCRAMBLE2);
    u = s[2];
    return make_float2(scr(__brev(r), scramble ^ SCRAMBLE0), scr(s[0], scramble ^ SCRAMBLE1));
  }
  B200_D float finalizeDim3(uint32_t revRes) const { return scr(revRes, scramble ^ SCRAMBLE3); }
  B200_D float2 getNext5Samples(uint32_t ss[3]) {
    nextGroup();
    const uint32_t r = owenHash2(revIndex, scramble) & idxMask;
    uint32_t s[4];
    revSample(r, s);
    ss[0] = s[1];
    ss[1] = s[2];
    ss[2] = s[3];
    return make_float2(scr(__brev(r), scramble ^ SCRAMBLE0), scr(s[0], scramble ^ SCRAMBLE1));
  }
  B200_D float2 finalizeDim23(const uint32_t rr[3]) const {
    return make_float2(scr(rr[0], scramble ^ SCRAMBLE2), scr(rr[1], scramble ^ SCRAMBLE3));
  }
  B200_D float finalizeDim4(const uint32_t rr[3]) const { return scr(rr[2], scramble ^ SCRAMBLE4); }
};

}  // namespace b200
