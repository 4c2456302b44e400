// pt_oracle_math.hpp -- vector arithmetic and samplers of the CPU oracle.
//
// ORACLE (test infrastructure only): a scalar restatement of the reference
// for checking the CUDA path.  Compiled with -ffp-contract=off so that every
// float operation is rounded separately, in the reference's order.
#pragma once
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <limits>

namespace orc {

constexpr double PI = 3.14159265358979323846;

// gl::vec<3,float> without GL_SIMD (include/utils/matrix.hpp:300-583)
struct V {
  float x = 0, y = 0, z = 0;
  V() = default;
  V(float a, float b, float c) : x(a), y(b), z(c) {}
  explicit V(float s) : x(s), y(s), z(s) {}
  float operator[](int i) const { return i == 0 ? x : i == 1 ? y : z; }
  float &operator[](int i) { return i == 0 ? x : i == 1 ? y : z; }
  float length() const { return std::sqrt(dot(*this)); }
  float dot(const V &o) const {
    float r = 0.0f;
    r += x * o.x;
    r += y * o.y;
    r += z * o.z;
    return r;
  }
  V normalize() const {
    float l = length();
    return V(x / l, y / l, z / l);
  }
  bool near_zero(float s = 1e-6f) const { return std::fabs(x) < s && std::fabs(y) < s && std::fabs(z) < s; }
};
inline V operator+(V a, V b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V operator-(V a, V b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V operator-(V a) { return V(-a.x, -a.y, -a.z); }
inline V operator*(V a, V b) { return V(a.x * b.x, a.y * b.y, a.z * b.z); }
inline V operator*(V a, float s) { return V(a.x * s, a.y * s, a.z * s); }
inline V operator*(float s, V a) { return V(s * a.x, s * a.y, s * a.z); }
inline V operator/(V a, float s) { return V(a.x / s, a.y / s, a.z / s); }
inline V operator/(V a, V b) { return V(a.x / b.x, a.y / b.y, a.z / b.z); }
inline V &operator+=(V &a, V b) { return a = a + b; }
inline V &operator*=(V &a, V b) { return a = a * b; }
inline float dot(V a, V b) { return a.dot(b); }
inline V cross(V a, V b) {
  return V(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline V normalize(V a) { return a.normalize(); }
inline float sqr(float x) { return x * x; }
inline float safe_sqrt(float x) { return std::sqrt(std::max(0.f, x)); }
inline float max_component(V a) { return std::max(a.x, std::max(a.y, a.z)); }

// OrthoBasis (utils/orthoBasis.hpp:15-36)
struct Onb {
  V ax[3];
  explicit Onb(V n) {
    ax[2] = n.normalize();
    V a = (std::abs(n.x) > 0.9) ? V(0, 1, 0) : V(1, 0, 0);
    ax[1] = normalize(cross(ax[2], a));
    ax[0] = cross(ax[2], ax[1]);
  }
  V at(V v) const { return v.x * ax[0] + v.y * ax[1] + v.z * ax[2]; }
  V local(V v) const { return V(dot(v, ax[0]), dot(v, ax[1]), dot(v, ax[2])); }
};

// ----------------------------------------------------------- hashing
inline uint64_t mix_bits(uint64_t v) {  // pbrt::mixBits (utils/hash.hpp:62-69)
  v ^= (v >> 31);
  v *= 0x7fb5d329728ea185ull;
  v ^= (v >> 27);
  v *= 0x81dadef4bc2dd44dull;
  v ^= (v >> 33);
  return v;
}

inline int permutation_element(uint32_t i, uint32_t l, uint32_t p) {  // utility.hpp:434-464
  uint32_t w = l - 1;
  w |= w >> 1;
  w |= w >> 2;
  w |= w >> 4;
  w |= w >> 8;
  w |= w >> 16;
  do {
    i ^= p;
    i *= 0xe170893d;
    i ^= p >> 16;
    i ^= (i & w) >> 4;
    i ^= p >> 8;
    i *= 0x0929eb3f;
    i ^= p >> 23;
    i ^= (i & w) >> 1;
    i *= 1 | p >> 27;
    i *= 0x6935fa69;
    i ^= (i & w) >> 11;
    i *= 0x74dcb303;
    i ^= (i & w) >> 2;
    i *= 0x9e501cc3;
    i ^= (i & w) >> 2;
    i *= 0xc860a3df;
    i &= w;
    i ^= i >> 5;
  } while (i >= l);
  return (int)((i + p) % l);
}

// MurmurHash64A (hash.hpp:10-58) and pbrt::hash of packed arguments (:84-91)
inline uint64_t murmur64a(const unsigned char *key, size_t len, uint64_t seed) {
  const uint64_t m = 0xc6a4a7935bd1e995ull;
  const int r = 47;
  uint64_t h = seed ^ (len * m);
  const unsigned char *end = key + 8 * (len / 8);
  while (key != end) {
    uint64_t k;
    std::memcpy(&k, key, 8);
    key += 8;
    k *= m;
    k ^= k >> r;
    k *= m;
    h ^= k;
    h *= m;
  }
  switch (len & 7) {
  case 7: h ^= uint64_t(key[6]) << 48; [[fallthrough]];
  case 6: h ^= uint64_t(key[5]) << 40; [[fallthrough]];
  case 5: h ^= uint64_t(key[4]) << 32; [[fallthrough]];
  case 4: h ^= uint64_t(key[3]) << 24; [[fallthrough]];
  case 3: h ^= uint64_t(key[2]) << 16; [[fallthrough]];
  case 2: h ^= uint64_t(key[1]) << 8; [[fallthrough]];
  case 1:
    h ^= uint64_t(key[0]);
    h *= m;
  }
  h ^= h >> r;
  h *= m;
  h ^= h >> r;
  return h;
}

static const int PRIMES[25] = {2,  3,  5,  7,  11, 13, 17, 19, 23, 29, 31, 37, 41,
                               43, 47, 53, 59, 61, 67, 71, 73, 79, 83, 89, 97};

// radicalInverse, float (utility.hpp:406-420)
inline float radical_inverse(int baseIndex, uint64_t a) {
  int base = PRIMES[baseIndex % 25];
  float invBase = (float)1 / (float)base, invBaseM = 1;
  uint64_t rev = 0;
  while (a) {
    uint64_t next = a / base;
    uint64_t digit = a - next * base;
    rev = rev * base + digit;
    invBaseM *= invBase;
    a = next;
  }
  return std::min(rev * invBaseM, (float)0x1.fffffep-1);
}

// owenScrambledRadicalInverse (digitPerm.hpp:99-133); dim >= 25 uses
// Primes[dim % 25] (the reference reads out of bounds there).
inline double owen_radical_inverse(int baseIndex, uint64_t a, uint32_t hash) {
  const int base = PRIMES[baseIndex % 25];
  const double invBase = 1.0 / (double)base;
  double invBaseM = 1.0;
  uint64_t rev = 0;
  int di = 0;
  while (1.0 - (base - 1) * invBaseM < 1.0) {
    uint64_t next = a / base;
    int digit = (int)(a - next * base);
    uint32_t dh = (uint32_t)mix_bits(hash ^ (uint32_t)rev ^ ((uint32_t)di << 16));
    digit = permutation_element((uint32_t)digit, (uint32_t)base, dh);
    rev = rev * (uint64_t)base + (uint64_t)digit;
    invBaseM *= invBase;
    ++di;
    a = next;
  }
  return std::min(invBaseM * (double)rev, std::nextafter(1.0, 0.0));
}

// DigitPermutation + scrambledRadicalInverse (digitPerm.hpp:12-97)
inline double permuted_radical_inverse(int baseIndex, uint64_t a, uint32_t seed) {
  const int base = PRIMES[baseIndex];
  const double invBase = 1.0 / (double)base;
  double invBaseM = 1.0;
  uint64_t rev = 0;
  int di = 0;
  while (1.0 - (base - 1) * invBaseM < 1.0) {
    uint64_t next = a / base;
    int digit = (int)(a - next * base);
    unsigned char buf[12];
    int32_t b32 = base, d32 = di;
    std::memcpy(buf, &b32, 4);
    std::memcpy(buf + 4, &d32, 4);
    std::memcpy(buf + 8, &seed, 4);
    uint64_t dseed = murmur64a(buf, 12, 0);
    int pv = permutation_element((uint32_t)digit, (uint32_t)base, (uint32_t)dseed);
    rev = rev * (uint64_t)base + (uint64_t)pv;
    invBaseM *= invBase;
    ++di;
    a = next;
  }
  return std::min(invBaseM * (double)rev, std::nextafter(1.0, 0.0));
}

// HaltonSampler::SampleDimension (sampler.hpp:54-73)
inline float halton_sample(int strategy, uint32_t seed, int dim, uint32_t index) {
  if (strategy == 0) return (float)radical_inverse(dim, index);
  if (strategy == 1) {
    if (dim >= 25) return (float)radical_inverse(dim, index);
    return (float)permuted_radical_inverse(dim, index, seed);
  }
  return (float)owen_radical_inverse(dim, index, (uint32_t)mix_bits(1u + ((uint32_t)dim << 4)));
}

// The build's counter-based replacement of gl::rand_num (SplitMix64 output
// function over key ^ slot * constant, 24 bits).
inline uint64_t splitmix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
inline float rand01(uint64_t key, uint32_t slot) {
  uint64_t h = splitmix64(key ^ ((uint64_t)slot * 0xd1b54a32d192ed03ull));
  return (float)(h >> 40) * (1.0f / 16777216.0f);
}
inline uint64_t path_key(uint32_t seed, uint64_t sample_id) {
  return splitmix64(((uint64_t)seed << 40) ^ sample_id);
}

}  // namespace orc
