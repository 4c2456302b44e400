// pt_common.cuh -- vector math, counter-based RNG and the Halton-family
// samplers shared by every kernel of the wavefront path integrator.
//
// Host+device functions.  Where the reference's result must be reproduced
// bit for bit (sampler sequences, ray/primitive tests) the arithmetic is
// written with explicitly rounded operations so that no multiply-add is
// contracted; everywhere else ordinary float arithmetic (FMA allowed) is used
// and parity is held to the 1e-4 relative bar of the BSDF tests.
#pragma once
#include <cstdint>
#include <cfloat>
#include <cmath>
#include <cstring>

#if defined(__CUDACC__)
#define PT_HD __host__ __device__ __forceinline__
#else
#define PT_HD inline
#endif

#ifndef PT_PI
#define PT_PI 3.14159265358979323846
#endif
#define PT_INV_PI_F 0.318309886183790671538f

namespace pt {

#if !defined(__CUDACC__)
using std::isinf;
#endif

// ------------------------------------------------------ exact arithmetic
// Rounded single-precision operations that are never fused.
#if defined(__CUDA_ARCH__)
PT_HD float xmul(float a, float b) { return __fmul_rn(a, b); }
PT_HD float xadd(float a, float b) { return __fadd_rn(a, b); }
PT_HD float xsub(float a, float b) { return __fsub_rn(a, b); }
PT_HD float xdiv(float a, float b) { return __fdiv_rn(a, b); }
PT_HD float xsqrt(float a) { return __fsqrt_rn(a); }
PT_HD double xdmul(double a, double b) { return __dmul_rn(a, b); }
#else
PT_HD float xmul(float a, float b) { return a * b; }
PT_HD float xadd(float a, float b) { return a + b; }
PT_HD float xsub(float a, float b) { return a - b; }
PT_HD float xdiv(float a, float b) { return a / b; }
PT_HD float xsqrt(float a) { return std::sqrt(a); }
PT_HD double xdmul(double a, double b) { return a * b; }
#endif

// sin/cos of pi*x and of x (device intrinsics; libm on the host).
PT_HD void sincospi_(float x, float *s, float *c) {
#if defined(__CUDA_ARCH__)
  sincospif(x, s, c);
#else
  *s = sinf(x * (float)PT_PI);
  *c = cosf(x * (float)PT_PI);
#endif
}
PT_HD void sincos_(float x, float *s, float *c) {
#if defined(__CUDA_ARCH__)
  sincosf(x, s, c);
#else
  *s = sinf(x);
  *c = cosf(x);
#endif
}

PT_HD uint32_t f2u(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}
PT_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}

// ------------------------------------------------------------ float3
struct V3 {
  float x, y, z;
};
PT_HD V3 v3(float x, float y, float z) { return V3{x, y, z}; }
PT_HD V3 v3(float s) { return V3{s, s, s}; }
PT_HD V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
PT_HD V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
PT_HD V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
PT_HD V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
PT_HD V3 operator*(float s, V3 a) { return V3{a.x * s, a.y * s, a.z * s}; }
PT_HD V3 operator*(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
PT_HD V3 operator/(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
PT_HD V3 operator/(V3 a, V3 b) { return V3{a.x / b.x, a.y / b.y, a.z / b.z}; }
PT_HD V3 &operator+=(V3 &a, V3 b) { a = a + b; return a; }
PT_HD V3 &operator*=(V3 &a, V3 b) { a = a * b; return a; }
PT_HD V3 &operator*=(V3 &a, float s) { a = a * s; return a; }
PT_HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
PT_HD V3 cross(V3 a, V3 b) {
  return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
PT_HD float length(V3 a) { return sqrtf(dot(a, a)); }
// gl::vec::normalize (matrix.hpp:337-343): each component divided by the length.
PT_HD V3 normalize(V3 a) {
  float l = length(a);
  return V3{a.x / l, a.y / l, a.z / l};
}
PT_HD float max_comp(V3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
PT_HD bool near_zero(V3 a) { return fabsf(a.x) < 1e-6f && fabsf(a.y) < 1e-6f && fabsf(a.z) < 1e-6f; }

// Exact (never fused) forms in the reference's operation order:
// dot = ((0 + a0*b0) + a1*b1) + a2*b2 (matrix.hpp:553-559),
// cross = a1*b2 - a2*b1 ... (matrix.hpp:571-579).
PT_HD float xdot(V3 a, V3 b) {
  return xadd(xadd(xmul(a.x, b.x), xmul(a.y, b.y)), xmul(a.z, b.z));
}
PT_HD V3 xcross(V3 a, V3 b) {
  return V3{xsub(xmul(a.y, b.z), xmul(a.z, b.y)), xsub(xmul(a.z, b.x), xmul(a.x, b.z)),
            xsub(xmul(a.x, b.y), xmul(a.y, b.x))};
}
PT_HD V3 xsubv(V3 a, V3 b) { return V3{xsub(a.x, b.x), xsub(a.y, b.y), xsub(a.z, b.z)}; }
PT_HD V3 xnormalize(V3 a) {
  float l = xsqrt(xdot(a, a));
  return V3{xdiv(a.x, l), xdiv(a.y, l), xdiv(a.z, l)};
}
// o + t*d with each product rounded before the add (Ray::at, ray.hpp:21).
PT_HD V3 xat(V3 o, V3 d, float t) {
  return V3{xadd(o.x, xmul(t, d.x)), xadd(o.y, xmul(t, d.y)), xadd(o.z, xmul(t, d.z))};
}

// Orthonormal basis around n (OrthoBasis, utils/orthoBasis.hpp:15-36).
struct Onb {
  V3 u, v, w;
};
PT_HD Onb make_onb(V3 n) {
  Onb b;
  b.w = normalize(n);
  V3 a = (fabsf(n.x) > 0.9f) ? v3(0.f, 1.f, 0.f) : v3(1.f, 0.f, 0.f);
  b.v = normalize(cross(b.w, a));
  b.u = cross(b.w, b.v);
  return b;
}
PT_HD V3 to_world(const Onb &b, V3 l) { return l.x * b.u + l.y * b.v + l.z * b.w; }
PT_HD V3 to_local(const Onb &b, V3 v) { return V3{dot(v, b.u), dot(v, b.v), dot(v, b.w)}; }

// ------------------------------------------------------------ hashing
// pbrt::mixBits (utils/hash.hpp:62-69): 64-bit finalizer of
// zimbry.blogspot.ch/2011/09 (variant 13 of Stafford's mixers).
PT_HD uint64_t mix_bits(uint64_t v) {
  v ^= (v >> 31);
  v *= 0x7fb5d329728ea185ull;
  v ^= (v >> 27);
  v *= 0x81dadef4bc2dd44dull;
  v ^= (v >> 33);
  return v;
}

// l - 1 with every bit below its highest set bit set.
PT_HD uint32_t fill_mask(uint32_t l) {
  uint32_t w = l - 1;
  w |= w >> 1;
  w |= w >> 2;
  w |= w >> 4;
  w |= w >> 8;
  w |= w >> 16;
  return w;
}

// The rejection loop of gl::permutationElement (utils/utility.hpp:434-464):
// Kensler's hashed permutation of [0, l) ("Correlated Multi-Jittered
// Sampling", 2013) before its final offset; w = fill_mask(l).
PT_HD uint32_t permutation_index(uint32_t i, uint32_t l, uint32_t w, uint32_t p) {
  do {
    i ^= p;
    i *= 0xe170893du;
    i ^= p >> 16;
    i ^= (i & w) >> 4;
    i ^= p >> 8;
    i *= 0x0929eb3fu;
    i ^= p >> 23;
    i ^= (i & w) >> 1;
    i *= 1u | p >> 27;
    i *= 0x6935fa69u;
    i ^= (i & w) >> 11;
    i *= 0x74dcb303u;
    i ^= (i & w) >> 2;
    i *= 0x9e501cc3u;
    i ^= (i & w) >> 2;
    i *= 0xc860a3dfu;
    i &= w;
    i ^= i >> 5;
  } while (i >= l);
  return i;
}

// gl::permutationElement: the permuted index, offset by p modulo l.
PT_HD uint32_t permutation_element(uint32_t i, uint32_t l, uint32_t p) {
  return (permutation_index(i, l, fill_mask(l), p) + p) % l;
}

// Counter-based uniform draws for everything the reference takes from
// gl::rand_num() (pixel-offset grid, lens, light pick, light-point jitter,
// Russian roulette).  SplitMix64's output function (Steele, Lea, Flood,
// OOPSLA 2014) over key ^ slot*golden; 24 high bits -> [0, 1).
PT_HD uint64_t splitmix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
PT_HD float rand01(uint64_t key, uint32_t slot) {
  uint64_t h = splitmix64(key ^ ((uint64_t)slot * 0xd1b54a32d192ed03ull));
  return (float)(h >> 40) * (1.0f / 16777216.0f);
}
PT_HD uint64_t path_key(uint32_t seed, uint64_t sample_id) {
  return splitmix64(((uint64_t)seed << 40) ^ sample_id);
}

// ------------------------------------------------------------ samplers
// Halton bases (gl::Primes, utility.hpp:400-402).  The reference indexes
// Primes[dim] without a bound (digitPerm.hpp:101), which is undefined for
// dim >= 25; this build defines it as Primes[dim % 25], the rule the
// unscrambled radicalInverse already uses (utility.hpp:408).
#define PT_PRIME_COUNT 25
struct HaltonTables {
  int32_t prime[PT_PRIME_COUNT];
  int32_t ndigits[PT_PRIME_COUNT];    // digits visited by the double loop test
  double inv_base_m[PT_PRIME_COUNT];  // invBase^ndigits, accumulated as the loop does
  int32_t perm_offset[PT_PRIME_COUNT];// into perm[] (PermuteDigits tables)
  // a / prime as a multiply-high and shifts (division by an invariant
  // integer, Granlund and Montgomery, PLDI 1994): magic 0 = power of two
  uint32_t div_magic[PT_PRIME_COUNT];
  int32_t div_shift[PT_PRIME_COUNT];  // shift; bit 6 set: the 33-bit (add) form
  // Owen-scrambled digits after which the value is tested for being settled
  // (the least k with prime^k >= 2^38), and prime^(ndigits - owen_check)
  int32_t owen_check[PT_PRIME_COUNT];
  uint64_t owen_tail[PT_PRIME_COUNT];
};

// The magic multiplier and shift of a / d for every 32-bit a (d >= 2):
// m = 2^(32 + floor(log2 d)) / d + 1 when that leaves an error below
// 2^floor(log2 d), else the 33-bit multiplier whose top bit the add form of
// div_prime supplies.
inline void div_invariant(uint32_t d, uint32_t &magic, int32_t &shift) {
  int l = 0;
  while ((d >> (l + 1)) != 0) ++l;  // floor(log2 d)
  if ((d & (d - 1)) == 0) {
    magic = 0;
    shift = l;
    return;
  }
  const uint64_t num = (uint64_t)1 << (32 + l);
  uint32_t m = (uint32_t)(num / d), rem = (uint32_t)(num % d);
  if (d - rem < (1u << l)) {
    shift = l;
  } else {
    m += m;
    const uint32_t twice = rem + rem;
    if (twice >= d || twice < rem) m += 1;
    shift = l | 64;
  }
  magic = m + 1;
}

// a / T.prime[bi] for every 32-bit a.
PT_HD uint32_t div_prime(const HaltonTables &T, int bi, uint32_t a) {
  const uint32_t m = T.div_magic[bi];
  const int s = T.div_shift[bi];
  if (!m) return a >> s;
#ifdef __CUDA_ARCH__
  const uint32_t q = __umulhi(m, a);
#else
  const uint32_t q = (uint32_t)(((uint64_t)m * a) >> 32);
#endif
  if (s & 64) return (((a - q) >> 1) + q) >> (s & 63);
  return q >> s;
}

// gl::radicalInverse (utility.hpp:406-420), float arithmetic.
PT_HD float radical_inverse(const HaltonTables &T, int dim, uint64_t a) {
  const int bi = dim % PT_PRIME_COUNT;
  const uint32_t base = (uint32_t)T.prime[bi];
  const float inv_base = xdiv(1.0f, (float)base);
  float inv_base_m = 1.0f;
  uint64_t rev = 0;
  while (a) {
    uint64_t next = a / base;
    uint64_t digit = a - next * base;
    rev = rev * base + digit;
    inv_base_m = xmul(inv_base_m, inv_base);
    a = next;
  }
  float r = xmul((float)rev, inv_base_m);
  const float one_minus_eps = 0x1.fffffep-1f;
  return r < one_minus_eps ? r : one_minus_eps;
}

PT_HD float clamp_to_float(double r) {
  const double one_minus_eps = 0x1.fffffffffffffp-1;
  return (float)(r < one_minus_eps ? r : one_minus_eps);
}

// gl::owenScrambledRadicalInverse (sampler/digitPerm.hpp:99-133) with the
// hash HaltonSampler passes (sampler.hpp:69-71).  The sample index is a
// uint32 in the reference, so the digit extraction runs on 32 bits.
//
// The value is rev * invBase^ndigits rounded to double and then to float,
// a non-decreasing function f of rev, and the digits still to come after
// the first k can only place rev in [rev_k * b^r, rev_k * b^r + b^r - 1]
// (r = ndigits - k).  Where f takes the same value at both ends, that is
// the result whatever the remaining digits are, so the loop stops there;
// after T.owen_check digits this settles all but a few in 10^4 samples
// (the rest run every digit as the reference does).
struct OwenDigits {
  uint32_t a;    // the index's digits not yet taken
  uint64_t rev;  // the scrambled digits so far, most significant first
};
template <bool BASE2>
PT_HD void owen_digit(const HaltonTables &T, int bi, uint32_t base, uint32_t w, uint32_t hash, int di,
                      OwenDigits &s) {
  const uint32_t dh = (uint32_t)mix_bits(hash ^ (uint32_t)s.rev ^ ((uint32_t)di << 16));
  if (BASE2) {
    // permutation_element(d, 2, p) = d ^ bit 0 of (p >> 8 ^ p >> 16 ^ p >> 23):
    // with w = 1 every odd multiplier keeps bit 0, every (i & w) >> k
    // shift is 0, the loop runs once and the final + p cancels p's bit 0
    // (checked for every p and d)
    const uint32_t digit = (s.a & 1u) ^ (((dh >> 8) ^ (dh >> 16) ^ (dh >> 23)) & 1u);
    s.rev = (s.rev << 1) | digit;
    s.a >>= 1;
  } else {
    const uint32_t next = div_prime(T, bi, s.a);
    const uint32_t digit = s.a - next * base;
    // permutation_element(digit, base, dh), its modulo by the base's divisor
    const uint32_t v = permutation_index(digit, base, w, dh) + dh;
    s.rev = s.rev * base + (v - div_prime(T, bi, v) * base);
    s.a = next;
  }
}
template <bool BASE2>
PT_HD float owen_digits(const HaltonTables &T, int bi, uint32_t hash, uint32_t index) {
  const uint32_t base = (uint32_t)T.prime[bi];
  const uint32_t w = fill_mask(base);
  const double scale = T.inv_base_m[bi];
  OwenDigits s{index, 0};
  const int nd = T.ndigits[bi], nc = T.owen_check[bi];
  int di = 0;
  for (; di < nc; ++di) owen_digit<BASE2>(T, bi, base, w, hash, di, s);
  const uint64_t lo = s.rev * T.owen_tail[bi];
  const float flo = clamp_to_float(xdmul(scale, (double)lo));
  if (flo == clamp_to_float(xdmul(scale, (double)(lo + (T.owen_tail[bi] - 1))))) return flo;
  for (; di < nd; ++di) owen_digit<BASE2>(T, bi, base, w, hash, di, s);
  return clamp_to_float(xdmul(scale, (double)s.rev));
}
PT_HD float owen_radical_inverse(const HaltonTables &T, int dim, uint32_t index) {
  const int bi = dim % PT_PRIME_COUNT;
  const uint32_t hash = (uint32_t)mix_bits(1u + ((uint32_t)dim << 4));
  return T.prime[bi] == 2 ? owen_digits<true>(T, bi, hash, index) : owen_digits<false>(T, bi, hash, index);
}

// gl::scrambledRadicalInverse with DigitPermutation tables
// (sampler/digitPerm.hpp:12-97); perm holds uint16 entries per base.
PT_HD float permuted_radical_inverse(const HaltonTables &T, const uint16_t *perm, int dim,
                                     uint32_t index) {
  if (dim >= PT_PRIME_COUNT) return radical_inverse(T, dim, index);  // sampler.hpp:60-63
  const uint32_t base = (uint32_t)T.prime[dim];
  const uint16_t *p = perm + T.perm_offset[dim];
  uint32_t a = index;
  uint64_t rev = 0;
  const int nd = T.ndigits[dim];
  for (int di = 0; di < nd; ++di) {
    uint32_t next = div_prime(T, dim, a);
    uint32_t digit = a - next * base;
    rev = rev * base + p[di * base + digit];
    a = next;
  }
  return clamp_to_float(xdmul(T.inv_base_m[dim], (double)rev));
}

}  // namespace pt
