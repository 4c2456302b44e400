// Host check of the sampler arithmetic in pt_common.cuh against the plain
// forms it replaces: division by a Halton base as a multiply-high by a
// precomputed reciprocal (div_invariant / div_prime), Kensler's permutation
// of {0, 1} as one parity bit of the hash, and the Owen-scrambled radical
// inverse with its early termination -- each against the straightforward
// computation (hardware division, permutation_element's modulo, every
// digit).  Prints one line per check and exits non-zero on a mismatch.
#include "../../pathtracer_gb300/csrc/pt_common.cuh"

#include <cstdio>

using namespace pt;

static const int kPrimes[PT_PRIME_COUNT] = {2,  3,  5,  7,  11, 13, 17, 19, 23, 29, 31, 37, 41,
                                            43, 47, 53, 59, 61, 67, 71, 73, 79, 83, 89, 97};

// The tables the library uploads (digit counts and radix powers as the
// reference's double loop computes them; reciprocals; early-exit points).
static HaltonTables tables() {
  HaltonTables T{};
  for (int b = 0; b < PT_PRIME_COUNT; ++b) {
    const int base = kPrimes[b];
    T.prime[b] = base;
    double m = 1.0;
    int nd = 0;
    while (1.0 - (base - 1) * m < 1.0) {
      ++nd;
      m *= 1.0 / (double)base;
    }
    T.ndigits[b] = nd;
    T.inv_base_m[b] = m;
    div_invariant((uint32_t)base, T.div_magic[b], T.div_shift[b]);
    int check = 0;
    for (uint64_t p = 1; p < (1ull << 38) && check < nd; p *= (uint64_t)base) ++check;
    uint64_t tail = 1;
    for (int r = check; r < nd; ++r) tail *= (uint64_t)base;
    T.owen_check[b] = check;
    T.owen_tail[b] = tail;
  }
  return T;
}

// Every digit, hardware division and permutation_element's own modulo.
static float owen_plain(const HaltonTables &T, int dim, uint32_t index) {
  const int bi = dim % PT_PRIME_COUNT;
  const uint32_t base = (uint32_t)T.prime[bi];
  const uint32_t hash = (uint32_t)mix_bits(1u + ((uint32_t)dim << 4));
  uint32_t a = index;
  uint64_t rev = 0;
  for (int di = 0; di < T.ndigits[bi]; ++di) {
    const uint32_t next = a / base;
    uint32_t digit = a - next * base;
    const uint32_t dh = (uint32_t)mix_bits(hash ^ (uint32_t)rev ^ ((uint32_t)di << 16));
    digit = permutation_element(digit, base, dh);
    rev = rev * base + digit;
    a = next;
  }
  return clamp_to_float(xdmul(T.inv_base_m[bi], (double)rev));
}

int main() {
  const HaltonTables T = tables();
  long long bad = 0, n = 0;
  // 1. a / p for the lowest and highest 2^20 operands and 2^22 hashed ones
  for (int b = 0; b < PT_PRIME_COUNT; ++b) {
    const uint32_t p = (uint32_t)kPrimes[b];
    for (uint64_t k = 0; k < (1u << 20); ++k) {
      const uint32_t lo = (uint32_t)k, hi = 0xffffffffu - (uint32_t)k;
      const uint32_t mid = (uint32_t)splitmix64(k * 25 + b);
      bad += div_prime(T, b, lo) != lo / p;
      bad += div_prime(T, b, hi) != hi / p;
      bad += div_prime(T, b, mid) != mid / p;
      n += 3;
    }
  }
  printf("div_prime: %lld mismatches in %lld operands\n", bad, n);
  long long bad2 = 0;
  // 2. Kensler's permutation of {0, 1}
  for (uint64_t k = 0; k < (1u << 22); ++k) {
    const uint32_t h = (uint32_t)splitmix64(k);
    for (uint32_t d = 0; d < 2; ++d)
      bad2 += permutation_element(d, 2, h) != (d ^ (((h >> 8) ^ (h >> 16) ^ (h >> 23)) & 1u));
  }
  printf("base-2 permutation: %lld mismatches\n", bad2);
  long long bad3 = 0, n3 = 0;
  // 3. the Owen-scrambled radical inverse against every digit
  for (int dim = 0; dim < 100; ++dim)
    for (uint64_t k = 0; k < (1u << 15); ++k) {
      const uint32_t idx = k < (1u << 14) ? (uint32_t)k : (uint32_t)splitmix64(k * 131 + dim);
      const float x = owen_radical_inverse(T, dim, idx), y = owen_plain(T, dim, idx);
      bad3 += std::memcmp(&x, &y, 4) != 0;
      ++n3;
    }
  printf("owen_radical_inverse: %lld mismatches in %lld values\n", bad3, n3);
  return (bad || bad2 || bad3) ? 1 : 0;
}
