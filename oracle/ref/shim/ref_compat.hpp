// Portability shim force-included (-include) into every translation unit of
// the reference build.  It changes no arithmetic of the reference: it only
// supplies library names that GCC 13 / libstdc++ 13 in C++17 mode lack, and
// one clamp overload for a mixed double/float call the reference makes.
#pragma once
#include <cmath>
#include <cstring>
#include <functional>
#include <memory>
#include <optional>
#include <random>
#include <algorithm>
#include <type_traits>
namespace std {
using ::logf;
#if __cplusplus < 202002L
template <class To, class From>
inline To bit_cast(const From &src) noexcept {
  static_assert(sizeof(To) == sizeof(From), "bit_cast size mismatch");
  To dst;
  std::memcpy(&dst, &src, sizeof(To));
  return dst;
}
#endif
// pattern.hpp calls std::clamp(fabs(float), 0.f, 1.f) with a double first
// argument; Apple's libc++ resolves fabs(float) to float there.
inline float clamp(double v, float lo, float hi) {
  float f = (float)v;
  return f < lo ? lo : (hi < f ? hi : f);
}
}  // namespace std
