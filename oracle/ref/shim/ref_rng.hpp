// Reproducibility shim force-included into every translation unit of the
// reference build (oracle infrastructure only).  The reference draws
// gl::rand_num() from `static std::mt19937 gen(rd())` declared in a header
// (include/utils/utility.hpp:540-547): one generator per translation unit,
// seeded from std::random_device and shared by all threads.  This shim keeps
// the engine type and the distribution code of the reference but routes every
// such generator to ONE thread-local std::mt19937 that the harness seeds, so a
// run is reproducible and thread-safe.  It must be included after <random>.
#pragma once
#include <cstdint>
#include <random>
inline thread_local std::mt19937 pt_ref_tls_engine(5489u);
namespace std {
struct pt_ref_tls_mt19937 {
  using result_type = std::mt19937::result_type;
  static constexpr result_type min() { return std::mt19937::min(); }
  static constexpr result_type max() { return std::mt19937::max(); }
  explicit pt_ref_tls_mt19937(result_type = 5489u) {}
  result_type operator()() { return pt_ref_tls_engine(); }
};
}  // namespace std
#define mt19937 pt_ref_tls_mt19937
