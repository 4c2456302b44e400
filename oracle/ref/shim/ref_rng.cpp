// Seeds the thread-local engine behind gl::rand_num (see ref_rng.hpp).
#include <cstdint>
#include <random>
#include "ref_rng.hpp"
extern "C" void ref_rng_seed(uint64_t seed) {
  std::seed_seq seq{(uint32_t)seed, (uint32_t)(seed >> 32)};
  pt_ref_tls_engine.seed(seq);
}
