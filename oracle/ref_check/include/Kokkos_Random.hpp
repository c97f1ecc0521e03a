// Kokkos_Random.hpp -- TEST INFRASTRUCTURE.  Serial stand-in for the random
// pool used by the reference's H84/C91 initial conditions (Init.h:15,
// 146-148, 170-172).  Those draws are not reproducible across Kokkos
// back-ends, so this stand-in only has to be deterministic: a 64-bit
// xorshift (Marsaglia 2003) advanced per draw.
#pragma once
#include <cstdint>
#include <memory>
#include "Kokkos_Core.hpp"

namespace Kokkos {
template <class Device = void>
class Random_XorShift64_Pool {
 public:
  struct generator {
    std::shared_ptr<uint64_t> s;
    double drand(double a, double b) {
      uint64_t x = *s;
      x ^= x << 13;
      x ^= x >> 7;
      x ^= x << 17;
      *s = x;
      return a + (b - a) * (double)(x >> 11) * 0x1.0p-53;
    }
  };
  explicit Random_XorShift64_Pool(uint64_t seed = 1) : s_(std::make_shared<uint64_t>(seed ? seed : 1)) {}
  generator get_state() const { return generator{s_}; }
  void free_state(const generator &) const {}

 private:
  std::shared_ptr<uint64_t> s_;
};
}  // namespace Kokkos
