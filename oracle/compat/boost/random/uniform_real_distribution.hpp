// Boost-API shim (oracle test infrastructure): uniform_real_distribution.
// For a 64-bit integer engine: u = x * 2^-64 * (b - a) + a, redrawn when it
// rounds up to b.
#pragma once
#include <cstdint>

namespace boost {
namespace random {
template <class RealType = double>
class uniform_real_distribution {
 public:
  explicit uniform_real_distribution(RealType a = RealType(0), RealType b = RealType(1)) : a_(a), b_(b) {}
  template <class Engine>
  RealType operator()(Engine &eng) const {
    for (;;) {
      const RealType u = static_cast<RealType>(eng() - (Engine::min)()) * RealType(5.421010862427522170037264e-20);
      const RealType r = u * (b_ - a_) + a_;
      if (r < b_) return r;
    }
  }

 private:
  RealType a_, b_;
};
}  // namespace random
}  // namespace boost
