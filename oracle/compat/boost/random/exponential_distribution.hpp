// Boost-API shim (oracle test infrastructure): exponential_distribution(rate)
// by inversion, -log(1 - U) / rate, one uniform draw.
#pragma once
#include <cmath>
#include <boost/random/uniform_01.hpp>

namespace boost {
namespace random {
template <class RealType = double>
class exponential_distribution {
 public:
  explicit exponential_distribution(RealType lambda = RealType(1)) : lambda_(lambda) {}
  template <class Engine>
  RealType operator()(Engine &eng) const {
    return -std::log(RealType(1) - uniform_01<RealType>()(eng)) / lambda_;
  }

 private:
  RealType lambda_;
};
}  // namespace random
}  // namespace boost
