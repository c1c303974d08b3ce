// Boost-API shim (oracle test infrastructure): poisson_distribution by
// sequential inversion of one uniform_01 draw (Boost's method for means below
// 10; used here for every mean).
#pragma once
#include <cmath>
#include <boost/random/uniform_01.hpp>

namespace boost {
namespace random {
template <class IntType = int, class RealType = double>
class poisson_distribution {
 public:
  explicit poisson_distribution(RealType mean = RealType(1)) : mean_(mean), exp_mean_(std::exp(-mean)) {}
  template <class Engine>
  IntType operator()(Engine &eng) const {
    RealType p = exp_mean_;
    IntType x = 0;
    RealType u = uniform_01<RealType>()(eng);
    while (u > p) {
      u = u - p;
      ++x;
      p = mean_ * p / x;
    }
    return x;
  }
  RealType mean() const { return mean_; }

 private:
  RealType mean_, exp_mean_;
};
}  // namespace random
}  // namespace boost
