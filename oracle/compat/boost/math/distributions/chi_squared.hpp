// Boost-API shim (oracle test infrastructure): chi_squared_distribution and
// quantile(), computed by the oracle's FP64 incomplete-gamma inversion.
#pragma once
#include "chi2.h"

namespace boost {
namespace math {
template <class RealType = double>
class chi_squared_distribution {
 public:
  explicit chi_squared_distribution(RealType dof) : dof_(dof) {}
  RealType degrees_of_freedom() const { return dof_; }

 private:
  RealType dof_;
};
template <class RealType>
RealType quantile(const chi_squared_distribution<RealType> &d, RealType p) {
  return oracle_chi2_quantile(d.degrees_of_freedom(), p);
}
}  // namespace math
}  // namespace boost
