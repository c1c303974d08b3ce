// Boost-API shim (oracle test infrastructure): declared for completeness; the
// reference includes it but draws its normals through Numerics::normcdfinv_as241.
#pragma once
namespace boost {
namespace random {
template <class RealType = double>
class normal_distribution {
 public:
  explicit normal_distribution(RealType mean = 0, RealType sigma = 1) : m_(mean), s_(sigma) {}

 private:
  RealType m_, s_;
};
}  // namespace random
}  // namespace boost
