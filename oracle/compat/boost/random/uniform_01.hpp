// Boost-API shim (oracle test infrastructure): uniform_01 = x * 2^-64, < 1.
#pragma once
namespace boost {
namespace random {
template <class RealType = double>
class uniform_01 {
 public:
  template <class Engine>
  RealType operator()(Engine &eng) const {
    for (;;) {
      const RealType u = static_cast<RealType>(eng() - (Engine::min)()) * RealType(5.421010862427522170037264e-20);
      if (u < RealType(1)) return u;
    }
  }
};
}  // namespace random
}  // namespace boost
