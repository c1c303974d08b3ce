// Must not compile: a Bates stepper (Merton jumps) for a Heston model (no jumps),
// the reference's compile-time error.
#include "myql_gpu/MonteCarloPricer.hpp"
using namespace myql_gpu;
int main() {
  HestonModel m(HestonParams{1.5, 0.04, 0.3, -0.7, 0.04});
  std::vector<double> s;
  MonteCarloPricer<HestonModel, BatesStepper<SchemeNV>, EuropeanOption<PayoffVanilla<OptionType::Call>>> p(
      m, MonteCarloConfig{});
  p.job(100.0, 0.02, 0.0, EuropeanOption<PayoffVanilla<OptionType::Call>>(100.0, 1.0), s);
  return 0;
}
