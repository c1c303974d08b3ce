// Must not compile: the GPU engine has xoshiro256++ streams only, so another
// random engine in the pricer's RNG parameter is a compile-time error.
#include <random>

#include "myql_gpu/MonteCarloPricer.hpp"
using namespace myql_gpu;
using Eur = EuropeanOption<PayoffVanilla<OptionType::Call>>;
int main() {
  HestonModel m(HestonParams{1.5, 0.04, 0.3, -0.7, 0.04});
  MonteCarloPricer<HestonModel, HestonStepper<SchemeNV>, Eur, GreekMode::None, std::mt19937_64> p(m, MonteCarloConfig{});
  (void)p;
  return 0;
}
