// Compiles: the pricers' fifth template parameter names the random engine, as in
// the reference (MonteCarloPricer.hpp:86), spelled with the drop-in's tag or with
// Boost's xoshiro256pp where Boost's header is on the include path.
#include "myql_gpu/MonteCarloPricer.hpp"
using namespace myql_gpu;
using Eur = EuropeanOption<PayoffVanilla<OptionType::Call>>;
int main() {
  HestonModel m(HestonParams{1.5, 0.04, 0.3, -0.7, 0.04});
  std::vector<double> s;
  MonteCarloPricer<HestonModel, HestonStepper<SchemeNV>, Eur, GreekMode::None, xoshiro256pp> a(m, MonteCarloConfig{});
  a.job(100.0, 0.02, 0.0, Eur(100.0, 1.0), s);
#ifdef MYQL_GPU_HAVE_BOOST_XOSHIRO
  MonteCarloPricer<HestonModel, HestonStepper<SchemeNV>, Eur, GreekMode::Essential, boost::random::xoshiro256pp> b(
      m, MonteCarloConfig{});
  b.job(100.0, 0.02, 0.0, Eur(100.0, 1.0), s);
  MultiLevelMonteCarloPricer<HestonModel, CoupledHestonStepper<SchemeNV>, Eur, GreekMode::None,
                             boost::random::xoshiro256pp>
      c(m, MLMCConfig{});
  (void)c;
#else
#error "this check is compiled with a Boost-API xoshiro header on the include path"
#endif
  return 0;
}
