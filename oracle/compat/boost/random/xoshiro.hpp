// Boost-API shim (oracle test infrastructure): boost::random::xoshiro256pp.
// xoshiro256++ (Blackman & Vigna) seeded from one 64-bit value with splitmix64,
// the generator the reference instantiates (MonteCarloPricer.hpp:86,191).
#pragma once
#include <cstdint>
#include <limits>

namespace boost {
namespace random {
class xoshiro256pp {
 public:
  using result_type = std::uint64_t;
  explicit xoshiro256pp(result_type value = 0) { seed(value); }
  void seed(result_type value) {
    std::uint64_t x = value;
    for (auto &w : s_) {
      std::uint64_t z = (x += 0x9e3779b97f4a7c15ull);
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
      w = z ^ (z >> 31);
    }
  }
  static constexpr result_type min() { return 0; }
  static constexpr result_type max() { return std::numeric_limits<result_type>::max(); }
  result_type operator()() {
    const std::uint64_t out = rotl(s_[0] + s_[3], 23) + s_[0];
    const std::uint64_t t = s_[1] << 17;
    s_[2] ^= s_[0];
    s_[3] ^= s_[1];
    s_[1] ^= s_[2];
    s_[0] ^= s_[3];
    s_[2] ^= t;
    s_[3] = rotl(s_[3], 45);
    return out;
  }

 private:
  static std::uint64_t rotl(std::uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  std::uint64_t s_[4];
};
}  // namespace random
}  // namespace boost
