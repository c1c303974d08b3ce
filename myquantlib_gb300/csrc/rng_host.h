// rng_host.h -- host side of the xoshiro256++ stream layout.
//
// A stream index k maps to the generator seeded from one 64-bit seed with
// splitmix64 (four successive outputs become s0..s3), advanced by k * 2^128
// steps.  An advance by 2^(128+i) steps is the linear map x^(2^(128+i)) mod p(x)
// applied to the state, p the characteristic polynomial of the xoshiro256
// state transition over GF(2).  p is recovered here with Berlekamp-Massey
// from 512 output bits of the transition itself, and the i = 0 polynomial
// equals the published jump() constants of xoshiro256 (checked at start-up).
#pragma once
#include <cstdint>

namespace myql {

struct XoState {
  uint64_t s[4];
};

uint64_t splitmix64_next(uint64_t &x);
XoState xo_seed(uint64_t seed);
void xo_step(XoState &st);         // state transition only
uint64_t xo_next_host(XoState &st);  // xoshiro256++ output + transition

// polys[i][0..3] = coefficients of x^(2^(128+i)) mod p, bit j of word w = x^(64w+j).
// Returns false if the derived i = 0 polynomial differs from the published jump().
bool xo_jump_polys(uint64_t polys[][4], int count);

// Applies a jump polynomial to a state (Vigna's jump loop).
void xo_apply_poly(XoState &st, const uint64_t poly[4]);

}  // namespace myql
