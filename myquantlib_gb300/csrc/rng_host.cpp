// rng_host.cpp -- GF(2) polynomial machinery for xoshiro256 jump-ahead.
#include "rng_host.h"

#include <cstring>
#include <vector>

namespace myql {

uint64_t splitmix64_next(uint64_t &x) {
  uint64_t z = (x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

XoState xo_seed(uint64_t seed) {
  XoState st;
  uint64_t x = seed;
  for (int i = 0; i < 4; ++i) st.s[i] = splitmix64_next(x);
  return st;
}

static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

void xo_step(XoState &st) {
  uint64_t *s = st.s;
  const uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl(s[3], 45);
}

uint64_t xo_next_host(XoState &st) {
  const uint64_t out = rotl(st.s[0] + st.s[3], 23) + st.s[0];
  xo_step(st);
  return out;
}

void xo_apply_poly(XoState &st, const uint64_t poly[4]) {
  uint64_t acc[4] = {0, 0, 0, 0};
  for (int w = 0; w < 4; ++w)
    for (int b = 0; b < 64; ++b) {
      if ((poly[w] >> b) & 1ull)
        for (int j = 0; j < 4; ++j) acc[j] ^= st.s[j];
      xo_step(st);
    }
  std::memcpy(st.s, acc, sizeof acc);
}

namespace {
// 512-bit polynomials over GF(2), little-endian words.
struct P512 {
  uint64_t w[9] = {0};
  bool bit(int i) const { return (w[i >> 6] >> (i & 63)) & 1ull; }
  void flip(int i) { w[i >> 6] ^= 1ull << (i & 63); }
};

P512 mulmod(const P512 &a, const P512 &b, const P512 &p, int deg) {
  // schoolbook carry-less product, then reduction by p (degree deg)
  P512 r;
  for (int i = 0; i < deg; ++i)
    if (b.bit(i))
      for (int j = 0; j < deg; ++j)
        if (a.bit(j)) r.flip(i + j);
  for (int k = 2 * deg - 2; k >= deg; --k)
    if (r.bit(k))
      for (int j = 0; j <= deg; ++j)
        if (p.bit(j)) r.flip(k - deg + j);
  return r;
}
}  // namespace

bool xo_jump_polys(uint64_t polys[][4], int count) {
  // Berlekamp-Massey on bit 0 of s0 along the transition.
  const int N = 512;
  std::vector<int> seq(N);
  XoState st = xo_seed(0);
  for (int n = 0; n < N; ++n) {
    seq[n] = (int)(st.s[0] & 1ull);
    xo_step(st);
  }
  std::vector<int> C(N + 1, 0), B(N + 1, 0), T;
  C[0] = B[0] = 1;
  int L = 0, m = 1;
  for (int n = 0; n < N; ++n) {
    int d = seq[n];
    for (int i = 1; i <= L; ++i) d ^= C[i] & seq[n - i];
    if (d == 0) {
      ++m;
    } else if (2 * L <= n) {
      T = C;
      for (int i = 0; i + m <= N; ++i) C[i + m] ^= B[i];
      L = n + 1 - L;
      B = T;
      m = 1;
    } else {
      for (int i = 0; i + m <= N; ++i) C[i + m] ^= B[i];
      ++m;
    }
  }
  if (L != 256) return false;
  P512 p;
  for (int j = 0; j <= L; ++j)
    if (C[L - j]) p.flip(j);
  P512 r;
  r.flip(1);  // x
  for (int k = 0; k < 128; ++k) r = mulmod(r, r, p, L);
  for (int i = 0; i < count; ++i) {
    for (int w = 0; w < 4; ++w) polys[i][w] = r.w[w];
    r = mulmod(r, r, p, L);
  }
  static const uint64_t kPublished[4] = {0x180ec6d33cfd0abaull, 0xd5a61266f0c9392cull,
                                         0xa9582618e03fc9aaull, 0x39abdc4529b1661cull};
  return std::memcmp(polys[0], kPublished, sizeof kPublished) == 0;
}

}  // namespace myql
