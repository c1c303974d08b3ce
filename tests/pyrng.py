"""Independent pure-Python (big-int) xoshiro256++ / splitmix64 / jump, used to
pin the engine's and the oracle's random streams bit for bit.

Algorithms as published by Blackman & Vigna (xoshiro256++ 1.0, splitmix64);
the jump polynomial is re-derived from the generator itself with
Berlekamp-Massey instead of being copied, and checked against the published
jump() constants.
"""
M64 = (1 << 64) - 1
JUMP = (0x180ec6d33cfd0aba, 0xd5a61266f0c9392c, 0xa9582618e03fc9aa, 0x39abdc4529b1661c)


def rotl(x, k):
    return ((x << k) | (x >> (64 - k))) & M64


def seed_state(seed):
    x = seed & M64
    out = []
    for _ in range(4):
        x = (x + 0x9e3779b97f4a7c15) & M64
        z = x
        z = ((z ^ (z >> 30)) * 0xbf58476d1ce4e5b9) & M64
        z = ((z ^ (z >> 27)) * 0x94d049bb133111eb) & M64
        out.append(z ^ (z >> 31))
    return out


def step(s):
    a, b, c, d = s
    t = (b << 17) & M64
    c ^= a
    d ^= b
    b ^= c
    a ^= d
    c ^= t
    d = rotl(d, 45)
    return [a, b, c, d]


def next_out(s):
    out = (rotl((s[0] + s[3]) & M64, 23) + s[0]) & M64
    return out, step(s)


def jump(s, poly=JUMP):
    acc = [0, 0, 0, 0]
    for w in poly:
        for b in range(64):
            if (w >> b) & 1:
                acc = [x ^ y for x, y in zip(acc, s)]
            s = step(s)
    return acc


def stream_state(seed, k):
    s = seed_state(seed)
    for _ in range(k):
        s = jump(s)
    return s


def derive_jump_poly():
    """x^(2^128) mod the characteristic polynomial of the state transition."""
    s = seed_state(0)
    seq = []
    for _ in range(512):
        seq.append(s[0] & 1)
        s = step(s)
    C, B, L, m = 1, 1, 0, 1
    for n in range(512):
        d = seq[n]
        for i in range(1, L + 1):
            if (C >> i) & 1:
                d ^= seq[n - i]
        if d == 0:
            m += 1
        elif 2 * L <= n:
            T = C
            C ^= B << m
            L = n + 1 - L
            B = T
            m = 1
        else:
            C ^= B << m
            m += 1
    p = 0
    for j in range(L + 1):
        if (C >> (L - j)) & 1:
            p |= 1 << j

    def mulmod(a, b):
        r = 0
        while b:
            if b & 1:
                r ^= a
            b >>= 1
            a <<= 1
            if (a >> L) & 1:
                a ^= p
        return r

    r = 2
    for _ in range(128):
        r = mulmod(r, r)
    return L, tuple((r >> (64 * i)) & M64 for i in range(4))
