"""Derives the coefficients of the device inverse-normal central polynomial.

    z = Phi^-1(p) = (p - 1/2) * R(w),   w = -log(4 p (1 - p)),   0 <= w <= 6

R is fitted by Chebyshev least squares (near-minimax) of degree 10 to
Phi^-1 evaluated with mpmath at 40 digits; its FP32 Horner evaluation has a
relative error of about 1.3e-7 over p in [6.2e-4, 1 - 6.2e-4].  The variable w
is bounded and smooth where (p - 1/2) approaches +-1/2, so the coefficients
stay small and the FP32 evaluation is well conditioned (Acklam's double
precision rational loses ~1e-4 there in FP32).  Outside that range the kernel
uses Acklam's tail rational in sqrt(-2 log min(p, 1-p)).

Run:  python myquantlib_gb300/csrc/fit_inverse_normal.py   (needs mpmath)
"""
import numpy as np
import mpmath as mp

mp.mp.dps = 40
WMAX, DEG = 6.0, 10


def main():
    ws = (1 - np.cos(np.linspace(0, np.pi, 6001))) / 2 * WMAX
    R = []
    for w in ws:
        if w < 1e-30:
            R.append(float(mp.sqrt(2 * mp.pi)))
            continue
        p = (1 - mp.sqrt(1 - mp.e ** (-mp.mpf(w)))) / 2
        z = mp.sqrt(2) * mp.erfinv(2 * p - 1)
        R.append(float(z / (p - mp.mpf(1) / 2)))
    R = np.array(R)
    cheb = np.polynomial.chebyshev.chebfit(ws / WMAX * 2 - 1, R, DEG)
    P = np.polynomial.Polynomial(np.polynomial.chebyshev.cheb2poly(cheb))
    coef = P(np.polynomial.Polynomial([-1.0, 2.0 / WMAX])).coef  # powers of w
    acc = np.float32(coef[-1])
    w32 = ws.astype(np.float32)
    for c in coef[-2::-1]:
        acc = (acc * w32 + np.float32(c)).astype(np.float32)
    print("fp32 max rel err %.3e" % np.max(np.abs(acc - R) / R))
    print("highest power first:")
    for c in coef[::-1]:
        print("  %.9ef," % c)


if __name__ == "__main__":
    main()
