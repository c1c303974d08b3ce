"""CPU checks of the SchemeNCI cell rules (the device's nci_cells_main_kernel restated in
numpy on scipy's quantile nodes): the mean of the chi-squared draw that the cells give,
integrated exactly, against the exact conditional mean.

* the reference's cells (harmonic-mean slopes, VolSchemes.hpp:292-310, first cell a cubic from
  y(0) = 0) fall short of the mean by 1e-5 to 4e-5 relative for many degrees of freedom;
* the opt-in cells (exact slopes 1 / f(y), a first cell that keeps the exact mean of [0, dx])
  integrate to it within 1e-7.
"""
import numpy as np
import pytest
from scipy import special, stats

D = 0.4938271604938271       # the Bates strip's 4 kappa theta / sigma^2
G = 10000
DX = 0.999 / (G - 1)


def cells(nu, exact):
    u = np.arange(G) * DX
    y = stats.chi2.ppf(u, nu)
    y[0] = 0.0
    if exact:
        m = np.empty(G)
        m[0] = (y[1] - y[0]) / DX
        m[1:] = np.exp(-stats.chi2.logpdf(y[1:], nu))
    else:
        d1 = np.diff(y) / DX
        m = np.empty(G)
        m[0], m[-1] = d1[0], d1[-1]
        a, b = d1[:-1], d1[1:]
        m[1:-1] = np.where(a * b > 0, 2 * a * b / (a + b), 0.0)
    h0, h1 = DX * m[:-1], DX * m[1:]
    c = [y[:-1].copy(), h0.copy(), 3 * (y[1:] - y[:-1]) - 2 * h0 - h1, 2 * (y[:-1] - y[1:]) + h0 + h1]
    if exact and nu >= D + 8:
        a_ = 0.5 * nu + 1.0
        mean = nu * special.gammainc(a_, 0.5 * y[1]) / DX
        q = 3 * (mean - y[1] + 0.5 * h1[0])
        c[0][0], c[1][0], c[2][0], c[3][0] = y[1] - h1[0] + q, h1[0] - 2 * q, q, 0.0
    return [np.asarray(x, dtype=np.float32).astype(np.float64) for x in c]


def cells_mean_rel_error(nu, exact):
    c0, c1, c2, c3 = cells(nu, exact)
    got = DX * np.sum(c0 + c1 / 2 + c2 / 3 + c3 / 4)
    want = nu * stats.chi2.cdf(stats.chi2.ppf(0.999, nu), nu + 2)   # int_0^0.999 Q(u) du
    return (got - want) / nu


@pytest.mark.parametrize("row", [25, 100, 1000])
def test_reference_cells_fall_short_of_the_mean(row):
    err = cells_mean_rel_error(D + 2 * row, exact=False)
    assert -5e-5 < err < -1e-5, err


@pytest.mark.parametrize("row", [0, 5, 25, 100, 1000])
def test_exact_cells_keep_the_mean(row):
    assert abs(cells_mean_rel_error(D + 2 * row, exact=True)) < 1e-7


def test_exact_first_cell_is_monotone_and_positive():
    for row in (4, 25, 1000):
        c0, c1, c2, c3 = cells(D + 2 * row, exact=True)
        t = np.linspace(0, 1, 101)
        v = c0[0] + t * (c1[0] + t * (c2[0] + t * c3[0]))
        assert v[0] > 0 and np.all(np.diff(v) >= 0)
