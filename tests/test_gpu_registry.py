"""GPU tests of the record front-end: a mixed list of records priced through
registry.price_records (one persistent batch for the scalar None / Essential requests,
price_mc for strips and Full Greeks) equals each request priced alone, and price_fourier
is the engine's FP64 Gil-Pelaez value (dispatcher::price_fourier, PricingDispatch.hpp:128-155)."""
import numpy as np
import pytest

import myquantlib_gb300 as m
from myquantlib_gb300 import registry as reg

pytestmark = pytest.mark.gpu

RECORDS = [
    {"model": "Heston", "heston1": [1.5, 0.04, 0.3, -0.7, 0.04], "instrument": "ArithAsian", "option_type": "Call",
     "strikes": [100.0], "maturity": 1.0, "r": 0.02, "paths": 1 << 16, "steps": 64, "seed": 3},
    {"model": "Bates", "heston1": [2.0, 0.05, 0.9, -0.6, 0.05], "merton": [0.5, -0.1, 0.15],
     "instrument": "Vanilla", "option_type": "Call", "strikes": [90.0, 100.0, 110.0], "maturity": 1.0,
     "r": 0.02, "paths": 1 << 16, "steps": 50, "mode": "Essential"},
    {"model": "BatesKou", "heston1": [1.5, 0.04, 0.3, -0.7, 0.04], "kou": [0.8, 0.4, 10.0, 5.0],
     "instrument": "UpAndOut", "option_type": "Call", "strikes": [100.0], "maturity": 1.0, "barrier": 130.0,
     "r": 0.02, "paths": 1 << 15, "steps": 100, "mode": "Essential", "scheme": "Exact"},
    {"model": "DoubleHeston", "heston1": [1.5, 0.04, 0.3, -0.7, 0.04], "heston2": [0.5, 0.03, 0.2, -0.3, 0.03],
     "instrument": "LookbackFloating", "option_type": "Put", "maturity": 0.5, "r": 0.01,
     "paths": 1 << 15, "steps": 32, "scheme": "NV"},
    {"model": "Bates", "heston1": [2.0, 0.05, 0.9, -0.6, 0.05], "merton": [0.5, -0.1, 0.15],
     "instrument": "Vanilla", "option_type": "Put", "strikes": [100.0], "maturity": 1.0,
     "r": 0.02, "paths": 1 << 15, "steps": 50, "mode": "Full"},
]


def test_price_records_equals_each_request_alone(engine):
    got = reg.price_records(RECORDS, engine)
    reqs = reg.load_requests(RECORDS)
    assert [reg.batchable(r) for r in reqs] == [True, False, True, True, False]
    for rq, g in zip(reqs, got):
        want = m.dispatch.price_mc(rq.model, rq.instrument, rq.cfg, rq.S0, rq.r, rq.q, rq.mode, rq.scheme, engine)
        # the batch sums each request in its own tiling: equal up to FP32 summation order
        np.testing.assert_allclose(g.prices, want.prices, rtol=2e-6, atol=1e-3 * max(want.prices_std_err))
        np.testing.assert_allclose(g.prices_std_err, want.prices_std_err, rtol=1e-4)
        if rq.mode != m.GreekMode.NONE:
            np.testing.assert_allclose(g.deltas, want.deltas, rtol=2e-6, atol=1e-3 * max(want.deltas_std_err))
        if rq.mode == m.GreekMode.FULL:
            assert g.vegas == want.vegas and g.thetas == want.thetas and g.rhos == want.rhos


def test_price_fourier_dispatch(engine):
    p = reg.RuntimeModelParams(heston1=m.HestonParams(1.5, 0.04, 0.3, -0.7, 0.04))
    model = reg.build_model("Heston", p)
    ins = reg.build_european("Vanilla", "Call", reg.RuntimeInstrumentParams(strikes=[90.0, 100.0, 110.0], maturity=1.0))
    res = reg.price_fourier(model, ins, 100.0, 0.02, 0.0, m.GreekMode.FULL, engine)
    assert abs(res.prices[1] - 8.628108103110) < 1e-8  # the reference's FP64 Fourier value of this call
    assert res.prices[0] > res.prices[1] > res.prices[2]
    assert len(res.deltas) == len(res.gammas) == len(res.thetas) == len(res.rhos) == 3
    assert res.prices_std_err == [] and res.vegas_std_err == []
    with pytest.raises(TypeError):
        reg.price_fourier(model, reg.build_instrument("ArithAsian", "Call",
                                                      reg.RuntimeInstrumentParams(strikes=[100.0], maturity=1.0)),
                          100.0, 0.02, 0.0)
