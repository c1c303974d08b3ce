"""GPU test of myql_mc_price_noalloc, the entry point for callers that cannot
allocate device memory while pricing (memory owned by their own pool or
another framework's allocator, or allocation forbidden after start-up).

It is called through the C ABI with a caller-owned output buffer and must
reproduce myql_mc_price on the same request, on two calls in a row (the
shared scratch array keeps the previous call's contents, which must not leak
into the next result).  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

import myquantlib_gb300 as m
from myquantlib_gb300 import _abi

pytestmark = pytest.mark.gpu


def _jobs():
    heston = m.HestonModel(m.HestonParams(1.5, 0.04, 0.3, -0.7, 0.04))
    cfg = m.MonteCarloConfig(num_paths=200000, time_steps=64, seed=7, n_streams=8192)
    a = m.make_job(heston, m.HestonStepper(m.SchemeNV), m.EuropeanOption([90.0, 100.0, 110.0], 1.0),
                   m.GreekMode.ESSENTIAL, cfg, 100.0, 0.02, 0.0)
    b = m.make_job(heston, m.HestonStepper(m.SchemeExact), m.DownAndOutPut(100.0, 85.0, 1.0),
                   m.GreekMode.NONE, m.MonteCarloConfig(num_paths=50000, time_steps=50, seed=3), 100.0, 0.02, 0.0)
    # 2^21 paths with the default stream count: above 2^20 paths the default is M / 8
    # streams (2^18 here), not 2^17, and both entry points must pick the same layout
    c = m.make_job(heston, m.HestonStepper(m.SchemeNV), m.EuropeanOption(100.0, 1.0),
                   m.GreekMode.NONE, m.MonteCarloConfig(num_paths=1 << 21, time_steps=16, seed=11),
                   100.0, 0.02, 0.0)
    return [a, b, c]


def test_noalloc_matches_the_allocating_entry_point():
    torch = pytest.importorskip("torch")
    from myquantlib_gb300 import build
    build.build()
    lib = _abi.load()
    eng = m.Engine(0)
    for job in _jobs():
        want, _ = eng.price(job)
        out = torch.empty(2 * _abi.Q_COUNT * job.n_strikes, dtype=torch.float64, device="cuda:0")
        for _ in range(2):  # two calls in a row on the shared scratch
            out.fill_(np.nan)
            _abi.check(lib.myql_mc_price_noalloc(0, C.byref(job.c), C.c_void_p(out.data_ptr()), None))
            got = out.cpu().numpy().reshape(2 * _abi.Q_COUNT, job.n_strikes)
            np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-15)


def test_noalloc_rejects_what_does_not_fit():
    torch = pytest.importorskip("torch")
    lib = _abi.load()
    job = _jobs()[0]
    job.c.config.num_paths = 1 << 26  # records alone exceed the fixed scratch
    out = torch.empty(2 * _abi.Q_COUNT * job.n_strikes, dtype=torch.float64, device="cuda:0")
    assert lib.myql_mc_price_noalloc(0, C.byref(job.c), C.c_void_p(out.data_ptr()), None) == _abi.ERR_TOO_LARGE
    nci = _jobs()[1]
    nci.c.config.scheme[0] = _abi.SCHEME_NCI
    assert lib.myql_mc_price_noalloc(0, C.byref(nci.c), C.c_void_p(out.data_ptr()), None) == _abi.ERR_UNSUPPORTED
