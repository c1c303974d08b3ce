"""CPU tests of the drop-in boundary: the C-ABI library loads and exports every
declared entry point, the ctypes mirror has the C layout, host-side validation
and the reference-style Python API behave like the reference."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import myquantlib_gb300 as m
from myquantlib_gb300 import _abi, build
from myquantlib_gb300.pricers import validate

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "myql_gpu.h"


def header_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:myql_status|size_t|int)\s+(myql_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    lib_path = build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib_path)], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r" T (myql_\w+)", out))
    declared = header_functions()
    assert declared, "no declarations parsed"
    missing = [f for f in declared if f not in exported]
    assert not missing, missing
    # the ctypes mirror binds exactly the declared set
    assert sorted(_abi.declared_symbols()) == declared
    lib = _abi.load()
    for f in declared:
        assert hasattr(lib, f)
    assert lib.myql_abi_version() == 1


def test_struct_layouts_match_c(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(r'''
#include <stdio.h>
#include <stddef.h>
#include "myql_gpu.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(myql_mc_job),
         offsetof(myql_mc_job, instrument), offsetof(myql_mc_job, config), offsetof(myql_mc_job, S0),
         offsetof(myql_instrument, strikes), offsetof(myql_mc_config, n_streams),
         sizeof(myql_mc_stats), sizeof(myql_mlmc_config), sizeof(myql_mlmc_result),
         offsetof(myql_model, jump_lambda));
  return 0;
}''')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    want = [C.sizeof(_abi.McJobC), _abi.McJobC.instrument.offset, _abi.McJobC.config.offset,
            _abi.McJobC.S0.offset, _abi.InstrumentC.strikes.offset, _abi.McConfigC.n_streams.offset,
            C.sizeof(_abi.McStatsC), C.sizeof(_abi.MlmcConfigC), C.sizeof(_abi.MlmcResultC),
            _abi.ModelC.jump_lambda.offset]
    assert got == want


def heston(sigma=0.3, kappa=1.5, theta=0.04):
    return m.HestonModel(m.HestonParams(kappa, theta, sigma, -0.7, 0.04))


def test_nv_condition_rejected_on_host():
    # VolSchemes.hpp:40-41 throws for sigma^2 > 4 kappa theta; the ABI returns a status
    job = m.make_job(heston(sigma=0.9), m.HestonStepper(m.SchemeNV), m.EuropeanOption(100.0, 1.0),
                     m.GreekMode.NONE, m.MonteCarloConfig(), 100.0, 0.02, 0.0)
    with pytest.raises(_abi.MyqlError) as e:
        validate(job)
    assert e.value.status == _abi.ERR_NV_CONDITION
    ok = m.make_job(heston(sigma=0.9), m.HestonStepper(m.SchemeNCI), m.EuropeanOption(100.0, 1.0),
                    m.GreekMode.NONE, m.MonteCarloConfig(), 100.0, 0.02, 0.0)
    validate(ok)


@pytest.mark.parametrize("mutate,status", [
    (lambda j: setattr(j.c, "S0", -1.0), _abi.ERR_INVALID_ARG),
    (lambda j: setattr(j.c.instrument, "maturity", 0.0), _abi.ERR_INVALID_ARG),
    (lambda j: setattr(j.c.config, "num_paths", 0), _abi.ERR_INVALID_ARG),
    (lambda j: setattr(j.c.config, "time_steps", 0), _abi.ERR_INVALID_ARG),
    (lambda j: setattr(j.c.instrument, "n_strikes", 0), _abi.ERR_INVALID_ARG),
    (lambda j: setattr(j.c.model, "num_factors", 3), _abi.ERR_INVALID_ARG),
    (lambda j: j.c.config.scheme.__setitem__(0, 9), _abi.ERR_INVALID_ARG),
    (lambda j: setattr(j.c.config, "greek_mode", 7), _abi.ERR_INVALID_ARG),
    (lambda j: setattr(j.c.config, "n_streams", 1 << 27), _abi.ERR_TOO_LARGE),
])
def test_invalid_jobs_rejected(mutate, status):
    job = m.make_job(heston(), m.HestonStepper(m.SchemeNV), m.EuropeanOption(100.0, 1.0),
                     m.GreekMode.NONE, m.MonteCarloConfig(num_paths=1 << 28), 100.0, 0.02, 0.0)
    mutate(job)
    with pytest.raises(_abi.MyqlError) as e:
        validate(job)
    assert e.value.status == status


def test_full_greeks_need_t_bump_below_maturity():
    job = m.make_job(heston(), m.HestonStepper(m.SchemeNV), m.EuropeanOption(100.0, 1e-4),
                     m.GreekMode.FULL, m.MonteCarloConfig(), 100.0, 0.02, 0.0)
    with pytest.raises(_abi.MyqlError):
        validate(job)


def test_kou_eta1_must_exceed_one():
    model = m.BatesKouModel(m.HestonParams(1.5, 0.04, 0.3, -0.7, 0.04), m.KouParams(1.0, 0.4, 0.9, 5.0))
    job = m.make_job(model, m.BatesKouStepper(m.SchemeNV), m.EuropeanOption(100.0, 1.0),
                     m.GreekMode.NONE, m.MonteCarloConfig(), 100.0, 0.02, 0.0)
    with pytest.raises(_abi.MyqlError):
        validate(job)


def test_stepper_model_instrument_mismatch_is_a_type_error():
    # the reference rejects these at compile time (Stepper::ModelParams / State types)
    opt = m.EuropeanOption(100.0, 1.0)
    with pytest.raises(TypeError):
        m.make_job(heston(), m.DoubleHestonStepper(m.SchemeNV, m.SchemeNV), opt, m.GreekMode.NONE,
                   m.MonteCarloConfig(), 100.0, 0.0, 0.0)
    with pytest.raises(TypeError):
        m.make_job(heston(), m.BatesStepper(m.SchemeNV), opt, m.GreekMode.NONE, m.MonteCarloConfig(),
                   100.0, 0.0, 0.0)
    with pytest.raises(TypeError):
        m.make_job(heston(), m.HestonStepper(m.SchemeNV, m.TrackerLookback), opt, m.GreekMode.NONE,
                   m.MonteCarloConfig(), 100.0, 0.0, 0.0)


def test_job_lowering_and_dispatcher_default():
    opt = m.EuropeanOption([90.0, 100.0, 110.0], 2.0, m.PayoffCashOrNothing(m.OptionType.Put, 0.5))
    job = m.make_job(heston(), None, opt, m.GreekMode.ESSENTIAL,
                     m.MonteCarloConfig(num_paths=123, time_steps=7, seed=9), 101.0, 0.03, 0.01)
    c = job.c
    assert c.config.scheme[0] == _abi.SCHEME_NCI  # StepperTraits.hpp:68 default scheme
    assert c.instrument.is_strip == 1 and c.instrument.n_strikes == 3
    assert c.instrument.payoff == _abi.PAYOFF_CASH and c.instrument.option_type == _abi.PUT
    assert c.instrument.payoff_eps == 0.5
    assert [c.instrument.strikes[i] for i in range(3)] == [90.0, 100.0, 110.0]
    assert (c.config.num_paths, c.config.time_steps, c.config.seed) == (123, 7, 9)
    assert (c.S0, c.r, c.q) == (101.0, 0.03, 0.01)


def test_result_unpacking_shapes():
    raw = np.arange(20 * 3, dtype=float).reshape(20, 3)
    r = m.result_from_raw(raw, m.GreekMode.FULL, True)
    assert np.array_equal(r.price, raw[0]) and np.array_equal(r.price_std_err, raw[1])
    assert np.array_equal(r.vega[1], raw[8]) and np.array_equal(r.charm_std_err, raw[19])
    r1 = m.result_from_raw(raw[:, :1], m.GreekMode.NONE, False)
    assert r1.price == 0.0 and r1.delta is None


def test_header_constants_match_the_python_mirror():
    """The #define constants of include/myql_gpu.h that the Python mirror repeats."""
    text = (Path(__file__).resolve().parents[1] / "include" / "myql_gpu.h").read_text()
    seed = re.search(r"#define MYQL_QMC_DEFAULT_DIRECTION_SEED (\d+)", text)
    assert seed and int(seed.group(1)) == _abi.QMC_DEFAULT_DIRECTION_SEED
