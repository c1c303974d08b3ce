"""CPU tests of the runtime registries and the record front-end (myquantlib_gb300.registry):
the model and instrument factories of dispatcher/ModelRegistry.hpp:35-72 and
dispatcher/InstrumentRegistry.hpp:142-257, their error behaviour, and JSON / CSV records
lowered to the same C-ABI jobs."""
import json

import pytest

import myquantlib_gb300 as m
from myquantlib_gb300 import _abi, registry as reg

H1 = m.HestonParams(2.0, 0.05, 0.9, -0.6, 0.05)
H2 = m.HestonParams(0.5, 0.02, 0.3, -0.3, 0.02)
MJ = m.MertonParams(0.5, -0.1, 0.15)
KJ = m.KouParams(0.8, 0.4, 10.0, 5.0)


def test_build_model_every_type():
    p = reg.RuntimeModelParams(heston1=H1, heston2=H2, vol=0.2, merton=MJ, kou=KJ)
    want = {
        "BlackScholes": m.BlackScholesModel(0.2), "Merton": m.MertonModel(0.2, MJ), "Kou": m.KouModel(0.2, KJ),
        "Heston": m.HestonModel(H1), "Bates": m.BatesModel(H1, MJ), "BatesKou": m.BatesKouModel(H1, KJ),
        "DoubleHeston": m.DoubleHestonModel(H1, H2), "DoubleBates": m.DoubleBatesModel(H1, H2, MJ),
        "DoubleBatesKou": m.DoubleBatesKouModel(H1, H2, KJ),
    }
    assert set(want) == set(reg.MODEL_TYPES)
    for name, model in want.items():
        assert reg.build_model(name, p) == model, name
    with pytest.raises(ValueError, match="Unknown model type: SABR"):
        reg.build_model("SABR", p)


@pytest.mark.parametrize("type_", reg.INSTRUMENT_TYPES)
@pytest.mark.parametrize("ot", ["Call", "Put"])
def test_build_instrument_every_type(type_, ot):
    ip = reg.RuntimeInstrumentParams(strikes=[95.0, 100.0], maturity=1.5, barrier_level=120.0, rebate=2.0,
                                     rate=0.03)
    ins = reg.build_instrument(type_, ot, ip)
    assert ins.T == 1.5
    assert ins.payoff.Type == (m.OptionType.Call if ot == "Call" else m.OptionType.Put)
    if type_ in reg.EUROPEAN_TYPES:
        assert ins.kind == _abi.INSTR_EUROPEAN and ins.is_strip and list(ins.strikes) == [95.0, 100.0]
        assert type(ins.payoff).__name__ == {"Vanilla": "PayoffVanilla", "CashOrNothing": "PayoffCashOrNothing",
                                             "AssetOrNothing": "PayoffAssetOrNothing"}[type_]
        assert reg.build_european(type_, ot, ip).kind == _abi.INSTR_EUROPEAN
        return
    assert not ins.is_strip and isinstance(ins.payoff, m.PayoffVanilla)
    floating = type_.endswith("Floating")
    assert ins.fixed_strike == (0 if floating else 1)
    assert float(ins.strikes[0]) == (0.0 if floating else 95.0)  # first strike for fixed exotics
    if "Asian" in type_:
        assert ins.kind == (_abi.INSTR_ASIAN_GEO if type_.startswith("Geo") else _abi.INSTR_ASIAN_ARITH)
    elif type_.startswith("Lookback"):
        assert ins.kind == _abi.INSTR_LOOKBACK
    else:
        assert ins.kind == _abi.INSTR_BARRIER and ins.barrier == 120.0 and ins.rebate == 2.0
        assert ins.barrier_rate == 0.03 and ins.rebate_timing == int(m.RebateTiming.NONE)
        assert ins.barrier_up == int(type_.startswith("Up"))
        assert ins.barrier_action == int(m.BarrierAction.Out if type_.endswith("Out") else m.BarrierAction.In)
    with pytest.raises(ValueError, match="Unknown European instrument: " + type_):
        reg.build_european(type_, ot, ip)


def test_unknown_instrument_and_option_type():
    ip = reg.RuntimeInstrumentParams(strikes=[100.0], maturity=1.0)
    with pytest.raises(ValueError, match="Unknown instrument: Rainbow Call"):
        reg.build_instrument("Rainbow", "Call", ip)
    with pytest.raises(ValueError, match="Unknown instrument: Vanilla Straddle"):
        reg.build_instrument("Vanilla", "Straddle", ip)
    with pytest.raises(ValueError, match="Unknown European instrument: Vanilla Straddle"):
        reg.build_european("Vanilla", "Straddle", ip)


RECORDS = [
    {"model": "Bates", "heston1": [2.0, 0.05, 0.9, -0.6, 0.05], "merton": [0.5, -0.1, 0.15],
     "instrument": "Vanilla", "option_type": "Call", "strikes": [90.0, 100.0, 110.0], "maturity": 1.0,
     "S0": 100.0, "r": 0.02, "q": 0.01, "paths": 65536, "steps": 50, "seed": 7, "mode": "Essential"},
    {"model": "DoubleHeston", "heston1": [1.5, 0.04, 0.3, -0.7, 0.04], "heston2": [0.5, 0.03, 0.2, -0.3, 0.03],
     "instrument": "ArithAsian", "option_type": "Put", "strikes": [100.0], "maturity": 2.0,
     "S0": 100.0, "r": 0.02, "paths": 16384, "steps": 64, "scheme": "NV"},
    {"model": "BatesKou", "heston1": [1.5, 0.04, 0.3, -0.7, 0.04], "kou": [0.8, 0.4, 10.0, 5.0],
     "instrument": "UpAndOut", "option_type": "Call", "strikes": [100.0], "maturity": 1.0, "barrier": 130.0,
     "rebate": 1.0, "S0": 100.0, "r": 0.03, "paths": 32768, "steps": 100, "mode": "Full", "scheme": "Exact",
     "t_bump": 1e-3},
]
CSV = """model,kappa,theta,sigma,rho,v0,kappa2,theta2,sigma2,rho2,v02,jump_lambda,merton_mu,merton_delta,kou_p_up,kou_eta1,kou_eta2,instrument,option_type,strikes,maturity,barrier,rebate,S0,r,q,paths,steps,seed,mode,scheme,t_bump
Bates,2.0,0.05,0.9,-0.6,0.05,,,,,,0.5,-0.1,0.15,,,,Vanilla,Call,90;100;110,1.0,,,100,0.02,0.01,65536,50,7,Essential,,
DoubleHeston,1.5,0.04,0.3,-0.7,0.04,0.5,0.03,0.2,-0.3,0.03,,,,,,,ArithAsian,Put,100,2.0,,,100,0.02,,16384,64,,,NV,
BatesKou,1.5,0.04,0.3,-0.7,0.04,,,,,,0.8,,,0.4,10.0,5.0,UpAndOut,Call,100,1.0,130,1.0,100,0.03,,32768,100,,Full,Exact,0.001
"""


def job_fields(rq):
    job = m.make_job(rq.model, m.stepper_for(rq.model, rq.instrument, rq.scheme), rq.instrument, rq.mode, rq.cfg,
                     rq.S0, rq.r, rq.q)
    c = job.c
    return (bytes(memoryview(c.model)), c.instrument.kind, c.instrument.payoff, c.instrument.option_type,
            c.instrument.fixed_strike, c.instrument.barrier, c.instrument.rebate, c.instrument.barrier_rate,
            c.instrument.n_strikes, [c.instrument.strikes[i] for i in range(c.instrument.n_strikes)],
            c.instrument.maturity, bytes(memoryview(c.config)), c.S0, c.r, c.q)


def test_json_and_csv_records_give_the_same_jobs(tmp_path):
    from_json = reg.load_requests(json.dumps(RECORDS))
    from_csv = reg.load_requests(CSV)
    p = tmp_path / "requests.csv"
    p.write_text(CSV)
    from_file = reg.load_requests(str(p))
    assert len(from_json) == len(from_csv) == len(from_file) == 3
    for a, b, c in zip(from_json, from_csv, from_file):
        assert job_fields(a) == job_fields(b) == job_fields(c)
    a, b, c = from_json
    assert a.mode == m.GreekMode.ESSENTIAL and b.mode == m.GreekMode.NONE and c.mode == m.GreekMode.FULL
    assert a.scheme is m.SchemeNCI and b.scheme is m.SchemeNV and c.scheme is m.SchemeExact
    assert c.cfg.t_bump == 1e-3 and c.instrument.barrier_rate == 0.03  # rebate discounting defaults to r
    assert [reg.batchable(r) for r in from_json] == [False, True, False]


def test_record_errors():
    bad = dict(RECORDS[0], mode="Partial")
    with pytest.raises(ValueError, match="Unknown GreekMode"):
        reg.request_from_record(bad)
    with pytest.raises(ValueError, match="Unknown vol scheme"):
        reg.request_from_record(dict(RECORDS[0], scheme="QE"))
    with pytest.raises(ValueError, match="Unknown model type: Vasicek"):
        reg.request_from_record(dict(RECORDS[0], model="Vasicek"))
