"""The C++20 drop-in header (include/myql_gpu/MonteCarloPricer.hpp): pricers
declared with the reference's template signatures lower to the same C-ABI
requests as the Python mirror, and a mismatched stepper fails to compile as
in the reference.  The GPU variant prices through the header."""
import json
import shutil
import subprocess
from pathlib import Path

import pytest

import myquantlib_gb300 as m
from myquantlib_gb300 import build as mbuild

ROOT = Path(__file__).resolve().parent.parent
CPP = ROOT / "tests" / "cpp"
pytestmark = pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")


def compile_check(tmp_path) -> Path:
    lib = mbuild.LIB
    exe = tmp_path / "header_check"
    cmd = ["g++", "-std=c++20", "-O1", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(CPP / "header_check.cpp"),
           f"-L{lib.parent}", "-lmyql_gpu", f"-Wl,-rpath,{lib.parent}", "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


H1 = m.HestonParams(kappa=1.5, theta=0.04, sigma=0.3, rho=-0.7, v0=0.04)
H2 = m.HestonParams(kappa=3.0, theta=0.02, sigma=0.2, rho=-0.3, v0=0.02)


def python_jobs():
    cfg = m.MonteCarloConfig(num_paths=1 << 18, time_steps=100)
    lb_pay = m.PayoffCashOrNothing(m.OptionType.Call, eps=0.5)
    return {
        "heston_eur": m.make_job(m.HestonModel(H1), m.HestonStepper(m.SchemeNV), m.EuropeanOption(100.0, 1.0),
                                 m.GreekMode.ESSENTIAL, cfg, 100.0, 0.02, 0.0),
        "dbk_asian_strip": m.make_job(
            m.DoubleBatesKouModel(H1, H2, m.KouParams(0.7, 0.4, 10.0, 5.0)),
            m.DoubleBatesKouStepper(m.SchemeNCI, m.SchemeExact, m.TrackerArithAsian),
            m.AsianOption(m.TrackerArithAsian, m.PayoffVanilla(m.OptionType.Put), False, [90.0, 100.0, 110.0], 2.0,
                          past_avg_S=101.0, past_avg_log=4.6, t_elapsed=0.25),
            m.GreekMode.FULL, cfg, 100.0, 0.03, 0.01),
        "bates_uo": m.make_job(m.BatesModel(H1, m.MertonParams(0.5, -0.1, 0.15)),
                               m.BatesStepper(m.SchemeExact, m.TrackerBarrier),
                               m.UpAndOutCall(95.0, 130.0, 1.0, 0.02, 1.5, Timing=m.RebateTiming.AtHit),
                               m.GreekMode.NONE, cfg, 100.0, 0.02, 0.0),
        "merton_lookback": m.make_job(m.MertonModel(0.2, m.MertonParams(1.0, -0.05, 0.1)),
                                      m.MertonJDStepper(m.TrackerLookback),
                                      m.LookbackOption(lb_pay, True, 100.0, 1.0, 95.0, 104.0),
                                      m.GreekMode.ESSENTIAL, cfg, 100.0, 0.02, 0.0),
    }


def fields(job):
    c = job.c
    md, ins, cf = c.model, c.instrument, c.config
    hp = lambda h: [h.kappa, h.theta, h.sigma, h.rho, h.v0]  # noqa: E731
    return {"num_factors": md.num_factors, "jump": md.jump, "vol": md.vol, "h0": hp(md.heston[0]),
            "h1": hp(md.heston[1]), "jump_params": [md.jump_lambda, md.merton_mu, md.merton_delta, md.kou_p_up,
                                                    md.kou_eta1, md.kou_eta2],
            "kind": ins.kind, "payoff": ins.payoff, "option_type": ins.option_type, "fixed_strike": ins.fixed_strike,
            "barrier_up": ins.barrier_up, "barrier_action": ins.barrier_action, "rebate_timing": ins.rebate_timing,
            "is_strip": ins.is_strip, "maturity": ins.maturity, "barrier": ins.barrier, "rebate": ins.rebate,
            "barrier_rate": ins.barrier_rate, "payoff_eps": ins.payoff_eps,
            "strikes": [ins.strikes[k] for k in range(ins.n_strikes)],
            "history": [ins.past_avg_log, ins.past_avg_S, ins.t_elapsed, ins.hist_min_S, ins.hist_max_S],
            "num_paths": cf.num_paths, "time_steps": cf.time_steps, "seed": cf.seed,
            "bumps": [cf.fd_bump, cf.vol_bump, cf.t_bump, cf.r_bump], "scheme": [cf.scheme[0], cf.scheme[1]],
            "greek_mode": cf.greek_mode, "S0": c.S0, "r": c.r, "q": c.q}


def test_header_lowers_like_the_python_mirror(tmp_path):
    exe = compile_check(tmp_path)
    out = subprocess.run([str(exe), "lower"], check=True, capture_output=True, text=True).stdout
    got = {d["name"]: d for d in map(json.loads, out.strip().splitlines())}
    want = python_jobs()
    assert set(got) == set(want)
    for name, job in want.items():
        g = dict(got[name])
        assert g.pop("valid") == 0, name  # myql_validate_job accepts the request
        g.pop("name")
        w = fields(job)
        # Python instruments without an explicit eps leave the automatic bandwidth (-1)
        assert g == w, (name, {k: (g[k], w[k]) for k in g if g[k] != w[k]})


def test_mismatched_stepper_does_not_compile():
    r = subprocess.run(["g++", "-std=c++20", "-fsyntax-only", f"-I{ROOT / 'include'}", str(CPP / "mismatch.cpp")],
                       capture_output=True, text=True)
    assert r.returncode != 0 and "jump policy must match" in r.stderr


def test_rng_template_parameter():
    """The fifth template parameter (the reference's RNG) accepts xoshiro256pp, Boost's spelling
    included where a Boost-API header is on the include path, and rejects other engines."""
    ok = subprocess.run(["g++", "-std=c++20", "-fsyntax-only", "-Wall", "-Werror", f"-I{ROOT / 'include'}",
                         f"-I{ROOT / 'oracle' / 'compat'}", str(CPP / "rng_param.cpp")], capture_output=True, text=True)
    assert ok.returncode == 0, ok.stderr
    bad = subprocess.run(["g++", "-std=c++20", "-fsyntax-only", f"-I{ROOT / 'include'}", str(CPP / "rng_mismatch.cpp")],
                         capture_output=True, text=True)
    assert bad.returncode != 0 and "RNG must be xoshiro256pp" in bad.stderr


@pytest.mark.gpu
def test_header_prices_on_the_gpu(tmp_path):
    exe = compile_check(tmp_path)
    out = subprocess.run([str(exe), "price"], check=True, capture_output=True, text=True, timeout=300).stdout
    lines = [json.loads(x) for x in out.strip().splitlines()]
    res = lines[0]
    assert abs(res["price"] - 8.628108103110) < 4 * res["price_std_err"]
    assert res["total_steps"] == (1 << 18) * 100
    assert 0.4 < res["delta"] < 0.8
    assert lines[1]["mlmc_levels"] >= 3 and lines[1]["mlmc_delta"] == 0.0
    assert 1.0 < lines[1]["mlmc_price"] < 4.0 and lines[1]["mlmc_se"] > 0
    fl = lines[2]
    assert fl["full_price"][0] == fl["full_price"][1]          # the base scenario is unchanged
    assert fl["full_theta"][0] != fl["full_theta"][1]          # the T-bumped scenarios are not
    assert abs(fl["full_theta"][0] - fl["full_theta"][1]) < fl["theta_se"]
    assert lines[3]["nv_error"] == "runtime_error"
