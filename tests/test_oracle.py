"""CPU tests of the oracle: the C restatement against the reference's own
outputs (golden fixtures made by tests/golden/make_golden.py from the
reference headers), against scipy for the numerics, and the random streams
against an independent big-int implementation."""
import json
from pathlib import Path

import numpy as np
import pytest
from scipy import stats

import jobspec
import pyrng

GOLDEN = Path(__file__).resolve().parent / "golden"
MC_SPECS = json.loads((GOLDEN / "reference_mc.json").read_text())
FOURIER_SPECS = json.loads((GOLDEN / "reference_fourier.json").read_text())


@pytest.mark.parametrize("spec", MC_SPECS, ids=[s["name"] for s in MC_SPECS])
def test_restatement_matches_reference_outputs(oracle_lib, spec):
    """The FP64 restatement reproduces MonteCarloPricer::calculate of the
    reference (same seeds, same OpenMP thread layout): bit for bit on one
    thread, to merge-order rounding on three."""
    job = jobspec.make_job(spec)
    for nt, tol in (("1", 0.0), ("3", 1e-12)):
        want = np.array(spec["outputs"][nt])
        got, _ = oracle_lib.mc_price(job, oracle_lib.LAYOUT_REFERENCE, int(nt))
        scale = np.maximum(np.abs(want), 1e-300)
        if tol == 0.0:
            np.testing.assert_array_equal(got, want)
        else:
            assert np.all(np.abs(got - want) <= tol * scale + 1e-15), spec["name"]


def test_restatement_matches_live_reference(oracle_lib):
    """Where the reference compiles (oracle/_ref), compare live on a fresh seed."""
    if not (oracle_lib.REF_ROOT / "include").exists():
        pytest.skip("reference sources not present on this machine")
    oracle_lib.build(ref=True)
    spec = jobspec.with_config(MC_SPECS[2], seed=2024, paths=1500)
    job = jobspec.make_job(spec)
    a, _ = oracle_lib.mc_price(job, oracle_lib.LAYOUT_REFERENCE, 2)
    b = oracle_lib.ref_mc_price(job, 2)
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-15)


def test_chi2_quantile_matches_scipy(oracle_lib):
    lib = oracle_lib.restatement()
    rng = np.random.default_rng(7)
    dofs = np.concatenate([[0.05, 0.494, 1.0, 2.0, 4.7], rng.uniform(0.1, 3000.0, 30)])
    ps = np.concatenate([[1e-12, 1e-6, 1e-4, 0.001, 0.3, 0.5, 0.9, 0.999, 0.9999999],
                         rng.uniform(0, 1, 10)])
    worst = 0.0
    for nu in dofs:
        for p in ps:
            got = lib.myql_oracle_chi2_quantile(nu, p)
            want = stats.chi2.ppf(p, nu)
            worst = max(worst, abs(got - want) / max(want, 1e-300))
    assert worst < 1e-9, worst


def test_acklam_inverse_normal(oracle_lib):
    lib = oracle_lib.restatement()
    p = np.concatenate([np.logspace(-15, -1, 60), np.linspace(0.02, 0.98, 97), 1 - np.logspace(-15, -1, 60)])
    got = np.array([lib.myql_oracle_normcdfinv(x) for x in p])
    want = stats.norm.ppf(p)
    # Acklam's approximation: relative error below 1.15e-9
    assert np.max(np.abs(got - want) / np.abs(want + (want == 0))) < 1.2e-9


def test_inverse_poisson_exact(oracle_lib):
    """poissinvcdf (Giles' algorithm as in Numerics.hpp) is the exact inverse CDF."""
    lib = oracle_lib.restatement()
    rng = np.random.default_rng(11)
    lams = np.concatenate([[0.01, 0.5, 3.9, 4.1, 9.5, 25.0, 150.0, 1200.0], rng.uniform(0.01, 500, 40)])
    U = np.concatenate([[1e-12, 1e-6, 0.5, 1 - 1e-9], rng.uniform(0, 1, 60)])
    bad = 0
    for lam in lams:
        for u in U:
            got = lib.myql_oracle_poissinvcdf(lam, u)
            want = stats.poisson.ppf(u, lam)
            # scipy's ppf can be off by one right at a boundary (its own rounding)
            if got != want and not (abs(stats.poisson.cdf(min(got, want), lam) - u) < 1e-12):
                bad += 1
    assert bad == 0


def test_jump_polynomial_derived_from_generator():
    L, poly = pyrng.derive_jump_poly()
    assert L == 256
    assert poly == pyrng.JUMP  # the published xoshiro256 jump() constants


def test_oracle_streams_match_bigint(oracle_lib):
    got = oracle_lib.stream_states(42, 0, 5)
    for k in range(5):
        assert [int(x) for x in got[k]] == pyrng.stream_state(42, k)
    got = oracle_lib.stream_states(2**64 - 5, 3, 2)
    assert [int(x) for x in got[0]] == pyrng.stream_state(2**64 - 5, 3)


def test_reference_seed_layout_first_draws():
    """The reference seeds thread t with seed + t*999983 (MonteCarloPricer.hpp:191).
    Known answers of the seeding used here (splitmix64 expansion)."""
    s = pyrng.seed_state(42)
    outs = []
    for _ in range(3):
        o, s = pyrng.next_out(s)
        outs.append(o)
    golden = json.loads((GOLDEN / "rng_kat.json").read_text())
    assert outs == golden["seed42_first3"]
    s = pyrng.seed_state(42 + 999983)
    o, _ = pyrng.next_out(s)
    assert o == golden["seed42_thread1_first"]


def test_reference_put_theta_is_not_its_price_derivative(oracle_lib):
    """The reference's FourierPricer reports a put theta that is not the T-derivative of
    its own put price (the call side is consistent).  Recorded because the GPU engine's
    Monte Carlo theta and its Fourier oracle follow the derivative."""
    if not oracle_lib.reference_available():
        pytest.skip("reference library not built here")
    spec = [s for s in FOURIER_SPECS if s["name"] == "heston_put_k95_t05"][0]

    def ref(T):
        s = json.loads(json.dumps(spec))
        s["instrument"]["T"] = T
        return np.asarray(oracle_lib.ref_fourier(jobspec.make_job(dict(s, mode="full", schemes=["Exact"]))))

    h = 1e-5
    base = ref(0.5)
    dPdT = (ref(0.5 + h)[0] - ref(0.5 - h)[0]) / (2 * h)
    assert base[5] == pytest.approx(5.316764368677, rel=1e-9)   # the reported theta
    assert dPdT == pytest.approx(4.154394, rel=1e-6)             # the derivative of its price
