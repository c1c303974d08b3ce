"""Python mirror of MyQuantLib's Monte Carlo pricer API on top of the C ABI.

Names, argument order and meaning follow the reference's C++ templates so that
code written against it reads the same:

    model   = HestonModel(HestonParams(kappa, theta, sigma, rho, v0))
    option  = EuropeanOption(100.0, 1.0, PayoffVanilla(OptionType.Call))
    stepper = HestonStepper(SchemeNV)
    pricer  = MonteCarloPricer(model, stepper, GreekMode.NONE, MonteCarloConfig(num_paths=2**20))
    res     = pricer.calculate(S0, r, q, option)      # res.price, res.price_std_err, ...

(MonteCarloPricer.hpp:84-96; models ASVJmodel.hpp:14-87; instruments
European.hpp / Asian.hpp / Lookback.hpp / Barrier.hpp; steppers
ASVJstepper.hpp:290-339.)  Mismatches the reference rejects at compile time
(stepper factors / jump policy / tracker versus model and instrument) raise
TypeError here; invalid parameters raise MyqlError from the engine.
"""
from __future__ import annotations

import ctypes as C
import enum
import threading
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import _abi


# --------------------------------------------------------------------------- enums
class GreekMode(enum.IntEnum):  # PricingTypes.hpp:8-12
    NONE = 0
    ESSENTIAL = 1
    FULL = 2


class OptionType(enum.IntEnum):  # Payoffs.hpp:6
    Call = 0
    Put = 1


class BarrierDirection(enum.IntEnum):  # Barrier.hpp:10
    Up = 1
    Down = 0


class BarrierAction(enum.IntEnum):  # Barrier.hpp:11
    In = 0
    Out = 1


class RebateTiming(enum.IntEnum):  # Barrier.hpp:12
    NONE = 0
    AtHit = 1
    AtMaturity = 2


# --------------------------------------------------------------------------- parameters
@dataclass(frozen=True)
class HestonParams:  # ModelParams.hpp:7-25
    kappa: float
    theta: float
    sigma: float
    rho: float
    v0: float

    def is_low_vol_regime(self) -> bool:
        return self.sigma * self.sigma <= 4.0 * self.kappa * self.theta

    def is_Feller_regime(self) -> bool:
        return self.sigma * self.sigma <= 2.0 * self.kappa * self.theta


@dataclass(frozen=True)
class NoJumpParams:
    pass


@dataclass(frozen=True)
class MertonParams:  # ModelParams.hpp:35-39
    lambda_: float
    mu: float
    delta: float


@dataclass(frozen=True)
class KouParams:  # ModelParams.hpp:42-47
    lambda_: float
    p_up: float
    eta1: float
    eta2: float


# --------------------------------------------------------------------------- models
@dataclass(frozen=True)
class ZeroFactorModel:  # ASVJmodel.hpp:14-21
    vol: float
    jump: object = NoJumpParams()
    num_variance_factors = 0


@dataclass(frozen=True)
class SingleFactorModel:  # ASVJmodel.hpp:25-33
    heston: HestonParams
    jump: object = NoJumpParams()
    num_variance_factors = 1


@dataclass(frozen=True)
class DoubleFactorModel:  # ASVJmodel.hpp:37-50
    heston1: HestonParams
    heston2: HestonParams
    jump: object = NoJumpParams()
    num_variance_factors = 2


def BlackScholesModel(vol: float) -> ZeroFactorModel:
    return ZeroFactorModel(vol)


def MertonModel(vol: float, j: MertonParams) -> ZeroFactorModel:
    return ZeroFactorModel(vol, j)


def KouModel(vol: float, j: KouParams) -> ZeroFactorModel:
    return ZeroFactorModel(vol, j)


def HestonModel(h: HestonParams) -> SingleFactorModel:
    return SingleFactorModel(h)


def BatesModel(h: HestonParams, j: MertonParams) -> SingleFactorModel:
    return SingleFactorModel(h, j)


def BatesKouModel(h: HestonParams, j: KouParams) -> SingleFactorModel:
    return SingleFactorModel(h, j)


def DoubleHestonModel(h1: HestonParams, h2: HestonParams) -> DoubleFactorModel:
    return DoubleFactorModel(h1, h2)


def DoubleBatesModel(h1: HestonParams, h2: HestonParams, j: MertonParams) -> DoubleFactorModel:
    return DoubleFactorModel(h1, h2, j)


def DoubleBatesKouModel(h1: HestonParams, h2: HestonParams, j: KouParams) -> DoubleFactorModel:
    return DoubleFactorModel(h1, h2, j)


# --------------------------------------------------------------------------- policies
class NullVolScheme:  # VolSchemes.hpp:19
    code = _abi.SCHEME_NONE


class SchemeNV:  # VolSchemes.hpp:24
    code = _abi.SCHEME_NV


class SchemeExact:  # VolSchemes.hpp:71
    code = _abi.SCHEME_EXACT


class SchemeNCI:  # VolSchemes.hpp:230
    code = _abi.SCHEME_NCI


class NoJumps:  # JumpPolicies.hpp:15
    code = _abi.JUMP_NONE
    params = NoJumpParams


class MertonJump:  # JumpPolicies.hpp:32
    code = _abi.JUMP_MERTON
    params = MertonParams


class KouJump:  # JumpPolicies.hpp:81
    code = _abi.JUMP_KOU
    params = KouParams


class TrackerEuropean:  # PathTrackers.hpp:8
    is_path_dependent = False


class TrackerGeoAsian:  # PathTrackers.hpp:31
    is_path_dependent = True


class TrackerArithAsian:  # PathTrackers.hpp:77
    is_path_dependent = True


class TrackerLookback:  # PathTrackers.hpp:126
    is_path_dependent = True


class TrackerBarrier:  # PathTrackers.hpp:166
    is_path_dependent = True


@dataclass(frozen=True)
class ASVJStepper:  # ASVJstepper.hpp:18-22
    VolScheme1: type = NullVolScheme
    VolScheme2: type = NullVolScheme
    JumpPolicy: type = NoJumps
    TrackerPolicy: type = TrackerEuropean

    @property
    def num_cirs(self) -> int:
        if self.VolScheme1 is NullVolScheme and self.VolScheme2 is NullVolScheme:
            return 0
        return 1 if self.VolScheme2 is NullVolScheme else 2


# convenience aliases (ASVJstepper.hpp:290-339); the tracker defaults to the
# instrument's when left as None
def BlackScholesStepper(Tracker=None):
    return ASVJStepper(NullVolScheme, NullVolScheme, NoJumps, Tracker)


def MertonJDStepper(Tracker=None):
    return ASVJStepper(NullVolScheme, NullVolScheme, MertonJump, Tracker)


def KouJDStepper(Tracker=None):
    return ASVJStepper(NullVolScheme, NullVolScheme, KouJump, Tracker)


def HestonStepper(VolScheme, Tracker=None):
    return ASVJStepper(VolScheme, NullVolScheme, NoJumps, Tracker)


def BatesStepper(VolScheme, Tracker=None):
    return ASVJStepper(VolScheme, NullVolScheme, MertonJump, Tracker)


def BatesKouStepper(VolScheme, Tracker=None):
    return ASVJStepper(VolScheme, NullVolScheme, KouJump, Tracker)


def DoubleHestonStepper(V1, V2, Tracker=None):
    return ASVJStepper(V1, V2, NoJumps, Tracker)


def DoubleBatesStepper(V1, V2, Tracker=None):
    return ASVJStepper(V1, V2, MertonJump, Tracker)


def DoubleBatesKouStepper(V1, V2, Tracker=None):
    return ASVJStepper(V1, V2, KouJump, Tracker)


# --------------------------------------------------------------------------- payoffs
@dataclass
class PayoffVanilla:  # Payoffs.hpp:14-26
    Type: OptionType = OptionType.Call
    code = _abi.PAYOFF_VANILLA
    needs_smoothing = False
    eps: float = -1.0


@dataclass
class PayoffCashOrNothing:  # Payoffs.hpp:39-52
    Type: OptionType = OptionType.Call
    eps: float = -1.0
    code = _abi.PAYOFF_CASH
    needs_smoothing = True


@dataclass
class PayoffAssetOrNothing:  # Payoffs.hpp:57-69
    Type: OptionType = OptionType.Call
    eps: float = -1.0
    code = _abi.PAYOFF_ASSET
    needs_smoothing = True


# --------------------------------------------------------------------------- instruments
def _strikes(K) -> tuple[np.ndarray, bool]:
    if np.isscalar(K):
        return np.array([float(K)], dtype=np.float64), False
    arr = np.ascontiguousarray(np.asarray(K, dtype=np.float64).ravel())
    return arr, True


@dataclass
class _Instrument:
    strikes: np.ndarray
    is_strip: bool
    T: float
    payoff: object
    kind: int
    Tracker: type
    fixed_strike: int = 1
    barrier_up: int = 0
    barrier_action: int = 0
    rebate_timing: int = 0
    barrier: float = 0.0
    rebate: float = 0.0
    barrier_rate: float = 0.0
    past_avg_log: float = 0.0
    past_avg_S: float = 0.0
    t_elapsed: float = 0.0
    hist_min_S: float = 0.0
    hist_max_S: float = 0.0

    def size(self) -> int:
        return int(self.strikes.size)

    def get_maturity(self) -> float:
        return self.T

    def get_strikes(self):
        return self.strikes if self.is_strip else float(self.strikes[0])


def EuropeanOption(K, T: float, payoff=None) -> _Instrument:  # European.hpp:10-27
    s, strip = _strikes(K)
    return _Instrument(s, strip, T, payoff or PayoffVanilla(), _abi.INSTR_EUROPEAN, TrackerEuropean)


def AsianOption(Tracker, payoff, FixedStrike: bool, K, T: float, *, past_avg_S: float = 0.0,
                past_avg_log: float = 0.0, t_elapsed: float = 0.0) -> _Instrument:  # Asian.hpp:7-149
    s, strip = _strikes(K)
    if Tracker is TrackerGeoAsian:
        kind = _abi.INSTR_ASIAN_GEO
    elif Tracker is TrackerArithAsian:
        kind = _abi.INSTR_ASIAN_ARITH
    else:
        raise TypeError("AsianOption needs TrackerGeoAsian or TrackerArithAsian")
    return _Instrument(s, strip, T, payoff, kind, Tracker, fixed_strike=int(FixedStrike),
                       past_avg_log=past_avg_log, past_avg_S=past_avg_S, t_elapsed=t_elapsed)


def LookbackOption(payoff, FixedStrike: bool, K, T: float, hist_min_S: float = 0.0,
                   hist_max_S: float = 0.0) -> _Instrument:  # Lookback.hpp:8-214
    s, strip = _strikes(K)
    return _Instrument(s, strip, T, payoff, _abi.INSTR_LOOKBACK, TrackerLookback,
                       fixed_strike=int(FixedStrike), hist_min_S=hist_min_S, hist_max_S=hist_max_S)


def BarrierOption(payoff, Dir: BarrierDirection, Action: BarrierAction, Timing: RebateTiming,
                  K, B: float, T: float, r: float = 0.0, rebate: float = 0.0) -> _Instrument:
    # Barrier.hpp:17-55
    s, strip = _strikes(K)
    return _Instrument(s, strip, T, payoff, _abi.INSTR_BARRIER, TrackerBarrier,
                       barrier_up=int(Dir == BarrierDirection.Up), barrier_action=int(Action),
                       rebate_timing=int(Timing), barrier=B, rebate=rebate, barrier_rate=r)


def _barrier_alias(ot, d, a):
    def make(K, B, T, r=0.0, rebate=0.0, Timing=RebateTiming.NONE):
        return BarrierOption(PayoffVanilla(ot), d, a, Timing, K, B, T, r, rebate)
    return make


UpAndOutCall = _barrier_alias(OptionType.Call, BarrierDirection.Up, BarrierAction.Out)
UpAndOutPut = _barrier_alias(OptionType.Put, BarrierDirection.Up, BarrierAction.Out)
UpAndInCall = _barrier_alias(OptionType.Call, BarrierDirection.Up, BarrierAction.In)
UpAndInPut = _barrier_alias(OptionType.Put, BarrierDirection.Up, BarrierAction.In)
DownAndOutCall = _barrier_alias(OptionType.Call, BarrierDirection.Down, BarrierAction.Out)
DownAndOutPut = _barrier_alias(OptionType.Put, BarrierDirection.Down, BarrierAction.Out)
DownAndInCall = _barrier_alias(OptionType.Call, BarrierDirection.Down, BarrierAction.In)
DownAndInPut = _barrier_alias(OptionType.Put, BarrierDirection.Down, BarrierAction.In)


# --------------------------------------------------------------------------- config / results
@dataclass
class MonteCarloConfig:  # MonteCarloPricer.hpp:16-26
    num_paths: int = 100000
    time_steps: int = 100
    seed: int = 42
    fd_bump: float = 1e-4
    vol_bump: float = 1e-4
    t_bump: float = 1e-4
    r_bump: float = 1e-4
    n_streams: int = 0  # xoshiro streams (0 = engine default)
    stream_offset: int = 0  # first stream index (disjoint ranges = independent replicas)


@dataclass
class MonteCarloResult:  # PricingTypes.hpp:46-97
    mode: GreekMode
    price: object = 0.0
    price_std_err: object = 0.0
    delta: object = None
    delta_std_err: object = None
    gamma: object = None
    gamma_std_err: object = None
    vega: list = field(default_factory=list)
    vega_std_err: list = field(default_factory=list)
    theta: object = None
    theta_std_err: object = None
    rho: object = None
    rho_std_err: object = None
    vanna: list = field(default_factory=list)
    vanna_std_err: list = field(default_factory=list)
    charm: object = None
    charm_std_err: object = None
    total_steps: int = 0
    stats: object = None
    raw: object = None  # (2*Q, n) array [quantity value/stderr rows][strike]


# --------------------------------------------------------------------------- engine
class Engine:
    """One engine context (device memory, tables, stream) on one GPU."""

    def __init__(self, device: int = 0):
        self.lib = _abi.load()
        h = C.c_void_p()
        _abi.check(self.lib.myql_ctx_create(C.byref(h), device))
        self.handle = h
        self.device = device

    def close(self):
        if self.handle:
            self.lib.myql_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_loop_cap(self, cap: int):
        _abi.check(self.lib.myql_ctx_set_loop_cap(self.handle, cap))

    def set_records_limit(self, nbytes: int):
        _abi.check(self.lib.myql_ctx_set_records_limit(self.handle, nbytes))

    def set_nci_slopes(self, mode: int):
        """SchemeNCI table cells: 0 the reference's (default), 1 exact slopes and a first cell
        that keeps its exact mean, so the draw's conditional mean is unbiased."""
        _abi.check(self.lib.myql_ctx_set_nci_slopes(self.handle, int(mode)))

    def set_nci_rows(self, max_rows: int):
        """Upper bound on the SchemeNCI table rows (0: the sizing rule); Poisson counts beyond
        the rows take the Wilson-Hilferty quantile and are counted in table_fallbacks."""
        _abi.check(self.lib.myql_ctx_set_nci_rows(self.handle, int(max_rows)))

    def set_precise_theta(self, on: bool):
        """Theta and charm of one-factor SchemeNCI Europeans with the T-bumped scenarios'
        constants carried to beyond FP32 (their FP32 rounding errors added back), so the
        difference over 2 t_bump keeps its precision; off (the default) keeps every
        scenario's records equal to a single-maturity request's."""
        _abi.check(self.lib.myql_ctx_set_precise_theta(self.handle, 1 if on else 0))

    def price(self, job: "_Job") -> tuple[np.ndarray, _abi.McStatsC]:
        out = np.zeros(2 * _abi.Q_COUNT * job.n_strikes, dtype=np.float64)
        st = _abi.McStatsC()
        _abi.check(self.lib.myql_mc_price(self.handle, C.byref(job.c), _ptr(out), C.byref(st)))
        return out.reshape(2 * _abi.Q_COUNT, job.n_strikes), st

    def price_batch(self, jobs: list["_Job"]) -> tuple[list[np.ndarray], _abi.McStatsC]:
        """All jobs in one persistent launch (scalar instruments, GreekMode NONE/ESSENTIAL)."""
        n = len(jobs)
        arr = (_abi.McJobC * n)(*[j.c for j in jobs])
        outs = [np.zeros(2 * _abi.Q_COUNT, dtype=np.float64) for _ in jobs]
        ptrs = (C.POINTER(C.c_double) * n)(*[_ptr(o) for o in outs])
        st = _abi.McStatsC()
        _abi.check(self.lib.myql_mc_price_batch(self.handle, arr, n, ptrs, C.byref(st)))
        return [o.reshape(2 * _abi.Q_COUNT, 1) for o in outs], st

    def batch_plan(self) -> list[dict]:
        """Per kernel class of the last batch: the launch shape the autotuner picked (threads per
        block, streams per thread, unroll depth, persistent grid) and its timings."""
        cap = 64
        arr = (_abi.BatchClassPlanC * cap)()
        n = C.c_size_t()
        _abi.check(self.lib.myql_batch_last_plan(self.handle, arr, cap, C.byref(n)))
        return [{f: getattr(arr[i], f) for f, _ in _abi.BatchClassPlanC._fields_} for i in range(min(n.value, cap))]

    def set_batch_shape(self, block: int = 0, streams_per_thread: int = 1, unroll: int = 0):
        """Forces one launch shape on every batch class (block 0: the autotuner decides)."""
        _abi.check(self.lib.myql_ctx_set_batch_shape(self.handle, block, streams_per_thread, unroll))

    # ---- neural control variate
    def cv_init(self, seed: int = 1):
        _abi.check(self.lib.myql_cv_init(self.handle, seed))

    def cv_params(self) -> np.ndarray:
        out = np.zeros(_abi.CV_PARAMS, dtype=np.float32)
        _abi.check(self.lib.myql_cv_get_params(self.handle, _fptr(out), out.size))
        return out

    def cv_set_params(self, params) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != _abi.CV_PARAMS:
            raise ValueError(f"need {_abi.CV_PARAMS} parameters")
        _abi.check(self.lib.myql_cv_set_params(self.handle, _fptr(p), p.size))

    def cv_forward(self, feats, dM, n_paths: int, n_hedge: int) -> tuple[np.ndarray, np.ndarray]:
        f = np.ascontiguousarray(feats, dtype=np.float32)
        d = np.ascontiguousarray(dM, dtype=np.float32)
        cv = np.zeros(n_paths, dtype=np.float32)
        g = np.zeros(n_paths * n_hedge, dtype=np.float32)
        _abi.check(self.lib.myql_cv_forward(self.handle, _fptr(f), _fptr(d), n_paths, n_hedge, _fptr(cv), _fptr(g)))
        return cv, g

    def cv_gradient(self, feats, dM, Y, n_paths: int, n_hedge: int) -> tuple[float, np.ndarray]:
        f = np.ascontiguousarray(feats, dtype=np.float32)
        d = np.ascontiguousarray(dM, dtype=np.float32)
        y = np.ascontiguousarray(Y, dtype=np.float32)
        grad = np.zeros(_abi.CV_PARAMS, dtype=np.float32)
        loss = C.c_double()
        _abi.check(self.lib.myql_cv_gradient(self.handle, _fptr(f), _fptr(d), _fptr(y), n_paths, n_hedge,
                                             _fptr(grad), C.byref(loss)))
        return loss.value, grad

    def cv_train(self, job: "_Job", cfg: "_abi.CvConfigC") -> "_abi.CvResultC":
        res = _abi.CvResultC()
        _abi.check(self.lib.myql_cv_train(self.handle, C.byref(job.c), C.byref(cfg), C.byref(res)))
        return res

    def cv_price(self, job: "_Job", cfg: "_abi.CvConfigC") -> "_abi.CvResultC":
        res = _abi.CvResultC()
        _abi.check(self.lib.myql_cv_price(self.handle, C.byref(job.c), C.byref(cfg), C.byref(res)))
        return res

    def cv_qmc_price(self, job: "_Job", cfg: "_abi.CvConfigC", n_replicates: int = 16) -> "_abi.CvResultC":
        """The trained control variate on randomized QMC paths (myql_cv_qmc_price): replicate
        means of the control-variate and plain estimators, standard errors from their spread."""
        res = _abi.CvResultC()
        _abi.check(self.lib.myql_cv_qmc_price(self.handle, C.byref(job.c), C.byref(cfg), n_replicates,
                                              C.byref(res)))
        return res

    def mlmc_price(self, job: "_Job", mlmc_cfg: "_abi.MlmcConfigC") -> "_abi.MlmcResultC":
        """MultiLevelMonteCarloPricer::calculate (MultiLevelMonteCarloPricer.hpp:46-238)."""
        res = _abi.MlmcResultC()
        _abi.check(self.lib.myql_mlmc_price(self.handle, C.byref(job.c), C.byref(mlmc_cfg), C.byref(res)))
        return res

    def set_qmc_direction_seed(self, seed: int):
        """The Sobol point set of this context's randomized QMC: the seed of its initial
        direction numbers (the job's seed draws the digital shifts)."""
        _abi.check(self.lib.myql_ctx_set_qmc_direction_seed(self.handle, int(seed)))

    def qmc_price(self, job: "_Job", n_replicates: int = 16):
        """Randomized quasi-Monte Carlo price rows (myql_qmc_price) and the run statistics."""
        out = np.zeros(2 * _abi.Q_COUNT * job.n_strikes, dtype=np.float64)
        st = _abi.McStatsC()
        _abi.check(self.lib.myql_qmc_price(self.handle, C.byref(job.c), n_replicates, _ptr(out), C.byref(st)))
        return out.reshape(2 * _abi.Q_COUNT, job.n_strikes), st

    def ml2r_price(self, job: "_Job", mlmc_cfg: "_abi.MlmcConfigC") -> "_abi.MlmcResultC":
        """Multilevel Richardson-Romberg extrapolation on the MLMC levels (myql_ml2r_price)."""
        res = _abi.MlmcResultC()
        _abi.check(self.lib.myql_ml2r_price(self.handle, C.byref(job.c), C.byref(mlmc_cfg), C.byref(res)))
        return res

    def mlmc_cv_price(self, job: "_Job", mlmc_cfg: "_abi.MlmcConfigC", cv_cfg: "_abi.CvConfigC | None"):
        """MLMC with the control variate on every level -> (result, plain level variances)."""
        res = _abi.MlmcResultC()
        pv = np.zeros(_abi.MLMC_MAX_LEVELS)
        _abi.check(self.lib.myql_mlmc_cv_price(self.handle, C.byref(job.c), C.byref(mlmc_cfg),
                                               C.byref(cv_cfg) if cv_cfg is not None else None, C.byref(res),
                                               _ptr(pv)))
        return res, pv

    def mlmc_cv_level(self, job: "_Job", mlmc_cfg: "_abi.MlmcConfigC", level: int, dN: int) -> np.ndarray:
        out = np.zeros(4)
        _abi.check(self.lib.myql_mlmc_cv_level(self.handle, C.byref(job.c), C.byref(mlmc_cfg), level, dN,
                                               _ptr(out)))
        return out

    def fourier(self, job: "_Job", mode: "GreekMode | int" = 0) -> np.ndarray:
        """FP64 Gil-Pelaez oracle of a European job -> (2Q, n) rows (standard errors 0)."""
        out = np.zeros(2 * _abi.Q_COUNT * job.n_strikes, dtype=np.float64)
        _abi.check(self.lib.myql_fourier_price(self.handle, C.byref(job.c), int(mode), _ptr(out)))
        return out.reshape(2 * _abi.Q_COUNT, job.n_strikes)

    def paths(self, job: "_Job") -> np.ndarray:
        nsc, nf = C.c_uint32(), C.c_uint32()
        _abi.check(self.lib.myql_mc_paths(self.handle, C.byref(job.c), None, 0, C.byref(nsc),
                                          C.byref(nf)))
        m = int(job.c.config.num_paths)
        rec = np.zeros(nsc.value * nf.value * m, dtype=np.float32)
        _abi.check(self.lib.myql_mc_paths(self.handle, C.byref(job.c),
                                          rec.ctypes.data_as(C.POINTER(C.c_float)), rec.size,
                                          C.byref(nsc), C.byref(nf)))
        return rec.reshape(nsc.value, nf.value, m)

    def stream_states(self, seed: int, first: int, n: int) -> np.ndarray:
        out = np.zeros(4 * n, dtype=np.uint64)
        _abi.check(self.lib.myql_rng_stream_states(self.handle, seed, first, n,
                                                   out.ctypes.data_as(C.POINTER(C.c_uint64))))
        return out.reshape(n, 4)

    def draws(self, seed: int, first: int, n: int, count: int) -> np.ndarray:
        out = np.zeros(n * count, dtype=np.uint64)
        _abi.check(self.lib.myql_rng_draws(self.handle, seed, first, n, count,
                                           out.ctypes.data_as(C.POINTER(C.c_uint64))))
        return out.reshape(n, count)

    def peak(self, kind: int) -> float:
        """Measured FP32-FMA (kind 0) or MUFU (kind 1) operations per second."""
        v = C.c_double()
        _abi.check(self.lib.myql_probe_peak(self.handle, kind, C.byref(v)))
        return v.value

    def chi2_quantile(self, dof, p) -> np.ndarray:
        dof = np.ascontiguousarray(dof, dtype=np.float64)
        p = np.ascontiguousarray(p, dtype=np.float64)
        out = np.zeros_like(p)
        _abi.check(self.lib.myql_chi2_quantile(self.handle, _ptr(dof), _ptr(p), _ptr(out), p.size))
        return out

    def nci_nodes(self, d: float, rows: int):
        """FP64 nodes of the SchemeNCI table of offset d: (main [rows, 10000], tail [rows, 512])."""
        main = np.zeros((rows, 10000))
        tail = np.zeros((rows, 512))
        _abi.check(self.lib.myql_probe_nci_nodes(self.handle, float(d), int(rows), _ptr(main), _ptr(tail)))
        return main, tail

    def sampler(self, kind: int, x, lam=None) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.uint64)
        out = np.zeros(x.size, dtype=np.float32)
        lam_arr = np.ascontiguousarray(lam, dtype=np.float64) if lam is not None else None
        _abi.check(self.lib.myql_probe_sampler(
            self.handle, kind, x.ctypes.data_as(C.POINTER(C.c_uint64)),
            _ptr(lam_arr) if lam_arr is not None else None,
            out.ctypes.data_as(C.POINTER(C.c_float)), x.size))
        return out


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


_default_engine: Engine | None = None
_engine_lock = threading.Lock()


def default_engine() -> Engine:
    global _default_engine
    with _engine_lock:
        if _default_engine is None:
            _default_engine = Engine(0)
        return _default_engine


# --------------------------------------------------------------------------- job lowering
class _Job:
    """A myql_mc_job plus the numpy buffers it points into."""

    def __init__(self, c: _abi.McJobC, strikes: np.ndarray):
        self.c = c
        self.strikes = strikes
        self.n_strikes = int(strikes.size)


def _model_c(model) -> _abi.ModelC:
    m = _abi.ModelC()
    m.num_factors = model.num_variance_factors
    j = model.jump
    if isinstance(j, MertonParams):
        m.jump, m.jump_lambda, m.merton_mu, m.merton_delta = _abi.JUMP_MERTON, j.lambda_, j.mu, j.delta
    elif isinstance(j, KouParams):
        m.jump, m.jump_lambda = _abi.JUMP_KOU, j.lambda_
        m.kou_p_up, m.kou_eta1, m.kou_eta2 = j.p_up, j.eta1, j.eta2
    else:
        m.jump = _abi.JUMP_NONE
    if isinstance(model, ZeroFactorModel):
        m.vol = model.vol
    hs = ([model.heston] if isinstance(model, SingleFactorModel)
          else [model.heston1, model.heston2] if isinstance(model, DoubleFactorModel) else [])
    for i, h in enumerate(hs):
        m.heston[i] = _abi.HestonParamsC(h.kappa, h.theta, h.sigma, h.rho, h.v0)
    return m


def stepper_for(model, instrument, scheme=SchemeNCI) -> ASVJStepper:
    """dispatcher::StepperFor (StepperTraits.hpp:67-81): scheme for every factor."""
    nf = model.num_variance_factors
    jp = {NoJumpParams: NoJumps, MertonParams: MertonJump, KouParams: KouJump}[type(model.jump)]
    v1 = scheme if nf >= 1 else NullVolScheme
    v2 = scheme if nf == 2 else NullVolScheme
    return ASVJStepper(v1, v2, jp, instrument.Tracker)


def make_job(model, stepper: ASVJStepper | None, instrument: _Instrument, mode: GreekMode,
             cfg: MonteCarloConfig, S0: float, r: float, q: float) -> _Job:
    if stepper is None:
        stepper = stepper_for(model, instrument)
    if stepper.num_cirs != model.num_variance_factors:
        raise TypeError(f"stepper has {stepper.num_cirs} CIR factors, model has "
                        f"{model.num_variance_factors}")
    if not isinstance(model.jump, stepper.JumpPolicy.params):
        raise TypeError(f"stepper jump policy {stepper.JumpPolicy.__name__} does not match "
                        f"model jump parameters {type(model.jump).__name__}")
    if stepper.TrackerPolicy is not None and stepper.TrackerPolicy is not instrument.Tracker:
        raise TypeError(f"stepper tracker {stepper.TrackerPolicy.__name__} does not match the "
                        f"instrument's {instrument.Tracker.__name__}")
    job = _abi.McJobC()
    job.model = _model_c(model)
    ins = job.instrument
    ins.kind = instrument.kind
    ins.payoff = instrument.payoff.code
    ins.option_type = int(instrument.payoff.Type)
    ins.fixed_strike = instrument.fixed_strike
    ins.barrier_up = instrument.barrier_up
    ins.barrier_action = instrument.barrier_action
    ins.rebate_timing = instrument.rebate_timing
    ins.is_strip = int(instrument.is_strip)
    ins.maturity = instrument.T
    ins.barrier = instrument.barrier
    ins.rebate = instrument.rebate
    ins.barrier_rate = instrument.barrier_rate
    ins.payoff_eps = getattr(instrument.payoff, "eps", -1.0)
    strikes = np.ascontiguousarray(instrument.strikes, dtype=np.float64)
    ins.strikes = _ptr(strikes)
    ins.n_strikes = strikes.size
    ins.past_avg_log = instrument.past_avg_log
    ins.past_avg_S = instrument.past_avg_S
    ins.t_elapsed = instrument.t_elapsed
    ins.hist_min_S = instrument.hist_min_S
    ins.hist_max_S = instrument.hist_max_S
    c = job.config
    c.num_paths, c.time_steps, c.seed = cfg.num_paths, cfg.time_steps, cfg.seed
    c.fd_bump, c.vol_bump, c.t_bump, c.r_bump = cfg.fd_bump, cfg.vol_bump, cfg.t_bump, cfg.r_bump
    c.scheme[0] = stepper.VolScheme1.code
    c.scheme[1] = stepper.VolScheme2.code
    c.greek_mode = int(mode)
    c.n_streams = cfg.n_streams
    c.stream_offset = cfg.stream_offset
    job.S0, job.r, job.q = S0, r, q
    return _Job(job, strikes)


def validate(job: _Job) -> None:
    """Host-side checks of the engine (no device needed); raises MyqlError."""
    lib = _abi.load()
    _abi.check(lib.myql_validate_job(C.byref(job.c)))


def result_from_raw(raw: np.ndarray, mode: GreekMode, is_strip: bool, stats=None) -> MonteCarloResult:
    def g(qi, se=False):
        row = raw[2 * qi + (1 if se else 0)]
        return row.copy() if is_strip else float(row[0])

    res = MonteCarloResult(mode=mode, raw=raw, stats=stats)
    res.price, res.price_std_err = g(0), g(0, True)
    if mode >= GreekMode.ESSENTIAL:
        res.delta, res.delta_std_err = g(1), g(1, True)
        res.gamma, res.gamma_std_err = g(2), g(2, True)
    if mode == GreekMode.FULL:
        res.vega, res.vega_std_err = [g(3), g(4)], [g(3, True), g(4, True)]
        res.theta, res.theta_std_err = g(5), g(5, True)
        res.rho, res.rho_std_err = g(6), g(6, True)
        res.vanna, res.vanna_std_err = [g(7), g(8)], [g(7, True), g(8, True)]
        res.charm, res.charm_std_err = g(9), g(9, True)
    return res


class MonteCarloPricer:
    """MonteCarloPricer<Model, Stepper, Instrument, Mode> (MonteCarloPricer.hpp:84-96).

    `stepper=None` resolves the stepper like the runtime dispatcher (SchemeNCI
    for every factor, the jump policy of the model, the instrument's tracker).
    """

    def __init__(self, model, stepper: ASVJStepper | None = None, mode: GreekMode = GreekMode.NONE,
                 cfg: MonteCarloConfig | None = None, engine: Engine | None = None):
        self.model = model
        self.stepper = stepper
        self.mode = GreekMode(mode)
        self.cfg = cfg or MonteCarloConfig()
        self.engine = engine

    def job(self, S0: float, r: float, q: float, instr: _Instrument) -> _Job:
        return make_job(self.model, self.stepper, instr, self.mode, self.cfg, S0, r, q)

    def calculate(self, S0: float, r: float, q: float, instr: _Instrument) -> MonteCarloResult:
        eng = self.engine or default_engine()
        raw, st = eng.price(self.job(S0, r, q, instr))
        return result_from_raw(raw, self.mode, instr.is_strip, st)


@dataclass
class ControlVariateConfig:
    """Settings of the neural martingale control variate (no counterpart in the reference)."""
    hedge_every: int = 8          # time steps per hedge interval
    iterations: int = 120         # Adam steps
    pilot_paths: int = 1 << 18    # training paths (independent seed)
    batch_paths: int = 4096       # paths per Adam step
    learning_rate: float = 5e-3
    seed: int = 1

    @classmethod
    def for_plain_time(cls, plain_seconds: float, time_steps: int | None = None, **kw) -> "ControlVariateConfig":
        """A training budget and hedging interval sized to the job: `plain_seconds` is the
        estimated time of plain Monte Carlo to the wanted standard error, `time_steps` the
        job's steps.  Training is a fixed cost and its variance ratio grows slowly with it
        (Double Bates Asian, 256 steps, GB300: ratio 7.8 after 15 Adam steps of 2048 paths on
        2^15 pilot paths in 3 ms, 17.6 after 120 steps of 4096 on 2^19 in 18 ms); hedge rows
        cost MLP evaluations on every priced path.  So a short job gets the short training and
        8 hedge times per path, a mid-size one 10, a long one the full training and 32.  Keyword
        arguments override any field (an explicit hedge_every wins over time_steps)."""
        if plain_seconds < 0.05:
            budget = dict(pilot_paths=1 << 15, iterations=15, batch_paths=2048)
            rows = 8
        elif plain_seconds < 0.5:
            budget = dict(pilot_paths=1 << 18, iterations=60, batch_paths=2048)
            rows = 10
        else:
            budget = dict(pilot_paths=1 << 19, iterations=120, batch_paths=4096)
            rows = 32
        if time_steps is not None:
            budget["hedge_every"] = max(1, int(time_steps) // rows)
        budget.update(kw)
        return cls(**budget)

    def c(self) -> _abi.CvConfigC:
        c = _abi.CvConfigC()
        c.hedge_every, c.iterations, c.pilot_paths = self.hedge_every, self.iterations, self.pilot_paths
        c.batch_paths, c.learning_rate, c.seed = self.batch_paths, self.learning_rate, self.seed
        return c


@dataclass
class ControlVariateResult:
    price: float
    price_std_err: float
    plain_price: float
    plain_std_err: float
    variance_ratio: float
    train: object = None
    raw: object = None


class NeuralCVPricer:
    """MonteCarloPricer with a learned martingale control variate (GreekMode::None).

    `train(S0, r, q, instrument)` fits the network on pilot paths of the model;
    `calculate(S0, r, q, instrument)` prices with it and also reports the plain
    Monte Carlo estimator of the same paths.  Scalar European / Asian instruments.
    With qmc_replicates = R > 0 the pricing paths are randomized QMC (R digital
    shifts, myql_cv_qmc_price) and the standard errors come from the replicates.
    """

    def __init__(self, model, stepper: ASVJStepper | None = None, cfg: MonteCarloConfig | None = None,
                 cv: ControlVariateConfig | None = None, engine: Engine | None = None, qmc_replicates: int = 0):
        self.model, self.stepper = model, stepper
        self.cfg = cfg or MonteCarloConfig()
        self.cv = cv or ControlVariateConfig()
        self.engine = engine
        self.qmc_replicates = qmc_replicates
        self.train_result = None

    def _job(self, S0, r, q, instr):
        return make_job(self.model, self.stepper, instr, GreekMode.NONE, self.cfg, S0, r, q)

    def train(self, S0: float, r: float, q: float, instr: _Instrument):
        eng = self.engine or default_engine()
        self.train_result = eng.cv_train(self._job(S0, r, q, instr), self.cv.c())
        return self.train_result

    def calculate(self, S0: float, r: float, q: float, instr: _Instrument) -> ControlVariateResult:
        eng = self.engine or default_engine()
        if self.train_result is None:
            self.train(S0, r, q, instr)
        job = self._job(S0, r, q, instr)
        if self.qmc_replicates:
            res = eng.cv_qmc_price(job, self.cv.c(), self.qmc_replicates)
        else:
            res = eng.cv_price(job, self.cv.c())
        return ControlVariateResult(res.price, res.price_std_err, res.plain_price, res.plain_std_err,
                                    res.variance_ratio, self.train_result, res)
