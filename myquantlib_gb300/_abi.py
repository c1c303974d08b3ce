"""ctypes mirror of include/myql_gpu.h and the loader of libmyql_gpu.so.

The library is built in-tree (myquantlib_gb300/build.py).  Loading fails loudly
when it is missing: there is no CPU fallback for the engine.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libmyql_gpu.so"

# enums (myql_gpu.h)
OK, ERR_INVALID_ARG, ERR_NV_CONDITION, ERR_OOM, ERR_CUDA, ERR_LOOP_CAP, ERR_TIMEOUT, \
    ERR_NO_DEVICE, ERR_UNSUPPORTED, ERR_TOO_LARGE = range(10)
SCHEME_NONE, SCHEME_NV, SCHEME_EXACT, SCHEME_NCI = range(4)
JUMP_NONE, JUMP_MERTON, JUMP_KOU = range(3)
INSTR_EUROPEAN, INSTR_ASIAN_GEO, INSTR_ASIAN_ARITH, INSTR_LOOKBACK, INSTR_BARRIER = range(5)
PAYOFF_VANILLA, PAYOFF_CASH, PAYOFF_ASSET = range(3)
CALL, PUT = 0, 1
GREEKS_NONE, GREEKS_ESSENTIAL, GREEKS_FULL = range(3)
BARRIER_IN, BARRIER_OUT = 0, 1
REBATE_NONE, REBATE_AT_HIT, REBATE_AT_MATURITY = range(3)
Q_NAMES = ("price", "delta", "gamma", "vega0", "vega1", "theta", "rho", "vanna0", "vanna1", "charm")
Q_COUNT = len(Q_NAMES)
MLMC_MAX_LEVELS = 24
QMC_DEFAULT_DIRECTION_SEED = 6  # MYQL_QMC_DEFAULT_DIRECTION_SEED


class HestonParamsC(C.Structure):
    _fields_ = [("kappa", C.c_double), ("theta", C.c_double), ("sigma", C.c_double),
                ("rho", C.c_double), ("v0", C.c_double)]


class ModelC(C.Structure):
    _fields_ = [("num_factors", C.c_int32), ("jump", C.c_int32), ("vol", C.c_double),
                ("heston", HestonParamsC * 2), ("jump_lambda", C.c_double),
                ("merton_mu", C.c_double), ("merton_delta", C.c_double),
                ("kou_p_up", C.c_double), ("kou_eta1", C.c_double), ("kou_eta2", C.c_double)]


class InstrumentC(C.Structure):
    _fields_ = [("kind", C.c_int32), ("payoff", C.c_int32), ("option_type", C.c_int32),
                ("fixed_strike", C.c_int32), ("barrier_up", C.c_int32),
                ("barrier_action", C.c_int32), ("rebate_timing", C.c_int32),
                ("is_strip", C.c_int32), ("maturity", C.c_double), ("barrier", C.c_double),
                ("rebate", C.c_double), ("barrier_rate", C.c_double), ("payoff_eps", C.c_double),
                ("strikes", C.POINTER(C.c_double)), ("n_strikes", C.c_int64),
                ("past_avg_log", C.c_double), ("past_avg_S", C.c_double), ("t_elapsed", C.c_double),
                ("hist_min_S", C.c_double), ("hist_max_S", C.c_double)]


class McConfigC(C.Structure):
    _fields_ = [("num_paths", C.c_uint64), ("time_steps", C.c_uint64), ("seed", C.c_uint64),
                ("fd_bump", C.c_double), ("vol_bump", C.c_double), ("t_bump", C.c_double),
                ("r_bump", C.c_double), ("scheme", C.c_int32 * 2), ("greek_mode", C.c_int32),
                ("n_streams", C.c_uint64), ("stream_offset", C.c_uint64)]


class McJobC(C.Structure):
    _fields_ = [("model", ModelC), ("instrument", InstrumentC), ("config", McConfigC),
                ("S0", C.c_double), ("r", C.c_double), ("q", C.c_double)]


class McStatsC(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("path_steps", C.c_uint64), ("scenarios", C.c_uint32),
                ("loop_cap_hits", C.c_uint32), ("table_fallbacks", C.c_uint32),
                ("kernel_launches", C.c_uint32), ("device_ms", C.c_double),
                ("simulate_ms", C.c_double), ("payoff_ms", C.c_double)]


class MlmcConfigC(C.Structure):
    _fields_ = [("epsilon", C.c_double), ("L_min", C.c_uint64), ("L_max", C.c_uint64),
                ("N0", C.c_uint64), ("base_steps", C.c_uint64), ("alpha", C.c_double),
                ("beta", C.c_double), ("adaptive_rates", C.c_int32), ("seed", C.c_uint64),
                ("fd_bump", C.c_double), ("n_streams", C.c_uint64)]


class MlmcResultC(C.Structure):
    _fields_ = [("price", C.c_double), ("price_std_err", C.c_double), ("total_steps", C.c_uint64),
                ("n_levels", C.c_uint32), ("paths_per_level", C.c_uint64 * MLMC_MAX_LEVELS),
                ("mean_diffs", C.c_double * MLMC_MAX_LEVELS),
                ("var_diffs", C.c_double * MLMC_MAX_LEVELS),
                ("alpha_estimated", C.c_double), ("beta_estimated", C.c_double),
                ("device_ms", C.c_double)]


CV_PARAMS = 35332


class CvConfigC(C.Structure):
    _fields_ = [("hedge_every", C.c_uint32), ("iterations", C.c_uint32), ("pilot_paths", C.c_uint64),
                ("batch_paths", C.c_uint64), ("learning_rate", C.c_double), ("seed", C.c_uint64)]


class CvResultC(C.Structure):
    _fields_ = [("price", C.c_double), ("price_std_err", C.c_double), ("plain_price", C.c_double),
                ("plain_std_err", C.c_double), ("variance_ratio", C.c_double), ("initial_loss", C.c_double),
                ("final_loss", C.c_double), ("train_ms", C.c_double), ("simulate_ms", C.c_double),
                ("mlp_ms", C.c_double), ("total_ms", C.c_double), ("paths", C.c_uint64),
                ("kernel_launches", C.c_uint32)]


class BatchClassPlanC(C.Structure):
    _fields_ = [("factors", C.c_int32), ("scheme1", C.c_int32), ("scheme2", C.c_int32),
                ("path_dependent", C.c_int32), ("block", C.c_int32), ("streams_per_thread", C.c_int32),
                ("unroll", C.c_int32), ("tuned", C.c_int32), ("grid", C.c_uint32), ("items", C.c_uint64),
                ("tuned_ms", C.c_double), ("default_ms", C.c_double)]


class MyqlError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[myql status {status}] {message}")
        self.status = status


_SIGS = {
    "myql_abi_version": (C.c_int, []),
    "myql_last_error": (C.c_size_t, [C.c_char_p, C.c_size_t]),
    "myql_ctx_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
    "myql_ctx_destroy": (C.c_int, [C.c_void_p]),
    "myql_ctx_set_loop_cap": (C.c_int, [C.c_void_p, C.c_uint32]),
    "myql_ctx_set_records_limit": (C.c_int, [C.c_void_p, C.c_uint64]),
    "myql_ctx_set_nci_slopes": (C.c_int, [C.c_void_p, C.c_int]),
    "myql_ctx_set_nci_rows": (C.c_int, [C.c_void_p, C.c_int]),
    "myql_ctx_set_precise_theta": (C.c_int, [C.c_void_p, C.c_int]),
    "myql_ctx_set_qmc_direction_seed": (C.c_int, [C.c_void_p, C.c_uint64]),
    "myql_ctx_set_batch_shape": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "myql_batch_last_plan": (C.c_int, [C.c_void_p, C.POINTER(BatchClassPlanC), C.c_size_t,
                                       C.POINTER(C.c_size_t)]),
    "myql_validate_job": (C.c_int, [C.POINTER(McJobC)]),
    "myql_mc_price": (C.c_int, [C.c_void_p, C.POINTER(McJobC), C.POINTER(C.c_double),
                                C.POINTER(McStatsC)]),
    "myql_mc_price_async": (C.c_int, [C.c_void_p, C.POINTER(McJobC), C.c_void_p, C.c_void_p]),
    "myql_mc_price_noalloc": (C.c_int, [C.c_int, C.POINTER(McJobC), C.c_void_p, C.c_void_p]),
    "myql_mc_price_batch": (C.c_int, [C.c_void_p, C.POINTER(McJobC), C.c_size_t,
                                      C.POINTER(C.POINTER(C.c_double)), C.POINTER(McStatsC)]),
    "myql_mc_paths": (C.c_int, [C.c_void_p, C.POINTER(McJobC), C.POINTER(C.c_float), C.c_size_t,
                                C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "myql_mlmc_price": (C.c_int, [C.c_void_p, C.POINTER(McJobC), C.POINTER(MlmcConfigC),
                                  C.POINTER(MlmcResultC)]),
    "myql_qmc_price": (C.c_int, [C.c_void_p, C.POINTER(McJobC), C.c_uint32, C.POINTER(C.c_double),
                                 C.POINTER(McStatsC)]),
    "myql_qmc_directions": (C.c_int, [C.c_uint32, C.c_uint64, C.POINTER(C.c_uint32)]),
    "myql_ml2r_price": (C.c_int, [C.c_void_p, C.POINTER(McJobC), C.POINTER(MlmcConfigC),
                                  C.POINTER(MlmcResultC)]),
    "myql_mlmc_level": (C.c_int, [C.c_void_p, C.POINTER(McJobC), C.POINTER(MlmcConfigC), C.c_uint32,
                                  C.c_uint64, C.POINTER(C.c_double)]),
    "myql_rng_stream_states": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint64,
                                         C.POINTER(C.c_uint64)]),
    "myql_rng_draws": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64,
                                 C.POINTER(C.c_uint64)]),
    "myql_chi2_quantile": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                     C.POINTER(C.c_double), C.c_size_t]),
    "myql_probe_nci_nodes": (C.c_int, [C.c_void_p, C.c_double, C.c_int, C.POINTER(C.c_double),
                                       C.POINTER(C.c_double)]),
    "myql_probe_sampler": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_uint64),
                                     C.POINTER(C.c_double), C.POINTER(C.c_float), C.c_size_t]),
    "myql_probe_peak": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
    "myql_cv_train": (C.c_int, [C.c_void_p, C.POINTER(McJobC), C.POINTER(CvConfigC), C.POINTER(CvResultC)]),
    "myql_cv_price": (C.c_int, [C.c_void_p, C.POINTER(McJobC), C.POINTER(CvConfigC), C.POINTER(CvResultC)]),
    "myql_cv_qmc_price": (C.c_int, [C.c_void_p, C.POINTER(McJobC), C.POINTER(CvConfigC), C.c_uint32,
                                    C.POINTER(CvResultC)]),
    "myql_cv_init": (C.c_int, [C.c_void_p, C.c_uint64]),
    "myql_cv_get_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_size_t]),
    "myql_cv_set_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_size_t]),
    "myql_cv_forward": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_uint64, C.c_uint32,
                                  C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "myql_cv_gradient": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                   C.c_uint64, C.c_uint32, C.POINTER(C.c_float), C.POINTER(C.c_double)]),
    "myql_mlmc_cv_price": (C.c_int, [C.c_void_p, C.POINTER(McJobC), C.POINTER(MlmcConfigC), C.POINTER(CvConfigC),
                                     C.POINTER(MlmcResultC), C.POINTER(C.c_double)]),
    "myql_mlmc_cv_level": (C.c_int, [C.c_void_p, C.POINTER(McJobC), C.POINTER(MlmcConfigC), C.c_uint32,
                                     C.c_uint64, C.POINTER(C.c_double)]),
    "myql_fourier_price": (C.c_int, [C.c_void_p, C.POINTER(McJobC), C.c_int32, C.POINTER(C.c_double)]),
    "myql_probe_mma": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                 C.POINTER(C.c_float)]),
}

_lib = None


def declared_symbols() -> list[str]:
    return sorted(_SIGS)


def load(path: Path | str | None = None) -> C.CDLL:
    """Loads libmyql_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with `python -m myquantlib_gb300.build` "
                           "(the engine has no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def last_error() -> str:
    lib = load()
    buf = C.create_string_buffer(1024)
    lib.myql_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(status: int) -> None:
    if status != OK:
        raise MyqlError(status, last_error())
