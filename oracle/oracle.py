"""ctypes access to the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module: it checks or times the GPU engine, it is never part of it.

  restatement  oracle/_build/liboracle[_fast].so  -- FP64 C restatement of the
               reference's Monte Carlo path (oracle/mc_oracle.c); builds
               anywhere with gcc.
  reference    oracle/_ref/libmyql_ref[_fast].so  -- the reference's own
               headers compiled against the Boost-API shim in oracle/compat;
               builds only where the reference sources are present.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LAYOUT_REFERENCE = 0
LAYOUT_STREAMS = 1
REF_ROOT = Path(os.environ.get("MYQL_REF_ROOT", "/root/reference"))

_libs: dict[str, C.CDLL] = {}


def build(ref: bool | None = None) -> None:
    """make -C oracle (and the reference shim when its sources exist)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    if ref is None:
        ref = (REF_ROOT / "include" / "myql").exists()
    if ref:
        subprocess.run(["make", "-s", "-j2", "-C", str(HERE), "ref", f"REF_ROOT={REF_ROOT}"], check=True)


def _load(name: str) -> C.CDLL:
    if name in _libs:
        return _libs[name]
    path = HERE / name
    if not path.exists():
        build(ref=name.startswith("_ref"))
    lib = C.CDLL(str(path))
    _libs[name] = lib
    return lib


def restatement(fast: bool = False) -> C.CDLL:
    lib = _load("_build/liboracle_fast.so" if fast else "_build/liboracle.so")
    lib.myql_oracle_mc_price.restype = C.c_int
    lib.myql_oracle_mc_price.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double),
                                         C.POINTER(C.c_double)]
    lib.myql_oracle_stream_states.restype = C.c_int
    lib.myql_oracle_stream_states.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, C.POINTER(C.c_uint64)]
    for fn in ("myql_oracle_normcdfinv", "myql_oracle_chi2_quantile"):
        getattr(lib, fn).restype = C.c_double
    lib.myql_oracle_normcdfinv.argtypes = [C.c_double]
    lib.myql_oracle_poissinvcdf.restype = C.c_double
    lib.myql_oracle_poissinvcdf.argtypes = [C.c_double, C.c_double]
    lib.myql_oracle_chi2_quantile.argtypes = [C.c_double, C.c_double]
    lib.myql_oracle_mlmc_price.restype = C.c_int
    lib.myql_oracle_mlmc_price.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    lib.myql_oracle_mlmc_level.restype = C.c_int
    lib.myql_oracle_mlmc_level.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_uint32,
                                           C.c_uint64, C.POINTER(C.c_double)]
    lib.myql_oracle_uniform_of.restype = C.c_double
    lib.myql_oracle_uniform_of.argtypes = [C.c_uint64]
    return lib


def reference_available() -> bool:
    return (HERE / "_ref" / "libmyql_ref.so").exists() or (REF_ROOT / "include" / "myql").exists()


def reference(fast: bool = False) -> C.CDLL:
    lib = _load("_ref/libmyql_ref_fast.so" if fast else "_ref/libmyql_ref.so")
    lib.myql_ref_mc_price.restype = C.c_int
    lib.myql_ref_mc_price.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
    lib.myql_ref_mlmc_price.restype = C.c_int
    lib.myql_ref_mlmc_price.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    lib.myql_ref_fourier.restype = C.c_int
    lib.myql_ref_fourier.argtypes = [C.c_void_p, C.c_double, C.POINTER(C.c_double)]
    return lib


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def mc_price(job, layout: int = LAYOUT_REFERENCE, n_threads: int = 1, records: bool = False,
             fast: bool = False):
    """Restatement price of a myquantlib_gb300 job -> ((2Q, n) array, records or None)."""
    lib = restatement(fast)
    n = job.n_strikes
    out = np.zeros(20 * n)
    rec = None
    if records:
        m = int(job.c.config.num_paths)
        rec = np.zeros(9 * m * 6)
    st = lib.myql_oracle_mc_price(C.byref(job.c), layout, n_threads, _dptr(out),
                                  _dptr(rec) if rec is not None else None)
    if st != 0:
        raise RuntimeError(f"oracle failed ({st})")
    if rec is not None:
        m = int(job.c.config.num_paths)
        rec = rec.reshape(9, m, 6)
    return out.reshape(20, n), rec


def ref_mc_price(job, n_threads: int = 1, fast: bool = False) -> np.ndarray | None:
    """The reference's own MonteCarloPricer (None when not instantiated in the shim)."""
    lib = reference(fast)
    n = job.n_strikes
    out = np.zeros(20 * n)
    st = lib.myql_ref_mc_price(C.byref(job.c), n_threads, _dptr(out))
    if st == -2:
        return None
    if st != 0:
        raise RuntimeError(f"reference failed ({st})")
    return out.reshape(20, n)


def ref_fourier(job, tol: float = 1e-10) -> np.ndarray:
    """The reference's FP64 Fourier price and Full Greeks (10 values) of a European."""
    lib = reference()
    out = np.zeros(10)
    if lib.myql_ref_fourier(C.byref(job.c), tol, _dptr(out)) != 0:
        raise RuntimeError("reference Fourier failed")
    return out


def stream_states(seed: int, first: int, n: int) -> np.ndarray:
    lib = restatement()
    out = np.zeros(4 * n, dtype=np.uint64)
    lib.myql_oracle_stream_states(seed, first, n, out.ctypes.data_as(C.POINTER(C.c_uint64)))
    return out.reshape(n, 4)


def mlmc_price(job, cfg, layout: int = LAYOUT_REFERENCE, n_threads: int = 1, fast: bool = False):
    """Restatement of MultiLevelMonteCarloPricer::calculate -> MlmcResultC."""
    from myquantlib_gb300 import _abi
    res = _abi.MlmcResultC()
    if restatement(fast).myql_oracle_mlmc_price(C.byref(job.c), C.byref(cfg), layout, n_threads, C.byref(res)) != 0:
        raise RuntimeError("oracle MLMC failed")
    return res


def ref_mlmc_price(job, cfg, n_threads: int = 1):
    """The reference's own MultiLevelMonteCarloPricer (None when not instantiated)."""
    from myquantlib_gb300 import _abi
    res = _abi.MlmcResultC()
    st = reference().myql_ref_mlmc_price(C.byref(job.c), C.byref(cfg), n_threads, C.byref(res))
    if st == -2:
        return None
    if st != 0:
        raise RuntimeError(f"reference MLMC failed ({st})")
    return res


def mlmc_level(job, cfg, level: int, dN: int, layout: int = LAYOUT_STREAMS, n_threads: int = 1):
    """One evaluate_level call of the restatement -> (sum, sum of squares)."""
    out = np.zeros(2)
    if restatement().myql_oracle_mlmc_level(C.byref(job.c), C.byref(cfg), layout, n_threads, level, dN,
                                            _dptr(out)) != 0:
        raise RuntimeError("oracle MLMC level failed")
    return out
