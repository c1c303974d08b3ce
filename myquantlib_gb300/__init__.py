"""GB300-native (sm_103a) Monte Carlo path-simulation engine for MyQuantLib's pricer API.

The compute runs in hand-written CUDA kernels inside libmyql_gpu.so (C ABI in
include/myql_gpu.h); this package is the Python host mirror of the reference's
MonteCarloPricer / MultiLevelMonteCarloPricer interface on top of that ABI.
"""
from .pricers import *  # noqa: F401,F403
from .pricers import (  # noqa: F401
    Engine, MonteCarloConfig, MonteCarloPricer, MonteCarloResult, default_engine, make_job,
    result_from_raw, stepper_for,
)
from . import _abi  # noqa: F401
from . import dispatch  # noqa: F401
from . import registry  # noqa: F401
from . import calibration  # noqa: F401
