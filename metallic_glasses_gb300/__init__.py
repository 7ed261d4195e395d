"""GB300-native shear-transformation-zone kinetic Monte Carlo engine.

The engine is the CUDA library built from metallic_glasses_gb300/csrc
(C ABI: include/stz_api.h); this package is its Python host mirror.
"""
from .api import *  # noqa: F401,F403
from .api import Engine, Params, default_params, load_library, params_from_input  # noqa: F401
from . import configs  # noqa: F401
