"""GB300 (sm_103a) VarElecCond time-step hot path: CUDA kernels behind a C-ABI."""
from .params import VecParams, default_params, config0, config1, convection_params  # noqa: F401
