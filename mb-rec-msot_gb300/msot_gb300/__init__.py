"""GB300 (sm_103a) implementation of the MSOT model-based operator A / A^T,
the non-negative solvers that call it and the analytic reconstructors,
behind the reference toolbox's interfaces (juestellab/mb-rec-msot).

All compute runs in the CUDA library libmsotgpu.so (C ABI in
include/msot_gpu.h); this package is the host-side mirror of the
reference's MATLAB classes and functions.
"""
from . import _build, _lib  # noqa: F401
from .model import Discretization, MSOTmodel, Probe, butter_zero_phase  # noqa: F401
from .analytic import backproject_waveeq, dmas_cf, reconstruct_dmas_cf  # noqa: F401
from .solvers import (ITV, SB_ITV, SB_ITV2, rec_nn_with_L1_eye_reg, rec_nn_with_L2_reg,  # noqa: F401
                      rec_nn_with_TV_reg)

__all__ = ["Probe", "Discretization", "MSOTmodel", "rec_nn_with_L2_reg",
           "rec_nn_with_L1_eye_reg", "butter_zero_phase", "dmas_cf", "reconstruct_dmas_cf",
           "backproject_waveeq", "rec_nn_with_TV_reg", "SB_ITV", "SB_ITV2", "ITV"]
