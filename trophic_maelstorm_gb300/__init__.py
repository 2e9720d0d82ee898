"""GB300-native spatial stochastic integrator (Dornic-split 2-D lattice Langevin).

The compute path is libtm.so (hand-written sm_103a kernels behind the C ABI in
include/tm.h); this package is its Python host side.  Build the library with
`python -m trophic_maelstorm_gb300.build`.
"""
from . import _lib
from ._lib import (TM_FP32, TM_FP64, TM_REM_EULER_EXACT, TM_REM_RK4, TM_SAMPLER_EXACT, TM_SAMPLER_OFF,
                   TM_SAMPLER_REF_GAUSS100, TM_STATUS_NAN, TM_STATUS_NEGATIVE, TM_STATUS_SAMPLER_CAP, TMError)
from .api import (Batch, Context, FKEParams, critical_exp_delta, critical_exp_finite_scaling_collapse,
                  critical_exp_finite_scaling_stationary, critical_exp_theta_delta, dp_model, fke_advdiff, fke_parameters,
                  gaussian_stencil, instances, layout, linspace,
                  logarithm10_time_bins, pack, pattern_wavelength, percolation_dornic_2d, reference_step_grid, replicate_rows,
                  rietkerk_model, run_dp, unpack)

__all__ = [
    "_lib", "TM_FP32", "TM_FP64", "TM_REM_EULER_EXACT", "TM_REM_RK4", "TM_SAMPLER_EXACT", "TM_SAMPLER_OFF",
    "TM_SAMPLER_REF_GAUSS100", "TM_STATUS_NAN", "TM_STATUS_NEGATIVE", "TM_STATUS_SAMPLER_CAP", "TMError",
    "Batch", "Context", "FKEParams", "critical_exp_delta", "critical_exp_finite_scaling_collapse",
    "critical_exp_finite_scaling_stationary", "critical_exp_theta_delta", "dp_model", "fke_advdiff", "fke_parameters",
    "gaussian_stencil", "instances", "layout", "linspace",
    "logarithm10_time_bins", "pack", "pattern_wavelength", "percolation_dornic_2d", "reference_step_grid", "replicate_rows",
    "rietkerk_model", "run_dp", "unpack",
]
