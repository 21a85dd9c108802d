"""sfhgpu: GB300 (sm_103a) Hess-diagram hot path of StarFormationHistories.jl.

Python mirror of the reference's Julia API over the C ABI in include/sfhgpu.h.
All compute runs in libsfhgpu.so; there is no CPU fallback.
"""
from ._lib import (SFH_BF16X2, SFH_F32, SFH_F64, EXPORTED, LIB_PATH, SFHArgumentError, SFHError,
                   load)
from .core import Context, Models, as_models, default_context
from .emulator import SyntheticGenerator, TemplateEmulator
from .fitting import (Galaxies, composite_, construct_x0, construct_x0_mdf, fg_, fg_batched,
                      fg_ragged, fit_templates, fixed_amr, truncate_relweights,
                      fit_templates_fast, fit_templates_lbfgsb, grad_loglikelihood,
                      fit_bfgs_device, FIT_LOG_MAP, FIT_LOG_MLE, FIT_SQRT,
                      grad_loglikelihood_, loglikelihood, renormalize_x0, stack_models)
from .sampling import (BFGSResult, CompositeBFGSResult, GaussianDispersion, LinearAMR,
                       LogarithmicAMR, MH_from_Z, PowerLawMZR, calculate_coeffs, dMH_dZ, fit_sfh,
                       fit_sfh_x0, hmc_sample, laplace_metric, logdensity_batched, sample_sfh)
from .templates import (BrokenPowerLawIMF, Histogram, Kroupa2001, Martin2016_complete,
                        bin_cmd_smooth, calculate_edges, calculate_weights, compl_model, err_model,
                        exp_photerr, histogram_data, histogram_pix, interpolate_mini, midpoints,
                        mini_spacing, partial_cmd_smooth, partial_cmd_smooth_batch,
                        partial_cmd_smooth_ragged, NoBinaries, RandomBinaryPairs, trapz,
                        binary_points, binary_hess_batch, partial_cmd_smooth_binary_batch,
                        bin_cmd, partial_cmd, partial_cmd_points, julia_range, julia_colon, Range,
                        model_cmd)

__all__ = [
    "SFH_BF16X2", "SFH_F32", "SFH_F64", "EXPORTED", "LIB_PATH", "SFHArgumentError", "SFHError",
    "load", "Context", "Models", "as_models", "default_context", "composite_", "construct_x0",
    "fg_", "fg_batched", "fit_templates", "fit_templates_fast", "fit_templates_lbfgsb", "fit_bfgs_device", "FIT_LOG_MAP",
    "FIT_LOG_MLE", "FIT_SQRT", "grad_loglikelihood",
    "grad_loglikelihood_", "loglikelihood", "renormalize_x0", "stack_models", "BrokenPowerLawIMF",
    "Histogram", "Kroupa2001", "Martin2016_complete", "bin_cmd", "bin_cmd_smooth", "calculate_edges",
    "partial_cmd", "partial_cmd_points", "julia_range", "julia_colon", "Range", "model_cmd",
    "calculate_weights", "compl_model", "err_model", "exp_photerr", "histogram_data",
    "histogram_pix", "interpolate_mini", "midpoints", "mini_spacing", "partial_cmd_smooth",
    "partial_cmd_smooth_batch", "NoBinaries", "RandomBinaryPairs", "trapz", "binary_points",
    "binary_hess_batch", "partial_cmd_smooth_binary_batch", "GaussianDispersion", "PowerLawMZR", "calculate_coeffs",
    "hmc_sample", "laplace_metric", "logdensity_batched", "sample_sfh", "Galaxies", "fg_ragged",
    "partial_cmd_smooth_ragged", "SyntheticGenerator", "TemplateEmulator", "LinearAMR",
    "construct_x0_mdf", "fixed_amr", "truncate_relweights", "LogarithmicAMR", "MH_from_Z",
    "dMH_dZ", "fit_sfh", "fit_sfh_x0", "BFGSResult", "CompositeBFGSResult",
]
