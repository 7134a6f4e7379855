"""mesolf_gb300 -- GB300 (sm_103a) light-field projector and phase-space RL deconvolver.

The compute lives in ``libmesolf_lf.so`` (C ABI: ``include/mesolf_lf.h``); this package
holds its build recipe, ctypes bindings, the reference-shaped Python entry points and
the seeded synthetic workload generators.
"""
from ._lib import MesoLFError, load as load_library  # noqa: F401
from .api import (BatchSolver, PhaseSpacePSF, RLSolver, mex_lfm_convolution_vec,  # noqa: F401
                  recon_theory_phase_space_LFM_with_filter,
                  recon_theory_phase_space_LFM_with_filter_simple_peeling, forwardProjectGPU,
                  forwardProjectACC, forwardProjectGPU_discrete, forwardProjectGPU_skip_2D,
                  mex_lfm_convolution_vec_accumulate, seed_library_projections)

__all__ = ["MesoLFError", "load_library", "BatchSolver", "PhaseSpacePSF", "RLSolver", "mex_lfm_convolution_vec",
           "recon_theory_phase_space_LFM_with_filter", "recon_theory_phase_space_LFM_with_filter_simple_peeling",
           "forwardProjectGPU", "forwardProjectACC", "forwardProjectGPU_discrete", "forwardProjectGPU_skip_2D",
           "mex_lfm_convolution_vec_accumulate", "seed_library_projections"]
