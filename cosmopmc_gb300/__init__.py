"""cosmopmc_gb300 — a GB300 (sm_103a) Population Monte Carlo iteration engine.

The product is the C-ABI shared library `libpmcg.so` (include/pmcg.h): CUDA
kernels for the draws, the mixture log-density, the SN Ia / template /
Gaussian-mixture likelihoods, the importance weights with evidence and
perplexity, and the Rao-Blackwellised EM update, behind pmclib's entry-point
names. `cosmopmc_gb300.pmcg` is its ctypes mirror.
"""
from . import pmcg  # noqa: F401
from .pmcg import (FP64, MIXED, MixMvdens, Parabox, PmcSimu, Posterior, PmcgError, Rng, Run,  # noqa: F401
                   load)

__all__ = ["pmcg", "FP64", "MIXED", "MixMvdens", "Parabox", "PmcSimu", "Posterior", "PmcgError", "Rng", "Run",
           "load"]
