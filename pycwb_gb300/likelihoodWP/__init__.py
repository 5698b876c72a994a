"""GB300 drop-in for PycWB's likelihoodWP sky loop.

Module substitution, as the reference's own GPU backend does
(pycwb/modules/likelihoodWPGPU/__init__.py): the functions here keep the
signatures of pycwb.modules.likelihoodWP.dpf.calculate_dpf and
pycwb.modules.likelihoodWP.sky_scan.scan_sky_for_best_fit.
"""

from .sky_scan import (N_STATS, STAT_NAMES, calculate_dpf, find_optimal_sky_localization,
                       scan_sky_for_best_fit, sky_loop)

__all__ = ["N_STATS", "STAT_NAMES", "calculate_dpf", "find_optimal_sky_localization",
           "scan_sky_for_best_fit", "sky_loop"]
