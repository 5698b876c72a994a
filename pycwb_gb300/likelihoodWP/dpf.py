"""GPU drop-in for pycwb/modules/likelihoodWP/dpf.py (calculate_dpf, dpf.py:7-34)."""

from .sky_scan import calculate_dpf

__all__ = ["calculate_dpf"]
