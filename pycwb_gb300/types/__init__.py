"""GPU drop-ins for pycwb/types containers on the hot path."""
