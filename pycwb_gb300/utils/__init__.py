"""GPU drop-ins for pycwb/utils modules on the hot path."""
