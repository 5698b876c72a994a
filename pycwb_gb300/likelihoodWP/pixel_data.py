"""Per-cluster inputs of the sky loop from the reference's pixel arrays.

Mirrors pycwb/modules/likelihoodWP/pixel_data.py:55-71
(_extract_pixel_array_time_delay_data) and :74-128
(build_sky_delay_and_antenna_patterns), plus the transposes of
likelihood.py:299-305 that turn them into the scan's layout.
"""

from __future__ import annotations

import numpy as np

from .. import sky


def _extract_pixel_array_time_delay_data(pixel_arrays):
    """(noise_weights (nIFO, P) float32, td_phase0, td_phase90, td_energy
    (nIFO, P, 2K+1)) from an object with ``noise_rms`` (nIFO, P) and
    ``td_amp_dense()`` (P, nIFO, 2(2K+1)), as pixel_data.py:55-71:
    w_i = (1/rms_i) / sqrt(sum_j 1/rms_j^2) in float64, cast to float32."""
    inv = 1.0 / np.asarray(pixel_arrays.noise_rms).astype(np.float64)
    norm = 1.0 / np.sqrt(np.sum(inv ** 2, axis=0))
    noise_weights = (inv * norm[np.newaxis, :]).astype(np.float32)
    td = np.asarray(pixel_arrays.td_amp_dense())
    if td.ndim != 3 or td.shape[2] % 2:
        raise ValueError("td_amp_dense() must be (n_pix, n_ifo, 2 * n_delay)")
    half = td.shape[2] // 2
    td_phase0 = td[:, :, :half].transpose(1, 0, 2)
    td_phase90 = td[:, :, half:].transpose(1, 0, 2)
    return noise_weights, td_phase0, td_phase90, td_phase0 ** 2 + td_phase90 ** 2


def extract_pixel_time_delay_data(pixels, nifo, pixel_arrays=None):
    """pixel_data.py:19-52 for the ``PixelArrays`` path (the only one with
    precomputed td amplitudes); per-pixel ``Pixel`` lists are not supported."""
    if pixel_arrays is None:
        raise ValueError("pixel_arrays with td amplitudes is required")
    out = _extract_pixel_array_time_delay_data(pixel_arrays)
    if out[0].shape[0] != int(nifo):
        raise ValueError(f"pixel_arrays has {out[0].shape[0]} detectors, expected {nifo}")
    return out


load_data_from_pixels = extract_pixel_time_delay_data
_load_data_from_pixel_arrays = _extract_pixel_array_time_delay_data


def scan_inputs(noise_weights, td_phase0, td_phase90):
    """The scan's layout (likelihood.py:303-305): rms (P, nIFO), td00/td90
    (2K+1, nIFO, P), float32, C-contiguous."""
    rms = np.ascontiguousarray(np.asarray(noise_weights).T, dtype=np.float32)
    td00 = np.ascontiguousarray(np.transpose(np.asarray(td_phase0, np.float32), (2, 0, 1)))
    td90 = np.ascontiguousarray(np.transpose(np.asarray(td_phase90, np.float32), (2, 0, 1)))
    return rms, td00, td90


def td_size_for(config) -> tuple[float, int]:
    """(TD rate, delay range K) of a config, as pixel_data.py:113-124:
    TDRate = rateANA * upTDF unless given; K = max(TDSize * upTDF,
    int(max_delay * TDRate) + 1)."""
    up = int(getattr(config, "upTDF", 1))
    rate = int(getattr(config, "TDRate", int(getattr(config, "rateANA")) * up))
    K = max(int(getattr(config, "TDSize")) * up, int(getattr(config, "max_delay", 0.0) * float(rate)) + 1)
    return float(rate), int(K)


def build_sky_delay_and_antenna_patterns(nIFO, strains=None, config=None, ml=None, FP=None,
                                         FX=None):
    """(ml (nIFO, n_sky) int32, FP, FX (nIFO, n_sky) float64); precomputed
    arrays pass through (pixel_data.py:74-128).  The grid is Earth-fixed, so
    the strains' GPS time is not needed."""
    if ml is not None and FP is not None and FX is not None:
        return np.asarray(ml), np.asarray(FP), np.asarray(FX)
    if config is None:
        raise ValueError("strains and config are required when ml/FP/FX are not provided")
    rate, K = td_size_for(config)
    ifos = list(getattr(config, "ifo"))[:int(nIFO)]
    order = int(getattr(config, "healpix", 0)) if hasattr(config, "healpix") else None
    return sky.compute_sky_delay_and_patterns(ifos, getattr(config, "refIFO"), rate, K,
                                              healpix_order=order)


load_data_from_ifo = build_sky_delay_and_antenna_patterns
