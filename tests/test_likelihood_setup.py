"""Segment setup and per-cluster input extraction (host side), on the CPU.

Follows the reference's contracts: likelihood_setup.py:133-147 (constants),
:215-237 (returned keys), pixel_data.py:55-71 and the reference's own
test_data_extraction.py:87-104 (rms normalisation), sky_mask.py:71-176
(Patch / Fixed masks), pixel_data.py:113-124 (TD rate and delay range).
"""

import math
from types import SimpleNamespace

import numpy as np
import pytest

from pycwb_gb300 import sky
from pycwb_gb300.likelihoodWP.likelihood_setup import (compute_sky_valid_indices,
                                                        prepare_likelihood_inputs,
                                                        setup_likelihood)
from pycwb_gb300.likelihoodWP.pixel_data import (_extract_pixel_array_time_delay_data,
                                                  build_sky_delay_and_antenna_patterns,
                                                  load_data_from_pixels, scan_inputs, td_size_for)

REFERENCE_KEYS = {
    "network_energy_threshold", "xgb_rho_mode", "gamma_regulator", "delta_regulator",
    "net_rho_threshold", "netEC_threshold", "netCC", "ml", "FP", "FX", "FP_t", "FX_t", "n_sky",
    "healpix_order", "phi_geo_arr", "latitude_arr", "ra_arr", "dec_arr", "sky_mask_config",
    "segment_start_gps", "sky_valid_indices", "ml_big_cluster", "FP_big_cluster_t",
    "FX_big_cluster_t", "n_sky_big_cluster", "big_cluster_healpix_order",
    "phi_geo_arr_big_cluster", "latitude_arr_big_cluster", "sky_valid_indices_big",
}


def _config(**kw):
    base = dict(Acore=1.7, gamma=0.5, delta=0.0, netRHO=4.0, netCC=0.5, ifo=["L1", "H1", "V1"],
                refIFO="L1", rateANA=512, upTDF=4, TDSize=12, max_delay=0.0325, healpix=3)
    base.update(kw)
    return SimpleNamespace(**base)


def test_constants_and_keys():
    out = prepare_likelihood_inputs(_config(), None, 3)
    assert set(out) == REFERENCE_KEYS
    assert out["network_energy_threshold"] == 2 * 1.7 * 1.7 * 3
    assert out["gamma_regulator"] == 0.5 * 0.5 * 2 / 3
    assert out["delta_regulator"] == 0.00001           # delta = 0 is stored as 1e-5
    assert out["net_rho_threshold"] == 4.0 and out["netEC_threshold"] == 32.0
    assert prepare_likelihood_inputs(_config(delta=-2.5), None, 3)["delta_regulator"] == 1
    assert prepare_likelihood_inputs(_config(delta=-0.3), None, 3)["delta_regulator"] == 0.3
    assert out["FP_t"].dtype == np.float32 and out["FP_t"].shape == (out["n_sky"], 3)
    assert np.array_equal(out["sky_valid_indices"], np.arange(out["n_sky"]))
    assert setup_likelihood is prepare_likelihood_inputs
    with pytest.raises(ValueError):
        prepare_likelihood_inputs(None, None, 3)


def test_sky_tables_from_config_and_passthrough():
    cfg = _config()
    rate, K = td_size_for(cfg)
    assert (rate, K) == (2048.0, 67)                  # max(12 * 4, int(0.0325 * 2048) + 1)
    ml, FP, FX = build_sky_delay_and_antenna_patterns(3, None, cfg)
    ml2, FP2, FX2 = sky.compute_sky_delay_and_patterns(["L1", "H1", "V1"], "L1", 2048.0, 67,
                                                       healpix_order=3)
    assert np.array_equal(ml, ml2) and np.array_equal(FP, FP2) and np.array_equal(FX, FX2)
    out = prepare_likelihood_inputs(cfg, None, 3, ml=ml[:, :10], FP=FP[:, :10], FX=FX[:, :10])
    assert out["n_sky"] == 10 and out["ml"] is not None
    big = prepare_likelihood_inputs(cfg, None, 3, ml_big=ml, FP_big=FP, FX_big=FX,
                                    big_cluster_healpix_order=3)
    assert big["n_sky_big_cluster"] == ml.shape[1]
    assert big["FP_big_cluster_t"].shape == (ml.shape[1], 3)


def test_sky_masks():
    order = 4
    n = 12 * 4 ** order
    phi, lat = sky.build_sky_directions(n, order)
    # Patch: every kept direction within the radius, every other one outside
    mask = {"type": "Patch", "coordsys": "geo",
            "patch": {"center": {"longitude": "-120 deg", "latitude": "30 deg"},
                      "radius": "15 deg"}}
    v = compute_sky_valid_indices(phi, lat, mask)
    c_phi, c_lat = math.radians(240.0), math.radians(30.0)
    d = np.degrees(np.arccos(np.clip(np.sin(lat) * math.sin(c_lat) + np.cos(lat) * math.cos(c_lat)
                                     * np.cos(phi - c_phi), -1, 1)))
    assert np.array_equal(v, np.flatnonzero(d <= 15.0)) and 30 < v.size < 80   # cap area: 52
    # the same patch in cWB coordinates (co-latitude) and in legacy radians
    cwb = {"type": "Patch", "coordsys": "cwb",
           "patch": {"center": {"phi_geo": "240 deg", "theta_cwb": "60 deg"}, "radius": "15 deg"}}
    assert np.array_equal(compute_sky_valid_indices(phi, lat, cwb), v)
    legacy = {"type": "Patch", "patch": {"center": {"phi": 240.0, "theta": 30.0}, "radius": 15.0,
                                         "unit": "deg"}}
    assert np.array_equal(compute_sky_valid_indices(phi, lat, legacy), v)
    # Fixed: the nearest grid direction
    fixed = {"type": "Fixed", "coordsys": "geo",
             "coordinates": {"longitude": "10 deg", "latitude": "-45 deg"}}
    f = compute_sky_valid_indices(phi, lat, fixed)
    d2 = np.sin(lat) * math.sin(math.radians(-45)) + np.cos(lat) * math.cos(
        math.radians(-45)) * np.cos(phi - math.radians(10))
    assert f.tolist() == [int(np.argmax(d2))]
    assert np.array_equal(compute_sky_valid_indices(phi, lat, {"type": "UniformAllSky"}),
                          np.arange(n))
    with pytest.raises(ValueError, match="requires a GPS reference time"):
        compute_sky_valid_indices(phi, lat, {"type": "Patch", "coordsys": "icrs",
                                             "patch": {"center": {"ra": "1 rad", "dec": "0 rad"},
                                                       "radius": "5 deg"}})
    with pytest.raises(KeyError):
        compute_sky_valid_indices(phi, lat, {"type": "Custom", "custom": {}})
    with pytest.raises(ValueError):
        compute_sky_valid_indices(phi, lat, {"type": "Ring"})
    with pytest.raises(ValueError):
        compute_sky_valid_indices(phi, lat, {"type": "Patch", "coordsys": "geo", "patch": {
            "center": {"longitude": "0 deg", "latitude": "95 deg"}, "radius": "5 deg"}})
    # the mask reaches the segment setup
    out = prepare_likelihood_inputs(_config(healpix=order, sky_mask=mask), None, 3)
    assert np.array_equal(out["sky_valid_indices"], v)


class _PixelArrays:
    def __init__(self, noise_rms, td):
        self.noise_rms = noise_rms
        self._td = td

    def td_amp_dense(self):
        return self._td


def test_rms_normalisation_and_layout():
    rng = np.random.RandomState(42)
    n_ifo, n_pix, D = 3, 7, 9
    td = (rng.randn(n_pix, n_ifo, 2 * D) * 0.1).astype(np.float32)
    noise = np.full((n_ifo, n_pix), 1.0, np.float32)
    noise[1] *= 1.5
    noise[2, 3] = 0.25
    pa = _PixelArrays(noise, td)
    w, p0, p90, e = load_data_from_pixels(None, n_ifo, pixel_arrays=pa)
    inv = 1.0 / noise.astype(np.float64)
    expect = (inv * (1.0 / np.sqrt(np.sum(inv ** 2, axis=0)))[None, :]).astype(np.float32)
    assert np.array_equal(w, expect)
    assert p0.shape == p90.shape == e.shape == (n_ifo, n_pix, D)
    assert np.array_equal(e, p0 ** 2 + p90 ** 2)
    assert np.array_equal(p0[1, 4], td[4, 1, :D]) and np.array_equal(p90[2, 0], td[0, 2, D:])
    rms, td00, td90 = scan_inputs(w, p0, p90)
    assert rms.shape == (n_pix, n_ifo) and td00.shape == (D, n_ifo, n_pix)
    assert td00.flags.c_contiguous and np.array_equal(td00[5, 2, 6], td[6, 2, 5])
    assert np.array_equal(td90[0, 1, 2], td[2, 1, D])
    with pytest.raises(ValueError):
        load_data_from_pixels(None, n_ifo)
    with pytest.raises(ValueError):
        load_data_from_pixels(None, 4, pixel_arrays=pa)
    _ = _extract_pixel_array_time_delay_data(pa)


def test_sky_mask_reference_cases():
    """The cases of the reference's own sky-mask tests
    (pycwb/modules/likelihoodWP/tests/test_compute_sky_valid_indices.py:
    None and UniformAllSky configs, a legacy Patch in radians and degrees, a
    zero radius on a grid point, the full sky) on a 300-direction spiral."""
    n = 300
    k = np.arange(n, dtype=np.float64)
    phi = (np.pi * (3.0 - np.sqrt(5.0)) * k) % (2.0 * np.pi)
    lat = np.arcsin(np.clip(1.0 - 2.0 * (k + 0.5) / n, -1.0, 1.0))
    assert np.array_equal(compute_sky_valid_indices(phi, lat, None), np.arange(n))
    assert compute_sky_valid_indices(phi, lat, None).dtype == np.int64
    assert compute_sky_valid_indices(np.array([1.0]), np.array([0.5]), None).tolist() == [0]
    rad = {"type": "Patch", "patch": {"center": {"phi": 1.0, "theta": 0.3}, "radius": 0.5,
                                      "unit": "rad"}}
    deg = {"type": "Patch", "patch": {"center": {"phi": math.degrees(1.0),
                                                 "theta": math.degrees(0.3)},
                                      "radius": math.degrees(0.5), "unit": "deg"}}
    v = compute_sky_valid_indices(phi, lat, rad)
    sep = np.arccos(np.clip(np.sin(lat) * math.sin(0.3) + np.cos(lat) * math.cos(0.3)
                            * np.cos(phi - 1.0), -1.0, 1.0))
    assert np.array_equal(v, np.flatnonzero(sep <= 0.5)) and v.size > 0
    assert np.array_equal(compute_sky_valid_indices(phi, lat, deg), v)
    zero = {"type": "Patch", "patch": {"center": {"phi": float(phi[5]), "theta": float(lat[5])},
                                       "radius": 0.0, "unit": "rad"}}
    assert compute_sky_valid_indices(phi, lat, zero).tolist() == [5]
    full = {"type": "Patch", "patch": {"center": {"phi": 1.0, "theta": 0.3}, "radius": math.pi,
                                       "unit": "rad"}}
    assert compute_sky_valid_indices(phi, lat, full).size == n
