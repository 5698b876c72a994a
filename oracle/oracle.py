"""ctypes front end of the CPU oracle (liboracle.so, built from this folder).

TEST INFRASTRUCTURE ONLY.  tests/ use it as the checker of the CUDA path and
bench.py times it as the CPU baseline.  The product never imports it.
The functions mirror the reference signatures:

* calculate_dpf          pycwb/modules/likelihoodWP/dpf.py:8
* scan_sky_for_best_fit  pycwb/modules/likelihoodWP/sky_scan.py:18
* batch_get_td_vecs      pycwb/utils/td_vector_kernels.py:134
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
N_STATS = 11

_lib = None


def build(force: bool = False) -> str:
    """Compile liboracle.so with the Makefile beside this file."""
    srcs = [os.path.join(HERE, f) for f in ("skyscan_oracle.c", "tdamp_oracle.c", "subnet_oracle.c",
                                             "Makefile")]
    if force or not os.path.exists(LIB_PATH) or any(
            os.path.getmtime(s) > os.path.getmtime(LIB_PATH) for s in srcs):
        subprocess.run(["make", "-s", "-B", "-C", HERE, "liboracle.so"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        i64, i32, f64 = ctypes.c_int64, ctypes.c_int, ctypes.c_double
        L.oracle_calculate_dpf_f32.argtypes = [P, P, P, i64, i32, i64, f64, f64, P, i64, i32, P]
        L.oracle_calculate_dpf_f64.argtypes = [P, P, P, i64, i32, i64, f64, f64, P, i64, i32, P]
        L.oracle_scan_sky_f32.argtypes = [i32, i64, i64, P, P, P, P, P, i32, P, P, f64, f64, f64,
                                          P, i64, i32, P, P, P, P, P]
        L.oracle_scan_sky_f64.argtypes = [i32, i64, i64, P, P, P, P, P, i32, P, P, f64, f64,
                                          P, i64, i32, P, P, P, P]
        L.oracle_batch_get_td_vecs.argtypes = [P, i64, P, P, i64, P, P, i32, i32, i32, i32, P,
                                               i32, P]
        f32 = ctypes.c_float
        for f in (L.oracle_subnet_sky_f32, L.oracle_subnet_sky_f64):
            f.argtypes = [i32, i64, i64, P, P, P, P, P, i32, P, f32, f64, f64, P]
        for f in (L.oracle_calculate_dpf_f32, L.oracle_calculate_dpf_f64, L.oracle_scan_sky_f32,
                  L.oracle_scan_sky_f64, L.oracle_batch_get_td_vecs, L.oracle_subnet_sky_f32,
                  L.oracle_subnet_sky_f64):
            f.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def calculate_dpf(FP, FX, rms, n_sky, n_ifo, gamma_regulator, network_energy_threshold,
                  sky_valid_indices, n_threads=0, precision="f32"):
    FP, FX, rms = _c(FP, np.float32), _c(FX, np.float32), _c(rms, np.float32)
    valid = _c(sky_valid_indices, np.int64)
    out = np.zeros(1, np.float64)
    fn = lib().oracle_calculate_dpf_f32 if precision == "f32" else lib().oracle_calculate_dpf_f64
    rc = fn(_p(FP), _p(FX), _p(rms), int(n_sky), int(n_ifo), int(rms.shape[0]),
            float(gamma_regulator), float(network_energy_threshold), _p(valid), valid.size,
            int(n_threads), _p(out))
    if rc:
        raise ValueError(f"oracle calculate_dpf failed ({rc})")
    return float(out[0])


def scan_sky_for_best_fit(n_ifo, n_pix, n_sky, FP, FX, rms, td00, td90, ml, REG, netCC,
                          delta_regulator, network_energy_threshold, sky_valid_indices,
                          n_threads=0, precision="f32", return_ellipticity=False):
    """Returns the reference's 13-tuple (sky_scan.py:191-192).

    return_ellipticity=True appends an (n_sky,) array holding
    the ellipticity Cr of every valid direction, also those that the netCC
    cut rejects (NaN elsewhere) -- used to recognise near-threshold cuts."""
    FP, FX, rms = _c(FP, np.float32), _c(FX, np.float32), _c(rms, np.float32)
    td00, td90 = _c(td00, np.float32), _c(td90, np.float32)
    ml = _c(ml, np.int32)
    valid = _c(sky_valid_indices, np.int64)
    l_max = np.zeros(1, np.int64)
    smax = np.zeros(1, np.float64)
    if precision == "f32":
        REGa = _c(REG, np.float32)
        stats = np.zeros((N_STATS, int(n_sky)), np.float32)
        found = np.zeros(1, np.int32)
        cr = np.full(int(n_sky), np.nan, np.float32)
        rc = lib().oracle_scan_sky_f32(int(n_ifo), int(n_pix), int(n_sky), _p(FP), _p(FX), _p(rms),
                                       _p(td00), _p(td90), td00.shape[0], _p(ml), _p(REGa),
                                       float(netCC), float(delta_regulator),
                                       float(network_energy_threshold), _p(valid), valid.size,
                                       int(n_threads), _p(stats), _p(l_max), _p(smax), _p(found),
                                       _p(cr))
    else:
        REGa = _c(REG, np.float64)
        stats = np.zeros((N_STATS, int(n_sky)), np.float64)
        cr = np.full(int(n_sky), np.nan, np.float64)
        rc = lib().oracle_scan_sky_f64(int(n_ifo), int(n_pix), int(n_sky), _p(FP), _p(FX), _p(rms),
                                       _p(td00), _p(td90), td00.shape[0], _p(ml), _p(REGa),
                                       float(netCC), float(network_energy_threshold), _p(valid),
                                       valid.size, int(n_threads), _p(stats), _p(l_max), _p(smax),
                                       _p(cr))
    if rc:
        raise ValueError(f"oracle scan_sky_for_best_fit failed ({rc})")
    out = (int(l_max[0]),) + tuple(stats[k] for k in range(N_STATS)) + (float(smax[0]),)
    if return_ellipticity:
        out = out + (cr,)
    return out


def batch_get_td_vecs(pixel_indices, padded00, padded90, T0, Tx, M, n_coeffs, K, J,
                      n_threads=0):
    from pycwb_gb300.tdamp import td_phase_table

    idx = _c(pixel_indices, np.int32)
    p00, p90 = _c(padded00, np.float32), _c(padded90, np.float32)
    T0, Tx = _c(T0, np.float64), _c(Tx, np.float64)
    phase = td_phase_table(int(M), int(J))
    out = np.zeros((idx.size, 4 * int(K) + 2), np.float32)
    rc = lib().oracle_batch_get_td_vecs(_p(idx), idx.size, _p(p00), _p(p90), p00.shape[0],
                                        _p(T0), _p(Tx), int(M), int(n_coeffs), int(K), int(J),
                                        _p(phase), int(n_threads), _p(out))
    if rc:
        raise ValueError("oracle batch_get_td_vecs failed")
    return out


def optimze_sky_loc_from_td(n_ifo, n_pix, n_sky, FP, FX, rms, td00, td90, ml,
                            network_energy_threshold, e2or, subcut, precision="f32"):
    """sub_net_cut.py:404-517; returns (l_max, stat, Em, Am, lm, Vm, suball, EE)."""
    FP, FX, rms = _c(FP, np.float32), _c(FX, np.float32), _c(rms, np.float32)
    td00, td90, ml = _c(td00, np.float32), _c(td90, np.float32), _c(ml, np.int32)
    out = np.zeros(8, np.float64)
    fn = lib().oracle_subnet_sky_f32 if precision == "f32" else lib().oracle_subnet_sky_f64
    rc = fn(int(n_ifo), int(n_pix), int(n_sky), _p(FP), _p(FX), _p(rms), _p(td00), _p(td90),
            int(td00.shape[0]), _p(ml), float(np.float32(network_energy_threshold)), float(e2or),
            float(subcut), _p(out))
    if rc:
        raise ValueError(f"oracle_subnet_sky failed ({rc})")
    return (int(out[0]), out[1], out[2], out[3], int(out[4]), int(out[5]), out[6], out[7])
