"""GPU drop-ins for the likelihoodWP sky loop, with the reference's signatures.

* ``calculate_dpf``          replaces pycwb/modules/likelihoodWP/dpf.py:7-34
* ``scan_sky_for_best_fit``  replaces pycwb/modules/likelihoodWP/sky_scan.py:17-192
* ``sky_loop``               both passes of one cluster in one launch
                             (the two calls at likelihood.py:310-325)

Arguments may be NumPy arrays (copied to the GPU for the call) or CUDA
torch tensors (used in place).  Results are NumPy, exactly as the reference
returns them, unless ``return_device=True``.  Shape errors raise ValueError
like the reference (dpf.py:14-22); device-detected errors raise
RuntimeError.  There is no CPU fallback.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _device as dv
from .. import _lib

N_STATS = 11
STAT_NAMES = ("nAntennaPrior", "nAlignment", "nLikelihood", "nNullEnergy", "nCorrEnergy",
              "nCorrelation", "nSkyStat", "nDisbalance", "nNetIndex", "nEllipticity",
              "nPolarisation")


def _check_tables(FP, FX, rms, n_sky, n_ifo):
    if (dv.shape_of(FP) != (n_sky, n_ifo) or dv.shape_of(FX) != (n_sky, n_ifo)
            or len(dv.shape_of(rms)) != 2 or dv.shape_of(rms)[1] != n_ifo):
        raise ValueError(
            "FP and FX must have shape (n_sky, n_ifo) and rms must have shape (n_pix, n_ifo), "
            f"got FP: {dv.shape_of(FP)}, FX: {dv.shape_of(FX)}, rms: {dv.shape_of(rms)}")


_order_cache = {}


def _sky_order_device(ml, sky_valid_indices, device):
    """Scan order grouped by delay tuple (pgw_sky_order), cached per (ml, valid) pair.

    The order only groups directions for speed; results do not depend on it,
    so a cache hit on arrays changed in place costs time, never correctness."""
    def ident(x):
        if isinstance(x, torch.Tensor):
            return ("t", x.data_ptr(), tuple(x.shape))
        a = np.asarray(x)
        return ("n", id(x), a.__array_interface__["data"][0], a.shape)
    key = (ident(ml), ident(sky_valid_indices))
    hit = _order_cache.get(key)
    if hit is not None:
        return hit
    ml_h = ml.cpu().numpy() if isinstance(ml, torch.Tensor) else np.asarray(ml)
    v_h = (sky_valid_indices.cpu().numpy() if isinstance(sky_valid_indices, torch.Tensor)
           else np.asarray(sky_valid_indices))
    order, _ = _lib.sky_order(ml_h, v_h)
    t = torch.from_numpy(order).to(device)
    if len(_order_cache) > 16:
        _order_cache.clear()
    _order_cache[key] = t
    return t


_reg_order_cache = {}


def _reg_order_device(FP, FX, sky_valid_indices, device, gamma_regulator=None):
    """Regulator order (pgw_regulator_order, or with gamma_regulator its
    longest-tiles-first grouping), cached per (FP, FX, valid, gamma) like the
    scan order: it orders work only, never changes a result."""
    def ident(x):
        if isinstance(x, torch.Tensor):
            return ("t", x.data_ptr(), tuple(x.shape))
        a = np.asarray(x)
        return ("n", id(x), a.__array_interface__["data"][0], a.shape)
    key = (ident(FP), ident(FX), ident(sky_valid_indices), gamma_regulator)
    hit = _reg_order_cache.get(key)
    if hit is not None:
        return hit
    host = (lambda x: x.cpu().numpy() if isinstance(x, torch.Tensor) else np.asarray(x))
    order = _lib.regulator_order(host(FP), host(FX), host(sky_valid_indices), gamma_regulator)
    t = torch.from_numpy(order).to(device)
    if len(_reg_order_cache) > 16:
        _reg_order_cache.clear()
    _reg_order_cache[key] = t
    return t


def _valid(sky_valid_indices, n_sky):
    v = dv.to_device(sky_valid_indices, torch.int64)
    if v.ndim != 1 or v.numel() == 0:
        raise ValueError("sky_valid_indices must be a non-empty 1-D index array")
    return v


def calculate_dpf(FP, FX, rms, n_sky, n_ifo, gamma_regulator, network_energy_threshold,
                  sky_valid_indices, *, return_device=False):
    """REG[1] = (n_valid^2 / (n_pass^2 + 1e-9) - 1) * E_thr (float64)."""
    n_sky, n_ifo = int(n_sky), int(n_ifo)
    _check_tables(FP, FX, rms, n_sky, n_ifo)
    L = _lib.load()
    s = dv.begin()
    FPd, FXd = dv.to_device(FP, torch.float32), dv.to_device(FX, torch.float32)
    rmsd = dv.to_device(rms, torch.float32)
    valid = _valid(sky_valid_indices, n_sky)
    n_pix = int(rmsd.shape[0])
    nbytes = L.pgw_workspace_bytes(n_ifo, 1, n_pix, 1)
    ws = dv.workspace(nbytes)
    with torch.cuda.stream(s):
        out = torch.empty(1, dtype=torch.float64, device=FPd.device)
    rc = L.pgw_calculate_dpf(FPd.data_ptr(), FXd.data_ptr(), rmsd.data_ptr(), n_sky, n_ifo, n_pix,
                             float(gamma_regulator), float(network_energy_threshold),
                             valid.data_ptr(), valid.numel(), out.data_ptr(), None,
                             ws.data_ptr(), ws.numel(), dv.stream_handle(s))
    _lib.check(rc, "calculate_dpf")
    if return_device:
        dv.end(s, out)
        return out
    with torch.cuda.stream(s):
        return float(out.item())


def _scan_outputs(stats, res, return_device, s):
    if return_device:
        dv.end(s, stats, res)
        return stats, res
    with torch.cuda.stream(s):
        st = stats.cpu().numpy()
        r = res.cpu().numpy().view(dv.RESULT_DTYPE)[0]
    _lib.check_device_status(int(r["status"]), "sky scan")
    smax = np.float32(r["sky_stat_max"]) if r["found"] else 0
    return (int(r["l_max"]),) + tuple(st[k] for k in range(N_STATS)) + (smax,)


def scan_sky_for_best_fit(n_ifo, n_pix, n_sky, FP, FX, rms, td00, td90, ml, REG, netCC,
                          delta_regulator, network_energy_threshold, sky_valid_indices, *,
                          return_device=False):
    """The reference's 13-tuple: (l_max, 11 per-sky float32 arrays, sky_stat_max)."""
    n_ifo, n_pix, n_sky = int(n_ifo), int(n_pix), int(n_sky)
    _check_tables(FP, FX, rms, n_sky, n_ifo)
    if dv.shape_of(ml) != (n_ifo, n_sky):
        raise ValueError(f"ml must have shape (n_ifo, n_sky), got {dv.shape_of(ml)}")
    n_delay = dv.shape_of(td00)[0]
    if (dv.shape_of(td00) != (n_delay, n_ifo, n_pix) or dv.shape_of(td90) != dv.shape_of(td00)
            or dv.shape_of(rms)[0] != n_pix):
        raise ValueError("td00/td90 must have shape (n_delay, n_ifo, n_pix) and rms (n_pix, n_ifo), "
                         f"got td00: {dv.shape_of(td00)}, td90: {dv.shape_of(td90)}, "
                         f"rms: {dv.shape_of(rms)}")
    L = _lib.load()
    s = dv.begin()
    FPd, FXd = dv.to_device(FP, torch.float32), dv.to_device(FX, torch.float32)
    rmsd = dv.to_device(rms, torch.float32)
    t0, t9 = dv.to_device(td00, torch.float32), dv.to_device(td90, torch.float32)
    mld = dv.to_device(ml, torch.int32)
    REGd = dv.to_device(np.asarray(REG, np.float32) if not isinstance(REG, torch.Tensor) else REG,
                        torch.float32)
    valid = _valid(sky_valid_indices, n_sky)
    order = _sky_order_device(ml, sky_valid_indices, FPd.device)
    ws = dv.workspace(L.pgw_workspace_bytes(n_ifo, n_delay, n_pix, 1))
    with torch.cuda.stream(s):
        stats = torch.empty((N_STATS, n_sky), dtype=torch.float32, device=FPd.device)
        res = torch.empty(dv.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=FPd.device)
    rc = L.pgw_scan_sky_for_best_fit(n_ifo, n_pix, n_sky, FPd.data_ptr(), FXd.data_ptr(),
                                     rmsd.data_ptr(), t0.data_ptr(), t9.data_ptr(), n_delay,
                                     mld.data_ptr(), REGd.data_ptr(), float(netCC),
                                     float(delta_regulator), float(network_energy_threshold),
                                     valid.data_ptr(), valid.numel(), order.data_ptr(),
                                     stats.data_ptr(), res.data_ptr(), ws.data_ptr(), ws.numel(),
                                     dv.stream_handle(s))
    _lib.check(rc, "scan_sky_for_best_fit")
    return _scan_outputs(stats, res, return_device, s)


def sky_loop(n_ifo, n_pix, n_sky, FP, FX, rms, td00, td90, ml, REG0, gamma_regulator, netCC,
             network_energy_threshold, sky_valid_indices, *, shape=None, sky_order=True,
             return_device=False):
    """Regulator + scan of one cluster in one launch (likelihood.py:308-325).

    Returns (regulator, scan 13-tuple); REG = [REG0, float32(regulator), 0].
    sky_order=False scans the directions in the given order (same results).
    """
    n_ifo, n_pix, n_sky = int(n_ifo), int(n_pix), int(n_sky)
    _check_tables(FP, FX, rms, n_sky, n_ifo)
    n_delay = dv.shape_of(td00)[0]
    if dv.shape_of(td00) != (n_delay, n_ifo, n_pix) or dv.shape_of(td90) != dv.shape_of(td00):
        raise ValueError("td00/td90 must have shape (n_delay, n_ifo, n_pix)")
    L = _lib.load()
    s = dv.begin()
    FPd, FXd = dv.to_device(FP, torch.float32), dv.to_device(FX, torch.float32)
    rmsd = dv.to_device(rms, torch.float32)
    t0, t9 = dv.to_device(td00, torch.float32), dv.to_device(td90, torch.float32)
    mld = dv.to_device(ml, torch.int32)
    valid = _valid(sky_valid_indices, n_sky)
    order = _sky_order_device(ml, sky_valid_indices, FPd.device) if sky_order else None
    rorder = (_reg_order_device(FP, FX, sky_valid_indices, FPd.device, float(gamma_regulator))
              if sky_order else None)
    ws = dv.workspace(L.pgw_workspace_bytes(n_ifo, n_delay, n_pix, 1))
    with torch.cuda.stream(s):
        stats = torch.empty((N_STATS, n_sky), dtype=torch.float32, device=FPd.device)
        res = torch.empty(dv.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=FPd.device)
        reg = torch.empty(1, dtype=torch.float64, device=FPd.device)
    rc = L.pgw_sky_loop(n_ifo, n_pix, n_sky, FPd.data_ptr(), FXd.data_ptr(), rmsd.data_ptr(),
                        t0.data_ptr(), t9.data_ptr(), n_delay, mld.data_ptr(), float(np.float32(REG0)),
                        float(gamma_regulator), float(netCC), float(network_energy_threshold),
                        valid.data_ptr(), valid.numel(), dv.ptr(order), dv.ptr(rorder),
                        stats.data_ptr(), res.data_ptr(),
                        reg.data_ptr(), None if shape is None else ctypes.byref(shape),
                        ws.data_ptr(), ws.numel(), dv.stream_handle(s))
    _lib.check(rc, "sky_loop")
    if return_device:
        dv.end(s, reg, stats, res)
        return reg, stats, res
    out = _scan_outputs(stats, res, False, s)
    with torch.cuda.stream(s):
        return float(reg.item()), out


# Legacy alias, as in the reference (sky_scan.py:197)
find_optimal_sky_localization = scan_sky_for_best_fit
