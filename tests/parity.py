"""Shared comparison rules of the parity tests.

Tolerance (stated once, used everywhere).  Per statistic and direction:

    |gpu - ref| <= 1e-4 * max(|ref|, 1e-3 * max|ref|) + 2 * |ref - f64|

where ref is the reference's float32 arithmetic (the oracle, bit-exact to
the reference) and f64 the same loop in float64.  The first term is the
1e-4 relative bar, with a floor so values that cancel to near zero do not
dominate; the second admits directions that are ill-conditioned in float32:
there the reference itself is |ref - f64| away from the float64 value and
two float32 evaluation orders can differ by twice that.  NaN positions must
agree exactly.

Two decisions of the reference are discontinuous and are checked apart:
* the netCC cut (sky_scan.py:135): a direction may be kept on one side and
  rejected on the other only where the reference's ellipticity Cr lies
  within 1e-4 * netCC + 2 * |Cr - Cr_f64| of netCC (the same conditioning
  allowance as above); such directions are left out of the value
  comparison and counted;
* the sky maximum (sky_scan.py:183-189): the selected index must be
  identical unless the two statistics tie within 1e-5 relative.
"""

import numpy as np

RTOL = 1e-4
FLOOR = 1e-3
TIE_RTOL = 1e-5
CUT_RTOL = 1e-4


def stat_errors(gpu_stats, ref_stats, f64_stats=None, skip=None):
    """Per-statistic max of |gpu-ref| / allowance-unit (<= RTOL passes)."""
    errs = []
    for idx, (a, b) in enumerate(zip(gpu_stats, ref_stats)):
        a = np.asarray(a, np.float64)
        b = np.asarray(b, np.float64)
        na, nb = np.isnan(a), np.isnan(b)
        keep = np.ones(a.shape, bool) if skip is None else ~skip
        if not np.array_equal(na[keep], nb[keep]):
            errs.append(np.inf)
            continue
        ok = ~nb & keep
        if not ok.any():
            errs.append(0.0)
            continue
        scale = np.max(np.abs(b[ok]))
        den = np.maximum(np.abs(b[ok]), FLOOR * scale if scale > 0 else 1.0)
        diff = np.abs(a[ok] - b[ok])
        if f64_stats is not None:
            c = np.asarray(f64_stats[idx], np.float64)[ok]
            cond = np.where(np.isnan(c), 0.0, np.abs(b[ok] - c))
            diff = np.maximum(diff - 2.0 * cond, 0.0)
        errs.append(float(np.max(diff / den)))
    return errs


def cut_flips(gpu_out, ref_out, ref_cr=None, netCC=None, f64_cr=None):
    """Directions kept on one side and rejected by the netCC cut on the other.

    Returns (flips mask, mask of flips not explained by a near-threshold
    ellipticity)."""
    kept_gpu = np.any(np.stack([np.asarray(x) for x in gpu_out[1:12]]) != 0, axis=0)
    kept_ref = np.any(np.stack([np.asarray(x) for x in ref_out[1:12]]) != 0, axis=0)
    flips = kept_gpu != kept_ref
    if not flips.any() or ref_cr is None or netCC is None:
        return flips, flips
    cr = np.asarray(ref_cr, np.float64)
    window = CUT_RTOL * max(abs(netCC), 1e-3)
    if f64_cr is not None:
        window = window + 2.0 * np.nan_to_num(np.abs(cr - np.asarray(f64_cr, np.float64)))
    near = np.abs(cr - netCC) <= window
    return flips, flips & ~near


def assert_scan_close(gpu_out, ref_out, f64_out=None, rtol=RTOL, ref_cr=None, netCC=None,
                      what=""):
    f64_cr = f64_out[13] if (f64_out is not None and len(f64_out) > 13) else None
    flips, bad = cut_flips(gpu_out, ref_out, ref_cr, netCC, f64_cr)
    if bad.any():
        where = np.flatnonzero(bad)[:5]
        detail = [(int(l), float(ref_cr[l]) if ref_cr is not None else None,
                   float(f64_cr[l]) if f64_cr is not None else None) for l in where]
        raise AssertionError(f"{what}: {int(bad.sum())} directions kept/rejected differently with "
                             f"an ellipticity away from netCC={netCC} ({int(flips.sum())} flips "
                             f"in all); (direction, Cr_ref, Cr_f64): {detail}")
    f64s = None if f64_out is None else f64_out[1:12]
    errs = stat_errors(gpu_out[1:12], ref_out[1:12], f64s, skip=flips if flips.any() else None)
    assert max(errs) <= rtol, f"{what}: per-statistic max rel errors {errs}"
    lg, lr = int(gpu_out[0]), int(ref_out[0])
    if lg != lr:
        sg = float(ref_out[7][lg])
        sr = float(ref_out[7][lr])
        assert abs(sg - sr) <= TIE_RTOL * max(abs(sr), 1e-30), (
            f"{what}: l_max {lg} != {lr} and not a near-tie ({sg} vs {sr})")
        return
    smax_ref = float(ref_out[12])
    allowance = rtol * abs(smax_ref)
    if f64_out is not None:
        allowance += 2.0 * abs(smax_ref - float(f64_out[12]))
    assert abs(float(gpu_out[12]) - smax_ref) <= allowance + 1e-30, what
    return int(flips.sum())


def f64_error_ratio(gpu_out, ref_out, f64_out):
    """max over statistics of (GPU error vs f64) / (reference error vs f64), floored."""
    ratios = []
    for a, b, c in zip(gpu_out[1:12], ref_out[1:12], f64_out[1:12]):
        a, b, c = (np.asarray(x, np.float64) for x in (a, b, c))
        ok = ~(np.isnan(a) | np.isnan(b) | np.isnan(c)) & (a != 0) & (b != 0) & (c != 0)
        if not ok.any():
            continue
        scale = max(np.max(np.abs(c[ok])), 1e-30)
        eg = np.max(np.abs(a[ok] - c[ok])) / scale
        er = np.max(np.abs(b[ok] - c[ok])) / scale
        ratios.append(eg / max(er, 1e-6))
    return max(ratios) if ratios else 0.0
