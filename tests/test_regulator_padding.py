"""The regulator's staged weights past a cluster's last pixel.

The regulator's fast pass adds every staged pixel pair without a mask: past
the last pixel the stage holds w = (1, 0, ...) with no pair products, so
the pixel's term det / fp / (ni + 1e-9) has det = 0 exactly and its value
is 0 as long as the denominator 4 s4 + 4e-9 fp^2 is a normal float (a
zero or subnormal one -- flushed on the GPU -- would give 0 * inf = NaN,
which sends the direction to the exact pass: still the reference's result,
but slow).  This checks, with the fast pass's float32 expressions and
flush-to-zero, that no direction of the HEALPix-7 sky for L1/H1/V1 (and of
the HEALPix-5 sky for 2 and 4 detectors) gets such a denominator, and that
the padding pixel adds exactly 0 to NI.  A second test checks the bound of
the fp sum that the conditioning test and the early-fail bound use.
"""

import numpy as np
import pytest

TINY = np.float32(1.1754944e-38)


def _ftz(x):
    x = np.asarray(x, np.float32)
    return np.where(np.abs(x) < TINY, np.float32(0), x).astype(np.float32)


def _pad_term(FP, FX):
    """Fast-pass term and fp of the padding pixel w = (1, 0, ...) for every
    direction (rows of FP, FX), float32 with subnormals flushed."""
    f32 = np.float32
    Fp, Fx = FP[:, 0].astype(f32), FX[:, 0].astype(f32)
    U, V = _ftz(Fp * Fp), _ftz(Fx * Fx)
    Ad, Cd, Sd = _ftz(U + V), _ftz(U - V), _ftz(f32(2) * _ftz(Fp * Fx))
    AP, co, si = Ad, Cd, Sd                     # w_0 = 1, every other weight 0
    det4 = np.zeros_like(AP)                    # no pair products
    nn = _ftz(np.sqrt(_ftz(_ftz(co * co) + _ftz(si * si))))
    fp = _ftz(f32(0.5) * _ftz(AP + nn))
    rn = _ftz(f32(1) / _ftz(nn + f32(1e-9)))
    c2, s2 = _ftz(co * rn), _ftz(si * rn)
    g = _ftz(Ad + _ftz(Cd * c2) + _ftz(Sd * s2))
    s4x = _ftz(g * g)
    den = _ftz(_ftz(f32(4e-9) * _ftz(fp * fp)) + s4x)
    with np.errstate(divide="ignore", invalid="ignore"):
        rd = np.where(den > 0, f32(1) / den, np.inf).astype(f32)
        term = _ftz(_ftz(det4 * fp) * rd)
    return term, fp, den, Ad


@pytest.mark.parametrize("ifos,order", [(("L1", "H1", "V1"), 7), (("L1", "H1"), 5),
                                        (("L1", "H1", "V1", "K1"), 5)])
def test_padding_pixel_adds_zero_for_every_direction(ifos, order):
    from pycwb_gb300 import sky
    _, FP, FX = sky.compute_sky_delay_and_patterns(list(ifos), ifos[0], 512.0, 20,
                                                   healpix_order=order)
    FP_t, FX_t = FP.T.astype(np.float32), FX.T.astype(np.float32)
    term, fp, den, Ad = _pad_term(FP_t, FX_t)
    assert np.all(np.isfinite(den)) and np.all(den >= TINY), "a padding pixel would give 0/0"
    assert np.all(term == 0)                    # NI unchanged
    # a rank-one Gram matrix: fp = |F_0|^2 up to rounding
    np.testing.assert_allclose(fp, Ad, rtol=1e-6)
    assert Ad.min() > 1e-6                      # far from the flush-to-zero range


def test_fp_sum_bound_covers_the_running_sum():
    """The conditioning test NI >= 1e-5 sum(fp) and the early-fail bound take
    SF = sum_i |F_i|^2 W_i (W_i the cluster's total weight of detector i) in
    place of the running sum of fp over the pixels seen: since
    fp = (AP + nn) / 2 <= AP = sum_i w_i |F_i|^2, SF bounds that sum after any
    number of pixels, so both tests only become more cautious."""
    from pycwb_gb300 import sky
    from pycwb_gb300.synthetic import make_cluster
    ifos = ["L1", "H1", "V1"]
    ml, FP, FX = sky.compute_sky_delay_and_patterns(ifos, "L1", 512.0, 20, healpix_order=4)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    rng = np.random.default_rng(11)
    for P in (1, 20, 300):
        _, _, rms, _ = make_cluster(rng, ml, FP_t, FX_t, P, 20, 20.0)
        w = rms.astype(np.float64) ** 2                      # (P, I)
        Fp, Fx = FP_t.astype(np.float64), FX_t.astype(np.float64)
        Ad, Cd, Sd = Fp * Fp + Fx * Fx, Fp * Fp - Fx * Fx, 2 * Fp * Fx
        AP, co, si = w @ Ad.T, w @ Cd.T, w @ Sd.T            # (P, n_sky)
        fp = 0.5 * (AP + np.sqrt(co * co + si * si))
        running = np.cumsum(fp, axis=0)                      # after each pixel
        # the kernel's float32 bound from the float32 totals
        W = w.sum(axis=0).astype(np.float32)
        SF = (Ad.astype(np.float32) * W[None, :]).sum(axis=1, dtype=np.float32)
        assert np.all(SF.astype(np.float64) >= running.max(axis=0) * (1 - 1e-6))
