"""Host sky tables (pycwb_gb300/sky.py) against known answers from the
reference's own files, on the CPU.

* HEALPix RING centres: an event of the reference's injection-consistency
  baseline (tests/injection_consistency/baseline.json:98,136) sits at
  theta = 102.6356 deg, phi = 219.7266 deg, a pixel centre of the order-7
  grid (ring 298, z = -0.21875).
* Geocentric delays: pycwb/types/tests/test_detector_geometry.py:388-400
  gives H1 and L1 delays from the Earth's centre, -R.n/c, for RA = dec = 0
  at GPS 1126259162.4 (from PyCBC with IERS UT1).  Here the sidereal time
  is the IAU 1982 GMST polynomial with UT1 = UTC, so the comparison allows
  the UT1 - UTC difference (< 0.9 s, at most 1.5e-6 s on these delays).
"""

import math

import numpy as np
import pytest

from pycwb_gb300 import sky


def test_healpix_order7_contains_the_baseline_event_direction():
    n_sky = 12 * 4 ** 7
    phi, lat = sky.build_sky_directions(n_sky, 7)
    theta_deg = 90.0 - np.degrees(lat)
    phi_deg = np.degrees(phi)
    d = np.abs(theta_deg - 102.63562774658203) + np.abs(phi_deg - 219.7265625)
    k = int(np.argmin(d))
    assert d[k] < 1e-4
    assert math.cos(math.radians(theta_deg[k])) == pytest.approx(-0.21875, abs=1e-12)


def _gmst(gps, gps_minus_utc=17.0):
    """Greenwich mean sidereal time (rad), IAU 1982 polynomial at 0h UT of
    the date plus the elapsed sidereal time; UT1 taken as UTC."""
    jd = 2444244.5 + (gps - gps_minus_utc) / 86400.0      # GPS epoch = JD 2444244.5
    jd0 = math.floor(jd - 0.5) + 0.5
    T = (jd0 - 2451545.0) / 36525.0
    s = 24110.54841 + 8640184.812866 * T + 0.093104 * T * T - 6.2e-6 * T ** 3
    s += (jd - jd0) * 86400.0 * 1.00273790935
    return (s % 86400.0) / 86400.0 * 2.0 * math.pi


@pytest.mark.parametrize("ifo,ref", [("H1", -0.0137897984), ("L1", -0.0120959516)])
def test_geocentric_delay_matches_reference(ifo, ref):
    phi_geo = -_gmst(1126259162.4)          # RA = 0 in Earth-fixed longitude
    n = np.array([math.cos(phi_geo), math.sin(phi_geo), 0.0])
    tau = -float(sky.DetectorSite(ifo).vertex @ n) / sky.C_LIGHT
    assert tau == pytest.approx(ref, abs=1.5e-6)


def test_delay_table_sign_and_reference_row():
    """ml[i, l] = rint(n . (R_i - R_ref) / c * rate): zero for the reference
    detector, antisymmetric between opposite directions."""
    ml, FP, FX = sky.compute_sky_delay_and_patterns(["L1", "H1", "V1"], "L1", 2048.0, 67,
                                                    healpix_order=3)
    assert not ml[0].any()
    phi, lat = sky.build_sky_directions(ml.shape[1], 3)
    n = np.stack([np.cos(lat) * np.cos(phi), np.cos(lat) * np.sin(phi), np.sin(lat)], 1)
    R = {d: sky.DetectorSite(d).vertex for d in ("L1", "H1", "V1")}
    x = n @ (R["H1"] - R["L1"]) / sky.C_LIGHT * 2048.0
    assert np.array_equal(ml[1], np.clip(np.rint(x), -67, 67).astype(np.int32))
    # the grid is antipodally symmetric: opposite directions, opposite delays
    anti = np.argmax(n @ (-n).T, axis=1)
    assert np.allclose(n[anti], -n, atol=1e-12)
    assert np.array_equal(ml[1][anti], -ml[1])


def test_baseline_and_response_known_answers():
    """pycwb/types/tests/test_detector_geometry.py:209-225, 680-683: the
    H1-L1 light travel time is 10.013 ms, vertices sit at the Earth's
    radius, response tensors are symmetric and traceless (two orthogonal
    unit arms, (x x^T - y y^T) / 2)."""
    h1, l1 = sky.DetectorSite("H1"), sky.DetectorSite("L1")
    assert np.linalg.norm(h1.vertex - l1.vertex) / sky.C_LIGHT == pytest.approx(0.010013,
                                                                                 rel=1e-4)
    for d in ("H1", "L1", "V1", "K1"):
        site = sky.DetectorSite(d)
        assert 6.3e6 < np.linalg.norm(site.vertex) < 6.4e6
        assert np.allclose(site.response, site.response.T)
        assert abs(np.trace(site.response)) < 1e-12
