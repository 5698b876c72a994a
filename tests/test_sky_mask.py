"""Sky masks in ICRS and from HEALPix maps, and the HEALPix pixel lookups
they rest on (CPU).

Cases follow the reference's own sky-mask tests
(pycwb/modules/likelihoodWP/tests/test_compute_sky_valid_indices.py:
the cWB sidereal-time sign of an ICRS Fixed mask, the GPS-time requirement,
a Custom ICRS map looked up at phi + GMST, an ICRS mask evaluated again at
the cluster's time, the cWB co-latitude convention) with HEALPix maps
written to real FITS files instead of a patched healpy reader.
"""

import math
from types import SimpleNamespace

import numpy as np
import pytest

from pycwb_gb300 import sky
from pycwb_gb300.likelihoodWP import sky_mask as sm

GPS = 1261873618.0


@pytest.mark.parametrize("order", [0, 1, 2, 3, 5])
def test_ang2pix_inverts_pix2ang_and_nests(order):
    nside = 1 << order
    p = np.arange(12 * nside * nside)
    th, ph = sky.healpix_pix2ang_ring(nside, p)
    assert np.array_equal(sky.healpix_ang2pix_ring(nside, th, ph), p)
    nest = sky.healpix_ang2pix_nest(nside, th, ph)
    assert np.array_equal(np.sort(nest), p)                    # a permutation
    rng = np.random.default_rng(order)
    t = np.arccos(rng.uniform(-1.0, 1.0, 20000))
    f = rng.uniform(0.0, 2.0 * math.pi, 20000)
    ring = sky.healpix_ang2pix_ring(nside, t, f)
    # RING and NESTED name the same pixel, and NESTED is hierarchical
    assert np.array_equal(sky.healpix_ring_to_nest(nside)[ring], sky.healpix_ang2pix_nest(nside, t, f))
    assert np.array_equal(sky.healpix_ang2pix_nest(2 * nside, t, f) // 4,
                          sky.healpix_ang2pix_nest(nside, t, f))
    # the pixel holding a point has the nearest centre among its neighbours
    ct, cp = sky.healpix_pix2ang_ring(nside, ring)
    d_own = np.sin(t) * np.sin(ct) * np.cos(f - cp) + np.cos(t) * np.cos(ct)
    assert np.all(d_own > math.cos(2.0 * math.sqrt(4 * math.pi / p.size) + 0.2))


def test_gmst_cwb_known_value():
    # J2000.0 (GPS 630763213) is 2000-01-01 11:58:55.816 UTC; the IAU 1982
    # polynomial gives GMST = 67310.54841 s + the elapsed fraction there
    assert abs(sm.gmst_cwb(sm.EPOCH_J2000_0_GPS) - math.radians(67310.54841 / 240.0)) < 1e-12
    # one sidereal day later (86164.0905 s) the angle comes back within 1e-6 rad
    d = sm.gmst_cwb(GPS + 86164.0905) - sm.gmst_cwb(GPS)
    assert abs((d + math.pi) % (2 * math.pi) - math.pi) < 1e-5


def test_fixed_icrs_uses_ra_minus_gmst():
    gmst = sm.gmst_cwb(GPS)
    cfg = {"type": "Fixed", "coordsys": "icrs",
           "coordinates": {"ra": f"{math.degrees(gmst)} deg", "dec": "0 deg"}}
    # ra = GMST lands on phi_geo = 0, not on phi_geo = GMST
    got = sm.compute_sky_valid_indices(np.array([0.0, gmst]), np.array([0.0, 0.0]), cfg, t_ref=GPS)
    assert got.tolist() == [0]


def test_icrs_needs_a_reference_time():
    cfg = {"type": "Fixed", "coordsys": "icrs", "coordinates": {"ra": "120 deg", "dec": "0 deg"}}
    with pytest.raises(ValueError, match="requires a GPS reference time"):
        sm.compute_sky_valid_indices(np.array([0.0]), np.array([0.0]), cfg)


def test_custom_icrs_map_is_read_at_phi_plus_gmst(tmp_path):
    nside = 8
    phi = np.array([0.0])
    lat = np.array([0.0])
    right = int(sky.healpix_ang2pix_ring(nside, np.array([math.pi / 2]),
                                         sm.convert_phi_to_ra(phi, GPS))[0])
    wrong = int(sky.healpix_ang2pix_ring(nside, np.array([math.pi / 2]), phi)[0])
    assert right != wrong
    m = np.zeros(12 * nside * nside)
    m[right] = 1.0
    path = str(tmp_path / "mask.fits")
    sm.write_healpix_map(path, m)
    cfg = {"type": "Custom", "coordsys": "icrs",
           "custom": {"healpix_map": path, "nside": nside, "ordering": "ring", "threshold": 0.0}}
    assert sm.compute_sky_valid_indices(phi, lat, cfg, t_ref=GPS).tolist() == [0]
    with pytest.raises(ValueError, match="requires a GPS reference time"):
        sm.compute_sky_valid_indices(phi, lat, cfg)
    with pytest.raises(ValueError, match="nside"):
        sm.compute_sky_valid_indices(phi, lat, dict(cfg, custom=dict(cfg["custom"], nside=4)),
                                     t_ref=GPS)


@pytest.mark.parametrize("file_nest,want_nest", [(False, False), (False, True), (True, False),
                                                 (True, True)])
def test_healpix_fits_round_trip_and_ordering(tmp_path, file_nest, want_nest):
    nside = 4
    n = 12 * nside * nside
    ring_map = np.arange(n, dtype=np.float64) * 0.5 - 3.0
    perm = sky.healpix_ring_to_nest(nside)
    nest_map = np.empty(n)
    nest_map[perm] = ring_map
    path = str(tmp_path / f"m{int(file_nest)}{int(want_nest)}.fits")
    sm.write_healpix_map(path, nest_map if file_nest else ring_map, nest=file_nest)
    got = sm.read_healpix_map(path, want_nest)
    assert np.array_equal(got, nest_map if want_nest else ring_map)


def test_custom_geo_mask_on_the_grid(tmp_path):
    """A map at the grid's own resolution keeps exactly its marked pixels,
    in either ordering of the file and of the lookup."""
    order = 3
    nside = 1 << order
    phi, lat = sky.build_sky_directions(12 * nside * nside, order)
    keep = np.zeros(12 * nside * nside)
    marked = np.array([0, 5, 100, 383, 767])
    keep[marked] = 2.0
    path = str(tmp_path / "geo.fits")
    sm.write_healpix_map(path, keep)
    for ordering in ("ring", "nested"):
        cfg = {"type": "Custom", "coordsys": "geo",
               "custom": {"healpix_map": path, "ordering": ordering, "threshold": 1.0}}
        assert sm.compute_sky_valid_indices(phi, lat, cfg).tolist() == marked.tolist()


def test_icrs_mask_follows_the_cluster_time():
    start, offset = GPS, 600.0
    target = sm.gmst_cwb(start + offset)
    cfg = {"type": "Fixed", "coordsys": "icrs",
           "coordinates": {"ra": f"{math.degrees(target)} deg", "dec": "0 deg"}}
    at_start = float((target - sm.gmst_cwb(start)) % (2 * math.pi))
    setup = {"sky_mask_config": cfg, "segment_start_gps": start,
             "phi_geo_arr": np.array([0.0, at_start]), "latitude_arr": np.array([0.0, 0.0]),
             "sky_valid_indices": np.array([1], dtype=np.int64)}
    assert sm.sky_valid_indices_for_cluster(setup, SimpleNamespace(cluster_time=offset)).tolist() == [0]
    # no cluster time: the cluster metadata's c_time
    meta = SimpleNamespace(cluster_time=0.0, cluster_meta=SimpleNamespace(c_time=offset))
    assert sm.sky_valid_indices_for_cluster(setup, meta).tolist() == [0]
    # an Earth-fixed mask keeps the cached indices
    geo = dict(setup, sky_mask_config={"type": "UniformAllSky"})
    assert sm.sky_valid_indices_for_cluster(geo, SimpleNamespace(cluster_time=offset)).tolist() == [1]
    with pytest.raises(ValueError, match="segment_start_gps"):
        sm.sky_valid_indices_for_cluster(dict(setup, segment_start_gps=None),
                                         SimpleNamespace(cluster_time=offset))


def test_cwb_colatitude_is_converted_to_latitude():
    cfg = {"type": "Fixed", "coordsys": "cwb",
           "coordinates": {"phi_geo": "0 deg", "theta_cwb": "60 deg"}}
    got = sm.compute_sky_valid_indices(np.array([0.0, 0.0]), np.deg2rad([30.0, -30.0]), cfg)
    assert got.tolist() == [0]


def test_fixed_and_empty_sky_reference_cases():
    ra = np.array([0.0, 1.0, 2.0])
    dec = np.array([0.0, 0.5, -0.5])
    cfg = {"type": "Fixed", "coordinates": {"sky_loc": {"phi": 1.0, "theta": 0.5}, "unit": "rad"}}
    assert sm.compute_sky_valid_indices(ra, dec, cfg).tolist() == [1]
    empty = np.array([])
    assert sm.compute_sky_valid_indices(empty, empty, None).size == 0
    patch = {"type": "Patch", "patch": {"center": {"phi": 0.0, "theta": 0.0}, "radius": 1.0,
                                        "unit": "rad"}}
    assert sm.compute_sky_valid_indices(empty, empty, patch).size == 0
    with pytest.raises(ValueError):
        sm.compute_sky_valid_indices(ra, dec, {"type": "Galaxy"})
