"""Per-segment sky tables: HEALPix RING directions, delay indices and F+/Fx.

This is the table builder that feeds the sky scan.  It runs once per job
segment on the host (it is not on the per-cluster hot path) and restates,
without healpy or astropy:

* ``_build_sky_directions``           pycwb/types/detector.py:1220-1240
* ``compute_sky_delay_and_patterns``  pycwb/types/detector.py:1243-1329
* ``earth_centered_vectors``          pycwb/types/detector.py:1061-1123
* ``Detector.atenna_pattern``         pycwb/types/detector.py:272-358 (tensor,
  frequency=0 branch, evaluated at gha = -phi_geo and psi = 0)

HEALPix RING ``pix2ang`` follows the published scheme of Gorski et al. 2005
(ApJ 622:759, section 4); healpy is not required.  Geodetic -> ECEF uses the
WGS84 ellipsoid, which is what ``astropy.coordinates.EarthLocation.from_geodetic``
uses by default.  Detector site constants are the ones in
pycwb/constants/detectors.py:2-161.
"""

from __future__ import annotations

import math

import numpy as np

C_LIGHT = 299792458.0  # m/s (astropy.constants.c)

# name: (lat, lon, elevation, x_az, x_alt, y_az, y_alt)  radians / metres
DETECTORS = {
    "H1": (0.81079526383, -2.08405676917, 142.554,
           5.65487724844, -0.00061950000, 4.08408092164, 0.00001250000),
    "L1": (0.53342313506, -1.58430937078, -6.574,
           4.40317772346, -0.00031210000, 2.83238139666, -0.00061070000),
    "V1": (0.76151183984, 0.18333805213, 51.884,
           0.33916285222, 0.0, 5.05155183261, 0.0),
    "K1": (0.6355068497, 2.396441015, 414.181,
           1.054113, 0.0031414, -0.5166798, -0.0036270),
}


def healpix_npix(order: int) -> int:
    nside = 1 << int(order)
    return 12 * nside * nside


def healpix_pix2ang_ring(nside: int, ipix: np.ndarray):
    """(theta, phi) in radians of RING-scheme pixel centres.

    Polar caps: ring i (from the nearer pole) holds 4i pixels at
    z = +-(1 - i^2 / (3 nside^2)), phi = (j - 1/2) pi / (2i).
    Equatorial belt: ring i in [nside, 3 nside] holds 4 nside pixels at
    z = (2 nside - i) * 2 / (3 nside), phi = (j - s/2) pi / (2 nside) with
    s = 1 when i + nside is odd and s = 1/2 ... (here ``fodd``) otherwise.
    """
    ipix = np.asarray(ipix, dtype=np.int64)
    nside = int(nside)
    npix = 12 * nside * nside
    ncap = 2 * nside * (nside - 1)
    theta = np.empty(ipix.shape, dtype=np.float64)
    phi = np.empty(ipix.shape, dtype=np.float64)

    north = ipix < ncap
    south = ipix >= npix - ncap
    belt = ~(north | south)

    if np.any(north):
        p = ipix[north]
        iring = (1 + _isqrt(1 + 2 * p)) >> 1
        iphi = (p + 1) - 2 * iring * (iring - 1)
        z = 1.0 - (iring * iring) * (4.0 / npix)
        theta[north] = np.arccos(z)
        phi[north] = (iphi - 0.5) * (0.5 * math.pi) / iring
    if np.any(belt):
        ip = ipix[belt] - ncap
        nl4 = 4 * nside
        tmp = ip // nl4
        iring = tmp + nside
        iphi = ip - nl4 * tmp + 1
        fodd = np.where(((iring + nside) & 1) == 1, 1.0, 0.5)
        z = (2 * nside - iring) * (2.0 / (3.0 * nside))
        theta[belt] = np.arccos(z)
        phi[belt] = (iphi - fodd) * math.pi / (2.0 * nside)
    if np.any(south):
        ip = npix - ipix[south]
        iring = (1 + _isqrt(2 * ip - 1)) >> 1
        iphi = 4 * iring + 1 - (ip - 2 * iring * (iring - 1))
        z = (iring * iring) * (4.0 / npix) - 1.0
        theta[south] = np.arccos(z)
        phi[south] = (iphi - 0.5) * (0.5 * math.pi) / iring
    return theta, phi


def _zphi(theta, phi):
    theta = np.asarray(theta, dtype=np.float64)
    phi = np.asarray(phi, dtype=np.float64)
    if theta.shape != phi.shape:
        theta, phi = np.broadcast_arrays(theta, phi)
    if np.any((theta < 0.0) | (theta > math.pi)):
        raise ValueError("theta must lie in [0, pi]")
    z = np.cos(theta)
    tt = np.mod(phi, 2.0 * math.pi) * (2.0 / math.pi)   # in [0, 4)
    tt = np.where(tt >= 4.0, 0.0, tt)
    return z, np.abs(z), tt


def healpix_ang2pix_ring(nside: int, theta, phi) -> np.ndarray:
    """RING-scheme pixel holding each direction (theta co-latitude, phi
    longitude, radians), by the published scheme (Gorski et al. 2005,
    section 4): in the equatorial belt |z| <= 2/3 the ring and the position
    along it follow from the two families of pixel-boundary lines
    j+ = nside (1/2 + t - 3z/4) and j- = nside (1/2 + t + 3z/4) (t = 2 phi / pi);
    in the polar caps from the same lines scaled by sqrt(3 (1 - |z|))."""
    nside = int(nside)
    z, za, tt = _zphi(theta, phi)
    out = np.empty(z.shape, dtype=np.int64)
    npix = 12 * nside * nside
    ncap = 2 * nside * (nside - 1)
    eq = za <= 2.0 / 3.0
    if np.any(eq):
        t1 = nside * (0.5 + tt[eq])
        t2 = nside * z[eq] * 0.75
        jp = (t1 - t2).astype(np.int64)
        jm = (t1 + t2).astype(np.int64)
        ir = nside + 1 + jp - jm                      # ring counted from z = 2/3, 1..2 nside+1
        kshift = 1 - (ir & 1)
        ip = (jp + jm - nside + kshift + 1) // 2
        ip = np.mod(ip, 4 * nside)
        out[eq] = ncap + (ir - 1) * 4 * nside + ip
    pol = ~eq
    if np.any(pol):
        t = tt[pol]
        tp = t - np.floor(t)
        tmp = nside * np.sqrt(3.0 * (1.0 - za[pol]))
        jp = (tp * tmp).astype(np.int64)
        jm = ((1.0 - tp) * tmp).astype(np.int64)
        ir = jp + jm + 1                              # ring counted from the nearer pole
        ip = (t * ir).astype(np.int64)
        ip = np.mod(ip, 4 * ir)
        north = z[pol] > 0
        out[pol] = np.where(north, 2 * ir * (ir - 1) + ip, npix - 2 * ir * (ir + 1) + ip)
    return out


def _spread_bits(v: np.ndarray) -> np.ndarray:
    """Bit k of v moved to bit 2k (v < 2^29)."""
    v = v.astype(np.uint64)
    out = np.zeros(v.shape, dtype=np.uint64)
    for k in range(29):
        out |= ((v >> np.uint64(k)) & np.uint64(1)) << np.uint64(2 * k)
    return out


def healpix_ang2pix_nest(nside: int, theta, phi) -> np.ndarray:
    """NESTED-scheme pixel holding each direction: the base face (0-3 north,
    4-7 equatorial, 8-11 south) from the same boundary lines as the RING
    scheme, then the pixel's (x, y) within the face with the bits of x and y
    interleaved (Gorski et al. 2005, section 4)."""
    nside = int(nside)
    if nside < 1 or nside & (nside - 1):
        raise ValueError("nside must be a power of two for the NESTED scheme")
    z, za, tt = _zphi(theta, phi)
    face = np.empty(z.shape, dtype=np.int64)
    ix = np.empty(z.shape, dtype=np.int64)
    iy = np.empty(z.shape, dtype=np.int64)
    eq = za <= 2.0 / 3.0
    if np.any(eq):
        t1 = nside * (0.5 + tt[eq])
        t2 = nside * (z[eq] * 0.75)
        jp = (t1 - t2).astype(np.int64)
        jm = (t1 + t2).astype(np.int64)
        ifp = jp // nside
        ifm = jm // nside
        face[eq] = np.where(ifp == ifm, ifp | 4, np.where(ifp < ifm, ifp, ifm + 8))
        ix[eq] = jm & (nside - 1)
        iy[eq] = nside - (jp & (nside - 1)) - 1
    pol = ~eq
    if np.any(pol):
        t = tt[pol]
        ntt = np.minimum(3, t.astype(np.int64))
        tp = t - ntt
        tmp = nside * np.sqrt(3.0 * (1.0 - za[pol]))
        jp = np.minimum((tp * tmp).astype(np.int64), nside - 1)
        jm = np.minimum(((1.0 - tp) * tmp).astype(np.int64), nside - 1)
        north = z[pol] >= 0
        face[pol] = np.where(north, ntt, ntt + 8)
        ix[pol] = np.where(north, nside - jm - 1, jp)
        iy[pol] = np.where(north, nside - jp - 1, jm)
    xy = _spread_bits(ix) | (_spread_bits(iy) << np.uint64(1))
    return face * nside * nside + xy.astype(np.int64)


def healpix_ring_to_nest(nside: int) -> np.ndarray:
    """NESTED index of every RING pixel (ring index order)."""
    nside = int(nside)
    theta, phi = healpix_pix2ang_ring(nside, np.arange(12 * nside * nside))
    return healpix_ang2pix_nest(nside, theta, phi)


def _isqrt(v: np.ndarray) -> np.ndarray:
    r = np.floor(np.sqrt(v.astype(np.float64))).astype(np.int64)
    # exact integer correction of the float estimate
    r = np.where(r * r > v, r - 1, r)
    r = np.where((r + 1) * (r + 1) <= v, r + 1, r)
    return r


def build_sky_directions(n_sky: int, healpix_order: int | None = None):
    """Earth-fixed (phi_geo, latitude) of every sky direction, radians.

    HEALPix RING grid when ``healpix_order > 0``; otherwise the Fibonacci
    grid of pycwb/types/detector.py:1234-1240.
    """
    if healpix_order is not None and int(healpix_order) > 0:
        nside = 1 << int(healpix_order)
        theta, phi = healpix_pix2ang_ring(nside, np.arange(12 * nside * nside))
        return phi.astype(np.float64), (np.pi / 2.0) - theta
    n_sky = int(max(1, n_sky))
    idx = np.arange(n_sky, dtype=np.float64)
    z = 1.0 - 2.0 * (idx + 0.5) / float(n_sky)
    phi = (np.pi * (3.0 - np.sqrt(5.0)) * idx) % (2.0 * np.pi)
    return phi.astype(np.float64), np.arcsin(np.clip(z, -1.0, 1.0))


def _rot(axis: str, ang: float) -> np.ndarray:
    """Coordinate-frame (passive) rotation matrix about one axis."""
    c, s = math.cos(ang), math.sin(ang)
    if axis == "z":
        return np.array([[c, s, 0.0], [-s, c, 0.0], [0.0, 0.0, 1.0]])
    if axis == "y":
        return np.array([[c, 0.0, -s], [0.0, 1.0, 0.0], [s, 0.0, c]])
    raise ValueError(axis)


def geodetic_to_ecef(lat: float, lon: float, h: float) -> np.ndarray:
    a = 6378137.0
    f = 1.0 / 298.257223563
    e2 = f * (2.0 - f)
    sl, cl = math.sin(lat), math.cos(lat)
    n = a / math.sqrt(1.0 - e2 * sl * sl)
    return np.array([(n + h) * cl * math.cos(lon),
                     (n + h) * cl * math.sin(lon),
                     (n * (1.0 - e2) + h) * sl])


class DetectorSite:
    """Vertex position (ECEF, metres), arm unit vectors and response tensor.

    The response is D = (u_x u_x^T - u_y u_y^T) / 2, built as in
    pycwb/types/detector.py:1088-1110: each arm's unit vector is the
    rotation rz(-lon) ry(-(pi/2-lat)) rz(azimuth) ry(-altitude) applied to
    (-1, 0, 0).
    """

    def __init__(self, name: str):
        if name not in DETECTORS:
            raise ValueError(f"unknown detector {name!r}")
        lat, lon, h, xaz, xalt, yaz, yalt = DETECTORS[name]
        self.name = name
        self.latitude, self.longitude = lat, lon
        base = np.array([[-1.0, 0.0, 0.0], [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]])
        rm2 = _rot("z", -lon)
        rm1 = _rot("y", -(np.pi / 2.0 - lat))
        resps, vecs = [], []
        for az, alt in ((yaz, yalt), (xaz, xalt)):
            rm = rm2 @ rm1 @ _rot("z", az) @ _rot("y", -alt)
            resps.append(rm @ base @ rm.T / 2.0)
            vecs.append(rm @ np.array([-1.0, 0.0, 0.0]))
        self.y_vec, self.x_vec = vecs
        self.response = resps[0] - resps[1]
        self.vertex = geodetic_to_ecef(lat, lon, h)

    def antenna_pattern_geo(self, phi_geo: np.ndarray, latitude: np.ndarray,
                            psi: float | np.ndarray = 0.0):
        """F+ and Fx for Earth-fixed directions (gha = -phi_geo)."""
        gha = -np.asarray(phi_geo, dtype=np.float64)
        dec = np.asarray(latitude, dtype=np.float64)
        cosgha, singha = np.cos(gha), np.sin(gha)
        cosdec, sindec = np.cos(dec), np.sin(dec)
        cospsi, sinpsi = np.cos(psi), np.sin(psi)
        x = np.stack([-cospsi * singha - sinpsi * cosgha * sindec,
                      -cospsi * cosgha + sinpsi * singha * sindec,
                      sinpsi * cosdec * np.ones_like(gha)])
        y = np.stack([sinpsi * singha - cospsi * cosgha * sindec,
                      sinpsi * cosgha + cospsi * singha * sindec,
                      cospsi * cosdec])
        dx = self.response @ x
        dy = self.response @ y
        fplus = (x * dx - y * dy).sum(axis=0)
        fcross = (x * dy + y * dx).sum(axis=0)
        return fplus, fcross


def compute_sky_delay_and_patterns(ifos, ref_ifo, sample_rate, td_size,
                                   healpix_order=None, n_sky=None):
    """ml (nIFO, n_sky) int32, FP, FX (nIFO, n_sky) float64.

    ml[i, l] = clip(rint(n_l . (R_i - R_ref) / c * rate), -td_size, td_size):
    the sample shift that synchronises detector i to the reference
    (pycwb/types/detector.py:1310-1321).
    """
    dets = [DetectorSite(d) if isinstance(d, str) else d for d in ifos]
    if not dets:
        raise ValueError("No detectors provided")
    if n_sky is None:
        n_sky = healpix_npix(healpix_order) if healpix_order else 3072
    phi_geo, lat = build_sky_directions(n_sky, healpix_order)
    n_sky = phi_geo.size
    ref = next((i for i, d in enumerate(dets) if d.name == ref_ifo), 0)
    n_hat = np.vstack((np.cos(lat) * np.cos(phi_geo),
                       np.cos(lat) * np.sin(phi_geo), np.sin(lat))).T
    td_size = int(max(1, td_size))
    ml = np.zeros((len(dets), n_sky), dtype=np.int32)
    FP = np.zeros((len(dets), n_sky), dtype=np.float64)
    FX = np.zeros((len(dets), n_sky), dtype=np.float64)
    for i, d in enumerate(dets):
        shift = n_hat @ (d.vertex - dets[ref].vertex) / C_LIGHT
        ml[i] = np.clip(np.rint(shift * float(sample_rate)).astype(np.int32),
                        -td_size, td_size)
        FP[i], FX[i] = d.antenna_pattern_geo(phi_geo, lat, 0.0)
    return ml, FP, FX


def compute_sky_delay_and_patterns_device(ifos, ref_ifo, sample_rate, td_size, healpix_order,
                                          device="cuda"):
    """compute_sky_delay_and_patterns for a HEALPix grid, built on the GPU
    (pgw_sky_tables_healpix): (ml (n_ifo, n_sky) int32, FP_t, FX_t
    (n_sky, n_ifo) float32) as CUDA tensors, in the layouts the sky scan
    takes."""
    import torch

    from . import _device as dv
    from . import _lib

    if int(healpix_order) < 1:
        raise ValueError("healpix_order must be >= 1 (order 0 selects the host's non-HEALPix grid)")
    dets = [DetectorSite(d) if isinstance(d, str) else d for d in ifos]
    if not dets:
        raise ValueError("No detectors provided")
    ref = next((i for i, d in enumerate(dets) if d.name == ref_ifo), 0)
    resp = np.ascontiguousarray(np.stack([d.response for d in dets]).reshape(len(dets), 9),
                                np.float64)
    base = np.ascontiguousarray(np.stack([d.vertex - dets[ref].vertex for d in dets]), np.float64)
    n_sky = healpix_npix(healpix_order)
    dev = torch.device(device)
    s = dv.begin()
    with torch.cuda.stream(s):
        FP = torch.empty((n_sky, len(dets)), dtype=torch.float32, device=dev)
        FX = torch.empty((n_sky, len(dets)), dtype=torch.float32, device=dev)
        ml = torch.empty((len(dets), n_sky), dtype=torch.int32, device=dev)
    rc = _lib.load().pgw_sky_tables_healpix(int(healpix_order), len(dets), resp.ctypes.data,
                                            base.ctypes.data, float(C_LIGHT), float(sample_rate),
                                            int(max(1, td_size)), FP.data_ptr(), FX.data_ptr(),
                                            ml.data_ptr(), s.cuda_stream)
    _lib.check(rc, "sky_tables_healpix")
    dv.end(s, FP, FX, ml)
    return ml, FP, FX
