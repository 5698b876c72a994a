"""Sky masks on the Earth-fixed likelihood grid.

Mirrors pycwb/modules/likelihoodWP/sky_mask.py (compute_sky_valid_indices
:71-176, sky_valid_indices_for_cluster :179-211) without healpy or astropy:

* UniformAllSky (or no mask): every direction;
* Patch: the directions within ``radius`` of a centre;
* Fixed: the one direction nearest a point;
* Custom: the directions whose HEALPix map value exceeds ``threshold``
  (map read from a FITS file by ``read_healpix_map``; RING or NESTED);

in the coordinate systems ``geo`` (longitude, latitude), ``cwb`` (phi_geo,
theta_cwb co-latitude) and ``icrs`` (ra, dec).  An ICRS point is brought to
the Earth-fixed grid at a GPS time with cWB's sidereal-time polynomial
(pycwb/utils/skymap_coord.py:252-267, cwb-core skymap.hh phiRA):
phi = (ra - GMST(t)) mod 2 pi; an ICRS HEALPix map is looked up at
ra = (phi + GMST(t)) mod 2 pi.  ICRS masks depend on the event time, so
``sky_valid_indices_for_cluster`` evaluates them at segment start + the
cluster's time, as cWB's sky loop does (network.cc).

Angles are radians, or strings "<value> deg|rad|arcmin|arcsec".  The
legacy ``phi``/``theta`` keys with a separate ``unit`` are accepted.
"""

from __future__ import annotations

import functools
import math

import numpy as np

from .. import sky

TWO_PI = 2.0 * math.pi
EPOCH_J2000_0_GPS = 630763213.0
COORDINATE_KEYS = {"icrs": ("ra", "dec"), "geo": ("longitude", "latitude"),
                   "cwb": ("phi_geo", "theta_cwb")}
_UNITS = {"deg": math.pi / 180.0, "rad": 1.0, "arcmin": math.pi / 10800.0,
          "arcsec": math.pi / 648000.0}


def gmst_cwb(gps_time):
    """cWB's Greenwich mean sidereal time, radians (skymap.hh phiRA; the
    IAU 1982 polynomial in Julian centuries from J2000.0)."""
    gps = np.asarray(gps_time, dtype=np.float64)
    t = (gps - EPOCH_J2000_0_GPS) / 86400.0 / 36525.0
    sec = (-6.2e-6 * t + 0.093104) * t * t + 67310.54841 + 8640184.812866 * t + \
        3155760000.0 * t
    out = np.deg2rad((360.0 * sec / 86400.0) % 360.0)
    return float(out) if out.ndim == 0 else out


def convert_ra_to_phi(ra, gps_time):
    return (np.asarray(ra) - gmst_cwb(gps_time)) % TWO_PI


def convert_phi_to_ra(phi, gps_time):
    return (np.asarray(phi) + gmst_cwb(gps_time)) % TWO_PI


def _angle(v, name: str, legacy_unit=None) -> float:
    """Radians of one angle: a '<value> <unit>' string, or a number in
    ``legacy_unit`` (radians when none is given)."""
    if isinstance(v, str):
        parts = v.split()
        if len(parts) != 2 or parts[1] not in _UNITS:
            raise ValueError(f"{name} must be '<value> deg|rad|arcmin|arcsec', got {v!r}")
        return float(parts[0]) * _UNITS[parts[1]]
    scale = _UNITS.get(str(legacy_unit), 1.0) if legacy_unit is not None else 1.0
    return float(v) * scale


def _coordsys(cfg) -> str:
    cs = str(cfg.get("coordsys", "geo")).lower()
    if cs not in COORDINATE_KEYS:
        raise ValueError(f"Coordinate system {cs!r} is not recognized; supported values are: "
                         f"{', '.join(sorted(COORDINATE_KEYS))}")
    return cs


def parse_sky_coordinates(values, coordsys: str, context: str, legacy_unit=None):
    """(first, second) radians of a point given in ``coordsys`` keys, with the
    ranges checked as pycwb/utils/skymap_coord.py:84-168 checks them."""
    a, b = COORDINATE_KEYS[coordsys]
    legacy = False
    if a in values and b in values:
        first, second = _angle(values[a], f"{context}.{a}"), _angle(values[b], f"{context}.{b}")
    elif "phi" in values and "theta" in values:
        if legacy_unit is None:
            raise ValueError(f"Legacy {context} phi/theta values require an explicit angular unit")
        legacy = True
        first = _angle(values["phi"], f"{context}.phi", legacy_unit)
        second = _angle(values["theta"], f"{context}.theta", legacy_unit)
    else:
        raise ValueError(f"{context} with coordsys={coordsys!r} requires keys {a!r} and {b!r}")
    if coordsys == "icrs":
        if not legacy and not 0.0 <= first <= TWO_PI:
            raise ValueError(f"{context}.ra must be within [0 deg, 360 deg]")
        if not -math.pi / 2 <= second <= math.pi / 2:
            raise ValueError(f"{context}.dec must be within [-90 deg, 90 deg]")
        return first % TWO_PI, second
    if coordsys == "geo":
        if not legacy and not -math.pi <= first <= math.pi:
            raise ValueError(f"{context}.longitude must be within [-180 deg, 180 deg]")
        if not -math.pi / 2 <= second <= math.pi / 2:
            raise ValueError(f"{context}.latitude must be within [-90 deg, 90 deg]")
        return (first + math.pi) % TWO_PI - math.pi, second
    if not legacy and not 0.0 <= first <= TWO_PI:
        raise ValueError(f"{context}.phi_geo must be within [0 deg, 360 deg]")
    if not 0.0 <= second <= math.pi:
        raise ValueError(f"{context}.theta_cwb must be within [0 deg, 180 deg]")
    return first % TWO_PI, second


def _to_earth_fixed(first, second, coordsys, t_ref, context):
    """(phi_geo, latitude) radians (sky_mask.py:41-49)."""
    if coordsys == "icrs":
        if t_ref is None:
            raise ValueError(f"{context} with coordsys='icrs' requires a GPS reference time")
        return float(convert_ra_to_phi(first, t_ref)), second
    if coordsys == "geo":
        return first % TWO_PI, second
    return first % TWO_PI, math.pi / 2.0 - second


def _cos_distance(lat, phi, c_lat, c_phi):
    return np.sin(lat) * math.sin(c_lat) + np.cos(lat) * math.cos(c_lat) * np.cos(phi - c_phi)


# --------------------------------------------------------------------------
# HEALPix maps in FITS files
# --------------------------------------------------------------------------
UNSEEN = -1.6375e30
_FITS_BLOCK = 2880
_TFORM = {"E": ">f4", "D": ">f8", "J": ">i4", "K": ">i8", "I": ">i2", "B": "u1"}


def _fits_header(buf: bytes, pos: int):
    """Cards of the header starting at ``pos`` and the offset of its data."""
    cards = {}
    while True:
        if pos + _FITS_BLOCK > len(buf):
            raise ValueError("FITS file ends inside a header")
        block = buf[pos:pos + _FITS_BLOCK]
        pos += _FITS_BLOCK
        for k in range(0, _FITS_BLOCK, 80):
            card = block[k:k + 80].decode("ascii", errors="replace")
            key = card[:8].strip()
            if key == "END":
                return cards, pos
            if card[8:10] != "= ":
                continue
            val = card[10:]
            if val.lstrip().startswith("'"):
                s = val.lstrip()[1:]
                end = s.find("'")
                cards[key] = s[:end].strip() if end >= 0 else s.strip()
            else:
                v = val.split("/")[0].strip()
                if v in ("T", "F"):
                    cards[key] = v == "T"
                else:
                    try:
                        cards[key] = int(v)
                    except ValueError:
                        try:
                            cards[key] = float(v)
                        except ValueError:
                            cards[key] = v


def _padded(n: int) -> int:
    return (n + _FITS_BLOCK - 1) // _FITS_BLOCK * _FITS_BLOCK


def _column_layout(h):
    """Per column: (byte offset in the row, numpy dtype, repeat count)."""
    cols, off = [], 0
    for k in range(1, int(h.get("TFIELDS", 0)) + 1):
        form = str(h[f"TFORM{k}"]).strip()
        digits = ""
        while form and form[0].isdigit():
            digits, form = digits + form[0], form[1:]
        rep = int(digits) if digits else 1
        code = form[:1]
        if code not in _TFORM:
            raise ValueError(f"unsupported FITS column format TFORM{k}={h[f'TFORM{k}']!r}")
        dt = np.dtype(_TFORM[code])
        cols.append((off, dt, rep))
        off += rep * dt.itemsize
    return cols


@functools.lru_cache(maxsize=16)
def read_healpix_map(path: str, nest: bool) -> np.ndarray:
    """First map of a HEALPix FITS file (binary table, as healpy writes it),
    float64, in NESTED order when ``nest`` else RING -- the file's ordering
    (its ORDERING card) is converted when it differs.  Partial-sky files
    (INDXSCHM = EXPLICIT: a PIXEL and a SIGNAL column) are expanded with
    UNSEEN at the missing pixels."""
    with open(path, "rb") as f:
        buf = f.read()
    h0, pos = _fits_header(buf, 0)
    if not h0.get("SIMPLE", False):
        raise ValueError(f"{path}: not a FITS file")
    n0 = 1
    for k in range(1, int(h0.get("NAXIS", 0)) + 1):
        n0 *= int(h0[f"NAXIS{k}"])
    pos += _padded(abs(int(h0.get("BITPIX", 8))) // 8 * n0) if int(h0.get("NAXIS", 0)) else 0
    h, pos = _fits_header(buf, pos)
    if str(h.get("XTENSION", "")).strip() != "BINTABLE":
        raise ValueError(f"{path}: the first extension is not a binary table")
    row, nrow = int(h["NAXIS1"]), int(h["NAXIS2"])
    data = np.frombuffer(buf, dtype=np.uint8, count=row * nrow, offset=pos).reshape(nrow, row)
    cols = _column_layout(h)

    def column(k):
        off, dt, rep = cols[k]
        raw = np.ascontiguousarray(data[:, off:off + rep * dt.itemsize]).reshape(-1)
        return np.frombuffer(raw.tobytes(), dtype=dt).astype(np.float64)

    nside = int(h.get("NSIDE", 0))
    if str(h.get("INDXSCHM", "IMPLICIT")).strip().upper() == "EXPLICIT":
        if nside <= 0 or len(cols) < 2:
            raise ValueError(f"{path}: a partial-sky map needs NSIDE and PIXEL/SIGNAL columns")
        m = np.full(12 * nside * nside, UNSEEN)
        m[column(0).astype(np.int64)] = column(1)
    else:
        m = column(0)
        if nside <= 0:
            nside = int(round(math.sqrt(m.size / 12)))
    if m.size != 12 * nside * nside:
        raise ValueError(f"{path}: {m.size} values do not form a HEALPix map of nside {nside}")
    ordering = str(h.get("ORDERING", "RING")).strip().upper()
    file_nest = ordering.startswith("NEST")
    if file_nest != bool(nest):
        perm = sky.healpix_ring_to_nest(nside)     # nested index of each ring pixel
        if file_nest:
            m = m[perm]                            # nested -> ring
        else:
            out = np.empty_like(m)
            out[perm] = m                          # ring -> nested
            m = out
    m.setflags(write=False)
    return m


def write_healpix_map(path: str, m, nest: bool = False, coord: str | None = None) -> None:
    """A full-sky HEALPix map as a FITS binary table of float64 (one column,
    1024 values per row when the map allows), the layout ``read_healpix_map``
    reads."""
    m = np.asarray(m, dtype=">f8").reshape(-1)
    nside = int(round(math.sqrt(m.size / 12)))
    if 12 * nside * nside != m.size:
        raise ValueError("map size is not 12 nside^2")
    rep = 1024 if m.size % 1024 == 0 else 1
    nrow = m.size // rep

    def cards(items):
        out = b""
        for key, val in items:
            if isinstance(val, bool):
                v = "T" if val else "F"
                s = f"{key:<8}= {v:>20}"
            elif isinstance(val, int):
                s = f"{key:<8}= {val:>20}"
            else:
                s = f"{key:<8}= '{val:<8}'"
            out += s.ljust(80).encode("ascii")
        out += b"END".ljust(80)
        return out.ljust(_padded(len(out)), b" ")

    hdr0 = cards([("SIMPLE", True), ("BITPIX", 8), ("NAXIS", 0), ("EXTEND", True)])
    items = [("XTENSION", "BINTABLE"), ("BITPIX", 8), ("NAXIS", 2), ("NAXIS1", 8 * rep),
             ("NAXIS2", nrow), ("PCOUNT", 0), ("GCOUNT", 1), ("TFIELDS", 1),
             ("TTYPE1", "SIGNAL"), ("TFORM1", f"{rep}D"), ("PIXTYPE", "HEALPIX"),
             ("ORDERING", "NESTED" if nest else "RING"), ("NSIDE", nside),
             ("INDXSCHM", "IMPLICIT"), ("OBJECT", "FULLSKY")]
    if coord:
        items.append(("COORDSYS", coord))
    body = m.tobytes()
    with open(path, "wb") as f:
        f.write(hdr0 + cards(items) + body + b"\0" * (_padded(len(body)) - len(body)))


# --------------------------------------------------------------------------
# masks
# --------------------------------------------------------------------------
def sky_mask_requires_event_time(sky_mask_config) -> bool:
    """True for a restricted mask given in ICRS, which rotates against the
    Earth-fixed grid (sky_mask.py:24-28)."""
    if not sky_mask_config or sky_mask_config.get("type", "UniformAllSky") == "UniformAllSky":
        return False
    return _coordsys(sky_mask_config) == "icrs"


def compute_sky_valid_indices(phi_geo_arr, latitude_arr, sky_mask_config, t_ref=None):
    """Sorted int64 indices of the directions the mask keeps
    (sky_mask.py:71-176).  ``phi_geo_arr``/``latitude_arr`` are the
    Earth-fixed longitude and latitude of the grid, radians; ``t_ref`` the
    GPS time at which an ICRS mask is evaluated."""
    phi = np.asarray(phi_geo_arr, np.float64)
    lat = np.asarray(latitude_arr, np.float64)
    if phi.shape != lat.shape:
        raise ValueError("Sky longitude and latitude arrays must have identical shapes")
    n_sky = phi.size
    if not sky_mask_config or sky_mask_config.get("type", "UniformAllSky") == "UniformAllSky":
        return np.arange(n_sky, dtype=np.int64)
    kind = sky_mask_config.get("type")
    coordsys = _coordsys(sky_mask_config)
    if kind == "Patch":
        patch = sky_mask_config["patch"]
        unit = patch.get("unit", "rad")
        first, second = parse_sky_coordinates(patch["center"], coordsys, "sky_mask.patch.center",
                                              legacy_unit=unit)
        legacy = "phi" in patch["center"] and "theta" in patch["center"]
        r = patch["radius"]
        if not isinstance(r, str) and not legacy:
            raise ValueError("sky_mask.patch.radius must carry a unit, e.g. '10 deg'")
        radius = _angle(r, "sky_mask.patch.radius", unit)
        if not 0.0 <= radius <= math.pi:
            raise ValueError("sky_mask.patch.radius must be within [0 deg, 180 deg]")
        c_phi, c_lat = _to_earth_fixed(first, second, coordsys, t_ref, "sky_mask.patch")
        cos_d = _cos_distance(lat, phi, c_lat, c_phi)
        return np.where(np.arccos(np.clip(cos_d, -1.0, 1.0)) <= radius)[0].astype(np.int64)
    if kind == "Fixed":
        coords = sky_mask_config["coordinates"]
        values = coords.get("sky_loc", coords)
        first, second = parse_sky_coordinates(values, coordsys, "sky_mask.coordinates",
                                              legacy_unit=coords.get("unit", "rad"))
        f_phi, f_lat = _to_earth_fixed(first, second, coordsys, t_ref, "sky_mask.coordinates")
        if n_sky == 0:
            return np.array([], dtype=np.int64)
        cos_d = _cos_distance(lat, phi, f_lat, f_phi)
        return np.array([int(np.argmax(np.clip(cos_d, -1.0, 1.0)))], dtype=np.int64)
    if kind == "Custom":
        if coordsys == "icrs" and t_ref is None:
            raise ValueError("sky_mask Custom with coordsys='icrs' requires a GPS reference time")
        custom = sky_mask_config["custom"]
        ordering = str(custom.get("ordering", "ring")).lower()
        if ordering not in ("ring", "nested"):
            raise ValueError("sky_mask.custom.ordering must be 'ring' or 'nested'")
        nest = ordering == "nested"
        m = read_healpix_map(str(custom["healpix_map"]), nest)
        map_nside = int(round(math.sqrt(m.size / 12)))
        nside = int(custom.get("nside", map_nside))
        if nside != map_nside or m.size != 12 * nside * nside:
            raise ValueError("sky_mask.custom.nside does not match the loaded HEALPix map")
        lon = convert_phi_to_ra(phi, t_ref) if coordsys == "icrs" else phi
        theta = np.clip(math.pi / 2.0 - lat, 0.0, math.pi)
        pix = (sky.healpix_ang2pix_nest if nest else sky.healpix_ang2pix_ring)(nside, theta, lon)
        threshold = float(custom.get("threshold", 0.0))
        return np.where(m[pix] > threshold)[0].astype(np.int64)
    raise ValueError(f"Unknown sky_mask type: {kind!r}; supported types are "
                     "UniformAllSky, Patch, Fixed, Custom")


def sky_valid_indices_for_cluster(setup, cluster, *, use_big_grid: bool = False):
    """The mask at the cluster's GPS time (segment start + cluster time, or
    the cluster's c_time when its cluster_time is 0), for ICRS masks; the
    setup's cached indices otherwise (sky_mask.py:179-211)."""
    mask = setup.get("sky_mask_config")
    cached = setup.get("sky_valid_indices_big" if use_big_grid else "sky_valid_indices")
    if not sky_mask_requires_event_time(mask):
        return cached
    start = setup.get("segment_start_gps")
    if start is None:
        raise ValueError("An ICRS sky mask requires segment_start_gps so it can be evaluated "
                         "at the cluster time")
    offset = float(getattr(cluster, "cluster_time", 0.0) or 0.0)
    if offset == 0.0:
        meta = getattr(cluster, "cluster_meta", None)
        offset = float(getattr(meta, "c_time", 0.0) or 0.0)
    if use_big_grid:
        phi, lat = setup.get("phi_geo_arr_big_cluster"), setup.get("latitude_arr_big_cluster")
    else:
        phi = setup.get("phi_geo_arr", setup.get("ra_arr"))
        lat = setup.get("latitude_arr", setup.get("dec_arr"))
    return compute_sky_valid_indices(phi, lat, mask, t_ref=float(start) + offset)
