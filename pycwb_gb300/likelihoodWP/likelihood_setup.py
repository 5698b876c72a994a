"""Segment-level inputs of the likelihood: constants, sky tables, sky mask.

Mirrors pycwb/modules/likelihoodWP/likelihood_setup.py:81-238
(prepare_likelihood_inputs) with the same returned keys, and adds the
device-resident sky tables of the batched loop (``"gpu_tables"``) when a
device is given.  Constants (likelihood_setup.py:133-147):

    network_energy_threshold = 2 Acore^2 nIFO
    gamma_regulator          = gamma^2 * 2 / 3
    delta_regulator          = |delta| if |delta| < 1 else 1   (delta = 0 -> 1e-5)
    net_rho_threshold        = |netRHO|
    netEC_threshold          = 2 netRHO^2

Sky masks (pycwb/modules/likelihoodWP/sky_mask.py:71-176): UniformAllSky,
and Patch / Fixed in Earth-fixed coordinates ("geo": longitude/latitude;
"cwb": phi_geo/theta_cwb, co-latitude) with angles as "<value> deg" or
"<value> rad" strings, or numbers in radians.  ICRS masks (a GPS-time
sidereal rotation) and Custom HEALPix-map masks are not supported and
raise NotImplementedError.
"""

from __future__ import annotations

import math

import numpy as np

from .. import sky
from .pixel_data import build_sky_delay_and_antenna_patterns

_COORD_KEYS = {"geo": ("longitude", "latitude"), "cwb": ("phi_geo", "theta_cwb")}


def _angle(v, name: str) -> float:
    """Radians from a number (radians) or a '<value> deg|rad' string."""
    if isinstance(v, str):
        parts = v.split()
        if len(parts) != 2 or parts[1] not in ("deg", "rad"):
            raise ValueError(f"{name} must be '<value> deg' or '<value> rad', got {v!r}")
        x = float(parts[0])
        return math.radians(x) if parts[1] == "deg" else x
    return float(v)


def _earth_fixed(values, coordsys: str, context: str, legacy_unit=None):
    """(phi_geo, latitude) radians of a mask point."""
    if coordsys not in _COORD_KEYS:
        raise NotImplementedError(f"{context}: coordsys {coordsys!r} needs the sidereal rotation "
                                  "of the event time; only 'geo' and 'cwb' are supported")
    a, b = _COORD_KEYS[coordsys]
    if a in values and b in values:
        first, second = _angle(values[a], f"{context}.{a}"), _angle(values[b], f"{context}.{b}")
    elif "phi" in values and "theta" in values:
        scale = math.pi / 180.0 if legacy_unit == "deg" else 1.0
        first, second = float(values["phi"]) * scale, float(values["theta"]) * scale
    else:
        raise ValueError(f"{context} needs keys {a!r} and {b!r}")
    if coordsys == "geo":
        if not -math.pi / 2 <= second <= math.pi / 2:
            raise ValueError(f"{context}.latitude must be within [-90 deg, 90 deg]")
        return first % (2 * math.pi), second
    if not 0.0 <= second <= math.pi:
        raise ValueError(f"{context}.theta_cwb must be within [0 deg, 180 deg]")
    return first % (2 * math.pi), math.pi / 2 - second


def compute_sky_valid_indices(phi_geo_arr, latitude_arr, sky_mask_config, t_ref=None):
    """Sorted int64 indices of the directions the mask keeps (sky_mask.py:71-176)."""
    phi = np.asarray(phi_geo_arr, np.float64)
    lat = np.asarray(latitude_arr, np.float64)
    if phi.shape != lat.shape:
        raise ValueError("Sky longitude and latitude arrays must have identical shapes")
    n_sky = phi.size
    if not sky_mask_config or sky_mask_config.get("type", "UniformAllSky") == "UniformAllSky":
        return np.arange(n_sky, dtype=np.int64)
    kind = sky_mask_config["type"]
    coordsys = str(sky_mask_config.get("coordsys", "geo")).lower()
    if kind == "Patch":
        patch = sky_mask_config["patch"]
        unit = patch.get("unit", "rad")
        c_phi, c_lat = _earth_fixed(patch["center"], coordsys, "sky_mask.patch.center", unit)
        r = patch["radius"]
        radius = _angle(r, "sky_mask.patch.radius") if isinstance(r, str) else \
            float(r) * (math.pi / 180.0 if unit == "deg" else 1.0)
        if not 0.0 <= radius <= math.pi:
            raise ValueError("sky_mask.patch.radius must be within [0 deg, 180 deg]")
        cos_d = np.sin(lat) * math.sin(c_lat) + np.cos(lat) * math.cos(c_lat) * np.cos(phi - c_phi)
        return np.where(np.arccos(np.clip(cos_d, -1.0, 1.0)) <= radius)[0].astype(np.int64)
    if kind == "Fixed":
        coords = sky_mask_config["coordinates"]
        coords = coords.get("sky_loc", coords)
        f_phi, f_lat = _earth_fixed(coords, coordsys, "sky_mask.coordinates",
                                    sky_mask_config["coordinates"].get("unit", "rad"))
        if n_sky == 0:
            return np.array([], dtype=np.int64)
        cos_d = np.sin(lat) * math.sin(f_lat) + np.cos(lat) * math.cos(f_lat) * np.cos(phi - f_phi)
        return np.array([int(np.argmax(np.clip(cos_d, -1.0, 1.0)))], dtype=np.int64)
    if kind == "Custom":
        raise NotImplementedError("Custom HEALPix-map sky masks need healpy's map reader")
    raise ValueError(f"Unknown sky_mask type: {kind!r}; supported types are "
                     "UniformAllSky, Patch, Fixed, Custom")


def prepare_likelihood_inputs(config, strains, nIFO, ml=None, FP=None, FX=None, ml_big=None,
                              FP_big=None, FX_big=None, big_cluster_healpix_order=None, *,
                              device=None) -> dict:
    """Everything per segment that the per-cluster calls reuse
    (likelihood_setup.py:81-238).  With ``device`` set, ``"gpu_tables"`` holds
    the batched loop's SkyTables (FP/FX, ml, valid directions and the
    execution orders resident on that device)."""
    if config is None:
        raise ValueError("config is required")
    acor = float(getattr(config, "Acore"))
    gamma = float(getattr(config, "gamma", 0.0))
    delta = float(getattr(config, "delta", 0.0))
    net_rho = float(getattr(config, "netRHO", 0.0))
    netCC = float(getattr(config, "netCC", 0.0))
    n = int(nIFO)
    network_energy_threshold = 2 * acor * acor * n
    gamma_regulator = gamma * gamma * 2 / 3
    if delta == 0.0:
        delta = 0.00001
    delta_regulator = abs(delta) if abs(delta) < 1 else 1
    ml_a, FP_a, FX_a = build_sky_delay_and_antenna_patterns(n, strains, config, ml, FP, FX)
    n_sky = int(ml_a.shape[1])
    healpix_order = int(getattr(config, "healpix", 0)) if hasattr(config, "healpix") else None
    phi, lat = sky.build_sky_directions(n_sky, healpix_order)
    mask = getattr(config, "sky_mask", None)
    t_ref = float(strains[0].t0) if strains is not None and len(strains) and \
        hasattr(strains[0], "t0") else None
    valid = compute_sky_valid_indices(phi, lat, mask, t_ref=t_ref)

    big = {}
    if ml_big is not None and FP_big is not None and FX_big is not None:
        n_big = int(np.asarray(ml_big).shape[1])
        phi_b, lat_b = sky.build_sky_directions(n_big, big_cluster_healpix_order)
        big = dict(ml_big_cluster=np.asarray(ml_big),
                   FP_big_cluster_t=np.asarray(FP_big).T.astype(np.float32),
                   FX_big_cluster_t=np.asarray(FX_big).T.astype(np.float32),
                   n_sky_big_cluster=n_big, phi_geo_arr_big_cluster=phi_b,
                   latitude_arr_big_cluster=lat_b,
                   sky_valid_indices_big=compute_sky_valid_indices(phi_b, lat_b, mask, t_ref))
    else:
        big = dict(ml_big_cluster=None, FP_big_cluster_t=None, FX_big_cluster_t=None,
                   n_sky_big_cluster=None, phi_geo_arr_big_cluster=None,
                   latitude_arr_big_cluster=None, sky_valid_indices_big=None)

    out = {
        "network_energy_threshold": network_energy_threshold,
        "xgb_rho_mode": bool(getattr(config, "xgb_rho_mode", False)),
        "gamma_regulator": gamma_regulator,
        "delta_regulator": delta_regulator,
        "net_rho_threshold": abs(net_rho),
        "netEC_threshold": abs(net_rho) * abs(net_rho) * 2,
        "netCC": netCC,
        "ml": ml_a, "FP": FP_a, "FX": FX_a,
        "FP_t": FP_a.T.astype(np.float32), "FX_t": FX_a.T.astype(np.float32),
        "n_sky": n_sky, "healpix_order": healpix_order,
        "phi_geo_arr": phi, "latitude_arr": lat, "ra_arr": phi, "dec_arr": lat,
        "sky_mask_config": mask, "segment_start_gps": t_ref,
        "sky_valid_indices": valid,
        "big_cluster_healpix_order": big_cluster_healpix_order,
        **big,
    }
    if device is not None:
        import torch

        from .batched import SkyTables
        with torch.cuda.device(torch.device(device)):
            out["gpu_tables"] = SkyTables.from_arrays(
                out["FP_t"], out["FX_t"], ml_a, valid,
                network_energy_threshold=network_energy_threshold,
                gamma_regulator=gamma_regulator, delta_regulator=delta_regulator, netCC=netCC)
    return out


setup_likelihood = prepare_likelihood_inputs
