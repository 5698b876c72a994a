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

Sky masks: ``sky_mask.compute_sky_valid_indices`` (UniformAllSky, Patch,
Fixed and Custom HEALPix maps in geo, cwb or ICRS coordinates), evaluated
at the segment start; ICRS masks are evaluated again per cluster at the
cluster's time by ``sky_mask.sky_valid_indices_for_cluster``.
"""

from __future__ import annotations

import numpy as np

from .. import sky
from .pixel_data import build_sky_delay_and_antenna_patterns
from .sky_mask import compute_sky_valid_indices, sky_valid_indices_for_cluster  # noqa: F401


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
