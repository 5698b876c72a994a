"""The likelihood stage at the reference's call signatures, on the GPU.

Drop-ins for pycwb/modules/likelihoodWP/likelihood.py:

* ``evaluate_fragment_clusters`` / ``likelihood_wrapper`` (:58-135): every
  surviving cluster of every lag;
* ``evaluate_cluster_likelihood`` / ``likelihood`` (:138-462): one cluster.

Both run the same path.  Per cluster, as the reference (:258-339): the
big-cluster switch bBB (a cluster with more than nRES * (precision mod
65536) pixels is scanned on the coarse sky grid, :264-283), the sky mask at
the cluster's time (:287-294), rejection of an empty mask; then, for all
clusters at once, the GPU: one batched launch of the regulator and sky scan
per distinct (grid, sky mask) -- REG[1] and the 11 sky maps of every
cluster -- the rejection of sky_stat_max <= 0 (:328-336), the statistics at
each sky maximum (:354-363, pgw_skystat_batched), the threshold cut on them
(get_likelihood_rejection_reason, :367-386) and, for the clusters it
accepts, the normalised sky probability (softmax of nSkyStat, :338-342,
pgw_sky_probability); then, on the host, the sky-localisation fields of the
cluster (:420-432).  Only accepted clusters' maps, probabilities and
per-pixel statistics leave the device; the reference computes the
probability of every cluster with sky_stat_max > 0, but a rejected
cluster's result is (None, None) either way.

The reference's remaining host post-processing of an accepted cluster --
populate_detection_statistics (waveform reconstruction, hrss),
update_chirp_mass_statistics and compute_sky_error_region (:389-418) -- is
not part of this path.  ``post`` takes it: a callable
``post(cluster, sky_statistics, skymap_statistics, context)`` run on every
accepted cluster; ``post=reference_post_processing`` calls the reference's
own functions when the pycwb package is importable, on the GPU statistics
(their per-pixel arrays come back for the accepted clusters only).

Inputs are the reference's objects, read by attribute: a cluster has
``pixel_arrays`` (``noise_rms`` (nIFO, P), ``td_amp_dense()`` (P, nIFO,
2(2K+1)), ``populate_noise_rms(nRMS)``), ``cluster_status``,
``cluster_time``, ``cluster_freq``, ``cluster_meta``; an xtalk catalog has
``get_xtalk_pixels(pixel_arrays, True) -> (lookup, rows)``; a fragment
cluster has ``clusters``.
"""

from __future__ import annotations

import hashlib
import logging
import math
import time
from dataclasses import dataclass

import numpy as np
import torch

from .. import _lib
from .batched import BatchedSkyLoop, ClusterBatch, SkyTables
from .detection_statistics import get_likelihood_rejection_reason
from .likelihood_setup import prepare_likelihood_inputs
from .pixel_data import extract_pixel_time_delay_data, scan_inputs
from .sky_mask import sky_valid_indices_for_cluster
from .sky_scan import STAT_NAMES
from .sky_statistics import SkyStatistics, pack_xtalk, statistics_batched

logger = logging.getLogger(__name__)

MAP_FIELDS = ("nAntennaPrior", "nAlignment", "nLikelihood", "nNullEnergy", "nCorrEnergy",
              "nCorrelation", "nSkyStat", "nDisbalance", "nNetIndex", "nEllipticity",
              "nPolarisation")
assert len(MAP_FIELDS) == len(STAT_NAMES)


@dataclass
class SkyMapStatistics:
    """The sky maps of one cluster (pycwb/modules/likelihoodWP/typing.py:73-98):
    l_max, the 11 per-direction float32 maps in the scan's order,
    sky_stat_max, the normalised probability map and per-stage timings."""

    l_max: int
    nAntennaPrior: np.ndarray
    nAlignment: np.ndarray
    nLikelihood: np.ndarray
    nNullEnergy: np.ndarray
    nCorrEnergy: np.ndarray
    nCorrelation: np.ndarray
    nSkyStat: np.ndarray
    nDisbalance: np.ndarray
    nNetIndex: np.ndarray
    nEllipticity: np.ndarray
    nPolarisation: np.ndarray
    sky_stat_max: float = 0
    nProbability: np.ndarray = None
    stage_timings: dict = None

    @classmethod
    def from_tuple(cls, t):
        return cls(*t)


def _skymap_class():
    """The reference's SkyMapStatistics when pycwb is importable (so callers
    that check its type see their own class), else the local one."""
    try:
        from pycwb.modules.likelihoodWP.typing import SkyMapStatistics as ref
        return ref
    except Exception:  # noqa: BLE001 - any import failure means "not available"
        return SkyMapStatistics


def is_big_cluster(config, setup, n_pixels: int) -> bool:
    """bBB of likelihood.py:264-269: csize = |precision| mod 65536, and a
    cluster of more than nRES * csize pixels uses the coarse grid when the
    setup has one."""
    precision = int(abs(getattr(config, "precision", 0) or 0))
    csize = precision % 65536
    nres = int(getattr(config, "nRES", 1) or 1)
    return csize > 0 and n_pixels > nres * csize and setup.get("ml_big_cluster") is not None


def _grid(setup, big: bool):
    """(ml, FP_t, FX_t, n_sky, phi_geo, latitude) of the main or coarse grid."""
    if big:
        return (setup["ml_big_cluster"], setup["FP_big_cluster_t"], setup["FX_big_cluster_t"],
                int(setup["n_sky_big_cluster"]), setup["phi_geo_arr_big_cluster"],
                setup["latitude_arr_big_cluster"])
    phi = setup.get("phi_geo_arr")
    lat = setup.get("latitude_arr")
    return (setup["ml"], setup["FP_t"], setup["FX_t"], int(setup["n_sky"]),
            setup["ra_arr"] if phi is None else phi, setup["dec_arr"] if lat is None else lat)


def _mask_digest(valid: np.ndarray, memo: dict | None = None) -> str:
    """Content digest of a set of valid directions.  Jobs usually share the
    setup's one array (a mask that does not depend on the event time), so
    `memo` keeps the digest per live array object: one hash per distinct
    array instead of one per cluster (1.5 MB per HEALPix-7 sky)."""
    if memo is not None:
        hit = memo.get(id(valid))
        if hit is not None and hit[0] is valid:
            return hit[1]
    d = hashlib.sha1(np.ascontiguousarray(valid, np.int64).tobytes()).hexdigest()
    if memo is not None:
        memo[id(valid)] = (valid, d)
    return d


def _tables(setup, big: bool, valid: np.ndarray, digest: str | None = None) -> SkyTables:
    """Device sky tables of one (grid, sky mask), kept in the setup dict so
    that later calls of the segment reuse them."""
    cache = setup.setdefault("_gpu_tables_by_mask", {})
    key = (bool(big), digest if digest is not None else _mask_digest(valid))
    t = cache.get(key)
    if t is None:
        ml, FP_t, FX_t, n_sky, _, _ = _grid(setup, big)
        t = SkyTables.from_arrays(np.asarray(FP_t, np.float32), np.asarray(FX_t, np.float32),
                                  np.asarray(ml, np.int32), valid,
                                  network_energy_threshold=setup["network_energy_threshold"],
                                  gamma_regulator=setup["gamma_regulator"],
                                  delta_regulator=setup["delta_regulator"], netCC=setup["netCC"])
        cache[key] = t
    return t


@dataclass
class _Job:
    """One cluster on its way through the GPU stage."""

    cluster: object
    cluster_id: int | None
    big: bool
    valid: np.ndarray
    rms: np.ndarray
    td00: np.ndarray
    td90: np.ndarray
    xtalk_lookup: np.ndarray
    xtalk_rows: np.ndarray
    timings: dict


def sky_probability(loop: BatchedSkyLoop, clusters) -> tuple[np.ndarray, np.ndarray]:
    """nProbability of the given clusters of a BatchedSkyLoop that has run
    (pgw_sky_probability on the loop's maps): float32 (n, n_sky), and per
    cluster (max nSkyStat, sum of exp, directions holding 50 % / 90 %)."""
    sel = np.ascontiguousarray(clusters, np.int32).reshape(-1)
    n_sky = loop.t.n_sky
    if sel.size == 0:
        return np.zeros((0, n_sky), np.float32), np.zeros((0, 4))
    dev = loop.stats.device
    with torch.cuda.stream(loop.stream):
        idx = torch.from_numpy(sel).to(dev, non_blocking=False)
        prob = torch.empty((sel.size, n_sky), dtype=torch.float32, device=dev)
        summ = torch.empty((sel.size, 4), dtype=torch.float64, device=dev)
    if loop.stats.shape[0] != loop.b.n_clusters:
        raise ValueError("the loop keeps no per-cluster maps")
    rc = _lib.load().pgw_sky_probability(int(sel.size), int(n_sky), loop.stats.data_ptr(),
                                         int(loop.stats.stride(0)), idx.data_ptr(),
                                         prob.data_ptr(), summ.data_ptr(),
                                         loop.stream.cuda_stream)
    _lib.check(rc, "sky_probability")
    with torch.cuda.stream(loop.stream):
        p_h = torch.empty(prob.shape, dtype=prob.dtype, pin_memory=True)
        p_h.copy_(prob, non_blocking=True)
        s_h = summ.cpu()
    loop.stream.synchronize()
    return p_h.numpy(), s_h.numpy()


def _prepare_job(nIFO, cluster, config, setup, xtalk, nRMS, cluster_id):
    """Host-side inputs of one cluster (likelihood.py:241-305), or None when
    its sky mask keeps no direction."""
    t0 = time.perf_counter()
    if nRMS is not None and len(nRMS) == nIFO:
        cluster.pixel_arrays.populate_noise_rms(nRMS)
    n_pixels = len(cluster.pixel_arrays)
    big = is_big_cluster(config, setup, n_pixels)
    if big:
        logger.info("Cluster-id=%s is big (%d px): using the coarse sky grid (%d directions)",
                    cluster_id, n_pixels, setup["n_sky_big_cluster"])
    valid = sky_valid_indices_for_cluster(setup, cluster, use_big_grid=big)
    if valid is None:
        valid = np.arange(_grid(setup, big)[3], dtype=np.int64)
    valid = np.asarray(valid, dtype=np.int64)
    if valid.size == 0:
        logger.info("Cluster-id=%s rejected: sky mask selects no grid directions", cluster_id)
        return None
    lookup, rows = xtalk.get_xtalk_pixels(cluster.pixel_arrays, True)
    noise_weights, td0, td90, _ = extract_pixel_time_delay_data(
        None, nIFO, pixel_arrays=cluster.pixel_arrays)
    rms, td00_s, td90_s = scan_inputs(noise_weights, td0, td90)
    return _Job(cluster=cluster, cluster_id=cluster_id, big=big, valid=valid, rms=rms,
                td00=td00_s, td90=td90_s,
                xtalk_lookup=np.asarray(lookup, np.int64).reshape(-1, 2),
                xtalk_rows=np.asarray(rows, np.float32).reshape(-1, 8),
                timings={"data_prep": time.perf_counter() - t0})


def _run_group(setup, jobs, big, valid, xgb_rho_mode, digest=None):
    """One batched launch for the jobs that share a (grid, sky mask).
    Returns per job (skymap statistics or None, sky statistics or None)."""
    t0 = time.perf_counter()
    tables = _tables(setup, big, valid, digest)
    batch = ClusterBatch.from_clusters([(j.td00, j.td90, j.rms) for j in jobs])
    loop = BatchedSkyLoop(tables, batch)
    res = loop.run()
    t_scan = time.perf_counter() - t0
    # sky_stat_max <= 0 rejects the cluster (likelihood.py:328-336); a cluster
    # whose directions all fail the netCC cut has sky_stat_max 0 too
    smax = np.where(res.found, res.sky_stat_max, np.float32(0.0))
    keep = np.flatnonzero(smax > 0.0)
    out = [(None, None)] * len(jobs)
    if keep.size == 0:
        return out
    n_ifo = tables.n_ifo
    # The threshold cut (likelihood.py:367-386) on the statistics at l_max,
    # before anything per direction or per pixel leaves the device: the
    # maps, probabilities and per-pixel arrays are read back for the
    # clusters it accepts only; a rejected cluster comes back as
    # (None, reason).
    reasons = {}

    def accepted(records):
        for c in keep:
            why = get_likelihood_rejection_reason(
                SkyStatistics.from_record(records[c], n_ifo), setup["network_energy_threshold"],
                setup["netEC_threshold"], net_rho_threshold=setup["net_rho_threshold"],
                xgb_rho_mode=xgb_rho_mode)
            if why:
                reasons[int(c)] = why
        return [c for c in keep if int(c) not in reasons]

    t2 = time.perf_counter()
    xt, lk = pack_xtalk([(j.xtalk_rows, j.xtalk_lookup) for j in jobs])
    stats, pixels = statistics_batched(loop, res.l_max, xt, lk, xgb_rho_mode=xgb_rho_mode,
                                       pixel_arrays=accepted)
    t_stat = time.perf_counter() - t2
    for c, why in reasons.items():
        out[c] = (None, why)
    keep = np.array([c for c in keep if int(c) not in reasons], dtype=np.int64)
    if keep.size == 0:
        return out
    t1 = time.perf_counter()
    prob, summary = sky_probability(loop, keep)
    t_prob = time.perf_counter() - t1
    cls = _skymap_class()
    # the accepted clusters' maps into page-locked memory (torch caches the
    # blocks, so repeated calls do not pay for the page locking again)
    with torch.cuda.stream(loop.stream):
        sel = loop.stats[torch.from_numpy(keep).to(loop.stats.device)]
        host = torch.empty(sel.shape, dtype=sel.dtype, pin_memory=True)
        host.copy_(sel, non_blocking=True)
    loop.stream.synchronize()
    maps = host.numpy()
    for k, c in enumerate(keep):
        sm = cls.from_tuple((int(res.l_max[c]),) + tuple(maps[k, s] for s in range(len(MAP_FIELDS)))
                            + (float(smax[c]),))
        sm.nProbability = prob[k]
        sm.stage_timings = dict(jobs[c].timings, sky_scan=t_scan / len(jobs),
                                sky_probability=t_prob / keep.size,
                                sky_statistics_at_lmax=t_stat / len(jobs))
        sm.regulator = float(res.regulator[c])
        sm.error_region = {"max_sky_stat": float(summary[k, 0]),
                           "probability_sum": float(summary[k, 1]),
                           "directions_50": int(summary[k, 2]) if summary[k, 2] == summary[k, 2] else -1,
                           "directions_90": int(summary[k, 3]) if summary[k, 3] == summary[k, 3] else -1}
        out[c] = (sm, SkyStatistics.from_record(stats[c], n_ifo, pixels[c]))
    return out


def evaluate_clusters(nIFO, clusters, config, setup, xtalk, nRMS=None, cluster_ids=None,
                      post=None, context=None):
    """The likelihood stage for many clusters at once: a list with one
    (cluster, SkyMapStatistics) or (None, None) per input cluster, the
    results of evaluate_cluster_likelihood for each."""
    clusters = list(clusters)
    ids = list(cluster_ids) if cluster_ids is not None else [None] * len(clusters)
    results = [(None, None)] * len(clusters)
    jobs = {}
    for n, (cl, cid) in enumerate(zip(clusters, ids)):
        logger.info("-> Processing cluster-id=%d|pixels=%d", int(cid) if cid is not None else -1,
                    len(cl.pixel_arrays))
        job = _prepare_job(nIFO, cl, config, setup, xtalk, nRMS, cid)
        if job is not None:
            jobs[n] = job
    # one launch per distinct (grid, sky mask)
    groups, memo = {}, {}
    for n, job in jobs.items():
        key = (job.big, _mask_digest(job.valid, memo))
        groups.setdefault(key, []).append(n)
    xgb = bool(setup["xgb_rho_mode"])
    for (big, digest), members in groups.items():
        grp = [jobs[n] for n in members]
        for n, (sm, st) in zip(members, _run_group(setup, grp, big, grp[0].valid, xgb,
                                                   digest=digest)):
            if sm is None:
                if st is None:
                    logger.info("Cluster rejected: non-positive sky_stat_max")
                else:
                    logger.debug("Cluster rejected due to threshold cuts: %s", st)
                continue
            results[n] = _finish(nIFO, jobs[n], sm, st, config, setup, post, context)
    return results


def _finish(nIFO, job, skymap, stats, config, setup, post, context):
    """Threshold cut and sky-localisation fields of one cluster
    (likelihood.py:344-386, 420-445)."""
    cl = job.cluster
    rejected = get_likelihood_rejection_reason(stats, setup["network_energy_threshold"],
                                               setup["netEC_threshold"],
                                               net_rho_threshold=setup["net_rho_threshold"],
                                               xgb_rho_mode=setup["xgb_rho_mode"])
    if rejected:
        logger.debug("Cluster rejected due to threshold cuts: %s", rejected)
        return None, None
    if post is not None:
        post(cl, stats, skymap, dict(context or {}, nIFO=nIFO, config=config, setup=setup,
                                     cluster_xtalk=job.xtalk_rows,
                                     cluster_xtalk_lookup=job.xtalk_lookup))
    ml, _, _, _, phi_arr, lat_arr = _grid(setup, job.big)
    l_max = int(skymap.l_max)
    theta = float(np.clip(np.degrees(math.pi / 2.0 - float(lat_arr[l_max])), 0.0, 180.0))
    phi = float(np.degrees(float(phi_arr[l_max]))) % 360.0
    meta = cl.cluster_meta
    meta.l_max = l_max
    meta.theta = theta
    meta.phi = phi
    if getattr(meta, "c_time", 0.0) == 0.0:
        meta.c_time = cl.cluster_time
    if getattr(meta, "c_freq", 0.0) == 0.0:
        meta.c_freq = cl.cluster_freq
    cl.sky_time_delay = [float(ml[i, l_max]) for i in range(nIFO)]
    cl.cluster_status = -1
    logger.info("   cluster-id|pixels: %5d|%d\t -> SELECTED !!!",
                int(job.cluster_id) if job.cluster_id is not None else -1, len(cl.pixel_arrays))
    return cl, skymap


def reference_post_processing(cluster, sky_statistics, skymap_statistics, context):
    """The reference's host post-processing of an accepted cluster
    (likelihood.py:389-418) from the installed pycwb package:
    populate_detection_statistics on the GPU statistics at the maximum (its
    scalars and per-pixel arrays: packets, masks, noise amplitudes),
    update_chirp_mass_statistics and compute_sky_error_region."""
    from pycwb.modules.likelihoodWP import detection_statistics as ds
    from pycwb.modules.reconstruction.getMRAwaveform import _create_wdm_set_python

    config, setup, nIFO = context["config"], context["setup"], context["nIFO"]
    ds.populate_detection_statistics(
        sky_statistics, skymap_statistics, cluster=cluster, n_ifo=nIFO, xtalk=context["xtalk"],
        network_energy_threshold=setup["network_energy_threshold"],
        xgb_rho_mode=setup["xgb_rho_mode"], config=config,
        cluster_xtalk=context["cluster_xtalk"], cluster_xtalk_lookup=context["cluster_xtalk_lookup"],
        wdm_list=_create_wdm_set_python(config))
    pat0 = getattr(config, "pattern", 10) == 0
    ds.update_chirp_mass_statistics(cluster, xgb_rho_mode=setup["xgb_rho_mode"], pat0=pat0)
    ds.compute_sky_error_region(cluster)


def _load_xtalk(MRAcatalog):
    from pycwb.modules.xtalk.type import XTalk
    return XTalk.load(MRAcatalog, dump=True)


def evaluate_cluster_likelihood(nIFO, cluster, config, MRAcatalog=None, strains=None,
                                cluster_id=None, nRMS=None, setup=None, xtalk=None,
                                supercluster_setup=None, *, post=None):
    """likelihood.py:138-462 for one cluster: (cluster, SkyMapStatistics), or
    (None, None) when the cluster is rejected.  The same validation of
    arguments as the reference (:192-226)."""
    if xtalk is None:
        if MRAcatalog is None:
            raise ValueError("likelihood(): xtalk or MRAcatalog must be provided. For "
                             "multi-cluster / multi-lag use, call evaluate_fragment_clusters() "
                             "instead.")
        xtalk = _load_xtalk(MRAcatalog)
    if setup is None:
        sc = supercluster_setup or {}
        ml = sc.get("ml_likelihood", sc.get("ml"))
        if strains is None and ml is None:
            raise ValueError("likelihood(): setup, strains, or supercluster_setup must be "
                             "provided. For multi-cluster / multi-lag use, call "
                             "evaluate_fragment_clusters() instead.")
        setup = prepare_likelihood_inputs(
            config, strains, nIFO, ml=ml, FP=sc.get("FP_likelihood", sc.get("FP")),
            FX=sc.get("FX_likelihood", sc.get("FX")), ml_big=sc.get("ml_big_cluster"),
            FP_big=sc.get("FP_big_cluster"), FX_big=sc.get("FX_big_cluster"),
            big_cluster_healpix_order=sc.get("big_cluster_healpix_order"))
    if config is None:
        raise ValueError("likelihood(): config must be provided. Without it, hrss/strain are "
                         "zero and gps_time/central_freq fall back to coarser supercluster "
                         "estimates.")
    return evaluate_clusters(nIFO, [cluster], config, setup, xtalk, nRMS=nRMS,
                             cluster_ids=[cluster_id], post=post, context={"xtalk": xtalk})[0]


def evaluate_fragment_clusters(config, fragment_clusters, strains, MRAcatalog, nRMS=None,
                               xtalk=None, *, setup=None, post=None):
    """likelihood.py:58-135: every cluster with cluster_status <= 0 of every
    lag, all of them in one GPU pass (one launch per distinct sky grid and
    mask).  Returns results[lag] = [(cluster, SkyMapStatistics), ...] of the
    accepted clusters.  ``setup`` may be given to reuse a segment's tables."""
    t0 = time.perf_counter()
    if xtalk is None:
        xtalk = _load_xtalk(MRAcatalog)
    if setup is None:
        setup = prepare_likelihood_inputs(config, strains, config.nIFO)
    todo, where = [], []
    for lag, fc in enumerate(fragment_clusters):
        for k, cl in enumerate(fc.clusters):
            if cl.cluster_status > 0:
                continue
            cl.cluster_id = k + 1
            todo.append(cl)
            where.append((lag, k + 1))
    out = evaluate_clusters(config.nIFO, todo, config, setup, xtalk, nRMS=nRMS,
                            cluster_ids=[w[1] for w in where], post=post,
                            context={"xtalk": xtalk})
    results = [[] for _ in fragment_clusters]
    for (lag, _), (cl, sm) in zip(where, out):
        if cl is not None and cl.cluster_status == -1:
            results[lag].append((cl, sm))
    logger.info("Likelihood wrapper done: %d accepted cluster(s) across %d lag(s) in %.2f s",
                sum(len(r) for r in results), len(fragment_clusters), time.perf_counter() - t0)
    return results


setup_likelihood = prepare_likelihood_inputs
likelihood = evaluate_cluster_likelihood
likelihood_wrapper = evaluate_fragment_clusters

__all__ = ["setup_likelihood", "likelihood", "likelihood_wrapper", "prepare_likelihood_inputs",
           "evaluate_cluster_likelihood", "evaluate_fragment_clusters", "evaluate_clusters",
           "reference_post_processing", "sky_probability", "SkyMapStatistics", "is_big_cluster"]
