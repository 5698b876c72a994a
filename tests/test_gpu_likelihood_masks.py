"""likelihood_wrapper on the GPU with per-cluster sky masks and the
big-cluster coarse grid, against the oracle per cluster.

HEALPix 4 (3,072 directions) as the main grid and HEALPix 3 (768) as the
coarse grid of big clusters (likelihood.py:264-283: csize = precision mod
65536 = 20, nRES = 2, so clusters above 40 pixels go to the coarse grid),
L1/H1/V1, K = 20, and an ICRS Patch mask (a 70-degree cap around a fixed
right ascension and declination) that sky_mask.py:179-211 evaluates at each
cluster's GPS time -- segment start + cluster_time -- so clusters hours
apart see different Earth-fixed directions (likelihood.py:287-294).  For
every cluster the oracle runs the reference's per-cluster sequence
(likelihood.py:258-386) on the grid and the valid directions that cluster
gets: REG[1] (calculate_dpf over the valid directions), the scan, the
sky_stat_max <= 0 rejection, the statistics at l_max and the threshold cut.
The accepted set must be the oracle's, each accepted cluster's maps must
agree within the parity tolerance (tests/parity.py) and be zero outside its
valid directions, and its l_max must be one of them.
"""

import math
import os
import sys
from types import SimpleNamespace

import numpy as np
import pytest

from parity import assert_scan_close

pytestmark = pytest.mark.gpu

K = 20
IFOS = ["L1", "H1", "V1"]
T0 = 1.26e9


class _Pixels:
    def __init__(self, rms, td00, td90):
        self.noise_rms = (1.0 / rms.astype(np.float64)).T
        self._td = np.concatenate([np.transpose(td00, (2, 1, 0)), np.transpose(td90, (2, 1, 0))],
                                  axis=2)

    def __len__(self):
        return self.noise_rms.shape[1]

    def td_amp_dense(self):
        return self._td


class _XTalk:
    def __init__(self):
        self.by_id = {}

    def get_xtalk_pixels(self, pixels, check=True):
        rows, lookup = self.by_id[id(pixels)]
        return lookup, rows


def test_icrs_masks_and_coarse_grid_match_oracle(oracle_mod):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import skystat_oracle
    from pycwb_gb300 import _lib, sky
    from pycwb_gb300.likelihoodWP.detection_statistics import get_likelihood_rejection_reason
    from pycwb_gb300.likelihoodWP.likelihood import is_big_cluster, likelihood_wrapper
    from pycwb_gb300.likelihoodWP.likelihood_setup import prepare_likelihood_inputs
    from pycwb_gb300.likelihoodWP.pixel_data import extract_pixel_time_delay_data, scan_inputs
    from pycwb_gb300.likelihoodWP.sky_mask import sky_valid_indices_for_cluster
    from pycwb_gb300.synthetic import make_cluster
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from make_golden import synthetic_xtalk

    _lib.build()
    mask = {"type": "Patch", "coordsys": "icrs",
            "patch": {"center": {"ra": "150 deg", "dec": "-25 deg"}, "radius": "70 deg"}}
    cfg = SimpleNamespace(nIFO=3, Acore=math.sqrt(2.0), gamma=0.5, delta=0.5, netRHO=3.5,
                          netCC=0.5, healpix=4, precision=65536 * 3 + 20, nRES=2, sky_mask=mask)
    ml, FP, FX = sky.compute_sky_delay_and_patterns(IFOS, "L1", 512.0, K, healpix_order=4)
    mlb, FPb, FXb = sky.compute_sky_delay_and_patterns(IFOS, "L1", 512.0, K, healpix_order=3)
    strains = [SimpleNamespace(t0=T0) for _ in IFOS]
    setup = prepare_likelihood_inputs(cfg, strains, 3, ml=ml, FP=FP, FX=FX, ml_big=mlb,
                                      FP_big=FPb, FX_big=FXb, big_cluster_healpix_order=3)
    rng = np.random.default_rng(606)
    xtalk = _XTalk()
    clusters = []
    # (pixels, hours after the segment start): small and big clusters at
    # three sidereal positions of the mask
    for P, hours in ((30, 0.0), (80, 0.0), (25, 3.0), (120, 3.0), (35, 7.5), (60, 7.5), (18, 7.5)):
        grid = (mlb, FPb.T.astype(np.float32).copy(), FXb.T.astype(np.float32).copy()) \
            if P > 40 else (ml, setup["FP_t"], setup["FX_t"])
        td00, td90, rms, _ = make_cluster(rng, grid[0], grid[1], grid[2], P, K,
                                          float(rng.uniform(10, 40)))
        meta = SimpleNamespace(l_max=None, theta=None, phi=None, c_time=0.0, c_freq=0.0)
        cl = SimpleNamespace(pixel_arrays=_Pixels(rms, td00, td90), cluster_status=0,
                             cluster_time=3600.0 * hours + 5.0, cluster_freq=200.0,
                             cluster_meta=meta)
        xtalk.by_id[id(cl.pixel_arrays)] = synthetic_xtalk(rng, P)
        clusters.append(cl)

    # the oracle's decision per cluster on its own grid and valid directions
    expect, valids = {}, set()
    REG0 = np.float32(setup["delta_regulator"] * math.sqrt(2))
    for cl in clusters:
        w, t0, t9, _ = extract_pixel_time_delay_data(None, 3, pixel_arrays=cl.pixel_arrays)
        rms, td00, td90 = scan_inputs(w, t0, t9)
        P = rms.shape[0]
        big = is_big_cluster(cfg, setup, P)
        assert big == (P > 40)
        if big:
            mlg, FPg, FXg = (setup["ml_big_cluster"], setup["FP_big_cluster_t"],
                             setup["FX_big_cluster_t"])
        else:
            mlg, FPg, FXg = setup["ml"], setup["FP_t"], setup["FX_t"]
        n_sky = mlg.shape[1]
        valid = sky_valid_indices_for_cluster(setup, cl, use_big_grid=big)
        assert 0 < valid.size < n_sky
        valids.add((big, tuple(valid.tolist())))
        reg1 = oracle_mod.calculate_dpf(FPg, FXg, rms, n_sky, 3, setup["gamma_regulator"],
                                        setup["network_energy_threshold"], valid)
        REG = np.array([REG0, reg1, 0.0], np.float32)
        args = (3, P, n_sky, FPg, FXg, rms, td00, td90, mlg)
        tail = (setup["netCC"], setup["delta_regulator"], setup["network_energy_threshold"], valid)
        ref = oracle_mod.scan_sky_for_best_fit(*args, REG, *tail, return_ellipticity=True)
        f64 = oracle_mod.scan_sky_for_best_fit(*args, REG.astype(np.float64), *tail,
                                               precision="f64", return_ellipticity=True)
        accepted = False
        if ref[12] > 0:
            rows, lookup = xtalk.by_id[id(cl.pixel_arrays)]
            st = skystat_oracle.statistics_at_sky_position(
                ref[0], 3, P, FPg, FXg, rms, td00, td90, mlg, REG,
                setup["network_energy_threshold"], rows, lookup)
            reason = get_likelihood_rejection_reason(
                SimpleNamespace(**st), setup["network_energy_threshold"],
                setup["netEC_threshold"], setup["net_rho_threshold"], False)
            accepted = reason is None
        expect[id(cl)] = (accepted, ref, f64, valid, mlg)
    # the three cluster times give distinct masks on each grid
    assert len(valids) >= 5
    assert any(a for a, *_ in expect.values())

    results = likelihood_wrapper(cfg, [SimpleNamespace(clusters=clusters)], strains, None,
                                 xtalk=xtalk, setup=setup)
    got_ids = {id(cl) for cl, _ in results[0]}
    assert got_ids == {k for k, (a, *_) in expect.items() if a}
    for cl, sm in results[0]:
        _, ref, f64, valid, mlg = expect[id(cl)]
        out = (sm.l_max, sm.nAntennaPrior, sm.nAlignment, sm.nLikelihood, sm.nNullEnergy,
               sm.nCorrEnergy, sm.nCorrelation, sm.nSkyStat, sm.nDisbalance, sm.nNetIndex,
               sm.nEllipticity, sm.nPolarisation, sm.sky_stat_max)
        assert_scan_close(out, ref, f64, ref_cr=ref[13], netCC=setup["netCC"])
        outside = np.ones(mlg.shape[1], bool)
        outside[valid] = False
        assert not np.any(sm.nSkyStat[outside]) and not np.any(sm.nLikelihood[outside])
        assert sm.l_max in set(valid.tolist())
        assert cl.sky_time_delay == [float(mlg[i, sm.l_max]) for i in range(3)]
