"""likelihood_wrapper / likelihood on the GPU against the oracle, per cluster.

Two lags of synthetic clusters (HEALPix 4, L1/H1/V1, K = 20, synthetic xtalk
overlaps) go through the reference-signature entry point
pycwb_gb300.likelihoodWP.likelihood.likelihood_wrapper
(pycwb/modules/likelihoodWP/likelihood.py:58-135).  For every cluster the
oracle runs the reference's per-cluster sequence (likelihood.py:258-386):
REG[1] (calculate_dpf), the scan, the sky_stat_max <= 0 rejection, the
statistics at l_max and the threshold cut.  The set of accepted clusters
must be the oracle's; for each accepted cluster the maps must agree within
the parity tolerance (tests/parity.py), nProbability must be the softmax of
the returned nSkyStat (likelihood.py:338-342, float64 arithmetic), and the
sky-localisation fields must point at l_max.
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


class _Pixels:
    def __init__(self, rms, td00, td90):
        self.noise_rms = (1.0 / rms.astype(np.float64)).T            # (nIFO, P)
        self._td = np.concatenate([np.transpose(td00, (2, 1, 0)), np.transpose(td90, (2, 1, 0))],
                                  axis=2)                            # (P, nIFO, 2(2K+1))

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


def _config():
    return SimpleNamespace(nIFO=3, Acore=math.sqrt(2.0), gamma=0.5, delta=0.5, netRHO=3.5,
                           netCC=0.5, healpix=4, precision=0, nRES=1)


def test_wrapper_matches_oracle_per_cluster(oracle_mod):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import skystat_oracle
    from pycwb_gb300 import _lib, sky
    from pycwb_gb300.likelihoodWP.detection_statistics import get_likelihood_rejection_reason
    from pycwb_gb300.likelihoodWP.likelihood import likelihood_wrapper
    from pycwb_gb300.likelihoodWP.likelihood_setup import prepare_likelihood_inputs
    from pycwb_gb300.likelihoodWP.pixel_data import extract_pixel_time_delay_data, scan_inputs
    from pycwb_gb300.synthetic import make_cluster
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from make_golden import synthetic_xtalk

    _lib.build()
    cfg = _config()
    ml, FP, FX = sky.compute_sky_delay_and_patterns(IFOS, "L1", 512.0, K, healpix_order=4)
    setup = prepare_likelihood_inputs(cfg, None, 3, ml=ml, FP=FP, FX=FX)
    FP_t, FX_t, n_sky = setup["FP_t"], setup["FX_t"], setup["n_sky"]
    rng = np.random.default_rng(404)
    xtalk = _XTalk()
    lags = []
    for sizes in ([40, 250, 3, 120], [600, 15, -30, 75]):
        cls = []
        for P in sizes:
            td00, td90, rms, _ = make_cluster(rng, ml, FP_t, FX_t, abs(P), K,
                                              float(rng.uniform(6, 40)))
            if P < 0:       # a quiet cluster: no pixel above the energy threshold anywhere
                td00, td90, P = td00 * np.float32(1e-3), td90 * np.float32(1e-3), -P
            meta = SimpleNamespace(l_max=None, theta=None, phi=None, c_time=0.0, c_freq=0.0)
            cl = SimpleNamespace(pixel_arrays=_Pixels(rms, td00, td90), cluster_status=0,
                                 cluster_time=5.0, cluster_freq=200.0, cluster_meta=meta)
            xtalk.by_id[id(cl.pixel_arrays)] = synthetic_xtalk(rng, P)
            cls.append(cl)
        lags.append(SimpleNamespace(clusters=cls))

    # the oracle's decision for every cluster, on the inputs the GPU path sees
    expect = {}
    valid = np.arange(n_sky, dtype=np.int64)
    REG0 = np.float32(setup["delta_regulator"] * math.sqrt(2))
    for lag in lags:
        for cl in lag.clusters:
            w, t0, t9, _ = extract_pixel_time_delay_data(None, 3, pixel_arrays=cl.pixel_arrays)
            rms, td00, td90 = scan_inputs(w, t0, t9)
            P = rms.shape[0]
            reg1 = oracle_mod.calculate_dpf(FP_t, FX_t, rms, n_sky, 3, setup["gamma_regulator"],
                                            setup["network_energy_threshold"], valid)
            REG = np.array([REG0, reg1, 0.0], np.float32)
            args = (3, P, n_sky, FP_t, FX_t, rms, td00, td90, ml)
            tail = (setup["netCC"], setup["delta_regulator"], setup["network_energy_threshold"],
                    valid)
            ref = oracle_mod.scan_sky_for_best_fit(*args, REG, *tail, return_ellipticity=True)
            f64 = oracle_mod.scan_sky_for_best_fit(*args, REG.astype(np.float64), *tail,
                                                   precision="f64", return_ellipticity=True)
            accepted = False
            if ref[12] > 0:
                rows, lookup = xtalk.by_id[id(cl.pixel_arrays)]
                st = skystat_oracle.statistics_at_sky_position(
                    ref[0], 3, P, FP_t, FX_t, rms, td00, td90, ml, REG,
                    setup["network_energy_threshold"], rows, lookup)
                reason = get_likelihood_rejection_reason(
                    SimpleNamespace(**st), setup["network_energy_threshold"],
                    setup["netEC_threshold"], setup["net_rho_threshold"], False)
                accepted = reason is None
            expect[id(cl)] = (accepted, ref, f64)

    n_expected = sum(a for a, _, _ in expect.values())
    assert 0 < n_expected < len(expect), "the case must accept some clusters and reject others"
    assert any(ref[12] <= 0 for _, ref, _ in expect.values()), "a sky_stat_max <= 0 case"

    results = likelihood_wrapper(cfg, lags, None, None, xtalk=xtalk, setup=setup)
    got_ids = {id(cl) for lag_res in results for cl, _ in lag_res}
    assert got_ids == {k for k, (a, _, _) in expect.items() if a}
    phi, lat = setup["phi_geo_arr"], setup["latitude_arr"]
    for lag_res in results:
        for cl, sm in lag_res:
            _, ref, f64 = expect[id(cl)]
            out = (sm.l_max, sm.nAntennaPrior, sm.nAlignment, sm.nLikelihood, sm.nNullEnergy,
                   sm.nCorrEnergy, sm.nCorrelation, sm.nSkyStat, sm.nDisbalance, sm.nNetIndex,
                   sm.nEllipticity, sm.nPolarisation, sm.sky_stat_max)
            assert_scan_close(out, ref, f64, ref_cr=ref[13], netCC=setup["netCC"])
            s = sm.nSkyStat.astype(np.float64)
            e = np.exp(s - s.max())
            np.testing.assert_allclose(sm.nProbability, (e / e.sum()).astype(np.float32),
                                       rtol=2e-6, atol=1e-30)
            l = sm.l_max
            assert cl.cluster_status == -1 and cl.cluster_meta.l_max == l
            assert cl.cluster_meta.theta == pytest.approx(math.degrees(math.pi / 2 - lat[l]))
            assert cl.cluster_meta.phi == pytest.approx(math.degrees(phi[l]) % 360.0)
            assert cl.sky_time_delay == [float(ml[i, l]) for i in range(3)]
            er = sm.error_region
            assert 1 <= er["directions_50"] <= er["directions_90"] <= n_sky
