"""LagPipeline: device td build -> batched sky loop -> refinement, 4 detectors.

The network is L1/H1/V1/K1 at a TD rate of 2048 Hz, where the reference's
delay range rule (K = max(TDSize * upTDF, int(max_delay * TDRate) + 1),
pycwb/modules/super_cluster_native/super_cluster.py:402-403) gives K = 67:
135 delays per detector, a pixel record three times longer than the
41-delay workloads'.  Checks:

* the device-built td amplitudes equal the oracle's batch_get_td_vecs
  rearranged to the scan's layout, bit for bit;
* the scan over them matches the oracle's scan under tests/parity.py's
  tolerance, and equals a BatchedSkyLoop run on host-built inputs exactly;
* refinement never returns a statistic below its start.
"""

import math

import numpy as np
import pytest

from parity import assert_scan_close

pytestmark = pytest.mark.gpu

IFOS = ["L1", "H1", "V1", "K1"]
RATE = 2048.0
K = 67
ORDER = 3


@pytest.fixture(scope="module")
def lag():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pycwb_gb300 import _lib, sky
    from pycwb_gb300.adjoint import detector_geometry
    from pycwb_gb300.likelihoodWP.batched import SkyTables
    from pycwb_gb300.likelihoodWP.lag_pipeline import LagPipeline
    from pycwb_gb300.synthetic import make_lag, regulators
    _lib.build()
    ml, FP, FX = sky.compute_sky_delay_and_patterns(IFOS, "L1", RATE, K, healpix_order=ORDER)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    reg = regulators(len(IFOS))
    tables = SkyTables.from_arrays(FP_t, FX_t, ml, None, **{k: reg[k] for k in (
        "network_energy_threshold", "gamma_regulator", "delta_regulator", "netCC")})
    planes, level, pixels, rms, _ = make_lag(4, IFOS, ml, FP_t, FX_t, layers=(8, 16, 32),
                                             duration=4.0, n_clusters=10, size_lo=5,
                                             size_hi=300)
    pipe = LagPipeline(tables, planes, level, pixels, rms, K,
                       geometry=detector_geometry(IFOS, "L1", RATE), healpix_order=ORDER)
    out = pipe.run(refine=True, timed=True)
    return dict(pipe=pipe, out=out, planes=planes, level=level, pixels=pixels, rms=rms,
                ml=ml, FP_t=FP_t, FX_t=FX_t, reg=reg, tables=tables)


def _host_td(oracle_mod, lag, c):
    """Cluster c's (2K+1, nIFO, P) td00/td90 from the oracle."""
    D = 2 * K + 1
    P = lag["pixels"][c].size
    td00 = np.zeros((D, len(IFOS), P), np.float32)
    td90 = np.zeros_like(td00)
    for i, t in enumerate(lag["planes"][int(lag["level"][c])]):
        v = oracle_mod.batch_get_td_vecs(lag["pixels"][c], t.padded00.cpu().numpy(),
                                         t.padded90.cpu().numpy(), t.T0.cpu().numpy(),
                                         t.Tx.cpu().numpy(), t.M, t.n_coeffs, K, t.J)
        td00[:, i, :] = v[:, :D].T
        td90[:, i, :] = v[:, D:].T
    return td00, td90


def test_device_td_equals_oracle(lag, oracle_mod):
    b = lag["pipe"].batch
    loop = lag["pipe"].loop
    td00 = loop.td00.cpu().numpy()
    td90 = loop.td90.cpu().numpy()
    for c in range(b.n_clusters):
        a, e = int(b.td_offsets[c]), int(b.td_offsets[c + 1])
        r00, r90 = _host_td(oracle_mod, lag, c)
        assert np.array_equal(td00[a:e].view(np.uint32), r00.ravel().view(np.uint32)), c
        assert np.array_equal(td90[a:e].view(np.uint32), r90.ravel().view(np.uint32)), c


def test_scan_matches_oracle_and_host_path(lag, oracle_mod):
    from pycwb_gb300.likelihoodWP.batched import BatchedSkyLoop, ClusterBatch

    res = lag["out"].scan
    reg, ml, FP_t, FX_t = lag["reg"], lag["ml"], lag["FP_t"], lag["FX_t"]
    n_sky = ml.shape[1]
    n_ifo = len(IFOS)
    valid = np.arange(n_sky, dtype=np.int64)
    REG0 = np.float32(reg["delta_regulator"] * math.sqrt(2))
    clusters = []
    for c in range(len(lag["pixels"])):
        td00, td90 = _host_td(oracle_mod, lag, c)
        rms = np.asarray(lag["rms"][c], np.float32)
        clusters.append((td00, td90, rms))
        reg1 = oracle_mod.calculate_dpf(FP_t, FX_t, rms, n_sky, n_ifo, reg["gamma_regulator"],
                                        reg["network_energy_threshold"], valid)
        assert np.float32(res.regulator[c]) == np.float32(reg1)
        REG = np.array([REG0, reg1, 0.0], np.float32)
        args = (n_ifo, rms.shape[0], n_sky, FP_t, FX_t, rms, td00, td90, ml)
        tail = (reg["netCC"], reg["delta_regulator"], reg["network_energy_threshold"], valid)
        ref = oracle_mod.scan_sky_for_best_fit(*args, REG, *tail, return_ellipticity=True)
        f64 = oracle_mod.scan_sky_for_best_fit(*args, REG.astype(np.float64), *tail,
                                               precision="f64", return_ellipticity=True)
        assert_scan_close(res.cluster_tuple(c), ref, f64, ref_cr=ref[13], netCC=reg["netCC"],
                          what=f"cluster {c} (P={rms.shape[0]}, 4 detectors, K={K})")
    host = BatchedSkyLoop(lag["tables"], ClusterBatch.from_clusters(clusters)).run()
    assert np.array_equal(host.l_max, res.l_max)
    assert np.array_equal(host.sky_stat_max.view(np.uint32), res.sky_stat_max.view(np.uint32))
    assert np.array_equal(host.maps.cpu().numpy().view(np.uint32),
                          res.maps.cpu().numpy().view(np.uint32))


def test_refinement_and_timing(lag):
    out = lag["out"]
    r = out.refined
    assert r is not None and out.refined_clusters.size == int(out.scan.found.sum())
    assert np.all(r.statistic >= r.start_statistic)
    assert set(out.stage_ms) == {"td_build_ms", "sky_loop_ms", "refine_ms"}
    assert all(v >= 0.0 for v in out.stage_ms.values())
    again = lag["pipe"].run(refine=False)       # a second run rebuilds the same inputs
    assert np.array_equal(again.scan.l_max, out.scan.l_max)
    assert np.array_equal(again.scan.sky_stat_max, out.scan.sky_stat_max)


def test_per_detector_pixel_rows(lag, oracle_mod):
    """cluster_pixels given as (n_ifo, P) rows (each detector's own, e.g.
    time-shifted, pixels): every detector's td block comes from its row."""
    from pycwb_gb300.likelihoodWP.lag_pipeline import LagPipeline
    rng = np.random.default_rng(9)
    D = 2 * K + 1
    pixels2 = []
    for c, p in enumerate(lag["pixels"]):
        M = int(lag["level"][c])
        t0 = lag["planes"][M][0]
        n_cells = (t0.padded00.shape[0] - 2 * t0.n_coeffs) * (M + 1)   # unpadded time slices
        rows = np.stack([np.roll(p, i) if i % 2 == 0 else
                         rng.choice(n_cells, size=p.size, replace=False).astype(np.int32)
                         for i in range(len(IFOS))])
        pixels2.append(rows)
    pipe = LagPipeline(lag["tables"], lag["planes"], lag["level"], pixels2, lag["rms"], K)
    pipe.build_td()
    pipe.loop.stream.synchronize()
    td00 = pipe.loop.td00.cpu().numpy()
    td90 = pipe.loop.td90.cpu().numpy()
    b = pipe.batch
    for c in range(b.n_clusters):
        P = pixels2[c].shape[1]
        a = int(b.td_offsets[c])
        blk = td00[a:a + D * len(IFOS) * P].reshape(D, len(IFOS), P)
        blk90 = td90[a:a + D * len(IFOS) * P].reshape(D, len(IFOS), P)
        for i, t in enumerate(lag["planes"][int(lag["level"][c])]):
            v = oracle_mod.batch_get_td_vecs(pixels2[c][i], t.padded00.cpu().numpy(),
                                             t.padded90.cpu().numpy(), t.T0.cpu().numpy(),
                                             t.Tx.cpu().numpy(), t.M, t.n_coeffs, K, t.J)
            assert np.array_equal(blk[:, i, :].view(np.uint32),
                                  np.ascontiguousarray(v[:, :D].T).view(np.uint32)), (c, i)
            assert np.array_equal(blk90[:, i, :].view(np.uint32),
                                  np.ascontiguousarray(v[:, D:].T).view(np.uint32)), (c, i)
