"""GPU sky loop against the oracle at production sky resolution.

HEALPix order 7 (196,608 directions), L1/H1/V1, K = 20: the configurations
the throughput figures are quoted on.

* one cluster of 1,000 pixels with an SNR-15 coherent signal: the whole sky
  through the plain launch, every direction compared with the oracle;
* one cluster of 3,000 pixels: REG[1] equal over the whole sky (the
  regulator's early pass/fail margins grow with the pixel count) and the
  scan on a random sky sample plus the neighbourhood of the maximum;
* 32 clusters of 20-3,000 pixels (log-spaced, so the largest is >= 2,900)
  in one batched launch over the whole sky: every cluster's REG[1] equal to
  the oracle's over the whole sky, and its maps at 2,000 random directions
  plus the 25 directions nearest its maximum within tolerance, with the
  maximum identical (or a documented near-tie).

Reference: pycwb/modules/likelihoodWP/sky_scan.py:17-192 (scan),
dpf.py:7-34 (regulator), likelihood.py:308-325 (call order).  Comparison
rules and tolerance: tests/parity.py.
"""

import math

import numpy as np
import pytest

from parity import assert_scan_close, f64_error_ratio

pytestmark = pytest.mark.gpu

ORDER = 7
K = 20
IFOS = ("L1", "H1", "V1")


@pytest.fixture(scope="module")
def sky7():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pycwb_gb300 import _lib, sky
    from pycwb_gb300.synthetic import regulators
    _lib.build()
    ml, FP, FX = sky.compute_sky_delay_and_patterns(list(IFOS), IFOS[0], 512.0, K,
                                                    healpix_order=ORDER)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    phi, lat = sky.build_sky_directions(ml.shape[1], healpix_order=ORDER)
    xyz = np.stack([np.cos(lat) * np.cos(phi), np.cos(lat) * np.sin(phi), np.sin(lat)], axis=1)
    return dict(ml=ml, FP_t=FP_t, FX_t=FX_t, reg=regulators(len(IFOS)), xyz=xyz,
                n_sky=ml.shape[1], valid=np.arange(ml.shape[1], dtype=np.int64))


def _neighbourhood(xyz, l, n=25):
    """The n directions nearest direction l (l itself included)."""
    return np.argsort(-(xyz @ xyz[l]), kind="stable")[:n]


def _sample(env, rng, around, n_random=2000):
    """Sorted valid positions: n_random random directions plus the
    neighbourhoods of the directions in `around`."""
    parts = [rng.choice(env["n_sky"], n_random, replace=False)]
    parts += [_neighbourhood(env["xyz"], int(l)) for l in around]
    return np.unique(np.concatenate(parts)).astype(np.int64)


def _restrict(out, keep):
    """The GPU's 13-tuple with every direction outside `keep` zeroed, as the
    reference leaves directions that are not valid."""
    maps = []
    for k in range(1, 12):
        m = np.zeros_like(out[k])
        m[keep] = out[k][keep]
        maps.append(m)
    return (out[0],) + tuple(maps) + (out[12],)


def _oracle_scan(oracle_mod, env, td00, td90, rms, reg1, valid):
    r = env["reg"]
    REG = np.array([r["delta_regulator"] * math.sqrt(2), reg1, 0.0], np.float32)
    args = (len(IFOS), rms.shape[0], env["n_sky"], env["FP_t"], env["FX_t"], rms, td00, td90,
            env["ml"])
    tail = (r["netCC"], r["delta_regulator"], r["network_energy_threshold"], valid)
    ref = oracle_mod.scan_sky_for_best_fit(*args, REG, *tail, return_ellipticity=True)
    f64 = oracle_mod.scan_sky_for_best_fit(*args, REG.astype(np.float64), *tail, precision="f64",
                                           return_ellipticity=True)
    return ref, f64


def _check_cluster(oracle_mod, env, got, reg_gpu, td00, td90, rms, rng, what, full_scan=False):
    r = env["reg"]
    reg1 = oracle_mod.calculate_dpf(env["FP_t"], env["FX_t"], rms, env["n_sky"], len(IFOS),
                                    r["gamma_regulator"], r["network_energy_threshold"],
                                    env["valid"])
    assert np.float32(reg_gpu) == np.float32(reg1), f"{what}: REG[1] {reg_gpu} != {reg1}"
    if full_scan:
        ref, f64 = _oracle_scan(oracle_mod, env, td00, td90, rms, reg1, env["valid"])
        cmp = got
    else:
        sub = _sample(env, rng, [got[0]])
        ref, f64 = _oracle_scan(oracle_mod, env, td00, td90, rms, reg1, sub)
        cmp = _restrict(got, sub)
        # the GPU's maximum over the whole sky is in the sample, so the
        # oracle's maximum over the sample must be it (or a near-tie)
    assert_scan_close(cmp, ref, f64, ref_cr=ref[13], netCC=r["netCC"], what=what)
    assert f64_error_ratio(cmp, ref, f64) <= 3.0, what
    return ref


def test_plain_order7_p1000_whole_sky(sky7, oracle_mod):
    """One 1,000-pixel cluster, SNR 15, every direction of the
    order-7 sky against the oracle; the selected direction identical."""
    from pycwb_gb300.likelihoodWP import sky_loop
    from pycwb_gb300.synthetic import make_cluster
    rng = np.random.default_rng(20261204)
    e = sky7
    td00, td90, rms, _ = make_cluster(rng, e["ml"], e["FP_t"], e["FX_t"], 1000, K, 15.0)
    r = e["reg"]
    REG0 = np.float32(r["delta_regulator"] * math.sqrt(2))
    reg, out = sky_loop(len(IFOS), 1000, e["n_sky"], e["FP_t"], e["FX_t"], rms, td00, td90,
                        e["ml"], REG0, r["gamma_regulator"], r["netCC"],
                        r["network_energy_threshold"], e["valid"])
    ref = _check_cluster(oracle_mod, e, out, reg, td00, td90, rms, rng, "order 7 P 1000",
                         full_scan=True)
    assert out[0] == ref[0]
    # the selected direction holds the largest statistic of the GPU's own map
    assert out[7][out[0]] == np.nanmax(out[7]) == out[12]


def test_plain_order7_p3000(sky7, oracle_mod):
    """P = 3,000: REG[1] equal over the whole sky, the scan on a sample."""
    from pycwb_gb300.likelihoodWP import sky_loop
    from pycwb_gb300.synthetic import make_cluster
    rng = np.random.default_rng(3000)
    e = sky7
    td00, td90, rms, _ = make_cluster(rng, e["ml"], e["FP_t"], e["FX_t"], 3000, K, 25.0)
    r = e["reg"]
    REG0 = np.float32(r["delta_regulator"] * math.sqrt(2))
    reg, out = sky_loop(len(IFOS), 3000, e["n_sky"], e["FP_t"], e["FX_t"], rms, td00, td90,
                        e["ml"], REG0, r["gamma_regulator"], r["netCC"],
                        r["network_energy_threshold"], e["valid"])
    _check_cluster(oracle_mod, e, out, reg, td00, td90, rms, rng, "order 7 P 3000")


def test_batched_order7_size_stratified(sky7, oracle_mod):
    """The 4,096-cluster batch in miniature: 32 clusters of 20-3,000 pixels (SNR 8-40,
    independent directions) in one batched launch over the whole order-7 sky."""
    from pycwb_gb300.likelihoodWP.batched import BatchedSkyLoop, ClusterBatch, SkyTables
    from pycwb_gb300.synthetic import make_cluster
    e = sky7
    r = e["reg"]
    rng = np.random.default_rng(32)
    sizes = np.unique(np.round(np.geomspace(20, 3000, 32)).astype(int))
    assert sizes.max() >= 2900 and sizes.size == 32
    clusters = []
    for P in rng.permutation(sizes):
        td00, td90, rms, _ = make_cluster(rng, e["ml"], e["FP_t"], e["FX_t"], int(P), K,
                                          float(rng.uniform(8, 40)))
        clusters.append((td00, td90, rms))
    tables = SkyTables.from_arrays(e["FP_t"], e["FX_t"], e["ml"], None, **{k: r[k] for k in (
        "network_energy_threshold", "gamma_regulator", "delta_regulator", "netCC")})
    loop = BatchedSkyLoop(tables, ClusterBatch.from_clusters(clusters))
    res = loop.run()
    for c, (td00, td90, rms) in enumerate(clusters):
        got = res.cluster_tuple(c)
        _check_cluster(oracle_mod, e, got, res.regulator[c], td00, td90, rms, rng,
                       f"batched cluster {c} (P={rms.shape[0]})")


def test_plain_order8_four_detectors_wide_window(oracle_mod):
    """The lag pipeline's sky and detectors: HEALPix 8 (786,432 directions),
    L1/H1/V1/K1, K = 67 (135 delays), one 800-pixel cluster: REG[1] equal
    over the whole sky, the maps on a sample plus the maximum's
    neighbourhood, the maximum identical."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pycwb_gb300 import _lib, sky
    from pycwb_gb300.likelihoodWP import sky_loop
    from pycwb_gb300.synthetic import make_cluster, regulators
    _lib.build()
    ifos = ("L1", "H1", "V1", "K1")
    K8 = 67
    ml, FP, FX = sky.compute_sky_delay_and_patterns(list(ifos), ifos[0], 2048.0, K8,
                                                    healpix_order=8)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    phi, lat = sky.build_sky_directions(ml.shape[1], healpix_order=8)
    xyz = np.stack([np.cos(lat) * np.cos(phi), np.cos(lat) * np.sin(phi), np.sin(lat)], axis=1)
    e = dict(ml=ml, FP_t=FP_t, FX_t=FX_t, reg=regulators(len(ifos)), xyz=xyz, n_sky=ml.shape[1],
             valid=np.arange(ml.shape[1], dtype=np.int64))
    rng = np.random.default_rng(88)
    td00, td90, rms, _ = make_cluster(rng, ml, FP_t, FX_t, 800, K8, 20.0)
    r = e["reg"]
    REG0 = np.float32(r["delta_regulator"] * math.sqrt(2))
    reg, out = sky_loop(len(ifos), 800, e["n_sky"], FP_t, FX_t, rms, td00, td90, ml, REG0,
                        r["gamma_regulator"], r["netCC"], r["network_energy_threshold"],
                        e["valid"])
    reg1 = oracle_mod.calculate_dpf(FP_t, FX_t, rms, e["n_sky"], len(ifos), r["gamma_regulator"],
                                    r["network_energy_threshold"], e["valid"])
    assert np.float32(reg) == np.float32(reg1)
    sub = _sample(e, rng, [out[0]])
    REG = np.array([REG0, reg1, 0.0], np.float32)
    args = (len(ifos), 800, e["n_sky"], FP_t, FX_t, rms, td00, td90, ml)
    tail = (r["netCC"], r["delta_regulator"], r["network_energy_threshold"], sub)
    ref = oracle_mod.scan_sky_for_best_fit(*args, REG, *tail, return_ellipticity=True)
    f64 = oracle_mod.scan_sky_for_best_fit(*args, REG.astype(np.float64), *tail, precision="f64",
                                           return_ellipticity=True)
    cmp = _restrict(out, sub)
    assert_scan_close(cmp, ref, f64, ref_cr=ref[13], netCC=r["netCC"], what="order 8, 4 ifo, K 67")
    assert f64_error_ratio(cmp, ref, f64) <= 3.0
