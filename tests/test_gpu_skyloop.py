"""GPU sky loop against the oracle and the reference's golden vectors.

Every call goes through the C ABI (libpycwb_gb300.so) via the drop-in
functions pycwb_gb300.likelihoodWP.{calculate_dpf, scan_sky_for_best_fit,
sky_loop}.  Comparison rules and tolerance: tests/parity.py.
"""

import glob
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN
from parity import assert_scan_close, f64_error_ratio, stat_errors

pytestmark = pytest.mark.gpu

SKY_CASES = sorted(glob.glob(os.path.join(GOLDEN, "sky_*.npz")))


@pytest.fixture(scope="module")
def lwp():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pycwb_gb300 import _lib
    _lib.build()
    import pycwb_gb300.likelihoodWP as m
    return m


def _golden_cr(oracle_mod, z):
    out = oracle_mod.scan_sky_for_best_fit(*_golden_args(z), z["REG"], float(z["netCC"]),
                                           float(z["delta_regulator"]),
                                           float(z["network_energy_threshold"]), z["valid"],
                                           return_ellipticity=True)
    return out[13]


def _golden_f64(oracle_mod, z):
    reg = np.array([z["REG"][0], z["REG"][1], 0.0], np.float64)
    return oracle_mod.scan_sky_for_best_fit(*_golden_args(z), reg, float(z["netCC"]),
                                            float(z["delta_regulator"]),
                                            float(z["network_energy_threshold"]), z["valid"],
                                            precision="f64", return_ellipticity=True)


def _golden_args(z):
    return (int(z["n_ifo"]), int(z["n_pix"]), int(z["n_sky"]), z["FP"], z["FX"], z["rms"],
            z["td00"], z["td90"], z["ml"])


@pytest.mark.parametrize("path", SKY_CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_regulator_equals_reference(lwp, path):
    z = np.load(path)
    reg = lwp.calculate_dpf(z["FP"], z["FX"], z["rms"], int(z["n_sky"]), int(z["n_ifo"]),
                            float(z["gamma_regulator"]), float(z["network_energy_threshold"]),
                            z["valid"])
    assert np.float32(reg) == z["REG"][1]


@pytest.mark.parametrize("path", SKY_CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_scan_matches_reference(lwp, oracle_mod, path):
    z = np.load(path)
    out = lwp.scan_sky_for_best_fit(*_golden_args(z), z["REG"], float(z["netCC"]),
                                    float(z["delta_regulator"]),
                                    float(z["network_energy_threshold"]), z["valid"])
    ref = (int(z["l_max"]),) + tuple(z["stats"]) + (float(z["sky_stat_max"]),)
    f64 = _golden_f64(oracle_mod, z)
    assert out[0] == ref[0]
    assert_scan_close(out, ref, f64, ref_cr=_golden_cr(oracle_mod, z), netCC=float(z["netCC"]))
    # no less accurate against float64 than the reference's own float32 arithmetic
    assert f64_error_ratio(out, ref, f64) <= 3.0
    # directions the reference leaves at zero (masked or rejected) are zero here too
    stored_ref = np.any(z["stats"] != 0, axis=0)
    stored_gpu = np.any(np.stack(out[1:12]) != 0, axis=0)
    assert np.array_equal(stored_ref, stored_gpu)


def _shape(spec):
    from pycwb_gb300._lib import TileShape
    return None if spec is None else TileShape(*spec)


# launch shapes: (threads, lanes_per_sky, chunk_pix, stages, min_blocks, fast_math)
# fast_math: 0 / 1 the refined division and approximate square root (the
# default), -1 IEEE rounding of every division and square root
SHAPES = [None, (256, 1, 0, 3, 4, 1), (256, 2, 5, 2, 4, -1), (128, 2, 0, 4, 4, -1),
          (128, 2, 7, 3, 4, 1), (256, 1, 0, 2, 3, -1)]
SHAPE_IDS = ["default", "t256l1s3fast", "t256l2c5s2ieee", "t128l2s4ieee", "t128l2c7s3fast",
             "t256l1m3ieee"]


@pytest.mark.parametrize("spec", SHAPES, ids=SHAPE_IDS)
@pytest.mark.parametrize("path", SKY_CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_fused_sky_loop_matches_reference(lwp, oracle_mod, path, spec):
    z = np.load(path)
    reg, out = lwp.sky_loop(*_golden_args(z), z["REG"][0], float(z["gamma_regulator"]),
                            float(z["netCC"]), float(z["network_energy_threshold"]), z["valid"],
                            shape=_shape(spec))
    assert np.float32(reg) == z["REG"][1]
    ref = (int(z["l_max"]),) + tuple(z["stats"]) + (float(z["sky_stat_max"]),)
    assert_scan_close(out, ref, _golden_f64(oracle_mod, z), ref_cr=_golden_cr(oracle_mod, z),
                      netCC=float(z["netCC"]), what=f"{os.path.basename(path)} {spec}")


def _synthetic(order, n_pix, seed, ifos=("L1", "H1", "V1"), K=20, snr=15.0, netCC=0.5):
    from pycwb_gb300 import sky
    from pycwb_gb300.synthetic import make_cluster, regulators
    rng = np.random.default_rng(seed)
    ml, FP, FX = sky.compute_sky_delay_and_patterns(list(ifos), ifos[0], 512.0, K,
                                                    healpix_order=order)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    td00, td90, rms, l_true = make_cluster(rng, ml, FP_t, FX_t, n_pix, K, snr)
    reg = regulators(len(ifos), netCC=netCC)
    return dict(n_ifo=len(ifos), n_pix=n_pix, n_sky=ml.shape[1], FP=FP_t, FX=FX_t, rms=rms,
                td00=td00, td90=td90, ml=ml, reg=reg, l_true=l_true,
                valid=np.arange(ml.shape[1], dtype=np.int64))


def _oracle_loop(oracle_mod, c, with_f64=False):
    reg1 = oracle_mod.calculate_dpf(c["FP"], c["FX"], c["rms"], c["n_sky"], c["n_ifo"],
                                    c["reg"]["gamma_regulator"],
                                    c["reg"]["network_energy_threshold"], c["valid"])
    REG = np.array([c["reg"]["delta_regulator"] * math.sqrt(2), reg1, 0.0], np.float32)
    args = (c["n_ifo"], c["n_pix"], c["n_sky"], c["FP"], c["FX"], c["rms"], c["td00"],
            c["td90"], c["ml"])
    tail = (c["reg"]["netCC"], c["reg"]["delta_regulator"], c["reg"]["network_energy_threshold"],
            c["valid"])
    out = oracle_mod.scan_sky_for_best_fit(*args, REG, *tail, return_ellipticity=True)
    if not with_f64:
        return reg1, REG, out
    f64 = oracle_mod.scan_sky_for_best_fit(*args, REG.astype(np.float64), *tail, precision="f64", return_ellipticity=True)
    return reg1, REG, out, f64


@pytest.mark.parametrize("spec", SHAPES, ids=SHAPE_IDS)
@pytest.mark.parametrize("order,n_pix,ifos", [
    (4, 250, ("L1", "H1", "V1")),
    (5, 120, ("L1", "H1", "V1")),
    (4, 180, ("L1", "H1", "V1", "K1")),
    (4, 97, ("L1", "H1")),
])
def test_synthetic_cluster_matches_oracle(lwp, oracle_mod, order, n_pix, ifos, spec):
    c = _synthetic(order, n_pix, seed=100 + order * 7 + n_pix, ifos=ifos)
    reg1, REG, ref, f64 = _oracle_loop(oracle_mod, c, with_f64=True)
    args = (c["n_ifo"], c["n_pix"], c["n_sky"], c["FP"], c["FX"], c["rms"], c["td00"],
            c["td90"], c["ml"])
    reg, out = lwp.sky_loop(*args, REG[0], c["reg"]["gamma_regulator"], c["reg"]["netCC"],
                            c["reg"]["network_energy_threshold"], c["valid"], shape=_shape(spec))
    assert np.float32(reg) == np.float32(reg1)
    assert_scan_close(out, ref, f64, ref_cr=ref[13], netCC=c["reg"]["netCC"],
                      what=f"order {order} P {n_pix} {ifos} {spec}")
    # no less accurate against float64 than the reference's float32, in
    # either arithmetic
    assert f64_error_ratio(out, ref, f64) <= 3.0


def test_sky_order_does_not_change_results(lwp):
    """Scanning in tuple order (with skipped sub-threshold pixels) or in the
    given order gives identical bits."""
    c = _synthetic(4, 300, seed=9)
    args = (c["n_ifo"], c["n_pix"], c["n_sky"], c["FP"], c["FX"], c["rms"], c["td00"],
            c["td90"], c["ml"], np.float32(0.7071068), c["reg"]["gamma_regulator"],
            c["reg"]["netCC"], c["reg"]["network_energy_threshold"], c["valid"])
    r1, a = lwp.sky_loop(*args, sky_order=True)
    r2, b = lwp.sky_loop(*args, sky_order=False)
    assert r1 == r2 and a[0] == b[0] and a[12] == b[12]
    for k in range(1, 12):
        np.testing.assert_array_equal(a[k], b[k])


def test_zero_pixels_and_sky_subset(lwp, oracle_mod):
    """Empty cluster (every direction 0/0) and a scattered sky mask."""
    c = _synthetic(3, 40, seed=7)
    c["valid"] = np.sort(np.random.default_rng(1).choice(c["n_sky"], 333, replace=False))
    reg1, REG, ref, f64 = _oracle_loop(oracle_mod, c, with_f64=True)
    args = (c["n_ifo"], c["n_pix"], c["n_sky"], c["FP"], c["FX"], c["rms"], c["td00"],
            c["td90"], c["ml"])
    out = lwp.scan_sky_for_best_fit(*args, REG, c["reg"]["netCC"], c["reg"]["delta_regulator"],
                                    c["reg"]["network_energy_threshold"], c["valid"])
    assert_scan_close(out, ref, f64, ref_cr=ref[13], netCC=c["reg"]["netCC"])
    # zero pixels with netCC = 0: NaN disbalance and correlation, as the reference
    z = dict(c)
    z["n_pix"] = 0
    z["rms"] = c["rms"][:0]
    z["td00"], z["td90"] = c["td00"][:, :, :0], c["td90"][:, :, :0]
    z["reg"] = dict(c["reg"], netCC=0.0)
    reg1, REG, ref = _oracle_loop(oracle_mod, z)
    reg = lwp.calculate_dpf(z["FP"], z["FX"], z["rms"], z["n_sky"], z["n_ifo"],
                            z["reg"]["gamma_regulator"], z["reg"]["network_energy_threshold"],
                            z["valid"])
    assert np.float32(reg) == np.float32(reg1)
    out = lwp.scan_sky_for_best_fit(z["n_ifo"], 0, z["n_sky"], z["FP"], z["FX"], z["rms"],
                                    z["td00"], z["td90"], z["ml"], REG, 0.0,
                                    z["reg"]["delta_regulator"],
                                    z["reg"]["network_energy_threshold"], z["valid"])
    assert out[0] == ref[0]
    assert max(stat_errors(out[1:12], ref[1:12])) == 0.0
    assert all(np.isnan(out[k]).any() for k in (6, 7, 8))  # 0/0 correlation, statistic, disbalance


def test_shape_errors_raise_value_error(lwp):
    c = _synthetic(2, 10, seed=3)
    with pytest.raises(ValueError):
        lwp.calculate_dpf(c["FP"][:, :2], c["FX"], c["rms"], c["n_sky"], c["n_ifo"], 0.1, 12.0,
                          c["valid"])
    with pytest.raises(ValueError):
        lwp.scan_sky_for_best_fit(c["n_ifo"], c["n_pix"], c["n_sky"], c["FP"], c["FX"], c["rms"],
                                  c["td00"][:, :2], c["td90"], c["ml"], np.zeros(3, np.float32),
                                  0.5, 0.5, 12.0, c["valid"])


def test_delay_outside_window_is_reported(lwp):
    """ml + K outside [0, 2K] is detected on the device and raised, not read."""
    c = _synthetic(2, 10, seed=4)
    ml = c["ml"].copy()
    ml[1, 5] = 21  # K = 20
    with pytest.raises(RuntimeError, match="delay index"):
        lwp.scan_sky_for_best_fit(c["n_ifo"], c["n_pix"], c["n_sky"], c["FP"], c["FX"], c["rms"],
                                  c["td00"], c["td90"], ml, np.array([0.7, 5.0, 0], np.float32),
                                  0.5, 0.5, 12.0, c["valid"])


@pytest.mark.parametrize("ifos", [("L1", "H1", "V1"), ("L1", "H1"), ("L1", "H1", "V1", "K1")])
def test_regulator_count_is_exact_across_gammas(lwp, oracle_mod, ifos):
    """REG[1] equals the reference for thresholds that cut through the bulk of
    the per-direction DPF qualities (many directions near the threshold take
    the exact fallback), with degenerate pixels (equal weights, zero weights)
    and a 2-detector network whose Gram matrices are ill-conditioned."""
    from pycwb_gb300 import sky
    rng = np.random.default_rng(len(ifos) * 101)
    ml, FP, FX = sky.compute_sky_delay_and_patterns(list(ifos), ifos[0], 512.0, 20,
                                                    healpix_order=3)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    n_sky, n_ifo = FP_t.shape
    for trial in range(4):
        P = int(rng.integers(1, 200))
        rms = rng.uniform(0.2, 2.0, size=(P, n_ifo)).astype(np.float32)
        rms[: P // 5] = np.float32(1.0 / np.sqrt(n_ifo))       # equal weights
        if P > 3:
            rms[1, 0] = 0.0                                      # a dead detector
        valid = np.sort(rng.choice(n_sky, int(rng.integers(50, n_sky)), replace=False))
        for gamma in (0.02, 0.1, 0.25, 0.5, 1.0):
            ref = oracle_mod.calculate_dpf(FP_t, FX_t, rms, n_sky, n_ifo, gamma, 12.0, valid)
            got = lwp.calculate_dpf(FP_t, FX_t, rms, n_sky, n_ifo, gamma, 12.0, valid)
            assert np.float32(got) == np.float32(ref), (trial, P, gamma, got, ref)
