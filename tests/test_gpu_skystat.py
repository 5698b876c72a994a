"""Statistics at the sky maximum on the GPU (pgw_skystat_batched) against
the reference's golden vectors and the oracle.

The kernel rounds every float32 operation of the per-pixel pass as the
reference does; its float64 sums run in pixel order where NumPy sums
pairwise, and dpf's sum of f^4 squares twice where NumPy calls pow, so the
statistics agree to rounding: |gpu - ref| <= 1e-4 max(|ref|, 1e-3 Em) +
1e-6 (Em sets the energy scale of the differences Dc, Lm).
"""

import glob
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CASES = sorted(glob.glob(os.path.join(GOLDEN, "skystat_*.npz")))
SCALARS = ("Gn", "Ec", "Dc", "Rc", "Eh", "Es", "Np", "Em", "Lm", "norm", "cc", "rho", "xrho",
           "Lo", "Eo")


@pytest.fixture(scope="module")
def ss():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pycwb_gb300 import _lib
    _lib.build()
    from pycwb_gb300.likelihoodWP import sky_statistics
    return sky_statistics


def _close(got, ref, em, what):
    tol = 1e-4 * max(abs(ref), 1e-3 * abs(em)) + 1e-6
    assert abs(got - ref) <= tol, (what, got, ref)


@pytest.mark.parametrize("path", CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_single_cluster_matches_reference(ss, path):
    z = np.load(path)
    n_ifo = int(z["n_ifo"])
    got = ss.compute_statistics_at_sky_position(
        int(z["sky_idx"]), n_ifo, int(z["n_pix"]), z["FP"], z["FX"], z["rms"], z["td00"],
        z["td90"], z["ml"], z["REG"], float(z["network_energy_threshold"]), z["xtalk"],
        z["xtalk_lookup"], xgb_rho_mode=bool(z["xgb_rho_mode"]))
    ref = dict(zip(SCALARS, (float(v) for v in z["scalars"])))
    for k in SCALARS:
        _close(float(getattr(got, k)), ref[k], ref["Em"], k)
    assert got.N_pix_effective == pytest.approx(float(z["N_pix_effective"]), rel=1e-6)
    s_ref = z["out_S_snr"]
    assert np.allclose(got.S_snr, s_ref, rtol=1e-5, atol=1e-7)


def test_batched_matches_oracle(ss, oracle_mod):
    from oracle import skystat_oracle
    from pycwb_gb300 import sky
    from pycwb_gb300.likelihoodWP.batched import BatchedSkyLoop, ClusterBatch, SkyTables
    from pycwb_gb300.synthetic import make_cluster, regulators
    sys_path_golden = os.path.join(os.path.dirname(__file__), "golden")
    import sys
    sys.path.insert(0, sys_path_golden)
    from make_golden import synthetic_xtalk

    ifos = ["L1", "H1", "V1"]
    rng = np.random.default_rng(7)
    ml, FP, FX = sky.compute_sky_delay_and_patterns(ifos, "L1", 512.0, 20, healpix_order=2)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    reg = regulators(3)
    tables = SkyTables.from_arrays(FP_t, FX_t, ml, None, **{k: reg[k] for k in (
        "network_energy_threshold", "gamma_regulator", "delta_regulator", "netCC")})
    sizes = [40, 1, 25, 60, 7]
    clusters, xts = [], []
    for P in sizes:
        td00, td90, rms, _ = make_cluster(rng, ml, FP_t, FX_t, P, 20, float(rng.uniform(10, 40)))
        clusters.append((td00, td90, rms))
        xts.append(synthetic_xtalk(rng, P))
    loop = BatchedSkyLoop(tables, ClusterBatch.from_clusters(clusters))
    res = loop.run()
    xt, lk = ss.pack_xtalk(xts)
    out = ss.statistics_batched(loop, res.l_max, xt, lk)
    assert out.shape == (len(sizes),) and np.all(out["status"] == 0)
    REG0 = np.float32(reg["delta_regulator"] * math.sqrt(2))
    for c, (td00, td90, rms) in enumerate(clusters):
        REG = np.array([REG0, np.float32(res.regulator[c]), 0.0], np.float32)
        ref = skystat_oracle.statistics_at_sky_position(
            int(res.l_max[c]), 3, sizes[c], FP_t, FX_t, rms, td00, td90, ml, REG,
            reg["network_energy_threshold"], xts[c][0], xts[c][1])
        for k in SCALARS:
            _close(float(out[k][c]), float(ref[k]), float(ref["Em"]), (c, k))
        assert out["n_pix"][c] == sizes[c]


def test_bad_xtalk_is_reported(ss):
    z = np.load(CASES[0])
    xt = np.array(z["xtalk"])
    # a neighbour outside the cluster, in a row of the most active pixel (rows
    # are read for pixels inside the event mask only, as in the reference)
    i = int(np.argmax(z["out_pixel_mask"]))
    assert z["out_pixel_mask"][i] > 0.5
    xt[int(z["xtalk_lookup"][i][0]), 0] = 10_000
    with pytest.raises(RuntimeError):
        ss.compute_statistics_at_sky_position(
            int(z["sky_idx"]), int(z["n_ifo"]), int(z["n_pix"]), z["FP"], z["FX"], z["rms"],
            z["td00"], z["td90"], z["ml"], z["REG"], float(z["network_energy_threshold"]), xt,
            z["xtalk_lookup"])
    with pytest.raises(ValueError):
        ss.compute_statistics_at_sky_position(
            int(z["sky_idx"]), int(z["n_ifo"]), int(z["n_pix"]), z["FP"], z["FX"], z["rms"],
            z["td00"], z["td90"], z["ml"], z["REG"], float(z["network_energy_threshold"]),
            z["xtalk"], z["xtalk_lookup"][:-1])


# per-pixel arrays: float32 quantities within float32 rounding of a few
# operations, float64 packets within 1e-6 relative of the largest entry
ARRAYS32 = ("energy_array_plus", "energy_array_cross", "pixel_mask", "gaussian_noise_correction",
            "coherent_energy", "noise_amplitude_00", "noise_amplitude_90", "f", "F")
ARRAYS64 = ("pd", "pD", "ps", "pS")


def _arr_close(got, ref, what, rtol):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    assert got.shape == ref.shape, (what, got.shape, ref.shape)
    scale = max(float(np.abs(ref).max()) if ref.size else 0.0, 1e-30)
    err = np.abs(got - ref)
    assert np.all(err <= rtol * np.maximum(np.abs(ref), 1e-3 * scale) + 1e-7), (
        what, float(err.max()), int(np.argmax(err)))


@pytest.mark.parametrize("path", CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_pixel_arrays_match_reference(ss, path):
    """The per-pixel SkyStatistics arrays (sky_statistics.py:26-262 fields)
    against the reference's own outputs for the same inputs."""
    z = np.load(path)
    n_ifo = int(z["n_ifo"])
    got = ss.compute_statistics_at_sky_position(
        int(z["sky_idx"]), n_ifo, int(z["n_pix"]), z["FP"], z["FX"], z["rms"], z["td00"],
        z["td90"], z["ml"], z["REG"], float(z["network_energy_threshold"]), z["xtalk"],
        z["xtalk_lookup"], xgb_rho_mode=bool(z["xgb_rho_mode"]))
    np.testing.assert_array_equal(got.pixel_mask, z["out_pixel_mask"])
    for k in ARRAYS32:
        _arr_close(getattr(got, k), z["out_" + k], k, 2e-5)
    for k in ARRAYS64:
        _arr_close(getattr(got, k), z["out_" + k], k, 1e-5)
    for pol in ("p00", "p90"):
        arr = getattr(got, pol + "_POL")
        assert arr.shape == (2, int(z["n_pix"]))
        _arr_close(arr[0], z[f"out_{pol}_POL_r"], pol + " r", 2e-5)
        # angles: compared where the radius is not negligible (atan2 of tiny vectors)
        r = z[f"out_{pol}_POL_r"]
        sel = r > 1e-4 * max(float(r.max()), 1e-30)
        d = np.abs(arr[1][sel] - z[f"out_{pol}_POL_a"][sel])
        d = np.minimum(d, 2 * np.pi - d)
        assert np.all(d <= 1e-4), (pol, float(d.max()) if d.size else 0.0)


def test_batched_pixel_arrays_subset(ss, oracle_mod):
    """statistics_batched with a cluster subset: only those clusters' arrays
    come back, each the same as the single-cluster call's."""
    from pycwb_gb300 import sky
    from pycwb_gb300.likelihoodWP.batched import BatchedSkyLoop, ClusterBatch, SkyTables
    from pycwb_gb300.synthetic import make_cluster, regulators
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from make_golden import synthetic_xtalk

    ifos = ["L1", "H1", "V1"]
    rng = np.random.default_rng(11)
    ml, FP, FX = sky.compute_sky_delay_and_patterns(ifos, "L1", 512.0, 20, healpix_order=2)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    reg = regulators(3)
    tables = SkyTables.from_arrays(FP_t, FX_t, ml, None, **{k: reg[k] for k in (
        "network_energy_threshold", "gamma_regulator", "delta_regulator", "netCC")})
    sizes = [30, 4, 55]
    clusters, xts = [], []
    for P in sizes:
        td00, td90, rms, _ = make_cluster(rng, ml, FP_t, FX_t, P, 20, float(rng.uniform(10, 40)))
        clusters.append((td00, td90, rms))
        xts.append(synthetic_xtalk(rng, P))
    loop = BatchedSkyLoop(tables, ClusterBatch.from_clusters(clusters))
    res = loop.run()
    xt, lk = ss.pack_xtalk(xts)
    out, pix = ss.statistics_batched(loop, res.l_max, xt, lk, pixel_arrays=[2, 0])
    assert pix[1] is None and pix[0] is not None and pix[2] is not None
    REG0 = np.float32(reg["delta_regulator"] * math.sqrt(2))
    for c in (0, 2):
        td00, td90, rms = clusters[c]
        REG = np.array([REG0, np.float32(res.regulator[c]), 0.0], np.float32)
        one = ss.compute_statistics_at_sky_position(
            int(res.l_max[c]), 3, sizes[c], FP_t, FX_t, rms, td00, td90, ml, REG,
            reg["network_energy_threshold"], xts[c][0], xts[c][1])
        for k in ARRAYS32 + ARRAYS64 + ("p00_POL", "p90_POL"):
            np.testing.assert_array_equal(pix[c][k], getattr(one, k), err_msg=f"{c} {k}")
