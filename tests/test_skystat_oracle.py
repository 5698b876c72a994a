"""The statistics-at-l_max oracle (oracle/skystat_oracle.py) against golden
vectors written by the reference's own compute_statistics_at_sky_position
(pycwb/modules/likelihoodWP/sky_statistics.py:26-262; tests/golden/
skystat_*.npz from tests/golden/make_golden.py, on synthetic xtalk
overlaps).  The per-pixel part comes from the C oracle, bit-exact to the
reference's sky scan; the packet part follows NumPy's rounding rules.  Every
float32 statistic equals the reference's bit for bit; the float64 packet
amplitudes may differ in the last bit where a BLAS dot product of the xtalk
overlaps sums in another order (tolerance 1e-14 of the array's scale).
"""

import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

CASES = sorted(glob.glob(os.path.join(GOLDEN, "skystat_*.npz")))
SCALARS = ("Gn", "Ec", "Dc", "Rc", "Eh", "Es", "Np", "Em", "Lm", "norm", "cc", "rho", "xrho",
           "Lo", "Eo")
ARRAYS = ("energy_array_plus", "energy_array_cross", "pixel_mask", "gaussian_noise_correction",
          "coherent_energy", "noise_amplitude_00", "noise_amplitude_90", "pd", "pD", "ps", "pS",
          "S_snr", "f", "F")


@pytest.mark.parametrize("path", CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_statistics_at_sky_position_match_reference(oracle_mod, path):
    from oracle import skystat_oracle
    z = np.load(path)
    out = skystat_oracle.statistics_at_sky_position(
        int(z["sky_idx"]), int(z["n_ifo"]), int(z["n_pix"]), z["FP"], z["FX"], z["rms"],
        z["td00"], z["td90"], z["ml"], z["REG"], float(z["network_energy_threshold"]),
        z["xtalk"], z["xtalk_lookup"], xgb_rho_mode=bool(z["xgb_rho_mode"]))
    for k, ref in zip(SCALARS, z["scalars"]):
        assert np.float32(out[k]) == np.float32(ref), (k, float(out[k]), float(ref))
    assert out["N_pix_effective"] == pytest.approx(float(z["N_pix_effective"]), rel=1e-14)
    for k in ARRAYS:
        ref = z[f"out_{k}"]
        got = np.asarray(out[k])
        assert got.shape == ref.shape and got.dtype == ref.dtype, k
        if ref.dtype == np.float32:
            assert np.array_equal(got, ref), k
        else:
            scale = max(1e-300, float(np.abs(ref).max()))
            assert np.abs(got - ref).max() <= 1e-14 * scale, k
    for k in ("p00_POL", "p90_POL"):
        for part, ref in ((0, z[f"out_{k}_r"]), (1, z[f"out_{k}_a"])):
            assert np.array_equal(np.asarray(out[k][part]), ref), k


def test_cases_cover_both_rho_modes_and_quiet_clusters():
    z = [np.load(p) for p in CASES]
    assert len(z) >= 6
    assert any(bool(x["xgb_rho_mode"]) for x in z) and any(not bool(x["xgb_rho_mode"]) for x in z)
    assert {int(x["n_ifo"]) for x in z} >= {2, 3, 4}


def test_packet_helpers_known_answers(oracle_mod):
    """The reference's own known-answer tests of the packet helpers
    (pycwb/modules/likelihoodWP/tests/test_packet_ops_contract.py:37-121),
    applied to the oracle's restatements."""
    from oracle import skystat_oracle as so
    # null packet: plain float32 differences (:37-50)
    d = np.array([[1.0, 2.0], [3.0, 4.0]], np.float32)
    D = np.array([[5.0, 6.0], [7.0, 8.0]], np.float32)
    h = np.array([[0.5, 1.0], [1.5, 2.0]], np.float32)
    H = np.array([[2.5, 3.0], [3.5, 4.0]], np.float32)
    n, N = so.null_packet(d, D, h, H)
    assert np.array_equal(n, d - h) and np.array_equal(N, D - H)
    # xtalk energy: an active pixel without neighbours contributes nothing (:53-70)
    p = np.array([[1.0, 0.5]])
    q = np.array([[2.0, 1.0]])
    assert so.xtalk_energy(p, q, np.zeros((0, 8)), np.array([[0, 0], [0, 0]]),
                           np.array([1.0, 0.0])) == 0.0
    # packet norms with every pixel masked: norms clamp at 2, SNR = q_E (:73-93)
    snr, norm, rn, qn = so.packet_norm(np.array([[1.0, 2.0]], np.float32),
                                       np.array([[3.0, 4.0]], np.float32), np.zeros((0, 8)),
                                       np.array([[0, 0], [0, 0]]), np.array([0.0, 0.0], np.float32),
                                       np.array([5.0], np.float32))
    assert np.allclose(snr, [5.0]) and np.all(norm == 2.0) and not rn.any() and not qn.any()
    # signal norms (:96-112): 2 p_E / q_E, the data norms kept
    total, snr, kept, p_norm = so.signal_norms(np.array([[0.5, 0.3]]), np.array([4.0]),
                                               np.array([3.0]), np.array([0.1, 0.0]))
    assert total > 0 and total == pytest.approx(1.5) and kept[0] == 4.0
    assert p_norm.tolist() == [[0.5, 0.0]]
