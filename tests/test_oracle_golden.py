"""The CPU oracle against golden vectors produced by PycWB's own kernels.

tests/golden/*.npz were written by tests/golden/make_golden.py, which runs
the reference's dpf.py, sky_stat.py, sky_scan.py and td_vector_kernels.py
unmodified.  The oracle restates that arithmetic operation for operation,
so the comparison is exact: identical float32 bits in every per-sky array,
the same l_max and sky_stat_max, and REG[1] equal after the reference's own
float32 store (likelihood.py:258,310).
"""

import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

SKY_CASES = sorted(glob.glob(os.path.join(GOLDEN, "sky_*.npz")))
TD_CASES = sorted(glob.glob(os.path.join(GOLDEN, "td_*.npz")))


def _same_bits(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("path", SKY_CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_regulator_matches_reference(oracle_mod, path):
    z = np.load(path)
    reg1 = oracle_mod.calculate_dpf(z["FP"], z["FX"], z["rms"], int(z["n_sky"]), int(z["n_ifo"]),
                                    float(z["gamma_regulator"]),
                                    float(z["network_energy_threshold"]), z["valid"])
    assert np.float32(reg1) == z["REG"][1]


@pytest.mark.parametrize("path", SKY_CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_scan_matches_reference_bit_for_bit(oracle_mod, path):
    z = np.load(path)
    out = oracle_mod.scan_sky_for_best_fit(
        int(z["n_ifo"]), int(z["n_pix"]), int(z["n_sky"]), z["FP"], z["FX"], z["rms"],
        z["td00"], z["td90"], z["ml"], z["REG"], float(z["netCC"]), float(z["delta_regulator"]),
        float(z["network_energy_threshold"]), z["valid"])
    assert out[0] == int(z["l_max"])
    assert out[12] == float(z["sky_stat_max"])
    for k in range(11):
        assert _same_bits(out[1 + k], z["stats"][k]), f"stat {k} differs"


@pytest.mark.parametrize("path", TD_CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_td_vectors_match_reference_bit_for_bit(oracle_mod, path):
    z = np.load(path)
    out = oracle_mod.batch_get_td_vecs(z["pixel_indices"], z["padded00"], z["padded90"], z["T0"],
                                       z["Tx"], int(z["M"]), int(z["n_coeffs"]), int(z["K"]),
                                       int(z["J"]))
    assert _same_bits(out, z["out"])


def test_f64_yardstick_is_close_to_reference(oracle_mod):
    """The FP64 loop agrees with the float32 reference to float32 accuracy."""
    z = np.load(os.path.join(GOLDEN, "sky_hlv_o2_p40.npz"))
    reg = np.array([z["REG"][0], z["REG"][1], 0.0], np.float64)
    out = oracle_mod.scan_sky_for_best_fit(
        int(z["n_ifo"]), int(z["n_pix"]), int(z["n_sky"]), z["FP"], z["FX"], z["rms"],
        z["td00"], z["td90"], z["ml"], reg, float(z["netCC"]), float(z["delta_regulator"]),
        float(z["network_energy_threshold"]), z["valid"], precision="f64")
    assert out[0] == int(z["l_max"])
    lik = z["stats"][2]
    sel = np.abs(lik) > 1.0
    np.testing.assert_allclose(out[3][sel], lik[sel], rtol=1e-4)


def test_golden_edge_cases_are_present():
    """The fixtures cover the edge cases the reference's tests exercise."""
    names = {os.path.basename(p) for p in SKY_CASES}
    assert "sky_hlv_o2_p40_netcc09.npz" in names       # every direction rejected: l_max=valid[0]
    assert "sky_hlv_o3_p24_subset.npz" in names        # sky mask (sky_valid_indices subset)
    assert "sky_hlv_o2_p1.npz" in names                # one pixel, directions with no pixel above E_thr
    z = np.load(os.path.join(GOLDEN, "sky_hlv_o2_p40_netcc09.npz"))
    assert int(z["l_max"]) == int(z["valid"][0]) and float(z["sky_stat_max"]) == 0.0
    z = np.load(os.path.join(GOLDEN, "sky_hlv_o2_p1.npz"))
    assert np.isnan(z["stats"][5]).any()                # 0/0 correlation where no pixel passes


SUBNET_CASES = sorted(glob.glob(os.path.join(GOLDEN, "subnet_*.npz")))


@pytest.mark.parametrize("path", SUBNET_CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_subnet_sky_loop_matches_reference_exactly(oracle_mod, path):
    """optimze_sky_loc_from_td (sub_net_cut.py:404-517): the oracle returns
    the reference's 8-tuple with identical float32 values."""
    z = np.load(path)
    got = oracle_mod.optimze_sky_loc_from_td(
        int(z["n_ifo"]), int(z["n_pix"]), int(z["n_sky"]), z["FP"], z["FX"], z["rms"],
        z["td00"], z["td90"], z["ml"], z["network_energy_threshold"], float(z["e2or"]),
        float(z["subcut"]))
    assert np.array_equal(np.array(got, np.float64), z["out"])


def test_subnet_golden_cover_the_gates():
    outs = {os.path.basename(p)[7:-4]: np.load(p) for p in SUBNET_CASES}
    assert len(outs) >= 7
    assert any(float(z["subcut"]) < 0 for z in outs.values())     # sky gate off
    assert any(int(z["n_ifo"]) == 4 for z in outs.values())
    assert any(int(z["n_ifo"]) == 2 for z in outs.values())
    assert any(float(z["out"][1]) == 0.0 for z in outs.values())  # no direction qualified
