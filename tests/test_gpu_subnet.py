"""Sub-network-cut sky loop on the GPU (pgw_subnet_sky_batched).

The kernel rounds every float32 operation as the reference does under NumPy
scalar semantics (no contraction; np.dot as float32 products summed in
float64), so its 8-tuple must equal the reference's golden vectors
(tests/golden/subnet_*.npz, written by the reference's own sub_net_cut.py)
and the oracle bit for bit, single cluster and batched.
"""

import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CASES = sorted(glob.glob(os.path.join(GOLDEN, "subnet_*.npz")))


@pytest.fixture(scope="module")
def snc():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pycwb_gb300 import _lib
    _lib.build()
    from pycwb_gb300.super_cluster import sub_net_cut
    return sub_net_cut


def _args(z):
    return (int(z["n_ifo"]), int(z["n_pix"]), int(z["n_sky"]), z["FP"], z["FX"], z["rms"],
            z["td00"], z["td90"], z["ml"], z["network_energy_threshold"], float(z["e2or"]),
            float(z["subcut"]))


@pytest.mark.parametrize("path", CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_single_cluster_equals_reference(snc, path):
    z = np.load(path)
    got = snc.optimze_sky_loc_from_td(*_args(z))
    assert np.array_equal(np.array([float(x) for x in got], np.float64), z["out"]), (got, z["out"])


@pytest.mark.parametrize("ifos,order,subcut,acore", [
    (("L1", "H1", "V1"), 3, 0.33, 1.7),
    (("L1", "H1", "V1"), 4, -1.0, 1.5),
    (("L1", "H1", "V1", "K1"), 3, 0.0, 1.7),
])
def test_batched_equals_oracle(snc, oracle_mod, ifos, order, subcut, acore):
    from pycwb_gb300 import sky
    from pycwb_gb300.synthetic import make_cluster, subnet_constants
    rng = np.random.default_rng(order * 10 + len(ifos))
    ml, FP, FX = sky.compute_sky_delay_and_patterns(list(ifos), ifos[0], 512.0, 20,
                                                    healpix_order=order)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    c = subnet_constants(len(ifos), acore=acore, subcut=subcut)
    sizes = [200, 1, 0, 37, 120, 5, 300]
    clusters = []
    for P in sizes:
        td00, td90, rms, _ = make_cluster(rng, ml, FP_t, FX_t, P, 20, float(rng.uniform(5, 40)))
        clusters.append((td00, td90, rms))
    res = snc.subnet_sky_batched(FP_t, FX_t, ml, clusters, c["network_energy_threshold"],
                                 c["e2or"], c["subcut"])
    n_sky = ml.shape[1]
    for k, (td00, td90, rms) in enumerate(clusters):
        ref = oracle_mod.optimze_sky_loc_from_td(len(ifos), rms.shape[0], n_sky, FP_t, FX_t, rms,
                                                 td00, td90, ml, c["network_energy_threshold"],
                                                 c["e2or"], c["subcut"])
        got = snc._tuple(res[k])
        assert np.array_equal(np.array([float(x) for x in got]), np.array(ref, np.float64)), \
            (k, sizes[k], got, ref)
    assert res["l_max"][2] == 0 and res["stat"][2] == 0.0   # the empty cluster


def test_delay_out_of_range_is_reported(snc):
    z = np.load(CASES[0])
    ml = np.array(z["ml"])
    ml[1, 3] = 10_000
    with pytest.raises(RuntimeError):
        snc.optimze_sky_loc_from_td(int(z["n_ifo"]), int(z["n_pix"]), int(z["n_sky"]), z["FP"],
                                    z["FX"], z["rms"], z["td00"], z["td90"], ml,
                                    z["network_energy_threshold"], float(z["e2or"]),
                                    float(z["subcut"]))
    with pytest.raises(ValueError):
        snc.optimze_sky_loc_from_td(int(z["n_ifo"]), int(z["n_pix"]) + 1, int(z["n_sky"]),
                                    z["FP"], z["FX"], z["rms"], z["td00"], z["td90"], z["ml"],
                                    z["network_energy_threshold"], float(z["e2or"]),
                                    float(z["subcut"]))
