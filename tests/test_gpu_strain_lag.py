"""A lag from strain to sky maximum on the GPU: WDM transform (T2) -> td
build (T1) -> batched regulator + scan, 4 detectors.

White noise with sine-Gaussian and Gaussian-pulse injections from known grid
directions (pycwb_gb300.synthetic.make_strain_lag); the clusters around
loud injections must be located at (or next to) their injected direction.
The same chain on the CPU oracle (oracle transform, the reference's td
amplitudes and sky scan) finds the injected grid direction exactly at
network SNR 40, and the antipode when the arrival-time convention is
reversed, so this test checks the device WDM transform and TD filters
against the physics the rest of the path assumes.
"""

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

IFOS = ["L1", "H1", "V1", "K1"]
RATE = 512.0
TD_RATE = 2048.0
K = 67
ORDER = 4


@pytest.fixture(scope="module")
def lag():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pycwb_gb300 import _lib, sky
    from pycwb_gb300.likelihoodWP.batched import SkyTables
    from pycwb_gb300.likelihoodWP.lag_pipeline import LagPipeline
    from pycwb_gb300.synthetic import make_strain_lag, regulators
    _lib.build()
    ml, FP, FX = sky.compute_sky_delay_and_patterns(IFOS, "L1", TD_RATE, K, healpix_order=ORDER)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    reg = regulators(len(IFOS))
    tables = SkyTables.from_arrays(FP_t, FX_t, ml, None, **{k: reg[k] for k in (
        "network_energy_threshold", "gamma_regulator", "delta_regulator", "netCC")})
    planes, level, pixels, rms, l_true, info = make_strain_lag(
        11, IFOS, ml, FP_t, FX_t, TD_RATE, layers=(16, 32, 64), duration=64.0, rate=RATE,
        n_inj=8, n_clusters=12, size_lo=50, size_hi=300, snr_lo=30.0, snr_hi=40.0)
    pipe = LagPipeline(tables, planes, level, pixels, rms, K)
    out = pipe.run(refine=False)
    phi, lat = sky.build_sky_directions(ml.shape[1], ORDER)
    vec = np.stack([np.cos(lat) * np.cos(phi), np.cos(lat) * np.sin(phi), np.sin(lat)], 1)
    return dict(out=out, l_true=l_true, vec=vec, info=info, pipe=pipe)


def test_injections_are_located(lag):
    res = lag["out"].scan
    inj = np.flatnonzero(lag["l_true"] >= 0)
    assert inj.size == 8 and res.found[inj].all()
    v = lag["vec"]
    ang = np.degrees(np.arccos(np.clip(np.einsum("ij,ij->i", v[res.l_max[inj]],
                                                 v[lag["l_true"][inj]]), -1.0, 1.0)))
    # HEALPix 4 directions are ~3.7 degrees apart
    assert np.median(ang) <= 4.0, ang
    assert np.sum(ang <= 10.0) >= 6, ang


def test_injection_statistic_above_noise(lag):
    res = lag["out"].scan
    inj = lag["l_true"] >= 0
    noise = ~inj
    assert np.median(res.sky_stat_max[inj]) > 2.0 * np.median(res.sky_stat_max[noise])
    assert lag["info"]["t2w_ms"] > 0.0
