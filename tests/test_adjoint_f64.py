"""The FP64 reference of the continuous sky statistic (tests/sky_stat_f64.py).

Pinned to the oracle: fed the grid's F+/Fx and integer-delay data of a grid
direction, its pipeline reproduces the oracle's float64 scan outputs of that
direction.  Its autograd gradient agrees with central finite differences
(h = 1e-6 rad) at points away from the statistic's kinks.
"""

import math

import numpy as np
import pytest
import torch

import sky_stat_f64 as ref64

K = 20


@pytest.fixture(scope="module")
def case():
    from pycwb_gb300 import sky
    from pycwb_gb300.adjoint import detector_geometry, grid_angles
    from pycwb_gb300.synthetic import make_cluster, regulators
    ifos = ["L1", "H1", "V1"]
    ml, FP, FX = sky.compute_sky_delay_and_patterns(ifos, "L1", 512.0, K, healpix_order=4)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    td00, td90, rms, l_true = make_cluster(np.random.default_rng(5), ml, FP_t, FX_t, 120, K, 30.0)
    r = regulators(3, netCC=0.0)
    theta, phi = grid_angles(ml.shape[1], 4)
    return dict(ml=ml, FP_t=FP_t, FX_t=FX_t, td00=td00, td90=td90, rms=rms, l_true=l_true,
                reg=r, geom=detector_geometry(ifos, "L1", 512.0), theta=theta, phi=phi)


def test_pipeline_matches_oracle_f64_on_grid(case, oracle_mod):
    c = case
    n_sky = c["ml"].shape[1]
    rr, RR = 0.5 * math.sqrt(2), 14.0
    valid = np.arange(n_sky, dtype=np.int64)
    out = oracle_mod.scan_sky_for_best_fit(3, c["rms"].shape[0], n_sky, c["FP_t"], c["FX_t"],
                                           c["rms"], c["td00"], c["td90"], c["ml"],
                                           np.array([rr, RR, 0.0]), 0.0, 0.5, 12.0, valid,
                                           precision="f64")
    names = {"statistic": 7, "likelihood": 3, "correlation": 6, "ellipticity": 10,
             "coherent_energy": 5, "null_energy": 4}
    for l in list(range(0, n_sky, 97)) + [c["l_true"]]:
        rows = c["ml"][:, l] + K
        v00 = torch.tensor(c["td00"][rows, np.arange(3)], dtype=torch.float64)
        v90 = torch.tensor(c["td90"][rows, np.arange(3)], dtype=torch.float64)
        acc = ref64.pipeline(torch.tensor(c["FP_t"][l], dtype=torch.float64),
                             torch.tensor(c["FX_t"][l], dtype=torch.float64), c["rms"], v00, v90,
                             rr, RR, 12.0)
        t = ref64.tail(acc, 3)
        for name, k in names.items():
            want = out[k][l]
            got = float(t[name])
            if math.isnan(want):
                assert math.isnan(got)
            else:
                assert abs(got - want) <= 1e-9 * max(abs(want), 1e-6), (l, name, got, want)


def clean_points(c, n=8, seed=0, spread=0.02, margin=1e-3):
    """Directions near the injected one whose margins to every kink exceed `margin`."""
    rng = np.random.default_rng(seed)
    th0, ph0 = c["theta"][c["l_true"]], c["phi"][c["l_true"]]
    pts = []
    for _ in range(400):
        th = float(np.clip(th0 + rng.normal(0, spread), 0.05, math.pi - 0.05))
        ph = float(ph0 + rng.normal(0, spread))
        o = ref64.sky_stat(torch.tensor(th, dtype=torch.float64), torch.tensor(ph, dtype=torch.float64),
                           c["geom"], c["td00"], c["td90"], c["rms"], K, 0.5 * math.sqrt(2), 14.0,
                           12.0)
        if min(o["margins"].values()) > margin and abs(float(o["statistic"])) > 1e-3:
            pts.append((th, ph))
        if len(pts) == n:
            break
    return pts


def test_f64_autograd_matches_central_differences(case):
    c = case
    pts = clean_points(c, n=6)
    assert len(pts) >= 3
    h = 1e-6
    args = (c["geom"], c["td00"], c["td90"], c["rms"], K, 0.5 * math.sqrt(2), 14.0, 12.0)
    for th, ph in pts:
        t = torch.tensor(th, dtype=torch.float64, requires_grad=True)
        p = torch.tensor(ph, dtype=torch.float64, requires_grad=True)
        s = ref64.sky_stat(t, p, *args)["statistic"]
        gt, gp = torch.autograd.grad(s, (t, p))

        def f(a, b):
            return float(ref64.sky_stat(torch.tensor(a, dtype=torch.float64),
                                        torch.tensor(b, dtype=torch.float64), *args)["statistic"])
        fd_t = (f(th + h, ph) - f(th - h, ph)) / (2 * h)
        fd_p = (f(th, ph + h) - f(th, ph - h)) / (2 * h)
        scale = max(abs(float(gt)), abs(float(gp)), 1e-3 * abs(float(s)))
        assert abs(float(gt) - fd_t) <= 1e-5 * scale, (th, ph, float(gt), fd_t)
        assert abs(float(gp) - fd_p) <= 1e-5 * scale, (th, ph, float(gp), fd_p)
