"""Gradient kernel of the continuous sky statistic (pgw_sky_stat_grad) and
off-grid refinement (pgw_refine_sky).

Reference: the FP64 torch re-implementation (tests/sky_stat_f64.py, pinned
to the oracle).  Tolerances: value within 1e-4 relative; gradient within
1e-3 relative of both FP64 autograd and FP64 central differences
(h = 1e-6 rad), measured against the larger gradient component with a
floor of 1e-3 of the statistic per radian; points are taken away from the
statistic's kinks (energy threshold, max(., 0) regulators, interpolation
knots), where a derivative is one-sided.
"""

import math

import numpy as np
import pytest
import torch

import sky_stat_f64 as ref64
from test_adjoint_f64 import K, clean_points

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pycwb_gb300 import _lib, sky
    from pycwb_gb300.adjoint import GradInputs, detector_geometry, grid_angles
    from pycwb_gb300.likelihoodWP.batched import BatchedSkyLoop, ClusterBatch, SkyTables
    from pycwb_gb300.synthetic import make_cluster, regulators
    _lib.build()
    ifos = ["L1", "H1", "V1"]
    ml, FP, FX = sky.compute_sky_delay_and_patterns(ifos, "L1", 512.0, K, healpix_order=4)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    rng = np.random.default_rng(5)
    clusters, ltrue = [], []
    for P, snr in ((120, 30.0), (300, 25.0), (60, 40.0)):
        td00, td90, rms, lt = make_cluster(rng, ml, FP_t, FX_t, P, K, snr)
        clusters.append((td00, td90, rms))
        ltrue.append(lt)
    r = regulators(3, netCC=0.0)
    tables = SkyTables.from_arrays(FP_t, FX_t, ml, None, **{k: r[k] for k in (
        "network_energy_threshold", "gamma_regulator", "delta_regulator", "netCC")})
    loop = BatchedSkyLoop(tables, ClusterBatch.from_clusters(clusters))
    res = loop.run()
    geom = detector_geometry(ifos, "L1", 512.0)
    theta, phi = grid_angles(ml.shape[1], 4)
    return dict(loop=loop, res=res, inp=GradInputs.from_loop(loop, geom, res.regulator),
                clusters=clusters, ltrue=ltrue, geom=geom, theta=theta, phi=phi, ml=ml)


def _ref_args(env, c):
    td00, td90, rms = env["clusters"][c]
    return (env["geom"], td00, td90, rms, K, env["loop"].t.REG0,
            float(np.float32(env["res"].regulator[c])), 12.0)


def _points(env, c):
    t = dict(theta=env["theta"], phi=env["phi"], l_true=env["ltrue"][c], geom=env["geom"])
    td00, td90, rms = env["clusters"][c]
    t.update(td00=td00, td90=td90, rms=rms)
    return clean_points(t, n=6, seed=c)


def test_gradient_matches_f64_autograd_and_differences(env):
    from pycwb_gb300.adjoint import sky_stat_grad
    n_checked = 0
    for c in range(len(env["clusters"])):
        args = _ref_args(env, c)
        pts = _points(env, c)
        if not pts:
            continue
        th = np.array([p[0] for p in pts])
        ph = np.array([p[1] for p in pts])
        out = sky_stat_grad(env["inp"], np.full(len(pts), c, np.int32), th, ph).cpu().numpy()
        for q, (a, b) in enumerate(pts):
            t = torch.tensor(a, dtype=torch.float64, requires_grad=True)
            p = torch.tensor(b, dtype=torch.float64, requires_grad=True)
            o = ref64.sky_stat(t, p, *args)
            gt, gp = (float(x) for x in torch.autograd.grad(o["statistic"], (t, p)))
            val = float(o["statistic"])
            assert abs(out[q, 0] - val) <= 1e-4 * abs(val) + 1e-6, (c, q, out[q, 0], val)
            scale = max(abs(gt), abs(gp), 1e-3 * abs(val))
            assert abs(out[q, 1] - gt) <= 1e-3 * scale, (c, q, out[q, 1], gt)
            assert abs(out[q, 2] - gp) <= 1e-3 * scale, (c, q, out[q, 2], gp)

            def f(x, y):
                return float(ref64.sky_stat(torch.tensor(x, dtype=torch.float64),
                                            torch.tensor(y, dtype=torch.float64),
                                            *args)["statistic"])
            h = 1e-6
            fd_t = (f(a + h, b) - f(a - h, b)) / (2 * h)
            fd_p = (f(a, b + h) - f(a, b - h)) / (2 * h)
            assert abs(out[q, 1] - fd_t) <= 1e-3 * scale, (c, q, out[q, 1], fd_t)
            assert abs(out[q, 2] - fd_p) <= 1e-3 * scale, (c, q, out[q, 2], fd_p)
            for k, name in ((3, "likelihood"), (4, "correlation"), (5, "ellipticity")):
                want = float(o[name])
                assert abs(out[q, k] - want) <= 1e-4 * max(abs(want), 1e-3), (name, out[q, k], want)
            n_checked += 1
    assert n_checked >= 6


def test_autograd_function_uses_the_kernel_gradient(env):
    from pycwb_gb300.adjoint import SkyStatistic, sky_stat_grad
    pts = _points(env, 0)[:3]
    th = torch.tensor([p[0] for p in pts], dtype=torch.float64, device="cuda", requires_grad=True)
    ph = torch.tensor([p[1] for p in pts], dtype=torch.float64, device="cuda", requires_grad=True)
    qc = np.zeros(len(pts), np.int32)
    s = SkyStatistic.apply(th, ph, env["inp"], qc)
    w = torch.arange(1, len(pts) + 1, dtype=torch.float64, device="cuda")
    (s * w).sum().backward()
    out = sky_stat_grad(env["inp"], qc, th.detach(), ph.detach()).cpu().numpy()
    np.testing.assert_allclose(th.grad.cpu().numpy(), w.cpu().numpy() * out[:, 1], rtol=1e-6)
    np.testing.assert_allclose(ph.grad.cpu().numpy(), w.cpu().numpy() * out[:, 2], rtol=1e-6)


def test_refinement_ascends_and_keeps_the_grid_as_fallback(env):
    from pycwb_gb300.adjoint import refine
    res = env["res"]
    r = refine(env["inp"], res.l_max, env["theta"], env["phi"], res.sky_stat_max, n_steps=10,
               healpix_order=4)
    tr = r.trace
    assert tr.shape == (len(res.l_max), 11, 3)
    assert np.all(np.diff(tr[:, :, 0], axis=1) >= 0)          # never descends
    # never worse than the grid direction under the same (continuous) statistic
    assert np.all(r.statistic >= r.start_statistic)
    kept = ~r.improved
    assert np.allclose(r.theta[kept], env["theta"][res.l_max[kept]])
    assert np.all(r.distance <= 2.0 * math.sqrt(4 * math.pi / (12 * 4 ** 4)) + 1e-12)
    assert r.improved.any()
