"""Sky statistic at continuous directions, its gradient, and refinement.

The grid scan gives the best HEALPix direction; here the statistic (the
reference's likelihood x network correlation, sky_scan.py:139-140) is
evaluated at any (theta, phi) with F+/Fx from the detector response tensors
and delays interpolated linearly between td samples, together with its
gradient (pgw_sky_stat_grad: dual-number tangents through the pipeline, in
the same kernel pass).  ``SkyStatistic`` exposes it to torch autograd;
``refine`` runs gradient ascent from each cluster's grid maximum
(pgw_refine_sky) and keeps the grid result when refinement does not improve
on it.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _device as dv
from . import _lib
from .sky import C_LIGHT, DetectorSite, build_sky_directions

N_OUT = 8
OUT_NAMES = ("statistic", "d_theta", "d_phi", "likelihood", "correlation", "ellipticity",
             "coherent_energy", "null_energy")


def detector_geometry(ifos, ref_ifo, sample_rate) -> np.ndarray:
    """(n_ifo, 12) float32: response tensor (row major) and baseline in TD samples.

    The baseline b_i = (R_i - R_ref) / c * rate makes tau_i = n . b_i the
    continuous form of the delay index of detector.py:1310-1321."""
    dets = [DetectorSite(d) if isinstance(d, str) else d for d in ifos]
    ref = next((d for d in dets if d.name == ref_ifo), dets[0])
    g = np.zeros((len(dets), 12), np.float64)
    for i, d in enumerate(dets):
        g[i, :9] = d.response.reshape(-1)
        g[i, 9:] = (d.vertex - ref.vertex) / C_LIGHT * float(sample_rate)
    return g.astype(np.float32)


def grid_angles(n_sky, healpix_order):
    """(theta, phi) of every grid direction: colatitude and Earth-fixed longitude."""
    phi, lat = build_sky_directions(n_sky, healpix_order)
    return np.pi / 2.0 - lat, phi


@dataclass
class GradInputs:
    """Device views of a batch (as BatchedSkyLoop holds them) + geometry."""
    n_ifo: int
    n_delay: int
    pix_off: torch.Tensor
    td_off: torch.Tensor
    rms: torch.Tensor
    td00: torch.Tensor
    td90: torch.Tensor
    geom: torch.Tensor
    REG0: float
    reg1: torch.Tensor          # float32 per cluster
    network_energy_threshold: float

    @classmethod
    def from_loop(cls, loop, geometry, regulators=None):
        """From a BatchedSkyLoop that has run (its REG[1] per cluster)."""
        if regulators is None:
            res = loop.results()
            regulators = res.regulator
        reg1 = torch.tensor(np.asarray(regulators, np.float32), device=loop.td00.device)
        return cls(n_ifo=loop.b.n_ifo, n_delay=loop.b.n_delay, pix_off=loop.pix_off,
                   td_off=loop.td_off, rms=loop.rms, td00=loop.td00, td90=loop.td90,
                   geom=dv.to_device(geometry, torch.float32), REG0=loop.t.REG0, reg1=reg1,
                   network_energy_threshold=loop.t.network_energy_threshold)


def sky_stat_grad(inp: GradInputs, query_cluster, theta, phi) -> torch.Tensor:
    """(n_queries, 8) float32 on the device (see OUT_NAMES)."""
    L = _lib.load()
    s = dv.begin()
    qc = dv.to_device(query_cluster, torch.int32)
    th = dv.to_device(theta, torch.float64)
    ph = dv.to_device(phi, torch.float64)
    n = int(qc.numel())
    with torch.cuda.stream(s):
        out = torch.empty((n, N_OUT), dtype=torch.float32, device=qc.device)
    rc = L.pgw_sky_stat_grad(inp.n_ifo, n, qc.data_ptr(), th.data_ptr(), ph.data_ptr(),
                             inp.pix_off.data_ptr(), inp.td_off.data_ptr(), inp.rms.data_ptr(),
                             inp.td00.data_ptr(), inp.td90.data_ptr(), inp.n_delay,
                             inp.geom.data_ptr(), inp.REG0, inp.reg1.data_ptr(),
                             inp.network_energy_threshold, out.data_ptr(), s.cuda_stream)
    _lib.check(rc, "sky_stat_grad")
    dv.end(s, out)
    return out


class SkyStatistic(torch.autograd.Function):
    """statistic(theta, phi) of each query's cluster; backward uses the
    kernel's exact gradient (computed in the forward pass)."""

    @staticmethod
    def forward(ctx, theta, phi, inp, query_cluster):
        out = sky_stat_grad(inp, query_cluster, theta.detach(), phi.detach())
        ctx.save_for_backward(out[:, 1].to(theta.dtype), out[:, 2].to(phi.dtype))
        return out[:, 0].to(theta.dtype)

    @staticmethod
    def backward(ctx, grad):
        gt, gp = ctx.saved_tensors
        return grad * gt, grad * gp, None, None


@dataclass
class Refined:
    theta: np.ndarray        # refined direction, or the grid direction where refinement failed
    phi: np.ndarray
    statistic: np.ndarray    # continuous statistic at the returned direction
    start_statistic: np.ndarray  # continuous statistic at the grid maximum
    grid_statistic: np.ndarray   # the grid scan's sky_stat_max (reported detection statistic)
    improved: np.ndarray     # bool: refinement moved to a better direction near the grid cell
    distance: np.ndarray     # arc between the grid direction and the refined one (radians)
    trace: np.ndarray        # (n, n_steps + 1, 3) statistic, theta, phi


def _arc(t1, p1, t2, p2):
    c = np.cos(t1) * np.cos(t2) + np.sin(t1) * np.sin(t2) * np.cos(p1 - p2)
    return np.arccos(np.clip(c, -1.0, 1.0))


def refine(inp: GradInputs, l_max, grid_theta, grid_phi, grid_stat, n_steps=10,
           step0=None, healpix_order=7, clusters=None, max_cells=2.0):
    """Off-grid refinement of each cluster's grid maximum.

    Gradient ascent on the continuous statistic starts at the grid maximum
    l_max.  The grid result is the fallback and the arbiter: the refined
    direction is kept only if its statistic beats the continuous statistic
    at the grid direction and it lies within `max_cells` grid spacings of
    it; otherwise the grid direction is returned.  The grid scan's
    sky_stat_max stays the detection statistic (`grid_statistic`).
    `clusters` maps each query to its cluster in the batch (default: query
    i is cluster i)."""
    L = _lib.load()
    s = dv.begin()
    n = len(l_max)
    spacing = math.sqrt(4 * math.pi / (12 * 4 ** healpix_order))
    if step0 is None:
        step0 = 0.5 * spacing
    th0 = np.asarray(grid_theta, np.float64)[np.asarray(l_max)]
    ph0 = np.asarray(grid_phi, np.float64)[np.asarray(l_max)]
    dev = inp.td00.device
    with torch.cuda.stream(s):
        qc = (torch.arange(n, dtype=torch.int32, device=dev) if clusters is None else
              torch.as_tensor(np.asarray(clusters, np.int32)).to(dev))
        t0 = torch.from_numpy(th0).to(dev)
        p0 = torch.from_numpy(ph0).to(dev)
        to = torch.empty(n, dtype=torch.float64, device=dev)
        po = torch.empty(n, dtype=torch.float64, device=dev)
        out = torch.empty((n, N_OUT), dtype=torch.float32, device=dev)
        tr = torch.empty((n, n_steps + 1, 3), dtype=torch.float32, device=dev)
    rc = L.pgw_refine_sky(inp.n_ifo, n, qc.data_ptr(), t0.data_ptr(), p0.data_ptr(),
                          inp.pix_off.data_ptr(), inp.td_off.data_ptr(), inp.rms.data_ptr(),
                          inp.td00.data_ptr(), inp.td90.data_ptr(), inp.n_delay,
                          inp.geom.data_ptr(), inp.REG0, inp.reg1.data_ptr(),
                          inp.network_energy_threshold, int(n_steps), float(step0),
                          to.data_ptr(), po.data_ptr(), out.data_ptr(), tr.data_ptr(),
                          s.cuda_stream)
    _lib.check(rc, "refine_sky")
    with torch.cuda.stream(s):
        o = out.cpu().numpy()
        tt, pp, trace = to.cpu().numpy(), po.cpu().numpy(), tr.cpu().numpy()
    start = trace[:, 0, 0].astype(np.float64)
    dist = _arc(th0, ph0, tt, pp)
    improved = (o[:, 0] > start) & (dist <= max_cells * spacing)
    return Refined(theta=np.where(improved, tt, th0), phi=np.where(improved, pp, ph0),
                   statistic=np.where(improved, o[:, 0], start), start_statistic=start,
                   grid_statistic=np.asarray(grid_stat, np.float64), improved=improved,
                   distance=np.where(improved, dist, 0.0), trace=trace)
