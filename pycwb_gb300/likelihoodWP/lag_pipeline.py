"""One lag's likelihood hot path, resident on the device from td build to sky maximum.

The reference's per-lag flow builds, for every cluster, the td-amplitude
vectors of its pixels at the cluster's WDM resolution
(pycwb/modules/likelihoodWP/pixel_batch_ops.py:150-200 through
pycwb/utils/td_vector_kernels.py:133-199), rearranges them to the scan's
(2K+1, nIFO, P) layout (likelihood.py:303-304), then runs the regulator and
the sky scan per cluster (likelihood.py:310-325).  LagPipeline keeps the
padded WDM planes and TD filters of every (resolution, detector) on the
device and, per call:

1. launches pgw_td_vecs_to_clusters once per (resolution, detector), each
   writing its pixels' amplitudes straight into the batched scan's inputs;
2. copies the per-pixel rms in (pinned host memory) and launches the batched
   regulator + sky scan (pgw_sky_loop_batched);
3. optionally refines every found cluster's sky maximum off the grid
   (pgw_refine_sky);

and only the per-cluster results come back to the host.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import torch

from .. import _device as dv
from .batched import BatchedSkyLoop, BatchResult, ClusterBatch, SkyTables


@dataclass
class LagResult:
    scan: BatchResult
    refined: object | None                       # adjoint.Refined for the found clusters
    refined_clusters: np.ndarray | None          # cluster index of each refined row
    stage_ms: dict = field(default_factory=dict)  # CUDA-event stage times when timed


class LagPipeline:
    """Device-resident td build -> batched sky loop -> refinement for one lag.

    tables: SkyTables of the network (n_ifo detectors).
    planes: {resolution key: [TDBatchInputs of detector 0..n_ifo-1]}, all of
        one resolution sharing M, n_coeffs and J.
    cluster_level: resolution key of each cluster.
    cluster_pixels: per cluster, its flat plane indices (n*(M+1)+m), shape
        (P_c,) when every detector uses the same pixels (zero lag) or
        (n_ifo, P_c) when each detector has its own (time-shifted) ones.
    rms: per cluster, the (P_c, n_ifo) normalised noise weights.
    K: delay range; the scan sees 2K+1 delays.
    geometry, healpix_order: detector geometry (adjoint.detector_geometry at
        the TD rate) and the sky grid's HEALPix order, needed for refine.
    """

    def __init__(self, tables: SkyTables, planes: dict, cluster_level, cluster_pixels, rms, K,
                 *, geometry=None, healpix_order=None, shape=None):
        n_ifo = tables.n_ifo
        self.K = int(K)
        self.tables = tables
        levels = list(cluster_level)
        pix = [np.asarray(p, np.int32) for p in cluster_pixels]
        if len(levels) != len(pix) or len(pix) != len(rms) or not pix:
            raise ValueError("cluster_level, cluster_pixels and rms need one entry per cluster")
        sizes = np.array([p.shape[-1] for p in pix], np.int64)
        for c, p in enumerate(pix):
            if p.ndim not in (1, 2) or (p.ndim == 2 and p.shape[0] != n_ifo):
                raise ValueError(f"cluster {c}: pixels must be (P,) or (n_ifo={n_ifo}, P)")
            if levels[c] not in planes:
                raise ValueError(f"cluster {c}: no planes for resolution {levels[c]!r}")
        self.batch = ClusterBatch(n_ifo, 2 * self.K + 1, sizes)
        for c in range(len(pix)):
            r = np.asarray(rms[c], np.float32)
            if r.shape != (sizes[c], n_ifo):
                raise ValueError(f"cluster {c}: rms must be ({sizes[c]}, {n_ifo})")
            p0, p1 = int(self.batch.pix_offsets[c]), int(self.batch.pix_offsets[c + 1])
            self.batch.rms[p0:p1] = torch.from_numpy(r)
        self.loop = BatchedSkyLoop(tables, self.batch, shape=shape)
        dev = self.loop.td00.device
        s = self.loop.stream

        # per resolution: resident planes/filters and the scatter lists
        self.levels = []
        with torch.cuda.stream(s):
            for key, per_ifo in planes.items():
                mine = [c for c in range(len(pix)) if levels[c] == key]
                if not mine:
                    continue
                if len(per_ifo) != n_ifo:
                    raise ValueError(f"resolution {key!r}: need planes of {n_ifo} detectors")
                t0 = per_ifo[0]
                M, nc, J = int(t0.M), int(t0.n_coeffs), int(t0.J)
                dcl = np.concatenate([np.full(sizes[c], c, np.int32) for c in mine])
                dpx = np.concatenate([np.arange(sizes[c], dtype=np.int32) for c in mine])
                src = [np.concatenate([pix[c] if pix[c].ndim == 1 else pix[c][i] for c in mine])
                       for i in range(n_ifo)]
                entry = dict(M=M, nc=nc, J=J,
                             dst_cluster=torch.from_numpy(dcl).to(dev),
                             dst_pixel=torch.from_numpy(dpx).to(dev),
                             src=[torch.from_numpy(x).to(dev) for x in src], ifo=[])
                for i, t in enumerate(per_ifo):
                    if (int(t.M), int(t.n_coeffs), int(t.J)) != (M, nc, J):
                        raise ValueError(f"resolution {key!r}: detectors disagree on M/n_coeffs/J")
                    entry["ifo"].append(tuple(dv.to_device(a, dt) for a, dt in (
                        (t.padded00, torch.float32), (t.padded90, torch.float32),
                        (t.T0, torch.float64), (t.Tx, torch.float64))))
                self.levels.append(entry)
        s.synchronize()
        self.geometry = geometry
        self.healpix_order = healpix_order
        self._angles = None

    @property
    def n_clusters(self) -> int:
        return self.batch.n_clusters

    @property
    def total_pix(self) -> int:
        return self.batch.total_pix

    @property
    def h2d_bytes(self) -> int:
        """Host -> device bytes of the scan: the rms only (the td amplitudes
        are built on the device)."""
        return 4 * self.batch.rms.numel()

    def build_td(self):
        """All td amplitudes of the lag, on the loop's stream."""
        from ..utils.td_vector_kernels import scatter_launch
        s = self.loop.stream
        for e in self.levels:
            for i, (p00, p90, T0, Tx) in enumerate(e["ifo"]):
                scatter_launch(self.loop, i, e["src"][i], e["dst_cluster"], e["dst_pixel"],
                               p00, p90, T0, Tx, e["M"], e["nc"], self.K, e["J"], s)

    def run(self, *, refine=True, n_steps=10, timed=False) -> LagResult:
        s = self.loop.stream
        s.wait_stream(torch.cuda.current_stream())
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)] if timed else None
        if timed:
            ev[0].record(s)
        self.build_td()
        if timed:
            ev[1].record(s)
        self.loop.upload(td=False)
        self.loop.launch()
        if timed:
            ev[2].record(s)
        self.loop.download()
        if timed:
            ev[3].record(s)
        s.synchronize()
        res = self.loop.results()
        refined = sel = None
        if refine:
            refined, sel = self._refine(res, n_steps)
        stage = {}
        if timed:
            ev[4].record(s)
            ev[4].synchronize()
            stage = {"td_build_ms": ev[0].elapsed_time(ev[1]),
                     "sky_loop_ms": ev[1].elapsed_time(ev[2]),
                     "refine_ms": ev[3].elapsed_time(ev[4]) if refine else 0.0}
        return LagResult(scan=res, refined=refined, refined_clusters=sel, stage_ms=stage)

    def _refine(self, res, n_steps):
        from ..adjoint import GradInputs, grid_angles, refine
        if self.geometry is None or self.healpix_order is None:
            raise ValueError("refine needs geometry and healpix_order")
        sel = np.flatnonzero(res.found)
        if sel.size == 0:
            return None, sel
        if self._angles is None:
            self._angles = grid_angles(self.tables.n_sky, self.healpix_order)
        theta, phi = self._angles
        inp = GradInputs.from_loop(self.loop, self.geometry, res.regulator)
        r = refine(inp, res.l_max[sel], theta, phi, res.sky_stat_max[sel], n_steps=n_steps,
                   healpix_order=self.healpix_order, clusters=sel)
        return r, sel
