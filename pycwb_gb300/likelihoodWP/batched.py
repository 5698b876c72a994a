"""Batched sky loop: thousands of clusters of one segment in one launch.

Replaces the per-cluster loop of evaluate_fragment_clusters
(pycwb/modules/likelihoodWP/likelihood.py:58-135) around its two sky-loop
calls (:310-325).  Per-segment tables (F+, Fx, delay indices, sky mask) are
uploaded once (SkyTables, the device side of prepare_likelihood_inputs,
likelihood_setup.py:81-238); the clusters of a lag are concatenated along
the pixel axis (ClusterBatch); one persistent kernel launch evaluates the
regulator and the scan of every cluster, taking (cluster, sky tile) work
items in decreasing cluster size.  The launch can be captured in a CUDA
graph and replayed.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np
import torch

from .. import _device as dv
from .. import _lib
from .sky_scan import N_STATS


@dataclass
class SkyTables:
    """Per-segment sky tables resident on the device.

    FP, FX (n_sky, n_ifo) float32, ml (n_ifo, n_sky) int32, valid (n_valid,)
    int64, plus the segment constants of likelihood_setup.py:140-147.
    """

    FP: torch.Tensor
    FX: torch.Tensor
    ml: torch.Tensor
    valid: torch.Tensor
    order: torch.Tensor          # scan order of valid positions grouped by delay tuple
    reg_order: torch.Tensor      # regulator order of valid positions (pgw_regulator_order)
    n_tuples: int
    n_ifo: int
    n_sky: int
    network_energy_threshold: float
    gamma_regulator: float
    delta_regulator: float
    netCC: float

    @classmethod
    def from_arrays(cls, FP_t, FX_t, ml, sky_valid_indices=None, *, network_energy_threshold,
                    gamma_regulator, delta_regulator, netCC):
        n_sky, n_ifo = dv.shape_of(FP_t)
        if dv.shape_of(FX_t) != (n_sky, n_ifo) or dv.shape_of(ml) != (n_ifo, n_sky):
            raise ValueError("FP/FX must be (n_sky, n_ifo) and ml (n_ifo, n_sky)")
        if sky_valid_indices is None:
            sky_valid_indices = np.arange(n_sky, dtype=np.int64)
        ml_h = ml.cpu().numpy() if isinstance(ml, torch.Tensor) else np.asarray(ml)
        v_h = (sky_valid_indices.cpu().numpy() if isinstance(sky_valid_indices, torch.Tensor)
               else np.asarray(sky_valid_indices))
        order, n_tuples = _lib.sky_order(ml_h, v_h)
        host = (lambda x: x.cpu().numpy() if isinstance(x, torch.Tensor) else np.asarray(x))
        reg_order = _lib.regulator_order(host(FP_t), host(FX_t), v_h, gamma_regulator)
        return cls(FP=dv.to_device(FP_t, torch.float32), FX=dv.to_device(FX_t, torch.float32),
                   ml=dv.to_device(ml, torch.int32),
                   valid=dv.to_device(sky_valid_indices, torch.int64),
                   order=dv.to_device(order, torch.int32),
                   reg_order=dv.to_device(reg_order, torch.int32), n_tuples=int(n_tuples),
                   n_ifo=int(n_ifo),
                   n_sky=int(n_sky), network_energy_threshold=float(network_energy_threshold),
                   gamma_regulator=float(gamma_regulator), delta_regulator=float(delta_regulator),
                   netCC=float(netCC))

    @classmethod
    def from_setup(cls, setup: dict):
        """From the dict of prepare_likelihood_inputs (likelihood_setup.py:207-238)."""
        return cls.from_arrays(setup["FP_t"], setup["FX_t"], setup["ml"],
                               setup.get("sky_valid_indices"),
                               network_energy_threshold=setup["network_energy_threshold"],
                               gamma_regulator=setup["gamma_regulator"],
                               delta_regulator=setup["delta_regulator"], netCC=setup["netCC"])

    @property
    def REG0(self) -> float:
        """REG[0] = delta * sqrt(2) as float32 (likelihood.py:258)."""
        return float(np.float32(self.delta_regulator * np.sqrt(2)))


class ClusterBatch:
    """Clusters concatenated along the pixel axis (host, pinned)."""

    def __init__(self, n_ifo: int, n_delay: int, sizes):
        self.n_ifo, self.n_delay = int(n_ifo), int(n_delay)
        self.sizes = np.asarray(sizes, dtype=np.int64)
        self.n_clusters = int(self.sizes.size)
        self.pix_offsets = np.concatenate([[0], np.cumsum(self.sizes)]).astype(np.int64)
        self.td_offsets = self.pix_offsets * (self.n_delay * self.n_ifo)
        self.total_pix = int(self.pix_offsets[-1])
        n_td = self.total_pix * self.n_delay * self.n_ifo
        self.td00 = torch.empty(n_td, dtype=torch.float32, pin_memory=True)
        self.td90 = torch.empty(n_td, dtype=torch.float32, pin_memory=True)
        self.rms = torch.empty((self.total_pix, self.n_ifo), dtype=torch.float32, pin_memory=True)

    @classmethod
    def from_clusters(cls, clusters):
        """clusters: iterable of (td00, td90, rms) with the reference's layouts
        (n_delay, n_ifo, n_pix), (n_delay, n_ifo, n_pix), (n_pix, n_ifo)."""
        clusters = list(clusters)
        if not clusters:
            raise ValueError("empty cluster list")
        n_delay, n_ifo, _ = np.shape(clusters[0][0])
        b = cls(n_ifo, n_delay, [np.shape(c[0])[2] for c in clusters])
        for c, (t0, t9, r) in enumerate(clusters):
            b.set_cluster(c, t0, t9, r)
        return b

    def set_cluster(self, c, td00, td90, rms):
        P = int(self.sizes[c])
        if (np.shape(td00) != (self.n_delay, self.n_ifo, P) or np.shape(td90) != np.shape(td00)
                or np.shape(rms) != (P, self.n_ifo)):
            raise ValueError(f"cluster {c}: td00/td90 must be (n_delay, n_ifo, {P}) and rms "
                             f"({P}, n_ifo)")
        a, b = int(self.td_offsets[c]), int(self.td_offsets[c + 1])
        self.td00[a:b] = torch.from_numpy(np.ascontiguousarray(td00, np.float32).ravel())
        self.td90[a:b] = torch.from_numpy(np.ascontiguousarray(td90, np.float32).ravel())
        p0, p1 = int(self.pix_offsets[c]), int(self.pix_offsets[c + 1])
        self.rms[p0:p1] = torch.from_numpy(np.ascontiguousarray(rms, np.float32))

    def cluster_views(self, c):
        a, b = int(self.td_offsets[c]), int(self.td_offsets[c + 1])
        P = int(self.sizes[c])
        shp = (self.n_delay, self.n_ifo, P)
        return (self.td00[a:b].numpy().reshape(shp), self.td90[a:b].numpy().reshape(shp),
                self.rms[int(self.pix_offsets[c]):int(self.pix_offsets[c + 1])].numpy())

    @property
    def h2d_bytes(self) -> int:
        return 4 * (self.td00.numel() + self.td90.numel() + self.rms.numel())


def copy_from_host(dst: torch.Tensor, src: torch.Tensor, stream: torch.cuda.Stream) -> None:
    """dst (device) <- src (page-locked host), asynchronously on `stream`.

    Large copies go through pgw_copy_from_host (SM loads): the copy engine's
    first pass over a large host buffer after a sky-loop launch ran at
    5-11 GB/s on GB300 against 80-130 GB/s for the kernel (both reach
    210 GB/s on a repeated pass).  Small or unpinned sources use torch."""
    n = src.numel() * src.element_size()
    if (n >= (1 << 20) and src.is_pinned() and src.is_contiguous() and dst.is_contiguous()
            and dst.is_cuda and dst.numel() * dst.element_size() == n):
        _lib.check(_lib.load().pgw_copy_from_host(dst.data_ptr(), src.data_ptr(), n,
                                                  stream.cuda_stream), "copy_from_host")
        return
    with torch.cuda.stream(stream):
        dst.copy_(src, non_blocking=True)


class BatchedSkyLoop:
    """Device buffers and launches of the batched sky loop for one batch shape."""

    def __init__(self, tables: SkyTables, batch: ClusterBatch, shape: _lib.TileShape | None = None,
                 keep_maps: bool = True):
        if batch.n_ifo != tables.n_ifo:
            raise ValueError("batch and tables disagree on n_ifo")
        self.t, self.b = tables, batch
        self.shape = shape
        self.L = _lib.load()
        self.stream = dv.stream()
        dev = dv.require_cuda()
        n = batch.n_clusters
        with torch.cuda.stream(self.stream):
            self.td00 = torch.empty(batch.td00.numel(), dtype=torch.float32, device=dev)
            self.td90 = torch.empty(batch.td90.numel(), dtype=torch.float32, device=dev)
            self.rms = torch.empty(tuple(batch.rms.shape), dtype=torch.float32, device=dev)
            self.pix_off = torch.from_numpy(batch.pix_offsets).to(dev)
            self.td_off = torch.from_numpy(batch.td_offsets).to(dev)
            self.stats = torch.empty((n if keep_maps else 1, N_STATS, tables.n_sky),
                                     dtype=torch.float32, device=dev)
            self.res = torch.empty((n, dv.RESULT_DTYPE.itemsize), dtype=torch.uint8, device=dev)
            self.regs = torch.empty(n, dtype=torch.float64, device=dev)
            nbytes = self.L.pgw_workspace_bytes(batch.n_ifo, batch.n_delay, batch.total_pix, n)
            self.ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        if not keep_maps and n > 1:
            raise ValueError("keep_maps=False needs the per-cluster maps buffer; not supported")
        self.res_host = torch.empty((n, dv.RESULT_DTYPE.itemsize), dtype=torch.uint8,
                                    pin_memory=True)
        self.regs_host = torch.empty(n, dtype=torch.float64, pin_memory=True)
        self.graph = None

    # -- steps -------------------------------------------------------------
    def upload(self, *, td=True):
        """Host (pinned) -> device copies of the cluster data, async on the stream.
        td=False copies the rms only, for batches whose td amplitudes were
        built on the device (utils.td_vector_kernels.td_vecs_to_clusters)."""
        self.stream.wait_stream(torch.cuda.current_stream())
        pairs = ([(self.td00, self.b.td00), (self.td90, self.b.td90)] if td else []) + \
            [(self.rms, self.b.rms)]
        for dst, src in pairs:
            copy_from_host(dst, src, self.stream)

    def launch(self):
        t, b = self.t, self.b
        rc = self.L.pgw_sky_loop_batched(
            b.n_ifo, b.n_clusters, self.pix_off.data_ptr(), self.td_off.data_ptr(), b.total_pix,
            t.n_sky, t.FP.data_ptr(), t.FX.data_ptr(), self.rms.data_ptr(), self.td00.data_ptr(),
            self.td90.data_ptr(), b.n_delay, t.ml.data_ptr(), t.REG0, t.gamma_regulator, t.netCC,
            t.network_energy_threshold, t.valid.data_ptr(), t.valid.numel(), t.order.data_ptr(),
            t.reg_order.data_ptr(), self.stats.data_ptr(), self.res.data_ptr(), self.regs.data_ptr(),
            None if self.shape is None else ctypes.byref(self.shape), self.ws.data_ptr(),
            self.ws.numel(), self.stream.cuda_stream)
        _lib.check(rc, "sky_loop_batched")

    def launch_regulators(self, out: torch.Tensor):
        """Regulator only for every cluster (pgw_calculate_dpf_batched) into
        `out` (n_clusters float64, device), on the loop's stream; the rms must
        be on the device (upload)."""
        t, b = self.t, self.b
        rc = self.L.pgw_calculate_dpf_batched(
            b.n_ifo, b.n_clusters, self.pix_off.data_ptr(), b.total_pix, t.n_sky,
            t.FP.data_ptr(), t.FX.data_ptr(), self.rms.data_ptr(), t.gamma_regulator,
            t.network_energy_threshold, t.valid.data_ptr(), t.valid.numel(), t.order.data_ptr(),
            t.reg_order.data_ptr(), out.data_ptr(), None if self.shape is None else ctypes.byref(self.shape),
            self.ws.data_ptr(), self.ws.numel(), self.stream.cuda_stream)
        _lib.check(rc, "calculate_dpf_batched")

    def regulators(self) -> np.ndarray:
        """REG[1] of every cluster (float64), regulator only."""
        with torch.cuda.stream(self.stream):
            out = torch.empty(self.b.n_clusters, dtype=torch.float64, device=self.regs.device)
        self.launch_regulators(out)
        with torch.cuda.stream(self.stream):
            return out.cpu().numpy()

    def download(self):
        """Device -> host (pinned) copies of the per-cluster results, async."""
        with torch.cuda.stream(self.stream):
            self.res_host.copy_(self.res, non_blocking=True)
            self.regs_host.copy_(self.regs, non_blocking=True)

    @property
    def d2h_bytes(self) -> int:
        return self.res_host.numel() + 8 * self.regs_host.numel()

    def capture(self):
        """Capture launch() in a CUDA graph (after one eager launch)."""
        self.launch()
        self.stream.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=self.stream):
            self.launch()
        self.graph = g
        return g

    def replay(self):
        """Replay the captured launch on this loop's stream (a CUDAGraph
        replays on the current stream, so it is made current here)."""
        if self.graph is None:
            self.capture()
        with torch.cuda.stream(self.stream):
            self.graph.replay()

    def run(self, *, upload=True, download=True):
        """The public one-call path: upload, launch, download, wait."""
        if upload:
            self.upload()
        self.launch()
        if download:
            self.download()
        self.stream.synchronize()
        return self.results() if download else None

    def run_many(self, batches):
        """Stream several batches of this loop's shape through it: yields one
        BatchResult per batch, in order.  Two device input sets alternate;
        batch k+1's host -> device copy runs on a copy stream (the copy
        engine, not the SMs) while batch k's launch computes, so every
        batch's inputs still cross the bus but only the first copy is
        exposed.  A yielded result's maps are valid until the next item is
        asked for (the next launch reuses them).  Each batch must be a
        ClusterBatch with this loop's offsets (the same cluster sizes).  The
        first copy, which nothing overlaps, goes through the SMs
        (copy_from_host); the others through the copy engine.  Afterwards
        the loop's device inputs hold whichever batch was staged into them
        last: upload() before a further launch()."""
        dev = self.td00.device
        copy_stream = torch.cuda.Stream(device=dev)
        spare = [(self.td00, self.td90, self.rms)]
        with torch.cuda.stream(self.stream):
            spare.append((torch.empty_like(self.td00), torch.empty_like(self.td90),
                          torch.empty_like(self.rms)))

        def stage(buf, batch, after_queued=False):
            if (batch.total_pix != self.b.total_pix or batch.n_clusters != self.b.n_clusters
                    or not np.array_equal(batch.pix_offsets, self.b.pix_offsets)):
                raise ValueError("run_many: every batch needs this loop's cluster sizes")
            if after_queued:
                # the first buffer is the loop's own: work queued on the
                # loop's stream before this call may still read it.  Later
                # buffers were last read by a launch that has completed.
                copy_stream.wait_stream(self.stream)
            with torch.cuda.stream(copy_stream):
                for dst, src in zip(buf, (batch.td00, batch.td90, batch.rms)):
                    if after_queued:
                        # nothing to overlap with: the SMs copy fastest
                        copy_from_host(dst, src, copy_stream)
                    else:
                        # alongside a launch that holds every SM: the copy engine
                        dst.copy_(src, non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(copy_stream)
            return ev

        it = iter(batches)
        cur = next(it, None)
        if cur is None:
            return
        ready = stage(spare[0], cur, after_queued=True)
        k = 0
        own = (self.td00, self.td90, self.rms)
        try:
            while cur is not None:
                buf = spare[k % 2]
                self.stream.wait_event(ready)
                self.td00, self.td90, self.rms = buf
                self.launch()
                nxt = next(it, None)
                if nxt is not None:
                    ready = stage(spare[(k + 1) % 2], nxt)
                self.download()
                self.stream.synchronize()
                yield self.results()
                cur = nxt
                k += 1
        finally:
            copy_stream.synchronize()
            self.td00, self.td90, self.rms = own

    # -- results -----------------------------------------------------------
    def results(self):
        r = self.res_host.numpy().view(dv.RESULT_DTYPE).reshape(-1)
        status = int(np.bitwise_or.reduce(r["status"])) if r.size else 0
        _lib.check_device_status(status, "sky_loop_batched")
        # the maps were allocated on the loop's stream and are read on the
        # caller's: keep the caching allocator from handing their memory to
        # new work on the loop's stream before the caller's queued reads ran
        cur = torch.cuda.current_stream(self.stats.device)
        if cur != self.stream:
            self.stats.record_stream(cur)
        return BatchResult(l_max=r["l_max"].copy(), sky_stat_max=r["sky_stat_max"].copy(),
                           found=r["found"].astype(bool), regulator=self.regs_host.numpy().copy(),
                           maps=self.stats, active_pairs=r["active_pairs"].copy())


@dataclass
class BatchResult:
    l_max: np.ndarray          # (n_clusters,) int64
    sky_stat_max: np.ndarray   # (n_clusters,) float32
    found: np.ndarray          # (n_clusters,) bool: some direction reached the >= comparison
    regulator: np.ndarray      # (n_clusters,) float64 REG[1]
    maps: torch.Tensor         # (n_clusters, 11, n_sky) float32 on the device
    active_pairs: np.ndarray   # (n_clusters,) int64 (direction, pixel) pairs above E_thr

    def cluster_tuple(self, c):
        """Cluster c as the reference's 13-tuple (sky_scan.py:191-192)."""
        st = self.maps[c].cpu().numpy()
        smax = np.float32(self.sky_stat_max[c]) if self.found[c] else 0
        return (int(self.l_max[c]),) + tuple(st[k] for k in range(N_STATS)) + (smax,)


def sky_loop_batched(tables: SkyTables, clusters, shape=None):
    """One-shot convenience: evaluate a list of (td00, td90, rms) clusters."""
    batch = clusters if isinstance(clusters, ClusterBatch) else ClusterBatch.from_clusters(clusters)
    loop = BatchedSkyLoop(tables, batch, shape=shape)
    return loop.run()


def shard_clusters(sizes, world: int, rank: int) -> np.ndarray:
    """Cluster indices of `rank` when clusters are spread over `world` GPUs.

    Clusters are independent (likelihood.py:58-135), so ranks share no data;
    the work of a cluster is proportional to its pixel count, and clusters
    are dealt largest first to the least-loaded rank (LPT).  Every rank
    computes the same assignment, so no communication is needed."""
    sizes = np.asarray(sizes, dtype=np.int64)
    if world < 1 or not (0 <= rank < world):
        raise ValueError("need world >= 1 and 0 <= rank < world")
    order = np.argsort(-sizes, kind="stable")
    load = np.zeros(world, dtype=np.int64)
    owner = np.empty(sizes.size, dtype=np.int64)
    for c in order:
        r = int(np.argmin(load))
        owner[c] = r
        load[r] += max(int(sizes[c]), 1)
    return np.flatnonzero(owner == rank)


def n_work_items(n_valid: int, n_clusters: int, shape: _lib.TileShape | None) -> int:
    threads = (shape.threads if shape and shape.threads else 256)
    lanes = (shape.lanes_per_sky if shape and shape.lanes_per_sky else 1)
    return 2 * n_clusters * math.ceil(n_valid / (threads // lanes))
