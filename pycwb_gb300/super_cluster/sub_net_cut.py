"""GPU drop-in for the sub-network-cut sky loop.

optimze_sky_loc_from_td keeps the reference's name (spelling included) and
signature (pycwb/modules/super_cluster_native/sub_net_cut.py:404-517) and
returns its 8-tuple (l_max, stat, Em, Am, lm, Vm, suball, EE);
subnet_sky_batched evaluates many clusters (a lag's superclusters, each
with its loudest pixels, utils.py:705-711) in one launch of
pgw_subnet_sky_batched.  FP/FX are (n_sky, n_ifo) float32 as the reference's
caller passes them after its transposes (sub_net_cut.py:49-53).
"""

from __future__ import annotations

import numpy as np
import torch

from .. import _device as dv
from .. import _lib

SUBNET_DTYPE = np.dtype([("key", "<u8"), ("l_max", "<i8"), ("stat", "<f4"), ("Em", "<f4"),
                         ("Am", "<f4"), ("suball", "<f4"), ("EE", "<f4"), ("Vm", "<i4"),
                         ("status", "<i4"), ("reserved", "<i4")])
assert SUBNET_DTYPE.itemsize == 48


def _tuple(r):
    l = int(r["l_max"])
    return (l, np.float32(r["stat"]), np.float32(r["Em"]), np.float32(r["Am"]), l, int(r["Vm"]),
            np.float32(r["suball"]), np.float32(r["EE"]))


def _run(n_ifo, n_clusters, pix_off, td_off, total_pix, FPd, FXd, rms, t0, t9, n_delay, mld,
         thr, e2or, subcut, s):
    with torch.cuda.stream(s):
        out = torch.empty((n_clusters, SUBNET_DTYPE.itemsize), dtype=torch.uint8, device=FPd.device)
    rc = _lib.load().pgw_subnet_sky_batched(
        int(n_ifo), int(n_clusters), dv.ptr(pix_off), dv.ptr(td_off), int(total_pix),
        int(FPd.shape[0]), FPd.data_ptr(), FXd.data_ptr(), dv.ptr(rms), dv.ptr(t0), dv.ptr(t9),
        int(n_delay), mld.data_ptr(), float(np.float32(thr)), float(e2or), float(subcut),
        out.data_ptr(), s.cuda_stream)
    _lib.check(rc, "subnet_sky_batched")
    with torch.cuda.stream(s):
        res = out.cpu().numpy().view(SUBNET_DTYPE).reshape(-1)
    status = int(np.bitwise_or.reduce(res["status"])) if res.size else 0
    _lib.check_device_status(status, "subnet_sky_batched")
    return res


def _tables(FP, FX, ml, n_sky, n_ifo):
    if dv.shape_of(FP) != (n_sky, n_ifo) or dv.shape_of(FX) != (n_sky, n_ifo):
        raise ValueError(f"FP and FX must have shape (n_sky, n_ifo) = ({n_sky}, {n_ifo}), got "
                         f"{dv.shape_of(FP)} and {dv.shape_of(FX)}")
    if dv.shape_of(ml) != (n_ifo, n_sky):
        raise ValueError(f"ml must have shape (n_ifo, n_sky) = ({n_ifo}, {n_sky})")
    return (dv.to_device(FP, torch.float32), dv.to_device(FX, torch.float32),
            dv.to_device(ml, torch.int32))


def optimze_sky_loc_from_td(n_ifo, n_pix, n_sky, FP, FX, rms, td00, td90, ml,
                            network_energy_threshold, e2or, subcut):
    """Best direction of one cluster for the sub-network cut
    (sub_net_cut.py:404-517): (l_max, stat, Em, Am, lm, Vm, suball, EE)."""
    n_ifo, n_pix, n_sky = int(n_ifo), int(n_pix), int(n_sky)
    n_delay = dv.shape_of(td00)[0]
    if dv.shape_of(td00) != (n_delay, n_ifo, n_pix) or dv.shape_of(td90) != dv.shape_of(td00):
        raise ValueError("td00/td90 must have shape (n_delay, n_ifo, n_pix)")
    if dv.shape_of(rms) != (n_pix, n_ifo):
        raise ValueError("rms must have shape (n_pix, n_ifo)")
    s = dv.begin()
    FPd, FXd, mld = _tables(FP, FX, ml, n_sky, n_ifo)
    t0, t9 = dv.to_device(td00, torch.float32), dv.to_device(td90, torch.float32)
    r = dv.to_device(rms, torch.float32)
    res = _run(n_ifo, 1, None, None, n_pix, FPd, FXd, r, t0, t9, n_delay, mld,
               network_energy_threshold, e2or, subcut, s)
    return _tuple(res[0])


def subnet_sky_batched(FP, FX, ml, clusters, network_energy_threshold, e2or, subcut):
    """optimze_sky_loc_from_td for every cluster of `clusters` (a ClusterBatch
    or a list of (td00, td90, rms)) in one launch; returns the per-cluster
    results as a SUBNET_DTYPE array (lm = l_max)."""
    from ..likelihoodWP.batched import ClusterBatch
    b = clusters if isinstance(clusters, ClusterBatch) else ClusterBatch.from_clusters(clusters)
    n_ifo = b.n_ifo
    n_sky = dv.shape_of(FP)[0]
    if b.n_clusters > 65535:
        raise ValueError("at most 65535 clusters per call")
    s = dv.begin()
    FPd, FXd, mld = _tables(FP, FX, ml, n_sky, n_ifo)
    dev = FPd.device
    with torch.cuda.stream(s):
        t0 = torch.empty(b.td00.numel(), dtype=torch.float32, device=dev)
        t9 = torch.empty(b.td90.numel(), dtype=torch.float32, device=dev)
        r = torch.empty(tuple(b.rms.shape), dtype=torch.float32, device=dev)
        pix_off = torch.from_numpy(b.pix_offsets).to(dev)
        td_off = torch.from_numpy(b.td_offsets).to(dev)
    from ..likelihoodWP.batched import copy_from_host
    for dst, src in ((t0, b.td00), (t9, b.td90), (r, b.rms)):
        copy_from_host(dst, src, s)
    return _run(n_ifo, b.n_clusters, pix_off, td_off, b.total_pix, FPd, FXd, r, t0, t9,
                b.n_delay, mld, network_energy_threshold, e2or, subcut, s)
