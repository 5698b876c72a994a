"""Statistics at the sky maximum on the GPU (pgw_skystat_batched).

Drop-in for pycwb/modules/likelihoodWP/sky_statistics.py:26-262
(compute_statistics_at_sky_position, legacy name calculate_sky_statistics):
the same arguments, returning SkyStatistics: the scalars Gn, Ec, Dc, Rc, Eh,
Es, Np, Em, Lm, norm, cc, rho, xrho, Lo, Eo, N_pix_effective, the
per-detector signal SNR S_snr, and the per-pixel arrays the reference's
populate_detection_statistics reads (energy_array_plus/cross, pixel_mask,
gaussian_noise_correction, coherent_energy, noise_amplitude_00/90, the
packets pd, pD, ps, pS, the antenna vectors f, F and the polar maps
p00_POL, p90_POL as (2, P) rows of radius and angle), from
pgw_skystat_pixel_arrays.

``statistics_batched`` evaluates every cluster of a BatchedSkyLoop at its
sky maximum in one launch, straight from the loop's device inputs.

xtalk overlaps come in the reference's packed form: rows (neighbour pixel
index within the cluster, 3 unused, 4 coefficients) and a per-pixel
(start, end) row range (pycwb/modules/xtalk; packet_ops.py:756-901).
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from .. import _device as dv
from .. import _lib

_F4 = np.float32
SKYSTAT_SCALARS = ("Gn", "Ec", "Dc", "Rc", "Eh", "Es", "Np", "Em", "Lm", "norm", "cc", "rho",
                   "xrho", "Lo", "Eo")
SKYSTAT_DTYPE = np.dtype([("N_pix_effective", np.float64)] + [(k, _F4) for k in SKYSTAT_SCALARS] +
                         [("S_snr", _F4, (8,)), ("status", np.int32), ("n_pix", np.int32),
                          ("reserved", np.int32)], align=True)
assert SKYSTAT_DTYPE.itemsize == 112


@dataclass
class SkyStatistics:
    """Event statistics at one direction (the scalar part of the reference's
    SkyStatistics, pycwb/modules/likelihoodWP/typing.py)."""

    Gn: np.float32
    Ec: np.float32
    Dc: np.float32
    Rc: np.float32
    Eh: np.float32
    Es: np.float32
    Np: np.float32
    Em: np.float32
    Lm: np.float32
    norm: np.float32
    cc: np.float32
    rho: np.float32
    xrho: np.float32
    Lo: np.float32
    Eo: np.float32
    N_pix_effective: float
    S_snr: np.ndarray
    # per-pixel arrays (None unless asked for): the reference's names and shapes
    energy_array_plus: np.ndarray = None
    energy_array_cross: np.ndarray = None
    pixel_mask: np.ndarray = None
    gaussian_noise_correction: np.ndarray = None
    coherent_energy: np.ndarray = None
    noise_amplitude_00: np.ndarray = None
    noise_amplitude_90: np.ndarray = None
    pd: np.ndarray = None
    pD: np.ndarray = None
    ps: np.ndarray = None
    pS: np.ndarray = None
    f: np.ndarray = None
    F: np.ndarray = None
    p00_POL: np.ndarray = None
    p90_POL: np.ndarray = None

    @classmethod
    def from_record(cls, r, n_ifo, pixels=None):
        return cls(**{k: np.float32(r[k]) for k in SKYSTAT_SCALARS},
                   N_pix_effective=float(r["N_pix_effective"]),
                   S_snr=np.array(r["S_snr"][:n_ifo], dtype=np.float64), **(pixels or {}))


def split_pixel_arrays(out32, out64, n_ifo, pix_offsets):
    """Per cluster, the reference's per-pixel SkyStatistics arrays from the
    records of pgw_skystat_pixel_arrays: a dict of numpy arrays with the
    reference's names and shapes ((P,), (n_ifo, P) or (P, n_ifo))."""
    I = int(n_ifo)
    out = []
    for c in range(len(pix_offsets) - 1):
        a, b = int(pix_offsets[c]), int(pix_offsets[c + 1])
        r32, r64 = out32[a:b], out64[a:b]
        out.append(dict(
            energy_array_plus=r32[:, 0].copy(), energy_array_cross=r32[:, 1].copy(),
            pixel_mask=r32[:, 2].copy(), gaussian_noise_correction=r32[:, 3].copy(),
            coherent_energy=r32[:, 4].copy(),
            p00_POL=np.stack([r32[:, 5], r32[:, 6]]), p90_POL=np.stack([r32[:, 7], r32[:, 8]]),
            noise_amplitude_00=r32[:, 9:9 + I].T.copy(), noise_amplitude_90=r32[:, 9 + I:9 + 2 * I].T.copy(),
            f=r32[:, 9 + 2 * I:9 + 3 * I].copy(), F=r32[:, 9 + 3 * I:9 + 4 * I].copy(),
            pd=r64[:, :I].T.copy(), pD=r64[:, I:2 * I].T.copy(),
            ps=r64[:, 2 * I:3 * I].T.copy(), pS=r64[:, 3 * I:4 * I].T.copy()))
    return out


def pack_xtalk(per_cluster):
    """Concatenate per-cluster packed xtalk (rows, lookup) into the batched
    form: rows (n, 8) float32 and a (total_pix, 2) int64 lookup whose ranges
    index the concatenated rows (neighbour indices stay cluster-local)."""
    rows, looks, base = [], [], 0
    for xt, lk in per_cluster:
        xt = np.asarray(xt, np.float32).reshape(-1, 8)
        lk = np.asarray(lk, np.int64).reshape(-1, 2)
        rows.append(xt)
        looks.append(lk + base)
        base += xt.shape[0]
    return (np.concatenate(rows) if rows else np.zeros((0, 8), np.float32),
            np.concatenate(looks) if looks else np.zeros((0, 2), np.int64))


def _run(n_ifo, pix_off, td_off, total_pix, FP, FX, rms, td00, td90, n_delay, ml, sky_idx, regs,
         REG0, ethr, xtalk, lookup, xgb, stream, pixel_arrays=False):
    L = _lib.load()
    dev = FP.device
    n = int(sky_idx.numel())
    xt_h = np.ascontiguousarray(xtalk, np.float32).reshape(-1, 8)
    lk_h = np.ascontiguousarray(lookup, np.int64).reshape(-1, 2)
    if lk_h.shape[0] != total_pix:
        raise ValueError(f"xtalk lookup must have one (start, end) row per pixel ({total_pix})")
    with torch.cuda.stream(stream):
        xt = torch.from_numpy(xt_h).to(dev)
        lk = torch.from_numpy(lk_h).to(dev)
        ws = torch.empty(int(L.pgw_skystat_workspace_bytes(n_ifo, total_pix)), dtype=torch.uint8,
                         device=dev)
        out = torch.empty((n, SKYSTAT_DTYPE.itemsize), dtype=torch.uint8, device=dev)
    P = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() else None
    rc = L.pgw_skystat_batched(
        n_ifo, n, P(pix_off), P(td_off), total_pix, int(FP.shape[0]), P(FP), P(FX), P(rms),
        P(td00), P(td90), n_delay, P(ml), P(sky_idx), P(regs), float(REG0), float(ethr),
        P(xt) if xt.numel() else None, int(xt.shape[0]), P(lk) if lk.numel() else None,
        int(bool(xgb)), P(ws),
        ws.numel(), P(out), ctypes.c_void_p(stream.cuda_stream))
    _lib.check(rc, "pgw_skystat_batched")
    pix = None
    if pixel_arrays is not False and total_pix > 0:
        with torch.cuda.stream(stream):
            o32 = torch.empty((total_pix, 9 + 4 * n_ifo), dtype=torch.float32, device=dev)
            o64 = torch.empty((total_pix, 4 * n_ifo), dtype=torch.float64, device=dev)
        rc = L.pgw_skystat_pixel_arrays(n_ifo, total_pix, P(ws), ws.numel(), P(o32), P(o64),
                                        ctypes.c_void_p(stream.cuda_stream))
        _lib.check(rc, "pgw_skystat_pixel_arrays")
        pix = (o32, o64)
    stream.synchronize()
    res = np.frombuffer(out.cpu().numpy().tobytes(), dtype=SKYSTAT_DTYPE).copy()
    bad = res["status"] != 0
    if bad.any():
        codes = sorted(set(int(x) for x in res["status"][bad]))
        raise RuntimeError(f"pgw_skystat_batched: cluster status {codes} "
                           f"({_lib.STATUS_NAMES.get(codes[0], codes[0])}) for "
                           f"{int(bad.sum())} clusters")
    if pixel_arrays is not False:
        offs = pix_off.cpu().numpy()
        n = len(offs) - 1
        if pixel_arrays is True:
            want = range(n)
        else:
            sel = pixel_arrays(res) if callable(pixel_arrays) else pixel_arrays
            want = sorted(set(int(c) for c in sel))
        arrays = [None] * n
        # only the wanted clusters' pixels leave the device, gathered there
        # into one block and copied back in one transfer per record type
        want = list(want)
        spans = [(int(offs[c]), int(offs[c + 1])) for c in want]
        local = np.concatenate([[0], np.cumsum([b - a for a, b in spans])]).astype(np.int64)
        r32 = np.zeros((0, 9 + 4 * n_ifo), np.float32)
        r64 = np.zeros((0, 4 * n_ifo))
        if pix is not None and local[-1] > 0:
            idx = np.concatenate([np.arange(a, b, dtype=np.int64) for a, b in spans])
            with torch.cuda.stream(stream):
                di = torch.from_numpy(idx).to(dev)
                r32 = pix[0].index_select(0, di).cpu().numpy()
                r64 = pix[1].index_select(0, di).cpu().numpy()
        for k, c in enumerate(want):
            arrays[c] = split_pixel_arrays(r32, r64, n_ifo, local[k:k + 2])[0] \
                if local[k + 1] > local[k] else \
                split_pixel_arrays(np.zeros((0, 9 + 4 * n_ifo), np.float32),
                                   np.zeros((0, 4 * n_ifo)), n_ifo, [0, 0])[0]
        return res, arrays
    return res


def statistics_batched(loop, l_max, xtalk, xtalk_lookup, *, regulators=None,
                       xgb_rho_mode=False, pixel_arrays=False):
    """Statistics of every cluster of a BatchedSkyLoop at its sky maximum
    (l_max, e.g. BatchResult.l_max), from the loop's device inputs.
    regulators: REG[1] per cluster (default: the loop's last regulators).
    Returns a structured array of SKYSTAT_DTYPE, one record per cluster; with
    pixel_arrays (True for every cluster, a sequence of cluster indices, or
    a function of the records returning such a sequence) also a list with,
    per cluster, a dict of the reference's per-pixel SkyStatistics arrays
    (split_pixel_arrays), None for clusters not asked for -- only their
    pixels are copied to the host."""
    t, b = loop.t, loop.b
    n = b.n_clusters
    dev = loop.td00.device
    l_h = np.ascontiguousarray(l_max, np.int64).reshape(-1)
    if l_h.size != n:
        raise ValueError(f"l_max needs one direction per cluster ({n})")
    with torch.cuda.stream(loop.stream):
        l = torch.from_numpy(l_h).to(dev)
        regs = (loop.regs if regulators is None else
                torch.from_numpy(np.asarray(regulators, np.float64).reshape(-1)).to(dev))
        regs = regs.to(torch.float32)
    if regs.numel() != n:
        raise ValueError(f"regulators needs one value per cluster ({n})")
    return _run(t.n_ifo, loop.pix_off, loop.td_off, b.total_pix, t.FP, t.FX, loop.rms, loop.td00,
                loop.td90, b.n_delay, t.ml, l, regs.contiguous(), t.REG0,
                t.network_energy_threshold, xtalk, xtalk_lookup, xgb_rho_mode, loop.stream,
                pixel_arrays=pixel_arrays)


def compute_statistics_at_sky_position(sky_idx, n_ifo, n_pix, FP, FX, rms, td00, td90, ml, REG,
                                       network_energy_threshold, cluster_xtalk,
                                       cluster_xtalk_lookup_table, DEBUG=False,
                                       xgb_rho_mode=False) -> SkyStatistics:
    """sky_statistics.py:26-262 for one cluster on the GPU: FP, FX (n_sky,
    nIFO) float32, rms (n_pix, nIFO), td00/td90 (2K+1, nIFO, n_pix), ml
    (nIFO, n_sky), REG (3,)."""
    dev = dv.require_cuda()
    n_ifo, n_pix = int(n_ifo), int(n_pix)
    FP_d = dv.to_device(FP, torch.float32)
    FX_d = dv.to_device(FX, torch.float32)
    if tuple(FP_d.shape) != tuple(FX_d.shape) or FP_d.shape[1] != n_ifo:
        raise ValueError("FP and FX must be (n_sky, n_ifo)")
    rms_d = dv.to_device(rms, torch.float32)
    if tuple(rms_d.shape) != (n_pix, n_ifo):
        raise ValueError(f"rms must be ({n_pix}, {n_ifo})")
    td00_d = dv.to_device(td00, torch.float32)
    td90_d = dv.to_device(td90, torch.float32)
    if td00_d.dim() != 3 or tuple(td00_d.shape[1:]) != (n_ifo, n_pix) or \
            tuple(td90_d.shape) != tuple(td00_d.shape):
        raise ValueError("td00/td90 must be (2K+1, n_ifo, n_pix)")
    ml_d = dv.to_device(ml, torch.int32)
    if tuple(ml_d.shape) != (n_ifo, FP_d.shape[0]):
        raise ValueError("ml must be (n_ifo, n_sky)")
    if not 0 <= int(sky_idx) < FP_d.shape[0]:
        raise ValueError(f"sky_idx {sky_idx} outside [0, {FP_d.shape[0]})")
    REG = np.asarray(REG, np.float32)
    s = dv.stream()
    with torch.cuda.stream(s):
        pix_off = torch.tensor([0, n_pix], dtype=torch.int64, device=dev)
        td_off = torch.tensor([0, td00_d.numel()], dtype=torch.int64, device=dev)
        l = torch.tensor([int(sky_idx)], dtype=torch.int64, device=dev)
        regs = torch.tensor([float(REG[1])], dtype=torch.float32, device=dev)
    res = _run(n_ifo, pix_off, td_off, n_pix, FP_d, FX_d, rms_d, td00_d, td90_d,
               int(td00_d.shape[0]), ml_d, l, regs, float(REG[0]),
               float(np.float32(network_energy_threshold)), cluster_xtalk,
               cluster_xtalk_lookup_table, xgb_rho_mode, s, pixel_arrays=True)
    res, pix = res
    return SkyStatistics.from_record(res[0], n_ifo, pix[0])


calculate_sky_statistics = compute_statistics_at_sky_position
