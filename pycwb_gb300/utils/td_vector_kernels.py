"""GPU drop-in for pycwb/utils/td_vector_kernels.py (batch_get_td_vecs, :133-199).

For every pixel index (time bin n, layer m of an (n_time, M+1) WDM plane)
and every delay dT in [-K, K], the 00 and 90 amplitudes the pixel would
have if the detector's data were delayed by dT TD-rate samples.  The
kernel (pgw_batch_get_td_vecs) is bit-identical to the reference: float64
accumulation in the reference's order, phase factors from the host libm.
"""

from __future__ import annotations

import numpy as np
import torch

from .. import _device as dv
from .. import _lib
from ..tdamp import td_phase_table_device


def batch_get_td_vecs(pixel_indices, padded00, padded90, T0, Tx, M, n_coeffs, K, J, *,
                      return_device=False):
    """(n_pixels, 4K+2) float32: [a00(-K..K), a90(-K..K)] per pixel."""
    M, n_coeffs, K, J = int(M), int(n_coeffs), int(K), int(J)
    if M < 1 or J < 1 or K < 0 or n_coeffs < 0:
        raise ValueError("need M >= 1, J >= 1, K >= 0, n_coeffs >= 0")
    rows = dv.shape_of(padded00)[0]
    if dv.shape_of(padded00) != (rows, M + 1) or dv.shape_of(padded90) != (rows, M + 1):
        raise ValueError(f"padded planes must be (rows, M+1={M + 1}), got "
                         f"{dv.shape_of(padded00)} and {dv.shape_of(padded90)}")
    if dv.shape_of(T0) != (2 * J + 1, 2 * n_coeffs + 1) or dv.shape_of(Tx) != dv.shape_of(T0):
        raise ValueError(f"T0/Tx must be (2J+1, 2*n_coeffs+1) = ({2 * J + 1}, {2 * n_coeffs + 1})")
    L = _lib.load()
    s = dv.begin()
    idx = dv.to_device(pixel_indices, torch.int32)
    p00, p90 = dv.to_device(padded00, torch.float32), dv.to_device(padded90, torch.float32)
    t0, tx = dv.to_device(T0, torch.float64), dv.to_device(Tx, torch.float64)
    ph = td_phase_table_device(M, J, idx.device)
    n = int(idx.numel())
    with torch.cuda.stream(s):
        out = torch.empty((n, 4 * K + 2), dtype=torch.float32, device=idx.device)
    rc = L.pgw_batch_get_td_vecs(idx.data_ptr(), n, p00.data_ptr(), p90.data_ptr(), rows,
                                 t0.data_ptr(), tx.data_ptr(), ph.data_ptr(), M, n_coeffs, K, J,
                                 out.data_ptr(), dv.stream_handle(s))
    _lib.check(rc, "batch_get_td_vecs")
    if return_device:
        dv.end(s, out)
        return out
    with torch.cuda.stream(s):
        return out.cpu().numpy()


def td_vecs_to_clusters(loop, td_inputs, ifo, pixel_indices, dst_cluster, dst_pixel, K):
    """Write the td vectors of one (WDM plane, detector) into a BatchedSkyLoop.

    td_inputs: a TDBatchInputs (arrays may be NumPy or CUDA tensors);
    pixel_indices: flat plane indices (n*(M+1)+m) of the pixels to build;
    dst_cluster/dst_pixel: where each lands in the batch.  The amplitudes
    go straight into the loop's device td buffers in the scan's layout, so
    a lag's clusters need no host round trip between the td build and the
    sky scan.  K must equal the batch's (n_delay - 1) / 2."""
    if 2 * int(K) + 1 != loop.b.n_delay:
        raise ValueError(f"K={K} does not match the batch's n_delay={loop.b.n_delay}")
    t = td_inputs
    s = dv.begin()
    idx = dv.to_device(pixel_indices, torch.int32)
    dc = dv.to_device(dst_cluster, torch.int32)
    dp = dv.to_device(dst_pixel, torch.int32)
    p00, p90 = dv.to_device(t.padded00, torch.float32), dv.to_device(t.padded90, torch.float32)
    t0, tx = dv.to_device(t.T0, torch.float64), dv.to_device(t.Tx, torch.float64)
    s.wait_stream(loop.stream)  # a launch still reading the td buffers finishes first
    scatter_launch(loop, int(ifo), idx, dc, dp, p00, p90, t0, tx, int(t.M), int(t.n_coeffs),
                   int(K), int(t.J), s)
    loop.stream.wait_stream(s)


def scatter_launch(loop, ifo, idx, dst_cluster, dst_pixel, p00, p90, T0, Tx, M, nc, K, J, s):
    """pgw_td_vecs_to_clusters on stream `s`, all arguments already CUDA
    tensors of the right dtype (int32 indices, float32 planes, float64
    filters); shapes are checked here."""
    rows = int(p00.shape[0])
    if tuple(p00.shape) != (rows, M + 1) or tuple(p90.shape) != (rows, M + 1):
        raise ValueError(f"padded planes must be (rows, M+1={M + 1})")
    if tuple(T0.shape) != (2 * J + 1, 2 * nc + 1) or tuple(Tx.shape) != tuple(T0.shape):
        raise ValueError(f"T0/Tx must be (2J+1, 2*n_coeffs+1) = ({2 * J + 1}, {2 * nc + 1})")
    if not (int(idx.numel()) == int(dst_cluster.numel()) == int(dst_pixel.numel())):
        raise ValueError("pixel_indices, dst_cluster and dst_pixel differ in length")
    ph = td_phase_table_device(M, J, idx.device)
    rc = _lib.load().pgw_td_vecs_to_clusters(
        idx.data_ptr(), int(idx.numel()), dst_cluster.data_ptr(), dst_pixel.data_ptr(),
        loop.b.n_clusters, loop.pix_off.data_ptr(), loop.td_off.data_ptr(), int(ifo),
        loop.b.n_ifo, p00.data_ptr(), p90.data_ptr(), rows, T0.data_ptr(), Tx.data_ptr(),
        ph.data_ptr(), M, nc, K, J, loop.td00.data_ptr(), loop.td90.data_ptr(), s.cuda_stream)
    _lib.check(rc, "td_vecs_to_clusters")
