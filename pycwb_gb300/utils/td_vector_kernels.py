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
from ..tdamp import td_phase_table


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
    ph = dv.to_device(td_phase_table(M, J), torch.float64)
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
