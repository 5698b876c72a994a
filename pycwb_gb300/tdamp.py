"""Host-side helpers of the td-amplitude build (WDM time-delay vectors).

The td vectors of a pixel are, for every delay dT in [-K, K], the WDM
amplitudes a00/a90 that the pixel would have if its detector's data were
shifted by dT samples of the TD rate (pycwb/utils/td_vector_kernels.py:15-199,
the Python form of cWB's WDM::getTDamp, cwb-core/WDM.cc:1103-1196).

The trigonometric factors of each term depend only on (layer m, delay dT):

    dt    = dT * M / J                              (td_vector_kernels.py:42)
    same  = m * pi * dt / M                         (:59)
    low   = (2m - 1) * dt * pi / (2M)               (:82)
    high  = (2m + 1) * dt * pi / (2M)               (:113)

``td_phase_table`` evaluates them once per (M, J) with the host's libm,
using the same float64 expressions in the same order, so that the device
kernel multiplies by bit-identical factors.
"""

from __future__ import annotations

import functools
import math

import numpy as np


@functools.lru_cache(maxsize=64)
def _phase_table_cached(M: int, J: int) -> bytes:
    tab = np.zeros((M + 1, 2 * J + 1, 4), dtype=np.float64)
    for m in range(M + 1):
        for dT in range(-J, J + 1):
            dt_val = float(dT) * float(M) / float(J)
            same = m * math.pi * dt_val / M
            low = (2.0 * m - 1.0) * dt_val * math.pi / (2.0 * M)
            high = (2.0 * m + 1.0) * dt_val * math.pi / (2.0 * M)
            tab[m, dT + J] = (math.cos(same), math.sin(same), math.sin(low), math.sin(high))
    return tab.tobytes()


def td_phase_table(M: int, J: int) -> np.ndarray:
    """(M+1, 2J+1, 4) float64: cos(same), sin(same), sin(low), sin(high)."""
    M, J = int(M), int(J)
    if M < 1 or J < 1:
        raise ValueError(f"td phase table needs M >= 1 and J >= 1, got M={M}, J={J}")
    return np.frombuffer(_phase_table_cached(M, J), dtype=np.float64).reshape(M + 1, 2 * J + 1, 4)


_device_tables: dict = {}


def td_phase_table_device(M: int, J: int, device):
    """td_phase_table(M, J) as a float64 CUDA tensor, copied to `device` once
    and kept (the largest, M = 512 and J = 2048, is 67 MB)."""
    import torch

    dev = torch.device(device)
    key = (int(M), int(J), dev.index if dev.index is not None else torch.cuda.current_device())
    t = _device_tables.get(key)
    if t is None:
        t = torch.from_numpy(td_phase_table(M, J).copy()).to(torch.device("cuda", key[2]))
        torch.cuda.synchronize(key[2])   # complete before any stream reads it
        _device_tables[key] = t
    return t
