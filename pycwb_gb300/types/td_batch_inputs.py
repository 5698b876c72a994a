"""GPU drop-in for pycwb/types/td_batch_inputs.py (TDBatchInputs, :6-67)."""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class TDBatchInputs:
    """Padded quadrature planes and TD filter tables of one (level, detector).

    padded00/padded90: (n_time + 2*n_coeffs, M+1) float32; T0/Tx:
    (2*J+1, 2*n_coeffs+1) float64; J = M * L (td_batch_inputs.py:14-38).
    """

    padded00: np.ndarray
    padded90: np.ndarray
    T0: np.ndarray
    Tx: np.ndarray
    M: int
    n_coeffs: int
    J: int

    def extract_td_vecs(self, pixel_indices, K, *, return_device=False):
        """(n_pixels, 4K+2) float32 td vectors (td_batch_inputs.py:40-67)."""
        from ..utils.td_vector_kernels import batch_get_td_vecs

        return batch_get_td_vecs(pixel_indices, self.padded00, self.padded90, self.T0, self.Tx,
                                 self.M, self.n_coeffs, K, self.J, return_device=return_device)
