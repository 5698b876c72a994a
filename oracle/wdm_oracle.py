"""NumPy restatement of cWB's WDM forward transform (both quadratures).

TEST INFRASTRUCTURE ONLY: tests/ use it as the checker of pgw_wdm_t2w; the
product never imports it.

Follows cwb-core/WDM.cc:1384-1535 (t2w, MM = -1) step by step:

* :1399-1409  the series is taken up to a multiple of M and copied into a
  buffer with nWDM samples of mirror image on each side
  (ts[nWDM - n] = x[n] for n <= nWDM; ts[nWDM + nTS + n] = x[nTS - 1 - n]);
* :1445-1475  per time slice n, centre nWDM + n M of that buffer, the
  products with the symmetric filter are folded modulo 2M (the j loop pairs
  sample +t with sample -t; the last tap, t = nWDM - 1, lands on m = 0);
* :1477-1479  real FFT of length 2M with FFTW's forward sign (here
  numpy.fft.rfft, the same transform);
* :1489-1506  both parts of layers 0 and M become Re/sqrt(2); quadratures by
  the parity of m + n: odd -> (a00, a90) = sqrt2 (Im, Re), even -> sqrt2
  (Re, -Im).

Parity status: the reference's transform is in the third-party
wdm_wavelet package (absent) or in cwb-core/WDM.cc (needs ROOT/FFTW), so
no reference output exists here; the tests pin this restatement through
the properties that define the WDM basis (orthonormality of each
quadrature's atoms, the TD filters reproducing time shifts).
"""

from __future__ import annotations

import math

import numpy as np
from numpy.lib.stride_tricks import sliding_window_view


def mirrored_buffer(x: np.ndarray, M: int, n_wdm: int) -> tuple[np.ndarray, int]:
    """(buffer, n_time): the reference's ts buffer of nWWS + 2 nWDM samples."""
    x = np.asarray(x, np.float64)
    n_ts = x.size
    n_wws = n_ts + ((M - n_ts % M) if n_ts % M else 0)
    m = n_wws + 2 * n_wdm
    ts = np.zeros(m, np.float64)
    for n in range(n_wdm + 1):
        ts[n_wdm - n] = x[n]
    ts[n_wdm:n_wdm + n_ts] = x
    for n in range(m - n_wdm - n_ts):
        ts[n + n_wdm + n_ts] = x[n_ts - n - 1]
    return ts, n_wws // M


def fold(x: np.ndarray, M: int, filt: np.ndarray) -> np.ndarray:
    """(n_time, 2M) folded windows of every time slice."""
    n_wdm = filt.size
    M2 = 2 * M
    k = (n_wdm - 1) // M2
    ts, N = mirrored_buffer(x, M, n_wdm)
    w = np.concatenate([filt[:0:-1], filt])                 # taps t = -(nWDM-1) .. nWDM-1
    win = sliding_window_view(ts, w.size)[1:1 + N * M:M]   # centre nWDM + nM
    prod = win * w[None, :]
    r = prod[:, :2 * k * M2].reshape(N, 2 * k, M2).sum(axis=1)
    r[:, 0] += prod[:, -1]
    return r


def t2w(x: np.ndarray, M: int, filt: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(map00, map90), each (n_time, M+1) float64, row n = time slice."""
    r = fold(x, M, filt)
    X = np.fft.rfft(r, axis=1)
    re = X.real.copy()
    im = X.imag.copy()
    s2 = math.sqrt(2.0)
    for m in (0, M):
        re[:, m] = re[:, m] / s2
        im[:, m] = re[:, m]
    N = r.shape[0]
    odd = ((np.arange(M + 1)[None, :] + (np.arange(N) % 2)[:, None]) % 2) == 1
    a00 = np.where(odd, s2 * im, s2 * re)
    a90 = np.where(odd, s2 * re, -(s2 * im))
    return a00, a90


def get_filter_scalar(M: int, K: int, fourier: np.ndarray, n: int) -> np.ndarray:
    """WDM.cc:497-548 getFilter(n) as scalar loops, in the reference's order
    (the package evaluates the same closed form vectorised)."""
    B = math.pi / K
    A = (K - M) * math.pi / 2.0 / K / M
    K2 = float(K) * K
    gNorm = math.sqrt(2 * M) / math.pi
    four = [float(v) for v in fourier]
    out = np.zeros(n, np.float64)
    out[0] = (A + four[0] * B) * gNorm
    four[0] /= math.sqrt(2.0)
    for i in range(1, n):
        di = float(i)
        i2 = di * di
        se = so = 0.0
        for j in range(len(four)):
            if i % K == 0 and j == i // K:
                continue
            t = di / (i2 - j * j * K2) * four[j]
            if j & 1:
                so += t
            else:
                se += t
        intAB = 0.0
        if i % K == 0 and i // K < len(four):
            intAB = four[i // K] * B / 2 * math.cos(i * A)
        intAB += 2 * (se * math.sin(i * B / 2) * math.cos(i * math.pi / (2 * M))
                      - so * math.sin(i * math.pi / (2 * M)) * math.cos(i * B / 2))
        out[i] = gNorm * (math.sin(i * A) / i + math.sqrt(2.0) * intAB)
    return out
