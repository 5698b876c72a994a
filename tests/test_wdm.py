"""WDM basis, TD filters and the forward-transform oracle, on the CPU.

Pins, in the absence of any runnable reference transform (the reference's
is the third-party wdm_wavelet package, or cwb-core/WDM.cc with ROOT):

* the edge's cosine-series coefficients, recomputed by quadrature, against
  cWB's own table (tests/golden/wdm_fourier_tables.npz, read from
  cwb-core/FourierCoefficients.icc by tests/golden/make_wdm_golden.py);
* the basis filter's norm and length rule (WDM.cc:150-162) and its closed
  form against a scalar restatement in the reference's loop order;
* the transform's defining property: the atoms of each quadrature are
  orthonormal (interior of the series, to the filter's truncation);
* the TD filters against the reference's own td-amplitude kernel
  (restated bit-exactly in the oracle): the td amplitude of a pixel at delay
  dT equals the transform of the series delayed by dT / L samples.
"""

import math
import os

import numpy as np
import pytest

from conftest import GOLDEN

from oracle import wdm_oracle
from pycwb_gb300 import wdm


@pytest.mark.parametrize("kind", ["cos", "cos2", "sincos"])
@pytest.mark.parametrize("d", [2, 3, 4, 5, 6, 7])
def test_edge_series_matches_cwb_table(kind, d):
    ref = np.load(os.path.join(GOLDEN, "wdm_fourier_tables.npz"))[f"{kind}_{d}"]
    got = wdm.edge_series(kind, d)
    assert got.shape == ref.shape
    # cWB's table carries ~1e-14 error in its j = 1 entries and drops terms
    # below ~3e-15 in two sincos tails
    assert np.abs(got - ref).max() < 3e-14


@pytest.mark.parametrize("M", [1, 2, 8, 16, 64, 512])
@pytest.mark.parametrize("beta,prec", [(2, 6), (4, 10), (6, 12), (7, 8)])
def test_filter_norm_and_length_rule(M, beta, prec):
    f = wdm.wdm_filter(M, M, beta, prec)
    N = f.size
    M2 = 2 * M
    assert (N - 1) % M2 == 0 and N // M2 >= 3
    resid = 1.0 - f[0] ** 2 - 2.0 * np.sum(f[1:] ** 2)
    assert resid <= 10.0 ** -prec
    # the first admissible length: one period shorter fails the norm (or the 3-period floor)
    Ns = N - M2
    if Ns // M2 >= 3:
        assert 1.0 - f[0] ** 2 - 2.0 * np.sum(f[1:Ns] ** 2) > 10.0 ** -prec


@pytest.mark.parametrize("M,beta", [(4, 2), (8, 4), (16, 6), (32, 3)])
def test_filter_closed_form_matches_scalar_loops(M, beta):
    f = wdm.wdm_filter(M, M, beta, 10)
    s = wdm_oracle.get_filter_scalar(M, M, wdm.edge_series("cos", beta), f.size)
    assert np.abs(f - s).max() < 1e-15


def _basis(M, n_ts, filt):
    """Atoms of both quadratures: the transforms of unit impulses."""
    N = wdm.t2w_n_time(n_ts, M)
    A00 = np.zeros((N, M + 1, n_ts))
    A90 = np.zeros_like(A00)
    for s in range(n_ts):
        x = np.zeros(n_ts)
        x[s] = 1.0
        a, b = wdm_oracle.t2w(x, M, filt)
        A00[:, :, s] = a
        A90[:, :, s] = b
    return A00, A90


@pytest.mark.parametrize("M,beta", [(8, 4), (4, 2), (16, 6)])
def test_atoms_orthonormal(M, beta):
    n_ts = 1024 if M < 16 else 2048
    f = wdm.wdm_filter(M, M, beta, 10)
    A00, A90 = _basis(M, n_ts, f)
    N = A00.shape[0]
    nW = f.size
    inner = [n for n in range(N) if n * M - (nW - 1) >= 0 and n * M + nW - 1 < n_ts]
    assert len(inner) >= 8
    for A in (A00, A90):
        R = A[inner][:, 1:M].reshape(-1, n_ts)
        G = R @ R.T
        assert np.abs(G - np.eye(G.shape[0])).max() < 2e-5
        # edge layers: unit norm too (their atoms live at every other slice)
        norms = np.einsum("nms,nms->nm", A[inner], A[inner])
        assert np.abs(norms - 1.0).max() < 1e-9


def test_orthonormality_needs_the_parity_rule():
    """Without the (m + n) alternation of real and imaginary parts the atoms
    of neighbouring slices overlap: the test above does pin the quadrature
    assignment."""
    M = 8
    f = wdm.wdm_filter(M, M, 4, 10)
    n_ts = 512
    N = wdm.t2w_n_time(n_ts, M)
    rows = []
    for s in range(n_ts):
        x = np.zeros(n_ts)
        x[s] = 1.0
        r = wdm_oracle.fold(x, M, f)
        X = np.fft.rfft(r, axis=1)
        rows.append(X.real * math.sqrt(2.0))
    A = np.stack(rows, axis=-1)
    inner = [n for n in range(N) if n * M - (f.size - 1) >= 0 and n * M + f.size - 1 < n_ts]
    R = A[inner][:, 1:M].reshape(-1, n_ts)
    G = R @ R.T
    assert np.abs(G - np.eye(G.shape[0])).max() > 0.1


def _no_nyquist(x):
    X = np.fft.rfft(x)
    X[-1] = 0.0
    return np.fft.irfft(X, x.size)


def _delayed(x, d):
    """x delayed by d samples (periodic, band-limited interpolation)."""
    f = np.fft.rfftfreq(x.size)
    return np.fft.irfft(np.fft.rfft(x) * np.exp(-2j * np.pi * f * d), x.size)


@pytest.mark.parametrize("M,nc,L,beta,tol", [
    (16, 12, 1, 4, 5e-4),
    (32, 16, 1, 4, 1e-4),
    (8, 20, 1, 6, 1e-4),
    (16, 24, 1, 4, 1e-4),
    (16, 12, 2, 4, 5e-4),     # half-sample delays
])
def test_td_filters_reproduce_delays(oracle_mod, M, nc, L, beta, tol):
    rng = np.random.default_rng(M * 100 + nc + L)
    w = wdm.WDM(M, M, beta, 10)
    tb = w.set_td_filter(nc, L)
    assert tb.T0.shape == tb.Tx.shape == (2 * M * L + 1, 2 * nc + 1)
    assert tb.max_delay == M * L
    x = _no_nyquist(rng.standard_normal(8192))
    a00, a90 = wdm_oracle.t2w(x, M, w.filter)
    N = a00.shape[0]
    p00 = np.pad(a00, ((nc, nc), (0, 0))).astype(np.float32)
    p90 = np.pad(a90, ((nc, nc), (0, 0))).astype(np.float32)
    nn, mm = np.meshgrid(np.arange(N // 4, 3 * N // 4), np.arange(M + 1), indexing="ij")
    nn, mm = nn.ravel(), mm.ravel()
    pix = (nn * (M + 1) + mm).astype(np.int32)
    J = tb.max_delay
    K = 2 * J
    v = oracle_mod.batch_get_td_vecs(pix, p00, p90, tb.T0, tb.Tx, M, nc, K, J)
    D = 2 * K + 1
    edge = (mm == 0) | (mm == M)
    ok00 = ~edge | (nn % 2 == 0)        # edge layers: 00 atoms at even slices,
    ok90 = ~edge | (nn % 2 == 1)        # 90 atoms at odd ones (td_vector_kernels.py:128-129)
    if L > 1:
        ok00 &= ~edge                    # no Nyquist content: the top layer is not comparable
        ok90 &= ~edge
    for dT in sorted({1, -1, J // 2, J - 1, J, J + 1, -J, 2 * J - 1, K, -K}):
        b00, b90 = wdm_oracle.t2w(_delayed(x, dT / L), M, w.filter)
        e00 = np.abs(v[:, K + dT] - b00[nn, mm])[ok00].max()
        e90 = np.abs(v[:, D + K + dT] - b90[nn, mm])[ok90].max()
        assert max(e00, e90) < tol, (dT, e00, e90)


def test_errors():
    with pytest.raises(ValueError):
        wdm.WDM(12, 12)
    with pytest.raises(ValueError):
        wdm.WDM(8192, 8192)
    with pytest.raises(ValueError):
        wdm.WDM(16, 16).t2w(np.zeros(100))
    with pytest.raises(ValueError):
        wdm.WDM(16, 16).t2w(np.zeros(10_000), MM=16)
    with pytest.raises(ValueError):
        wdm.WDM(16, 16).td_inputs(np.zeros(10_000))     # no TD filters yet
    with pytest.raises(ValueError):
        wdm.edge_series("cos", 9)


@pytest.mark.parametrize("M,m0", [(16, 5), (32, 20), (8, 1)])
def test_layer_m_holds_frequency_m_df(M, m0):
    """Layer m covers the band around m * rate / (2M) (df = rate / 2M): a
    sinusoid at that frequency puts nearly all of its energy in layer m, and
    the 00 and 90 maps share it evenly."""
    rate = 512.0
    n = 8192
    t = np.arange(n) / rate
    x = np.sin(2 * np.pi * m0 * rate / (2 * M) * t + 0.3)
    w = wdm.WDM(M, M, 4, 10)
    a00, a90 = wdm_oracle.t2w(x, M, w.filter)
    inner = slice(a00.shape[0] // 4, 3 * a00.shape[0] // 4)
    e = (a00[inner] ** 2 + a90[inner] ** 2).sum(axis=0)
    assert e[m0] / e.sum() > 0.99
    assert (a00[inner, m0] ** 2).sum() == pytest.approx((a90[inner, m0] ** 2).sum(), rel=0.05)
