"""WDM forward transform on the GPU (pgw_wdm_t2w) against the oracle.

Both compute in float64; the device folds with FMAs and runs its own
radix-2 FFT, the oracle sums products and calls numpy's FFT, so the maps
agree to rounding: |gpu - oracle| <= 1e-12 max|oracle|.  The padded
float32 planes must be the float32 rounding of the device's own maps, bit
for bit, with zero padding rows.  End to end, td vectors built on the
device from a strain series must match the oracle chain (oracle transform
-> float32 planes -> oracle td vectors) up to the planes' float32 rounding.
"""

import numpy as np
import pytest

from oracle import wdm_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wdm_mod():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pycwb_gb300 import _lib, wdm
    _lib.build()
    return wdm


@pytest.mark.parametrize("M,n_ts,beta", [
    (1, 1000, 4), (2, 4099, 2), (16, 20_000, 4), (64, 70_001, 6), (512, 300_000, 4),
    (1024, 400_003, 4), (4096, 600_000, 4),
])
def test_t2w_matches_oracle(wdm_mod, M, n_ts, beta):
    rng = np.random.default_rng(M + n_ts)
    x = rng.standard_normal(n_ts)
    w = wdm_mod.WDM(M, M, beta, 10)
    out = w.t2w(x, sample_rate=512.0, t0=3.0)
    r00, r90 = wdm_oracle.t2w(x, M, w.filter)
    assert out.n_time == r00.shape[0] == -(-n_ts // M)
    assert out.dt == M / 512.0 and out.df == 256.0 / M
    g00, g90 = out.map00.cpu().numpy(), out.map90.cpu().numpy()
    scale = max(np.abs(r00).max(), np.abs(r90).max())
    assert np.abs(g00 - r00).max() <= 1e-12 * scale
    assert np.abs(g90 - r90).max() <= 1e-12 * scale
    d = out.data
    assert d.shape == (M + 1, out.n_time) and np.array_equal(d.real, g00.T)


@pytest.mark.parametrize("M,nc", [(16, 12), (256, 6), (1, 3)])
def test_padded_planes_are_the_maps(wdm_mod, M, nc):
    import torch
    x = np.random.default_rng(M).standard_normal(50_000)
    w = wdm_mod.WDM(M, M, 4, 10)
    w.set_td_filter(nc, 1)
    m = w.t2w(x)
    td = w.td_inputs(x)
    N = m.n_time
    assert tuple(td.padded00.shape) == (N + 2 * nc, M + 1)
    for p, full in ((td.padded00, m.map00), (td.padded90, m.map90)):
        assert torch.equal(p[nc:nc + N], full.to(torch.float32))
        assert not p[:nc].any() and not p[nc + N:].any()
    ref = m.prepare_td_inputs(w.td_filters)
    assert torch.equal(ref.padded00, td.padded00) and torch.equal(ref.padded90, td.padded90)


def test_strain_to_td_vectors(wdm_mod, oracle_mod):
    """T2 then T1 on the device from one strain series, against the oracle chain."""
    M, nc, L, K = 32, 12, 4, 100
    x = np.random.default_rng(5).standard_normal(200_000)
    w = wdm_mod.WDM(M, M, 4, 10)
    tb = w.set_td_filter(nc, L)
    td = w.td_inputs(x)
    rng = np.random.default_rng(6)
    N = wdm_mod.t2w_n_time(x.size, M)
    pix = rng.choice(N * (M + 1), size=3000, replace=False).astype(np.int32)
    got = td.extract_td_vecs(pix, K)
    r00, r90 = wdm_oracle.t2w(x, M, w.filter)
    p00 = np.pad(r00, ((nc, nc), (0, 0))).astype(np.float32)
    p90 = np.pad(r90, ((nc, nc), (0, 0))).astype(np.float32)
    ref = oracle_mod.batch_get_td_vecs(pix, p00, p90, tb.T0, tb.Tx, M, nc, K, tb.max_delay)
    assert got.shape == ref.shape == (pix.size, 4 * K + 2)
    # planes may differ by one float32 ulp where the two FFTs round differently
    assert np.abs(got - ref).max() <= 1e-5 * max(1.0, np.abs(ref).max())


def test_rejects_bad_shapes(wdm_mod):
    import ctypes

    import torch

    from pycwb_gb300 import _lib
    L = _lib.load()
    x = torch.zeros(10_000, dtype=torch.float64, device="cuda")
    f = torch.zeros(33, dtype=torch.float64, device="cuda")
    out = torch.zeros((700, 17), dtype=torch.float64, device="cuda")
    P = ctypes.c_void_p
    # M not a power of two / filter length not 1 + k 2M / series too short / no output
    for M, nf, n, o in ((12, 33, 10_000, out), (16, 40, 10_000, out), (16, 33, 20, out),
                        (16, 33, 10_000, None)):
        op = P(o.data_ptr()) if o is not None else None
        rc = L.pgw_wdm_t2w(P(x.data_ptr()), n, M, P(f.data_ptr()), nf, op, op, None, None, 0,
                           None)
        assert rc == 1 or rc == 2
    assert L.pgw_wdm_n_time(1000, 16) == 63 and L.pgw_wdm_n_time(1024, 16) == 64
