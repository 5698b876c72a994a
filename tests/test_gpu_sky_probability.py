"""pgw_sky_probability against NumPy: the reference caller's softmax of the
sky-statistic map (pycwb/modules/likelihoodWP/likelihood.py:338-342,
float64 softmax over all n_sky entries, cast to float32) and the error-region
counts (the directions, largest probability first, holding 50 % / 90 %).

Maps: a peaked statistic spanning hundreds of units (most probabilities far
below float32's range), a flat map, one with masked (zero) directions, one
with a NaN (every probability NaN, as NumPy's max and sum propagate it).
The exponentials are float32-accurate on the device, so probabilities agree
with NumPy's float64 result cast to float32 within 2e-6 relative.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_SKY = 3072
N_STATS = 11


def _smallest_count(p, level):
    """#(p >= t*) with t* the largest value whose upper set holds >= level."""
    v = np.sort(p.astype(np.float64))[::-1]
    cum = np.cumsum(v)
    i = int(np.searchsorted(cum, level, side="left"))
    t = v[min(i, v.size - 1)]
    return int(np.sum(p >= t))


def test_probability_matches_numpy_softmax():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pycwb_gb300 import _lib
    _lib.build()
    L = _lib.load()
    rng = np.random.default_rng(7)
    maps = []
    l = np.arange(N_SKY)
    maps.append(400.0 * np.exp(-0.5 * ((l - 1500) / 40.0) ** 2) + rng.normal(0, 3, N_SKY))
    maps.append(np.full(N_SKY, 2.5))
    m = rng.uniform(0, 60, N_SKY)
    m[rng.random(N_SKY) < 0.7] = 0.0
    maps.append(m)
    m = rng.uniform(0, 10, N_SKY)
    m[17] = np.nan
    maps.append(m)
    n = len(maps)
    stats = np.zeros((n + 1, N_STATS, N_SKY), np.float32)   # cluster 0 unused
    for c, m in enumerate(maps):
        stats[c + 1, 6] = m.astype(np.float32)
    dev = torch.device("cuda")
    st = torch.from_numpy(stats).to(dev)
    sel = torch.arange(1, n + 1, dtype=torch.int32, device=dev)
    prob = torch.empty((n, N_SKY), dtype=torch.float32, device=dev)
    summ = torch.empty((n, 4), dtype=torch.float64, device=dev)
    rc = L.pgw_sky_probability(n, N_SKY, st.data_ptr(), N_STATS * N_SKY, sel.data_ptr(),
                               prob.data_ptr(), summ.data_ptr(),
                               ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, L.pgw_last_error()
    torch.cuda.synchronize()
    got, sm = prob.cpu().numpy(), summ.cpu().numpy()
    for c in range(n):
        s = stats[c + 1, 6].astype(np.float64)
        if np.isnan(s).any():
            assert np.isnan(got[c]).all() and np.isnan(sm[c]).all()
            continue
        e = np.exp(s - s.max())
        ref = (e / e.sum()).astype(np.float32)
        np.testing.assert_allclose(got[c], ref, rtol=2e-6, atol=1e-30)
        assert sm[c, 0] == s.max()
        assert abs(sm[c, 1] - e.sum()) <= 1e-6 * e.sum()
        for k, level in ((2, 0.5), (3, 0.9)):
            want = _smallest_count(got[c], level)
            assert abs(int(sm[c, k]) - want) <= max(2, int(1e-3 * want)), (c, level, sm[c, k], want)
        assert 1 <= sm[c, 2] <= sm[c, 3] <= N_SKY
