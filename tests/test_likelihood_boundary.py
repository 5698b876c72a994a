"""Host logic of the reference-signature likelihood entry points (CPU).

pycwb_gb300.likelihoodWP.likelihood.{likelihood_wrapper, likelihood} with
the GPU stage replaced by a fake (as the reference's own contract tests
replace its kernels, pycwb/modules/likelihoodWP/tests/
test_gpu_sky_mask_contract.py:15-93): which clusters reach the GPU, on
which sky grid (the big-cluster switch, likelihood.py:264-283) and mask
(:287-294), how they are grouped into launches, and what happens to the
results -- rejection of sky_stat_max <= 0 (:328-336), the threshold cut
(:367-386), the sky-localisation fields of accepted clusters (:420-445)
and the per-lag result lists (:112-131).
"""

import math
from types import SimpleNamespace

import numpy as np
import pytest

from pycwb_gb300.likelihoodWP import likelihood as lk
from pycwb_gb300.likelihoodWP.detection_statistics import get_likelihood_rejection_reason

N_IFO, K = 3, 2
N_SKY, N_BIG = 48, 12


class _Pixels:
    def __init__(self, P, seed):
        rng = np.random.default_rng(seed)
        self.noise_rms = rng.uniform(0.5, 2.0, (N_IFO, P))
        self._td = rng.standard_normal((P, N_IFO, 2 * (2 * K + 1))).astype(np.float32)
        self.populated = None

    def __len__(self):
        return self.noise_rms.shape[1]

    def td_amp_dense(self):
        return self._td

    def populate_noise_rms(self, nRMS):
        self.populated = nRMS


def _cluster(P, seed, status=0, t=10.0):
    meta = SimpleNamespace(l_max=None, theta=None, phi=None, c_time=0.0, c_freq=0.0)
    return SimpleNamespace(pixel_arrays=_Pixels(P, seed), cluster_status=status,
                           cluster_time=t, cluster_freq=100.0 + P, cluster_meta=meta)


class _XTalk:
    def get_xtalk_pixels(self, pixels, check=True):
        assert check
        return np.zeros((len(pixels), 2), np.int64), np.zeros((0, 8), np.float32)


def _setup(mask=None, big=True):
    rng = np.random.default_rng(0)
    phi = np.linspace(0.0, 2 * math.pi, N_SKY, endpoint=False)
    lat = np.linspace(-1.2, 1.2, N_SKY)
    s = {"network_energy_threshold": 12.0, "xgb_rho_mode": False, "gamma_regulator": 0.1,
         "delta_regulator": 0.5, "net_rho_threshold": 4.0, "netEC_threshold": 32.0, "netCC": 0.5,
         "ml": rng.integers(-K, K + 1, (N_IFO, N_SKY)).astype(np.int32),
         "FP_t": rng.standard_normal((N_SKY, N_IFO)).astype(np.float32),
         "FX_t": rng.standard_normal((N_SKY, N_IFO)).astype(np.float32), "n_sky": N_SKY,
         "healpix_order": None, "phi_geo_arr": phi, "latitude_arr": lat, "ra_arr": phi,
         "dec_arr": lat, "sky_mask_config": mask, "segment_start_gps": 1.26e9,
         "sky_valid_indices": np.arange(N_SKY, dtype=np.int64),
         "ml_big_cluster": None, "sky_valid_indices_big": None}
    if big:
        s.update(ml_big_cluster=rng.integers(-K, K + 1, (N_IFO, N_BIG)).astype(np.int32),
                 FP_big_cluster_t=np.ones((N_BIG, N_IFO), np.float32),
                 FX_big_cluster_t=np.ones((N_BIG, N_IFO), np.float32), n_sky_big_cluster=N_BIG,
                 phi_geo_arr_big_cluster=np.linspace(0.0, 6.0, N_BIG),
                 latitude_arr_big_cluster=np.linspace(-1.0, 1.0, N_BIG),
                 sky_valid_indices_big=np.arange(N_BIG, dtype=np.int64))
    return s


def _stats(**kw):
    base = dict(Gn=1.0, Ec=100.0, Dc=90.0, Rc=0.9, Eh=1.0, Es=50.0, Np=10.0, Em=200.0,
                Lm=150.0, norm=1.0, cc=1.0, rho=9.0, xrho=9.0, Lo=120.0, Eo=160.0,
                N_pix_effective=20.0, S_snr=np.ones(N_IFO))
    base.update(kw)
    return lk.SkyStatistics(**{k: (np.float32(v) if k not in ("N_pix_effective", "S_snr") else v)
                               for k, v in base.items()})


class _FakeGPU:
    """Stands in for _run_group: records each launch and answers per cluster
    from its pixel count P: sky_stat_max = P - 10 (so P <= 10 is rejected),
    l_max = P mod n_sky; P = 13 fails the threshold cut (Lm < 0)."""

    def __init__(self):
        self.launches = []

    def __call__(self, setup, jobs, big, valid, xgb, digest=None):
        self.launches.append((big, valid.tolist(), [j.rms.shape[0] for j in jobs]))
        n_sky = setup["n_sky_big_cluster"] if big else setup["n_sky"]
        out = []
        for j in jobs:
            P = j.rms.shape[0]
            assert j.td00.shape == (2 * K + 1, N_IFO, P) and j.xtalk_lookup.shape == (P, 2)
            smax = float(P - 10)
            if smax <= 0:
                out.append((None, None))
                continue
            maps = tuple(np.full(n_sky, float(s), np.float32) for s in range(11))
            sm = lk.SkyMapStatistics.from_tuple((P % n_sky,) + maps + (smax,))
            sm.nProbability = np.full(n_sky, 1.0 / n_sky, np.float32)
            out.append((sm, _stats(Lm=-1.0 if P == 13 else 150.0)))
        return out


@pytest.fixture
def fake(monkeypatch):
    f = _FakeGPU()
    monkeypatch.setattr(lk, "_run_group", f)
    monkeypatch.setattr(lk, "_skymap_class", lambda: lk.SkyMapStatistics)
    return f


def _config(**kw):
    return SimpleNamespace(nIFO=N_IFO, precision=kw.pop("precision", 0), nRES=kw.pop("nRES", 1),
                           **kw)


def test_wrapper_groups_filters_and_reports_per_lag(fake):
    lag0 = SimpleNamespace(clusters=[_cluster(30, 1), _cluster(5, 2), _cluster(40, 3, status=1),
                                     _cluster(13, 4)])
    lag1 = SimpleNamespace(clusters=[_cluster(25, 5), _cluster(60, 6)])
    res = lk.likelihood_wrapper(_config(), [lag0, lag1], None, None, xtalk=_XTalk(),
                                setup=_setup())
    # one launch: every surviving cluster of both lags shares grid and mask;
    # the cluster with status 1 never reaches it
    assert len(fake.launches) == 1 and fake.launches[0][2] == [30, 5, 13, 25, 60]
    assert [len(r) for r in res] == [1, 2]
    c30, sm30 = res[0][0]
    assert c30 is lag0.clusters[0] and c30.cluster_status == -1 and c30.cluster_id == 1
    assert sm30.sky_stat_max == 20.0 and sm30.l_max == 30 % N_SKY
    # rejected: sky_stat_max <= 0 (P = 5) and the threshold cut (P = 13)
    assert lag0.clusters[1].cluster_status == 0 and lag0.clusters[3].cluster_status == 0
    assert [c.cluster_id for c, _ in res[1]] == [1, 2]


def test_sky_localisation_fields(fake):
    s = _setup()
    cl = _cluster(30, 7)
    got, sm = lk.likelihood(N_IFO, cl, _config(), setup=s, xtalk=_XTalk(), cluster_id=3)
    l = 30 % N_SKY
    assert got is cl and cl.cluster_meta.l_max == l
    assert cl.cluster_meta.theta == pytest.approx(math.degrees(math.pi / 2 - s["latitude_arr"][l]))
    assert cl.cluster_meta.phi == pytest.approx(math.degrees(s["phi_geo_arr"][l]) % 360.0)
    assert cl.sky_time_delay == [float(s["ml"][i, l]) for i in range(N_IFO)]
    # supercluster estimates fill c_time / c_freq left at 0
    assert cl.cluster_meta.c_time == cl.cluster_time and cl.cluster_meta.c_freq == cl.cluster_freq


def test_big_clusters_use_the_coarse_grid(fake):
    s = _setup()
    cfg = _config(precision=65536 * 3 + 20, nRES=2)     # csize = 20, big above 40 pixels
    small, big = _cluster(40, 1), _cluster(41, 2)
    lag = SimpleNamespace(clusters=[small, big])
    res = lk.likelihood_wrapper(cfg, [lag], None, None, xtalk=_XTalk(), setup=s)
    launches = sorted(fake.launches)
    assert launches == [(False, list(range(N_SKY)), [40]), (True, list(range(N_BIG)), [41])]
    assert len(res[0]) == 2
    assert big.sky_time_delay == [float(s["ml_big_cluster"][i, 41 % N_BIG]) for i in range(N_IFO)]
    # without coarse tables there is no switch
    assert not lk.is_big_cluster(cfg, _setup(big=False), 1000)
    assert lk.is_big_cluster(cfg, s, 41) and not lk.is_big_cluster(cfg, s, 40)
    assert not lk.is_big_cluster(_config(precision=65536 * 7), s, 10 ** 6)   # csize 0


def test_icrs_masks_split_launches_by_cluster_time(fake):
    from pycwb_gb300.likelihoodWP.sky_mask import gmst_cwb
    s = _setup(big=False)
    start = s["segment_start_gps"]
    # a Fixed ICRS mask aimed at phi_geo[7] at t = start + 100 s
    ra = (s["phi_geo_arr"][7] + gmst_cwb(start + 100.0)) % (2 * math.pi)
    s["sky_mask_config"] = {"type": "Fixed", "coordsys": "icrs",
                            "coordinates": {"ra": f"{ra} rad", "dec": f"{s['latitude_arr'][7]} rad"}}
    a, b, c = _cluster(30, 1, t=100.0), _cluster(31, 2, t=100.0), _cluster(32, 3, t=100.0 + 3 * 3600)
    lk.likelihood_wrapper(_config(), [SimpleNamespace(clusters=[a, b, c])], None, None,
                          xtalk=_XTalk(), setup=s)
    masks = sorted((tuple(v), p) for _, v, p in fake.launches)
    assert len(masks) == 2 and ((7,), [30, 31]) in masks
    assert [m for m in masks if m[0] != (7,)][0][1] == [32]


def test_empty_mask_rejects_before_the_gpu(fake):
    s = _setup(big=False)
    s["sky_valid_indices"] = np.zeros(0, np.int64)
    got = lk.likelihood(N_IFO, _cluster(30, 1), _config(), setup=s, xtalk=_XTalk())
    assert got == (None, None) and fake.launches == []


def test_post_hook_sees_accepted_clusters_only(fake):
    seen = []
    lag = SimpleNamespace(clusters=[_cluster(30, 1), _cluster(13, 2), _cluster(4, 3)])
    lk.likelihood_wrapper(_config(), [lag], None, None, xtalk=_XTalk(), setup=_setup(),
                          post=lambda cl, st, sm, ctx: seen.append((len(cl.pixel_arrays), ctx["nIFO"])))
    assert seen == [(30, N_IFO)]


def test_nrms_is_passed_to_the_pixels(fake):
    cl = _cluster(30, 1)
    nrms = ["a", "b", "c"]
    lk.likelihood(N_IFO, cl, _config(), setup=_setup(), xtalk=_XTalk(), nRMS=nrms)
    assert cl.pixel_arrays.populated is nrms


def test_argument_errors_match_the_reference():
    cl = _cluster(30, 1)
    with pytest.raises(ValueError, match="xtalk or MRAcatalog"):
        lk.likelihood(N_IFO, cl, _config())
    with pytest.raises(ValueError, match="setup, strains, or supercluster_setup"):
        lk.likelihood(N_IFO, cl, _config(), xtalk=_XTalk())
    with pytest.raises(ValueError, match="config must be provided"):
        lk.likelihood(N_IFO, cl, None, xtalk=_XTalk(), setup=_setup())


@pytest.mark.parametrize("xgb", [False, True])
def test_rejection_reason_cases(xgb):
    ok = _stats()
    assert get_likelihood_rejection_reason(ok, 12.0, 32.0, 4.0, xgb) is None
    assert "Lm" in get_likelihood_rejection_reason(_stats(Lm=0.0), 12.0, 32.0, 4.0, xgb)
    assert "(Eo - Eh)" in get_likelihood_rejection_reason(_stats(Eh=160.0), 12.0, 32.0, 4.0, xgb)
    assert "N < 1" in get_likelihood_rejection_reason(_stats(N_pix_effective=0.5), 12.0, 32.0,
                                                      4.0, xgb)
    if not xgb:
        # Ec Rc / cc = 100 * 0.9 / 1 = 90 against netEC thresholds either side
        assert get_likelihood_rejection_reason(ok, 12.0, 90.5, 4.0, xgb) is not None
        assert get_likelihood_rejection_reason(ok, 12.0, 89.5, 4.0, xgb) is None
    else:
        assert "rho" in get_likelihood_rejection_reason(_stats(rho=3.9), 12.0, 32.0, 4.0, xgb)
        assert "rho" in get_likelihood_rejection_reason(_stats(rho=float("nan")), 12.0, 32.0,
                                                        4.0, xgb)
        # default |netRHO| = sqrt(netEC / 2)
        assert get_likelihood_rejection_reason(_stats(rho=3.9), 12.0, 32.0, None, xgb) is not None
        assert get_likelihood_rejection_reason(_stats(rho=4.1), 12.0, 32.0, None, xgb) is None


def test_mask_digest_memo():
    """One digest per live array object (the per-cluster masks of a call
    usually are the setup's one array), equal digests for equal contents."""
    v = np.arange(1000, dtype=np.int64)
    memo = {}
    d = lk._mask_digest(v, memo)
    assert memo[id(v)] == (v, d) and lk._mask_digest(v, memo) == d
    w = v.copy()
    assert lk._mask_digest(w, memo) == d and len(memo) == 2
    w2 = v[:-1].copy()
    assert lk._mask_digest(w2, memo) != d
    assert lk._mask_digest(v) == d          # without a memo


def test_split_pixel_arrays_of_a_gathered_block():
    """split_pixel_arrays on the records of several clusters gathered into one
    block: each cluster's arrays come from its own rows, in the reference's
    shapes."""
    from pycwb_gb300.likelihoodWP.sky_statistics import split_pixel_arrays
    I = 3
    sizes = [4, 0, 7]
    off = np.concatenate([[0], np.cumsum(sizes)])
    n = int(off[-1])
    r32 = np.arange(n * (9 + 4 * I), dtype=np.float32).reshape(n, -1)
    r64 = np.arange(n * 4 * I, dtype=np.float64).reshape(n, -1) + 0.5
    out = split_pixel_arrays(r32, r64, I, off)
    assert len(out) == 3
    a, b, c = out
    assert a["energy_array_plus"].shape == (4,) and b["pd"].shape == (I, 0)
    np.testing.assert_array_equal(c["energy_array_plus"], r32[4:11, 0])
    np.testing.assert_array_equal(c["noise_amplitude_00"], r32[4:11, 9:9 + I].T)
    np.testing.assert_array_equal(c["f"], r32[4:11, 9 + 2 * I:9 + 3 * I])
    np.testing.assert_array_equal(c["pS"], r64[4:11, 3 * I:4 * I].T)
    np.testing.assert_array_equal(a["p90_POL"], np.stack([r32[0:4, 7], r32[0:4, 8]]))
