"""Seeded synthetic clusters with the shapes of the sky-scan workloads.

No detector data, WDM library or injection package is available offline,
so the td-amplitude blocks that the sky scan consumes are drawn directly:

* td00/td90: (2K+1, nIFO, n_pix) float32, unit-variance Gaussian noise plus
  a coherent signal of a chosen network SNR projected from one sky
  direction ``l_true``.  The signal sits at delay index ml[i, l_true] + K of
  each detector and leaks into neighbouring delay samples with a Gaussian
  profile (width 1.5 samples), which mimics the time-delay filter response.
* rms: (n_pix, nIFO) float32 normalised inverse-noise weights
  r_i = s_i^-1 / sqrt(sum_k s_k^-2) with per-detector noise s ~ U[0.5, 2],
  the normalisation of pycwb/modules/likelihoodWP/pixel_data.py:60-62.

``regulators`` derives the per-segment constants exactly as
pycwb/modules/likelihoodWP/likelihood_setup.py:133-147 does.
"""

from __future__ import annotations

import math

import numpy as np


def regulators(n_ifo, acore=math.sqrt(2.0), gamma=0.5, delta=0.5, netCC=0.5, netRHO=0.0):
    """Segment constants from the analysis config (likelihood_setup.py:133-147)."""
    network_energy_threshold = 2 * acore * acore * n_ifo
    gamma_regulator = gamma * gamma * 2 / 3
    if delta == 0.0:
        delta = 0.00001
    delta_regulator = abs(delta) if abs(delta) < 1 else 1
    return dict(network_energy_threshold=network_energy_threshold,
                gamma_regulator=gamma_regulator, delta_regulator=delta_regulator,
                netCC=float(netCC), net_rho_threshold=abs(netRHO),
                netEC_threshold=abs(netRHO) * abs(netRHO) * 2)


def subnet_constants(n_ifo, acore=1.7, subcut=0.33):
    """Constants of the sub-network cut (super_cluster.py:575-577,
    sub_net_cut.py:190): network_energy_threshold = float32(2 Acore^2 nIFO)
    and e2or from Acore as cWB's network::setAcore derives it
    (pycwb/types/detector.py:1188-1217): p = Q(nIFO, Acore^2 nIFO) with Q the
    regularised upper incomplete gamma, e2or = Q^-1(nIFO - 1, p)."""
    from scipy.special import gammaincc, gammainccinv
    n = int(max(1, n_ifo))
    if n < 2:
        e2or = float(max(0.0, acore))
    else:
        prob = float(np.clip(gammaincc(float(n), acore * acore * n), 1.0e-12, 1.0 - 1.0e-12))
        e2or = float(gammainccinv(float(n - 1), prob))
    return dict(network_energy_threshold=float(np.float32(2 * acore * acore * n)), e2or=e2or,
                subcut=float(subcut))


def make_rms(rng, n_pix, n_ifo):
    sigma = rng.uniform(0.5, 2.0, size=(n_ifo, n_pix))
    inv = 1.0 / sigma
    norm = 1.0 / np.sqrt(np.sum(inv ** 2, axis=0))
    return np.ascontiguousarray((inv * norm[np.newaxis, :]).astype(np.float32).T)


def make_cluster(rng, ml, FP_t, FX_t, n_pix, K, snr, l_true=None, spread=1.5):
    """One synthetic cluster; returns (td00, td90, rms, l_true)."""
    n_ifo, n_sky = ml.shape
    D = 2 * K + 1
    if l_true is None:
        l_true = int(rng.integers(n_sky))
    rms = make_rms(rng, n_pix, n_ifo)
    td00 = rng.standard_normal((D, n_ifo, n_pix), dtype=np.float32)
    td90 = rng.standard_normal((D, n_ifo, n_pix), dtype=np.float32)

    w = np.exp(rng.standard_normal(n_pix))
    w /= w.sum()
    h = rng.standard_normal((4, n_pix)) * np.sqrt(w)[None, :]   # hp00, hx00, hp90, hx90
    fp = FP_t[l_true].astype(np.float64)
    fx = FX_t[l_true].astype(np.float64)
    r = rms.astype(np.float64)                                   # (n_pix, n_ifo)
    s00 = r * (fp[None, :] * h[0][:, None] + fx[None, :] * h[1][:, None])
    s90 = r * (fp[None, :] * h[2][:, None] + fx[None, :] * h[3][:, None])
    e = float(np.sum(s00 ** 2 + s90 ** 2))
    if e > 0.0:
        scale = snr / math.sqrt(e)
        s00 *= scale
        s90 *= scale
    d = np.arange(D)
    for i in range(n_ifo):
        d0 = int(ml[i, l_true]) + K
        prof = np.exp(-0.5 * ((d - d0) / spread) ** 2)[:, None]
        td00[:, i, :] += (prof * s00[:, i][None, :]).astype(np.float32)
        td90[:, i, :] += (prof * s90[:, i][None, :]).astype(np.float32)
    return td00, td90, rms, l_true


def log_uniform_sizes(rng, n, lo, hi):
    return np.exp(rng.uniform(math.log(lo), math.log(hi), size=n)).astype(np.int64)


def make_batch_device(seed, sizes, ml, FP_t, FX_t, K, snr_lo=8.0, snr_hi=40.0, spread=1.5,
                      device="cuda"):
    """Many clusters at once, generated on the GPU with torch.

    Same model as make_cluster (noise N(0,1), per-pixel weights from
    s ~ U[0.5, 2], a coherent signal of network SNR ~ U[snr_lo, snr_hi] from
    an independent random direction per cluster), laid out for
    ClusterBatch: cluster c's (2K+1, nIFO, P_c) block at td_offsets[c].
    Returns (td00, td90, rms, l_true, snr) as device tensors / numpy.
    """
    import torch

    dev = torch.device(device)
    g = torch.Generator(device=dev)
    g.manual_seed(int(seed))
    rng = np.random.default_rng(seed)
    sizes = np.asarray(sizes, np.int64)
    n = sizes.size
    n_ifo, n_sky = ml.shape
    D = 2 * K + 1
    P_tot = int(sizes.sum())
    pix_off = np.concatenate([[0], np.cumsum(sizes)])
    l_true = rng.integers(n_sky, size=n)
    snr = rng.uniform(snr_lo, snr_hi, size=n)

    cl = torch.from_numpy(np.repeat(np.arange(n), sizes)).to(dev)           # cluster of pixel
    j = torch.arange(P_tot, device=dev) - torch.from_numpy(pix_off[:-1]).to(dev)[cl]
    Pc = torch.from_numpy(sizes).to(dev)[cl]
    td_base = torch.from_numpy(pix_off[:-1] * D * n_ifo).to(dev)[cl]

    sigma = torch.rand((P_tot, n_ifo), generator=g, device=dev, dtype=torch.float64) * 1.5 + 0.5
    inv = 1.0 / sigma
    rms = (inv / torch.sqrt((inv * inv).sum(1, keepdim=True))).to(torch.float32)

    td00 = torch.randn(P_tot * D * n_ifo, generator=g, device=dev, dtype=torch.float32)
    td90 = torch.randn(P_tot * D * n_ifo, generator=g, device=dev, dtype=torch.float32)

    w = torch.exp(torch.randn(P_tot, generator=g, device=dev, dtype=torch.float64))
    wsum = torch.zeros(n, device=dev, dtype=torch.float64).index_add_(0, cl, w)
    w = w / wsum[cl]
    h = torch.randn((4, P_tot), generator=g, device=dev, dtype=torch.float64) * torch.sqrt(w)
    lt = torch.from_numpy(l_true).to(dev)[cl]
    fp = torch.from_numpy(FP_t.astype(np.float64)).to(dev)[lt]             # (P, I)
    fx = torch.from_numpy(FX_t.astype(np.float64)).to(dev)[lt]
    r = rms.to(torch.float64)
    s00 = r * (fp * h[0][:, None] + fx * h[1][:, None])
    s90 = r * (fp * h[2][:, None] + fx * h[3][:, None])
    e = torch.zeros(n, device=dev, dtype=torch.float64).index_add_(
        0, cl, (s00 * s00 + s90 * s90).sum(1))
    scale = torch.from_numpy(snr).to(dev) / torch.sqrt(torch.clamp(e, min=1e-300))
    s00 = s00 * scale[cl][:, None]
    s90 = s90 * scale[cl][:, None]
    d0 = torch.from_numpy(ml.astype(np.int64).T).to(dev)[lt] + K          # (P, I)
    for d in range(D):
        prof = torch.exp(-0.5 * ((d - d0).to(torch.float64) / spread) ** 2)
        for i in range(n_ifo):
            idx = td_base + (d * n_ifo + i) * Pc + j
            td00.index_add_(0, idx, (prof[:, i] * s00[:, i]).to(torch.float32))
            td90.index_add_(0, idx, (prof[:, i] * s90[:, i]).to(torch.float32))
    return td00, td90, rms, l_true, snr


def make_lag(seed, ifos, ml, FP_t, FX_t, *, layers=(16, 32, 64, 128, 256, 512), duration=600.0,
             rate_ana=512, up_tdf=4, n_coeffs=12, n_clusters=1024, size_lo=50, size_hi=5000,
             snr_lo=8.0, snr_hi=40.0, device="cuda"):
    """A synthetic lag for LagPipeline: WDM planes, TD filters and clusters.

    Per resolution M (M+1 layers over duration * rate_ana samples) and
    detector, padded 00/90 planes of unit-variance Gaussian noise (on the
    device) and TD filters T0/Tx of shape (2J+1, 2*n_coeffs+1), J = M * up_tdf:
    T0 carries a unit centre tap tapered with the delay plus small random
    taps, Tx small random taps.  The filters are not the WDM basis's (the
    WDM library is not available offline); they give td amplitudes of the
    right shapes, magnitudes and cost.  Each cluster picks a resolution and
    P ~ log-uniform[size_lo, size_hi] distinct pixels in a compact
    time-frequency box; its pixels carry a coherent signal of network SNR
    ~ U[snr_lo, snr_hi] from a random direction (F+/Fx weighted as in
    make_cluster), added to every detector's planes.
    Returns (planes, cluster_level, cluster_pixels, rms, l_true)."""
    import torch

    from .types.td_batch_inputs import TDBatchInputs

    rng = np.random.default_rng(seed)
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    n_ifo = len(ifos)
    n_sky = ml.shape[1]
    nc = int(n_coeffs)
    planes, shapes = {}, {}
    for M in layers:
        M = int(M)
        n_time = int(duration * rate_ana) // M
        rows = n_time + 2 * nc
        J = M * int(up_tdf)
        d = np.arange(-J, J + 1, dtype=np.float64)
        per = []
        for _ in range(n_ifo):
            p00 = torch.zeros((rows, M + 1), dtype=torch.float32, device=device)
            p90 = torch.zeros_like(p00)
            p00[nc:nc + n_time] = torch.randn((n_time, M + 1), generator=g, device=device)
            p90[nc:nc + n_time] = torch.randn((n_time, M + 1), generator=g, device=device)
            T0 = rng.standard_normal((2 * J + 1, 2 * nc + 1)) * (0.05 / math.sqrt(2 * nc + 1))
            T0[:, nc] += np.cos(0.5 * math.pi * d / J)
            Tx = rng.standard_normal((2 * J + 1, 2 * nc + 1)) * (0.1 / math.sqrt(2 * nc + 1))
            per.append(TDBatchInputs(p00, p90, torch.from_numpy(T0).to(device),
                                     torch.from_numpy(Tx).to(device), M, nc, J))
        planes[M] = per
        shapes[M] = (n_time, M + 1)

    sizes = log_uniform_sizes(rng, n_clusters, size_lo, size_hi)
    level = rng.choice(np.asarray(layers, np.int64), size=n_clusters)
    pixels, rms, l_true = [], [], rng.integers(n_sky, size=n_clusters)
    for c in range(n_clusters):
        M = int(level[c])
        n_time, n_f = shapes[M]
        P = int(min(sizes[c], n_time * n_f // 2))
        wf = int(min(n_f, max(1, math.ceil(math.sqrt(2 * P)))))
        wt = int(min(n_time, math.ceil(2 * P / wf)))
        n0 = int(rng.integers(0, n_time - wt + 1))
        m0 = int(rng.integers(0, n_f - wf + 1))
        box = rng.choice(wt * wf, size=P, replace=False)
        n, m = n0 + box // wf, m0 + box % wf
        idx = (n * n_f + m).astype(np.int32)
        pixels.append(idx)
        r = make_rms(rng, P, n_ifo)
        rms.append(r)
        w = np.exp(rng.standard_normal(P))
        w /= w.sum()
        h = rng.standard_normal((4, P)) * np.sqrt(w)[None, :]
        fp = FP_t[l_true[c]].astype(np.float64)
        fx = FX_t[l_true[c]].astype(np.float64)
        rr = r.astype(np.float64)
        s00 = rr * (fp[None, :] * h[0][:, None] + fx[None, :] * h[1][:, None])
        s90 = rr * (fp[None, :] * h[2][:, None] + fx[None, :] * h[3][:, None])
        e = float(np.sum(s00 ** 2 + s90 ** 2))
        if e > 0.0:
            k = rng.uniform(snr_lo, snr_hi) / math.sqrt(e)
            s00 *= k
            s90 *= k
        rows_t = torch.from_numpy((n + nc).astype(np.int64)).to(device)
        cols_t = torch.from_numpy(m.astype(np.int64)).to(device)
        for i, t in enumerate(planes[M]):
            t.padded00.index_put_((rows_t, cols_t), torch.from_numpy(
                s00[:, i].astype(np.float32)).to(device), accumulate=True)
            t.padded90.index_put_((rows_t, cols_t), torch.from_numpy(
                s90[:, i].astype(np.float32)).to(device), accumulate=True)
    return planes, level, pixels, rms, l_true


def make_strain_lag(seed, ifos, ml, FP_t, FX_t, td_rate, *, layers=(16, 32, 64, 128, 256, 512),
                    duration=600.0, rate=512.0, n_inj=200, n_clusters=1024, size_lo=50,
                    size_hi=5000, snr_lo=8.0, snr_hi=40.0, f_lo=32.0, f_hi=224.0, q=9.0,
                    beta_order=4, precision=10, td_size=12, device="cuda"):
    """A synthetic lag built from strain: LagPipeline inputs through the WDM.

    Every detector gets `duration` s of white unit-variance noise at `rate`
    Hz plus n_inj injections from grid directions l_true: sine-Gaussians
    (f0 ~ U[f_lo, f_hi], quality q, random phase and ellipticity) and, one in
    five, Gaussian pulses (width 4-16 ms), scaled to a network SNR ~
    U[snr_lo, snr_hi].  Detector i sees h(t + ml[i, l_true] / td_rate)
    projected on F+/Fx of the direction, the arrival-time convention of the
    td amplitudes (the amplitude at delay d is that of the series delayed
    by d).  The series are transformed on the device (pycwb_gb300.wdm: every
    level of `layers`, TD filters of 2 td_size + 1 taps at upTDF = td_rate /
    rate), as the reference's td inputs cache does (td_vector_batch.py:35-144).
    The first n_inj clusters are the injections' (pixels: the P loudest of a
    time-frequency box around the injection, at the level whose time step
    best matches the injection's duration, P ~ log-uniform[size_lo,
    10 size_lo]), the others noise boxes at random levels with P ~
    log-uniform[size_lo, size_hi], picked the same way.  rms is 1/sqrt(n_ifo) for every pixel (equal white noise).
    Returns (planes, cluster_level, cluster_pixels, rms, l_true, info);
    l_true is -1 for noise clusters, info carries the injections and the
    transform's device time (t2w_ms)."""
    import torch

    from .wdm import WDM, t2w_n_time

    up = int(round(td_rate / rate))
    if up < 1 or abs(up * rate - td_rate) > 1e-9 * td_rate:
        raise ValueError("td_rate must be an integer multiple of rate")
    rng = np.random.default_rng(seed)
    n_ifo = len(ifos)
    n_sky = ml.shape[1]
    n = int(round(duration * rate))
    x = rng.standard_normal((n_ifo, n))
    t = np.arange(n) / rate
    margin = 4.0
    kinds = np.where(rng.random(n_inj) < 0.8, 0, 1)
    t0s = rng.uniform(margin, duration - margin, n_inj)
    f0s = rng.uniform(f_lo, f_hi, n_inj)
    snrs = rng.uniform(snr_lo, snr_hi, n_inj)
    l_inj = rng.integers(n_sky, size=n_inj)
    taus = np.where(kinds == 0, q / (math.sqrt(2.0) * math.pi * f0s),
                    rng.uniform(0.004, 0.016, n_inj))
    for k in range(n_inj):
        tau = float(taus[k])
        ph, ell = rng.uniform(0, 2 * math.pi), rng.uniform(0.0, 1.0)
        a = max(0, int((t0s[k] - 0.2 - 6 * tau) * rate))
        b = min(n, int((t0s[k] + 0.2 + 6 * tau) * rate) + 1)
        fp = FP_t[l_inj[k]].astype(np.float64)
        fx = FX_t[l_inj[k]].astype(np.float64)
        h = np.zeros((n_ifo, b - a))
        for i in range(n_ifo):
            u = t[a:b] + ml[i, l_inj[k]] / td_rate - t0s[k]
            env = np.exp(-(u / tau) ** 2)
            if kinds[k] == 0:
                hp = env * np.sin(2 * math.pi * f0s[k] * u + ph)
                hx = ell * env * np.cos(2 * math.pi * f0s[k] * u + ph)
            else:
                hp, hx = env, np.zeros_like(env)
            h[i] = fp[i] * hp + fx[i] * hx
        e = float(np.sum(h * h))
        if e > 0.0:
            x[:, a:b] += h * (snrs[k] / math.sqrt(e))

    dev = torch.device(device)
    strains = [torch.from_numpy(x[i]).to(dev) for i in range(n_ifo)]
    s = torch.cuda.current_stream(dev)
    bases = {}
    for M in layers:
        w = WDM(int(M), int(M), beta_order, precision)
        w.set_td_filter(td_size, up)
        bases[int(M)] = w
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s)
    planes = {M: [w.td_inputs(xs, stream=s) for xs in strains] for M, w in bases.items()}
    e1.record(s)
    e1.synchronize()
    t2w_ms = e0.elapsed_time(e1)

    nc = int(td_size)
    energy = {}
    for M, per in planes.items():
        N = t2w_n_time(n, M)
        energy[M] = sum((p.padded00[nc:nc + N].double() ** 2 + p.padded90[nc:nc + N].double() ** 2)
                        for p in per)

    sizes = log_uniform_sizes(rng, n_clusters, size_lo, size_hi)
    level = rng.choice(np.asarray(layers, np.int64), size=n_clusters)
    lay = np.asarray(layers, np.float64)
    for k in range(min(n_inj, n_clusters)):
        # the resolution whose time step best matches the injection's duration
        level[k] = int(lay[np.argmin(np.abs(np.log(lay / rate / (2.0 * taus[k]))))])
    sizes[:n_inj] = log_uniform_sizes(rng, min(n_inj, n_clusters), size_lo,
                                      max(size_lo, min(size_hi, 10 * size_lo)))
    pixels, rms, l_true = [], [], np.full(n_clusters, -1, np.int64)
    for c in range(n_clusters):
        M = int(level[c])
        E = energy[M]
        N, n_f = E.shape
        P = int(min(sizes[c], N * n_f // 2))
        wf = int(min(n_f, max(1, math.ceil(math.sqrt(2 * P)))))
        wt = int(min(N, math.ceil(2 * P / wf)))
        P = min(P, wt * wf)
        if c < n_inj:
            l_true[c] = l_inj[c]
            nc0 = int(round(t0s[c] * rate / M))
            mc0 = int(round(f0s[c] / (rate / (2.0 * M)))) if kinds[c] == 0 else 0
            n0 = int(np.clip(nc0 - wt // 2, 0, N - wt))
            m0 = int(np.clip(mc0 - wf // 2, 0, n_f - wf))
        else:
            n0 = int(rng.integers(0, N - wt + 1))
            m0 = int(rng.integers(0, n_f - wf + 1))
        box = E[n0:n0 + wt, m0:m0 + wf].reshape(-1)
        top = torch.topk(box, P).indices.cpu().numpy()
        nn, mm = n0 + top // wf, m0 + top % wf
        pixels.append((nn * n_f + mm).astype(np.int32))
        rms.append(np.full((P, n_ifo), 1.0 / math.sqrt(n_ifo), np.float32))
    info = {"t0": t0s, "f0": f0s, "snr": snrs, "kind": kinds, "tau": taus, "t2w_ms": t2w_ms,
            "samples": n, "bases": bases}
    return planes, level, pixels, rms, l_true, info
