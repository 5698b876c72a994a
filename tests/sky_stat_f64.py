"""FP64 torch re-implementation of the sky statistic at continuous directions.

Test infrastructure for the gradient kernel (pgw_sky_stat_grad): the same
pipeline as the reference's scan (sky_stat.py:74-405, dpf.py:396-446,
sky_scan.py:131-140) in float64 with torch autograd, so that the kernel's
gradient can be checked against autograd and against central finite
differences.  ``pipeline`` takes per-direction F+/Fx and delayed data and is
itself pinned to the oracle's float64 scan at grid directions
(tests/test_adjoint_f64.py).
"""

import math

import torch

F64 = torch.float64


def direction_inputs(theta, phi, geom):
    """F+ (I,), Fx (I,), tau (I,) for scalar tensors theta, phi; geom (I, 12)."""
    geom = torch.as_tensor(geom, dtype=F64)
    st, ct = torch.sin(theta), torch.cos(theta)
    sp, cp = torch.sin(phi), torch.cos(phi)
    sgha, cgha = -sp, cp            # gha = -phi
    sdec, cdec = ct, st             # dec = pi/2 - theta
    x = torch.stack([-sgha, -cgha, torch.zeros_like(st)])
    y = torch.stack([-cgha * sdec, sgha * sdec, cdec])
    n = torch.stack([st * cp, st * sp, ct])
    D = geom[:, :9].reshape(-1, 3, 3)
    dx = D @ x
    dy = D @ y
    Fp = (x * dx - y * dy).sum(-1)
    Fx = (x * dy + y * dx).sum(-1)
    tau = geom[:, 9:] @ n
    return Fp, Fx, tau


def interpolate(td00, td90, tau, K):
    """v00, v90 (I, P) at continuous delays tau (I,), linear between samples."""
    td00 = torch.as_tensor(td00, dtype=F64)
    td90 = torch.as_tensor(td90, dtype=F64)
    D = 2 * K + 1
    I = td00.shape[1]
    t = torch.clamp(tau, -K, K)
    pos = t + K
    k0 = torch.clamp(torch.floor(pos.detach()).long(), 0, D - 2)
    fr = pos - k0.to(F64)
    idx = torch.arange(I)
    lo0, hi0 = td00[k0, idx], td00[k0 + 1, idx]
    lo9, hi9 = td90[k0, idx], td90[k0 + 1, idx]
    v00 = lo0 + fr[:, None] * (hi0 - lo0)
    v90 = lo9 + fr[:, None] * (hi9 - lo9)
    return v00, v90, fr


def pipeline(Fp, Fx, rms, v00, v90, rr, RR, ethr):
    """Accumulators of the scan for one direction; v00, v90: (I, P)."""
    rms = torch.as_tensor(rms, dtype=F64)             # (P, I)
    v0, v9 = v00.T, v90.T                             # (P, I)
    e = (v0 * v0).sum(1) + (v9 * v9).sum(1) + 1e-12
    mk = e > ethr
    v0, v9, r, et = v0[mk], v9[mk], rms[mk], e[mk]
    f = r * Fp[None, :]
    F = r * Fx[None, :]
    ff, FF, fF = (f * f).sum(1), (F * F).sum(1), (F * f).sum(1)
    si2, co2, AP = 2 * fF, ff - FF, ff + FF
    nn = torch.sqrt(co2 * co2 + si2 * si2)
    cc = co2 / (nn + 1e-9)
    fp = (AP + nn) / 2
    si = torch.sqrt(torch.clamp((1 - cc) / 2, min=0))
    cq = torch.sqrt(torch.clamp((1 + cc) / 2, min=0))
    co = torch.where(si2 > 0, cq, -cq)
    f, F = f * co[:, None] + F * si[:, None], F * co[:, None] - f * si[:, None]
    fFn = (f * F).sum(1) / (fp + 1e-9)
    F = F - f * fFn[:, None]
    fx = (F * F).sum(1)
    ni = ((f * f) ** 2).sum(1) / (fp * fp + 1e-9)
    xp, XP = (v0 * f).sum(1), (v9 * f).sum(1)
    xx, XX = (v0 * F).sum(1), (v9 * F).sum(1)
    eto = et + 1e-9
    g = torch.clamp(torch.sqrt(ni * (xp * xp + XP * XP) / eto) * rr - fp, min=0)
    fd = 1.0 / (fp + g + 1e-9)
    h = (xp * fd) ** 2 + (XP * fd) ** 2
    H2 = xx * xx + XX * XX
    Fd = torch.sqrt(H2 / (h + 1e-9))
    R = 0.1 + RR / eto
    G = torch.clamp(Fd * R - fx, min=0)
    Gd = 1.0 / (fx + G + 1e-9)
    au, AU, av, AV = xp * fd, XP * fd, xx * Gd, XX * Gd
    msk = fd * fp + Gd * fx
    s = f * au[:, None] + F * av[:, None]
    S = f * AU[:, None] + F * AV[:, None]
    a2, A2, aA = (s * s).sum(1), (S * S).sum(1), (s * S).sum(1)
    osi, oco = 2 * aA, a2 - A2
    onn = torch.sqrt(oco * oco + osi * osi)
    occ = oco / (onn + 1e-21)
    sgn = torch.where(osi > 0, 1.0, -1.0).to(F64)
    osi = torch.sqrt(torch.clamp((1 - occ) / 2, min=0))
    oco = torch.sqrt(torch.clamp((1 + occ) / 2, min=0)) * sgn
    s_ = s * oco[:, None] + S * osi[:, None]
    x_ = v0 * oco[:, None] + v9 * osi[:, None]
    S_ = S * oco[:, None] - s * osi[:, None]
    X_ = v9 * oco[:, None] - v0 * osi[:, None]
    q, Q = s_ * x_, S_ * X_
    xs, XS = q.sum(1), Q.sum(1)
    c = (q * q).sum(1) / (xs * xs + 1e-9)
    C = (Q * Q).sum(1) / (XS * XS + 1e-9)
    ss, SS = (s_ * s_).sum(1), (S_ * S_).sum(1)
    rn = ((s - v0) ** 2).sum(1) + ((S - v9) ** 2).sum(1)
    ll = ss + SS
    ec = ss * (1 - c) + SS * (1 - C)
    gn = 2 * msk
    ccn = ec / (2 * torch.abs(ec) + rn + gn + 1e-9)
    margins = {
        "energy": torch.min(torch.abs(e - ethr) / ethr).item() if e.numel() else math.inf,
        "kink_g": torch.min(torch.abs(torch.sqrt(ni * (xp * xp + XP * XP) / eto) * rr - fp)
                            / (fp + 1e-30)).item() if fp.numel() else math.inf,
        "kink_G": torch.min(torch.abs(Fd * R - fx) / (fx + 1e-30)).item() if fx.numel() else math.inf,
    }
    return dict(EE=et.sum(), LL=ll.sum(), Lr=(ll * ccn).sum(), EC=ec.sum(), GN=gn.sum(),
                RN=rn.sum(), Mo=int(mk.sum()), margins=margins)


def tail(acc, n_ifo):
    Eo = acc["EE"] / 2
    Cr = 2 * acc["Lr"] / (acc["LL"] + 1e-9)
    No = (acc["GN"] + acc["RN"]) / 2
    Mo = acc["Mo"]
    CH = No / (n_ifo * Mo + math.sqrt(Mo))
    cc = torch.where(CH > 1, CH, torch.ones_like(CH))
    Co = acc["EC"] / (acc["EC"] + No * cc - Mo * (n_ifo - 1))
    Lk = torch.where(Eo > 0, Eo - No, torch.zeros_like(Eo))
    return dict(statistic=Lk * Co, likelihood=Eo - No, correlation=Co, ellipticity=Cr,
                coherent_energy=acc["EC"], null_energy=No)


def sky_stat(theta, phi, geom, td00, td90, rms, K, rr, RR, ethr):
    """Statistic and outputs at (theta, phi) in float64 (autograd-capable)."""
    Fp, Fx, tau = direction_inputs(theta, phi, geom)
    v00, v90, fr = interpolate(td00, td90, tau, K)
    acc = pipeline(Fp, Fx, rms, v00, v90, rr, RR, ethr)
    out = tail(acc, len(Fp))
    fr = fr.detach()
    moving = torch.as_tensor(geom, dtype=F64)[:, 9:].abs().sum(1) > 0  # the reference never moves
    acc["margins"]["knot"] = (torch.min(torch.minimum(fr, 1 - fr)[moving]).item()
                              if bool(moving.any()) else math.inf)
    out["margins"] = acc["margins"]
    return out
