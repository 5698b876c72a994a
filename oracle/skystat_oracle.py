"""Statistics at the sky maximum: a restatement of the reference's
compute_statistics_at_sky_position (pycwb/modules/likelihoodWP/
sky_statistics.py:26-262) and the packet operations it calls
(pycwb/modules/likelihoodWP/packet_ops.py).

TEST INFRASTRUCTURE ONLY: the checker for a future device implementation;
the product never imports it.

The per-pixel part at the direction (delayed data, DPF vectors, energy
mask, GW projection, orthogonalisation, coherent statistics:
sky_statistics.py:94-133) comes from the C oracle
(oracle_direction_pixels_f32, the same arithmetic as its sky scan).  The
packet part follows the reference's NumPy semantics: float32 where it keeps
float32 arrays and scalars (avx_packet_ps; Python floats are weak scalars,
NEP 50), float64 where it converts (the xtalk norms, the noise correction,
the packet amplitudes after avx_setAMP_ps).  Pinned by
tests/golden/skystat_*.npz, written by the reference's own functions.

The xtalk input is the reference's packed form: rows (neighbour index, 3
unused columns, 4 overlap coefficients) and a (start, end) row range per
pixel.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np

from . import oracle as _orc

F32 = np.float32


def direction_pixels(sky_idx, n_ifo, n_pix, FP, FX, rms, td00, td90, ml, REG, ethr):
    """Per-pixel quantities of one direction from the C oracle."""
    L = _orc.lib()
    fn = L.oracle_direction_pixels_f32
    V, i32, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64
    fn.argtypes = [i32, i64, i64, V, V, V, V, V, i32, i64, V, V, ctypes.c_double] + [V] * 19
    fn.restype = ctypes.c_int
    P, I = int(n_pix), int(n_ifo)
    FP = np.ascontiguousarray(FP, np.float32)
    FX = np.ascontiguousarray(FX, np.float32)
    rms = np.ascontiguousarray(rms, np.float32)
    td00 = np.ascontiguousarray(td00, np.float32)
    td90 = np.ascontiguousarray(td90, np.float32)
    ml = np.ascontiguousarray(ml, np.int32)
    REG = np.ascontiguousarray(REG, np.float32)
    o = {k: np.zeros((I, P), np.float32) for k in ("v0", "v9", "s", "S")}
    o.update({k: np.zeros((P, I), np.float32) for k in ("f", "F")})
    o.update({k: np.zeros(P, np.float32) for k in ("fp", "fx", "ni", "et", "msk", "ee", "EE",
                                                    "osi", "oco", "ec", "gn", "rn")})
    o["mk"] = np.zeros(P, np.int32)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    rc = fn(I, P, int(sky_idx), p(FP), p(FX), p(rms), p(td00), p(td90), int(td00.shape[0]),
            int(ml.shape[1]), p(ml), p(REG), ctypes.c_double(float(ethr)),
            *[p(o[k]) for k in ("v0", "v9", "f", "F", "fp", "fx", "ni", "et", "mk", "msk", "s",
                                "S", "ee", "EE", "osi", "oco", "ec", "gn", "rn")])
    if rc != 0:
        raise ValueError(f"oracle_direction_pixels_f32 failed ({rc})")
    return o


def packet(v0, v9, msk):
    """avx_packet_ps (packet_ops.py:659-753), float32 with weak Python floats."""
    I, P = v0.shape
    o = 1e-9
    mk = np.where(msk > 0, F32(1.0), F32(0.0))
    aa = np.zeros(I, F32)
    AA = np.zeros(I, F32)
    aA = np.zeros(I, F32)
    for j in range(I):                         # sequential float32 sums over pixels
        for i in range(P):
            aa[j] += mk[i] * (v0[j, i] * v0[j, i])
            AA[j] += mk[i] * (v9[j, i] * v9[j, i])
            aA[j] += mk[i] * (v0[j, i] * v9[j, i])
    si = np.empty(I, F32)
    co = np.empty(I, F32)
    a = np.empty(I, F32)
    A = np.empty(I, F32)
    E = np.empty(I, F32)
    for j in range(I):
        s2 = F32(2.0) * aA[j]
        c2 = aa[j] - AA[j]
        x = aa[j] + AA[j] + F32(o)
        nn = math.sqrt(float(c2 * c2 + s2 * s2))          # a Python float (double)
        a[j] = math.sqrt(float((x + F32(nn)) / F32(2.0)))
        A[j] = math.sqrt(float(abs((x - F32(nn)) / F32(2.0))))
        cc = c2 / F32(nn + o)
        sg = F32(1.0) if s2 > F32(0.0) else F32(-1.0)
        si[j] = math.sqrt(float((F32(1.0) - cc) / F32(2.0)))
        co[j] = F32(math.sqrt(float((F32(1.0) + cc) / F32(2.0)))) * sg
        E[j] = (a[j] + A[j]) ** 2 / F32(2.0)
    a_save, A_save = a.copy(), A.copy()
    ia = F32(1.0) / (a + F32(o))
    iA = F32(1.0) / (A + F32(o))
    Ep = F32(0.0)
    for j in range(I):
        Ep = Ep + E[j]
    pa = (v0 * co[:, None] + v9 * si[:, None])
    pA = (v9 * co[:, None] - v0 * si[:, None])
    pd = (mk[None, :] * pa * ia[:, None]).astype(F32)
    pD = (mk[None, :] * pA * iA[:, None]).astype(F32)
    return Ep / F32(2.0), pd, pD, E, si, co, a_save, A_save


def _xtalk_terms(p, q, xt, lookup, i):
    r0, r1 = int(lookup[i][0]), int(lookup[i][1])
    rows = xt[r0:r1]
    idx = rows[:, 0].astype(np.int32)
    cc = rows[:, 4:8].T.astype(np.float64)
    pn = p[:, idx].astype(np.float64)
    qn = q[:, idx].astype(np.float64)
    return pn @ cc[0], pn @ cc[1], qn @ cc[2], qn @ cc[3]


def packet_norm(p, q, xt, lookup, msk, q_E):
    """packet_norm_numpy (packet_ops.py:814-901): xtalk-corrected per-detector
    norms (clamped at 2), per-pixel norms and the halo noise."""
    I, P = p.shape
    q_norm = np.zeros((I, P))
    norm = np.zeros(I)
    rn = np.zeros(P)
    for i in range(P):
        if msk[i] <= 0.0:
            continue
        x0, x1, x2, x3 = _xtalk_terms(p, q, xt, lookup, i)
        pi = p[:, i].astype(np.float64)
        qi = q[:, i].astype(np.float64)
        t = x0 * pi + x1 * qi + x2 * pi + x3 * qi
        t = np.where(t < 0, 0.0, t)
        norm += t
        e = (pi * pi + qi * qi) / (t + 1e-12)
        q_norm[:, i] = np.where(e >= 1, 0.0, e)
        u, v = x0 + x2, x1 + x3
        rn[i] = np.sum(u * u + v * v)
    norm = np.where(norm < 2.0, 2.0, norm)
    return q_E.astype(np.float64) * 2.0 / norm, norm, rn, q_norm


def xtalk_energy(p, q, xt, lookup, msk):
    """xtalk_energy_sum_numpy (packet_ops.py:756-810): the unclamped sum."""
    I, P = p.shape
    g = np.zeros(I)
    for i in range(P):
        if msk[i] <= 0.0:
            continue
        x0, x1, x2, x3 = _xtalk_terms(p, q, xt, lookup, i)
        pi = np.asarray(p[:, i], np.float64)
        qi = np.asarray(q[:, i], np.float64)
        t = x0 * pi + x1 * qi + x2 * pi + x3 * qi
        g += np.where(t > 0.0, t, 0.0)
    return float(np.sum(g))


def signal_norms(q_norm, q_E, p_E, ec):
    """gw_norm_numpy (packet_ops.py:905-948): (total SNR, per-detector SNR
    2 p_E / q_E, the data norms q_E, the signal pixel norms)."""
    snr = (np.asarray(p_E) * 2) / np.asarray(q_E, np.float64)
    p_norm = np.where(np.asarray(ec)[None, :] > 0, q_norm, 0.0)
    return float(np.sum(snr)), snr, np.asarray(q_E, np.float64).copy(), p_norm


def null_packet(d, D, h, H):
    """avx_loadNULL_ps (packet_ops.py:333-361): data minus signal, float32."""
    return (np.asarray(d, F32) - np.asarray(h, F32), np.asarray(D, F32) - np.asarray(H, F32))


def noise_correction(p_norm, q_norm, et, msk, ec, gn, rn):
    """avx_noise_ps (packet_ops.py:93-231); gn is updated in place."""
    I = p_norm.shape[0]
    ns = np.asarray(p_norm, np.float64).sum(axis=0) / I
    nx = np.asarray(q_norm, np.float64).sum(axis=0) / I
    mk = (msk > 0).astype(np.float64)
    core = mk * (nx > 0).astype(np.float64)
    EC = float(np.sum(core * ec))
    NC = float(np.sum(core))
    ES = float(np.sum((mk - core) * rn))
    rc = np.where(gn < 2.0, 1.0, 0.0)
    rc = rc + gn * (1.0 - rc) * 0.5
    rc = ec / (rc + 1e-9)
    sig = mk * (ns > 0).astype(np.float64)
    gn[:] = mk * gn * nx
    SC = float(np.sum(sig * ec))
    RC = float(np.sum(sig * rc))
    GN = float(np.sum(sig * gn))
    NS = float(np.sum(sig))
    EH = float(np.sum((mk - sig) * et))
    return GN, EC, SC - EC, RC / (SC + 0.01), EH / 2, ES / 2, NC, NS


def set_amplitudes(p, q, q_norm, si, co, a, A, msk):
    """avx_setAMP_ps (packet_ops.py:234-330): float64 amplitudes."""
    I = p.shape[0]
    mk = 0.5 * (msk > 0).astype(p.dtype)
    n = (a + A)[:, None] * mk[None, :] * q_norm
    new_p = n * (p * co[:, None] - q * si[:, None])
    new_q = n * (q * co[:, None] + p * si[:, None])
    Np = float(np.sum(q_norm.sum(axis=0) * mk))
    return Np * 4 / I, new_p, new_q


def polar(p, q, msk, fp, fx, f, F):
    """The deterministic outputs of avx_pol_ps (packet_ops.py:564-655): the
    network-plane radius and angle of both quadratures."""
    o = 1e-9
    mk = (msk > 0).astype(np.float64)
    mp = np.asarray(p, np.float64) * mk[None, :]
    mq = np.asarray(q, np.float64) * mk[None, :]
    f64, F64 = np.asarray(f, np.float64), np.asarray(F, np.float64)
    xp, XP = (f64 * mp.T).sum(axis=1), (f64 * mq.T).sum(axis=1)
    xx, XX = (F64 * mp.T).sum(axis=1), (F64 * mq.T).sum(axis=1)
    fp64, fx64 = np.asarray(fp, np.float64), np.asarray(fx, np.float64)
    sfp, sfx = np.sqrt(fp64) + o, np.sqrt(fx64) + o
    r = np.sqrt(xp * xp / (fp64 + o) + xx * xx / (fx64 + o)).astype(F32)
    R = np.sqrt(XP * XP / (fp64 + o) + XX * XX / (fx64 + o)).astype(F32)
    return (r, np.arctan2(xx / sfx, xp / sfp).astype(F32)), \
        (R, np.arctan2(XX / sfx, XP / sfp).astype(F32))


def statistics_at_sky_position(sky_idx, n_ifo, n_pix, FP, FX, rms, td00, td90, ml, REG,
                               network_energy_threshold, xtalk, xtalk_lookup,
                               xgb_rho_mode=False):
    """Scalars and arrays of SkyStatistics (sky_statistics.py:94-262) as a dict."""
    d = direction_pixels(sky_idx, n_ifo, n_pix, FP, FX, rms, td00, td90, ml, REG,
                         network_energy_threshold)
    I = int(n_ifo)
    msk, et, ec = d["msk"], d["et"], d["ec"]
    gn = d["gn"].copy()
    Eo, pd, pD, E_d, si_d, co_d, a_d, A_d = packet(d["v0"], d["v9"], msk)
    Lo, ps, pS, E_s, si_s, co_s, a_s, A_s = packet(d["s"], d["S"], msk)
    _, norm_d, rn_x, qn_d = packet_norm(pd, pD, xtalk, xtalk_lookup, msk, E_d)
    _, s_snr, _, p_norm = signal_norms(qn_d, norm_d, E_s, ec)
    Gn, Ec, Dc, Rc, Eh, Es, NC, NS = noise_correction(p_norm, qn_d, et, msk, ec, gn, rn_x)
    N_eff, pd, pD = set_amplitudes(pd, pD, qn_d, si_d, co_d, a_d, A_d, msk)
    N_eff = N_eff - 1
    _, ps, pS = set_amplitudes(ps, pS, p_norm, si_s, co_s, a_s, A_s, msk)
    n00, n90 = null_packet(pd, pD, ps, pS)
    Em = xtalk_energy(pd, pD, xtalk, xtalk_lookup, msk)
    Np = xtalk_energy(n00, n90, xtalk, xtalk_lookup, msk)
    Lm = Em - Np - Gn
    norm = (Eo - F32(Eh)) / F32(Em) if Em > 0 else 1.e9
    if norm < 1:
        norm = 1
    if isinstance(norm, np.floating):            # a float32 ratio: the quotient is float32
        Ec, Dc = F32(Ec) / norm, F32(Dc) / norm
    else:                                        # the int 1 or the float 1e9
        Ec, Dc = Ec / norm, Dc / norm
    ch = (Np + Gn) / (N_eff * I)
    xrho = 0.0
    cc = ch if ch > 1 else 1
    if not xgb_rho_mode:
        rho = np.sqrt(Ec * Rc / 2.) if Ec > 0 else 0
    else:
        rho = (np.sqrt(Ec / (1 + ch * (max(1.0, ch) - 1))) if Ec > 0 else 0)
        xrho = np.sqrt(Ec * Rc / 2.) if Ec > 0 else 0
    pol00, pol90 = polar(d["v0"], d["v9"], msk, d["fp"], d["fx"], d["f"], d["F"])
    scalars = dict(Gn=Gn, Ec=Ec, Dc=Dc, Rc=Rc, Eh=Eh, Es=Es, Np=Np, Em=Em, Lm=Lm, norm=norm,
                   cc=cc, rho=rho, xrho=xrho, Lo=Lo, Eo=Eo)
    out = {k: np.float32(v) for k, v in scalars.items()}
    out.update(N_pix_effective=N_eff, energy_array_plus=d["ee"], energy_array_cross=d["EE"],
               pixel_mask=msk, gaussian_noise_correction=gn, coherent_energy=ec,
               noise_amplitude_00=n00, noise_amplitude_90=n90, pd=pd, pD=pD, ps=ps, pS=pS,
               p00_POL=pol00, p90_POL=pol90, S_snr=s_snr, f=d["f"], F=d["F"])
    return out
