"""Threshold cut of the likelihood stage (host side).

get_likelihood_rejection_reason restates
pycwb/modules/likelihoodWP/detection_statistics.py:444-517: a cluster is
rejected when, at its sky maximum,

* 2G statistics:  Lm <= 0, or Eo - Eh <= 0, or Ec Rc / cc < netEC_threshold,
  or N < 1 (N = the effective pixel count of avx_setAMP_ps minus one);
* XGB rho0:       Lm <= 0, or Eo - Eh <= 0, or rho not finite or below
  |netRHO| (default sqrt(netEC_threshold / 2)), or N < 1.

It returns the reason as text, or None when the cluster passes.  The
quantities come from the statistics at the sky maximum (the GPU's
pgw_skystat_batched, or the reference's SkyStatistics: the same names).
"""

from __future__ import annotations

import math


def get_likelihood_rejection_reason(sky_statistics, network_energy_threshold, netEC_threshold,
                                    net_rho_threshold=None, xgb_rho_mode=False):
    s = sky_statistics
    Lm, Eo, Eh, Ec, Rc, cc, rho = s.Lm, s.Eo, s.Eh, s.Ec, s.Rc, s.cc, s.rho
    N = s.N_pix_effective
    c1 = Lm <= 0.0
    c2 = (Eo - Eh) <= 0.0
    c4 = N < 1
    if not xgb_rho_mode:
        c3 = Ec * Rc / cc < netEC_threshold
    else:
        if net_rho_threshold is None:
            net_rho_threshold = (netEC_threshold / 2.0) ** 0.5
        c3 = (not math.isfinite(float(rho))) or rho < net_rho_threshold
    if not (c1 or c2 or c3 or c4):
        return None
    reason = ""
    if c1:
        reason += f"Lm > 0 but Lm = {Lm};"
    if c2:
        reason += f" (Eo - Eh) > 0 but (Eo - Eh) = {Eo - Eh};"
    if c3:
        if not xgb_rho_mode:
            reason += (f" Ec * Rc / cc >= netEC_threshold but Ec * Rc / cc = {Ec * Rc / cc:.4f}"
                       f" < {netEC_threshold:.4f};")
        else:
            reason += f" rho >= |netRHO| but rho = {rho} < {net_rho_threshold};"
    if c4:
        reason += f" N < 1 but N = {N};"
    return reason

