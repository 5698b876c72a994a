"""Generate golden input/output vectors by running PycWB's own kernels.

The reference's hot-path kernel files import only numpy, math and numba:

* pycwb/modules/likelihoodWP/dpf.py       (calculate_dpf, dpf_np_loops_vec)
* pycwb/modules/likelihoodWP/sky_stat.py  (load_data_from_td, avx_GW_ps, ...)
* pycwb/modules/likelihoodWP/sky_scan.py  (scan_sky_for_best_fit)
* pycwb/utils/td_vector_kernels.py        (batch_get_td_vecs)

numba is not installed here, so this script installs a small stand-in
module under the name ``numba``: ``njit`` returns the Python function,
``prange`` is ``range``, ``vectorize`` casts scalar arguments and the result
to the declared signature, and the type objects (``float32`` ...) construct
NumPy scalars and carry a ``.dtype``.  The reference files are then loaded
unmodified by file path and executed with NumPy scalar semantics.  The
outputs are written as ``.npz`` fixtures next to this script.

Also pycwb/modules/super_cluster_native/sub_net_cut.py (the sub-network-cut
sky loop, optimze_sky_loc_from_td), whose other imports are given empty
modules.

Also pycwb/modules/likelihoodWP/sky_statistics.py (statistics at the sky
maximum, compute_statistics_at_sky_position) with its packet operations,
on synthetic xtalk overlaps (the overlap catalog is not in the checkout).

Usage (needs the reference checkout; not used at test time)::

    python tests/golden/make_golden.py /path/to/pycwb-reference [subnet|skystat]
"""

from __future__ import annotations

import importlib.util
import math
import os
import sys
import types
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)


# --------------------------------------------------------------------------
# numba stand-in
# --------------------------------------------------------------------------
class _NbType:
    def __init__(self, np_type):
        self.np_type = np_type
        self.dtype = np.dtype(np_type)

    def __call__(self, *args):
        if args and all(isinstance(a, _NbType) for a in args):
            return (self, args)  # a signature: (return type, argument types)
        return self.np_type(*args)

    def __getitem__(self, item):  # array type spelling, e.g. float32[:]
        return self


def _install_numba_stub():
    nb = types.ModuleType("numba")

    def njit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    def vectorize(sigs, **kwargs):
        ret_t, arg_ts = sigs[0]

        def deco(f):
            def wrapped(*a):
                cast = [t.np_type(x) for t, x in zip(arg_ts, a)]
                return ret_t.np_type(f(*cast))
            return wrapped
        return deco

    def guvectorize(sigs, layout, **kwargs):
        return lambda f: f

    nb.njit = njit
    nb.jit = njit
    nb.vectorize = vectorize
    nb.guvectorize = guvectorize
    nb.prange = range
    for name, t in (("float32", np.float32), ("float64", np.float64),
                    ("int32", np.int32), ("int64", np.int64),
                    ("uint32", np.uint32)):
        setattr(nb, name, _NbType(t))
    sys.modules["numba"] = nb


def _load(name, path, package=None):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    if package:
        mod.__package__ = package
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def load_reference(ref_root):
    _install_numba_stub()
    lwp = os.path.join(ref_root, "pycwb", "modules", "likelihoodWP")
    pkg = types.ModuleType("ref_lwp")
    pkg.__path__ = [lwp]
    sys.modules["ref_lwp"] = pkg
    dpf = _load("ref_lwp.dpf", os.path.join(lwp, "dpf.py"), "ref_lwp")
    stat = _load("ref_lwp.sky_stat", os.path.join(lwp, "sky_stat.py"), "ref_lwp")
    scan = _load("ref_lwp.sky_scan", os.path.join(lwp, "sky_scan.py"), "ref_lwp")
    tdk = _load("ref_tdk", os.path.join(ref_root, "pycwb", "utils", "td_vector_kernels.py"))
    return dpf, stat, scan, tdk


def load_subnet(ref_root, dpf):
    """pycwb/modules/super_cluster_native/sub_net_cut.py under the stand-in.

    Its module-level imports outside numpy/numba (the xtalk catalog reader,
    pixel_data) serve other functions of the file; they get empty modules,
    and `pycwb.modules.likelihoodWP.dpf` resolves to the reference's dpf.py
    loaded above."""
    for name in ("pycwb", "pycwb.modules", "pycwb.modules.likelihoodWP", "pycwb.modules.xtalk",
                 "pycwb.modules.super_cluster_native"):
        m = types.ModuleType(name)
        m.__path__ = []
        sys.modules[name] = m
    sys.modules["pycwb.modules.likelihoodWP.dpf"] = dpf
    for name, attrs in (("pycwb.modules.xtalk.monster", ("getXTalk_pixels_fast",)),
                        ("pycwb.modules.xtalk.type", ("XTalk",)),
                        ("pycwb.modules.likelihoodWP.pixel_data", ("load_data_from_pixels",))):
        m = types.ModuleType(name)
        for a in attrs:
            setattr(m, a, object)
        sys.modules[name] = m
    path = os.path.join(ref_root, "pycwb", "modules", "super_cluster_native", "sub_net_cut.py")
    return _load("pycwb.modules.super_cluster_native.sub_net_cut", path,
                 "pycwb.modules.super_cluster_native")


# --------------------------------------------------------------------------
# cases
# --------------------------------------------------------------------------
def _sky_case(name, ifos, healpix_order, n_pix, K, seed, snr=15.0, valid=None,
              netCC=0.5, delta=0.5, gamma=0.5, acore=math.sqrt(2.0),
              random_tables=False, n_sky=None, delta_regulator=None):
    from pycwb_gb300.synthetic import make_cluster, regulators
    from pycwb_gb300 import sky

    rng = np.random.default_rng(seed)
    n_ifo = len(ifos)
    if random_tables:
        n_sky = int(n_sky)
        ml = rng.integers(-K, K + 1, size=(n_ifo, n_sky)).astype(np.int32)
        ml[0] = 0
        FP = rng.uniform(-1, 1, size=(n_ifo, n_sky))
        FX = rng.uniform(-1, 1, size=(n_ifo, n_sky))
    else:
        ml, FP, FX = sky.compute_sky_delay_and_patterns(
            ifos, ifos[0], 512.0, K, healpix_order=healpix_order)
        n_sky = ml.shape[1]
    FP_t = FP.T.astype(np.float32).copy()
    FX_t = FX.T.astype(np.float32).copy()
    td00, td90, rms, l_true = make_cluster(rng, ml, FP_t, FX_t, n_pix, K, snr)
    reg = regulators(n_ifo, acore=acore, gamma=gamma, delta=delta, netCC=netCC)
    if delta_regulator is not None:
        # scan_sky_for_best_fit takes any delta_regulator; a negative one
        # selects the likelihood-only sky statistic (sky_scan.py:141)
        reg["delta_regulator"] = delta_regulator
    if valid is None:
        valid = np.arange(n_sky, dtype=np.int64)
    return dict(name=name, n_ifo=n_ifo, n_pix=n_pix, n_sky=n_sky, FP=FP_t, FX=FX_t,
                rms=rms, td00=td00, td90=td90, ml=ml, valid=np.asarray(valid, np.int64),
                netCC=reg["netCC"], delta_regulator=reg["delta_regulator"],
                gamma_regulator=reg["gamma_regulator"],
                network_energy_threshold=reg["network_energy_threshold"],
                l_true=l_true)


def run_sky_case(ref, case):
    dpf, _, scan, _ = ref
    REG = np.array([case["delta_regulator"] * np.sqrt(2), 0.0, 0.0], dtype=np.float32)
    REG[1] = dpf.calculate_dpf(case["FP"], case["FX"], case["rms"], case["n_sky"],
                               case["n_ifo"], case["gamma_regulator"],
                               case["network_energy_threshold"], case["valid"])
    out = scan.scan_sky_for_best_fit(
        case["n_ifo"], case["n_pix"], case["n_sky"], case["FP"], case["FX"], case["rms"],
        case["td00"], case["td90"], case["ml"], REG, case["netCC"],
        case["delta_regulator"], case["network_energy_threshold"], case["valid"])
    res = dict(REG=REG, l_max=np.int64(out[0]), sky_stat_max=np.float64(out[12]),
               stats=np.stack([np.asarray(a, np.float32) for a in out[1:12]]))
    return res


def _td_case(name, seed, M, n_coeffs, L, K, n_time, n_pix):
    rng = np.random.default_rng(seed)
    J = M * L
    rows = n_time + 2 * n_coeffs
    padded00 = np.zeros((rows, M + 1), np.float32)
    padded90 = np.zeros((rows, M + 1), np.float32)
    padded00[n_coeffs:n_coeffs + n_time] = rng.standard_normal((n_time, M + 1))
    padded90[n_coeffs:n_coeffs + n_time] = rng.standard_normal((n_time, M + 1))
    T0 = rng.standard_normal((2 * J + 1, 2 * n_coeffs + 1)) * 0.3
    Tx = rng.standard_normal((2 * J + 1, 2 * n_coeffs + 1)) * 0.1
    # keep every tap row in range: n_eff = n - wdm_shift stays in [0, n_time)
    max_shift = (K + J - 1) // J
    n = rng.integers(max_shift, n_time - max_shift, size=n_pix)
    m = rng.integers(0, M + 1, size=n_pix)
    m[:4] = [0, 1, M - 1, M]  # edge layers
    idx = (n * (M + 1) + m).astype(np.int32)
    return dict(name=name, pixel_indices=idx, padded00=padded00, padded90=padded90,
                T0=T0, Tx=Tx, M=np.int64(M), n_coeffs=np.int64(n_coeffs),
                K=np.int64(K), J=np.int64(J))


def _subnet_case(name, ifos, healpix_order, n_pix, K, seed, snr=20.0, acore=1.7, subcut=0.33,
                 random_tables=False, n_sky=None):
    from pycwb_gb300.synthetic import make_cluster, subnet_constants
    from pycwb_gb300 import sky

    rng = np.random.default_rng(seed)
    n_ifo = len(ifos)
    if random_tables:
        n_sky = int(n_sky)
        ml = rng.integers(-K, K + 1, size=(n_ifo, n_sky)).astype(np.int32)
        ml[0] = 0
        FP = rng.uniform(-1, 1, size=(n_ifo, n_sky))
        FX = rng.uniform(-1, 1, size=(n_ifo, n_sky))
    else:
        ml, FP, FX = sky.compute_sky_delay_and_patterns(
            ifos, ifos[0], 512.0, K, healpix_order=healpix_order)
        n_sky = ml.shape[1]
    FP_t = FP.T.astype(np.float32).copy()
    FX_t = FX.T.astype(np.float32).copy()
    td00, td90, rms, l_true = make_cluster(rng, ml, FP_t, FX_t, n_pix, K, snr)
    c = subnet_constants(n_ifo, acore=acore, subcut=subcut)
    return dict(name=name, n_ifo=n_ifo, n_pix=n_pix, n_sky=n_sky, FP=FP_t, FX=FX_t, rms=rms,
                td00=td00, td90=td90, ml=ml, network_energy_threshold=np.float32(
                    c["network_energy_threshold"]), e2or=np.float64(c["e2or"]),
                subcut=np.float64(c["subcut"]), l_true=l_true)


def run_subnet_case(snc, case):
    out = snc.optimze_sky_loc_from_td(
        case["n_ifo"], case["n_pix"], case["n_sky"], case["FP"], case["FX"], case["rms"],
        case["td00"], case["td90"], case["ml"], case["network_energy_threshold"],
        float(case["e2or"]), float(case["subcut"]))
    return dict(out=np.array([float(x) for x in out], np.float64))


def main(ref_root):
    ref = load_reference(ref_root)
    sky_cases = [
        _sky_case("hlv_o2_p40", ["L1", "H1", "V1"], 2, 40, 20, seed=11),
        _sky_case("hlv_o3_p24_subset", ["L1", "H1", "V1"], 3, 24, 20, seed=12,
                  valid=np.sort(np.random.default_rng(5).choice(768, 300, replace=False))),
        _sky_case("hlvk_o2_p30", ["L1", "H1", "V1", "K1"], 2, 30, 20, seed=13, snr=25.0),
        _sky_case("hl_o2_p32", ["L1", "H1"], 2, 32, 20, seed=14),
        _sky_case("hlv_o2_p40_deltaneg", ["L1", "H1", "V1"], 2, 40, 20, seed=15,
                  delta_regulator=-0.3, netCC=0.0),
        _sky_case("hlv_o2_p1", ["L1", "H1", "V1"], 2, 1, 20, seed=16, snr=8.0, netCC=0.0),
        _sky_case("rand_s150_p50", ["L1", "H1", "V1"], None, 50, 20, seed=17,
                  random_tables=True, n_sky=150, netCC=0.3),
        _sky_case("hlv_o2_p40_netcc09", ["L1", "H1", "V1"], 2, 40, 20, seed=18, netCC=0.9),
        _sky_case("hlv_o2_p20_k8", ["L1", "H1", "V1"], 2, 20, 8, seed=19),
    ]
    for case in sky_cases:
        res = run_sky_case(ref, case)
        path = os.path.join(HERE, f"sky_{case['name']}.npz")
        np.savez_compressed(path, **{k: v for k, v in case.items() if k != "name"}, **res)
        print(case["name"], "l_max", int(res["l_max"]), "stat", float(res["sky_stat_max"]),
              "REG1", float(res["REG"][1]), "->", os.path.relpath(path, REPO))

    tdk = ref[3]
    td_cases = [
        _td_case("m16_nc6_l1_k8", 21, M=16, n_coeffs=6, L=1, K=8, n_time=40, n_pix=64),
        _td_case("m8_nc5_l1_k12", 22, M=8, n_coeffs=5, L=1, K=12, n_time=40, n_pix=48),
        _td_case("m8_nc4_l2_k20", 23, M=8, n_coeffs=4, L=2, K=20, n_time=40, n_pix=48),
        _td_case("m4_nc3_l1_k9", 24, M=4, n_coeffs=3, L=1, K=9, n_time=30, n_pix=32),
    ]
    for case in td_cases:
        out = tdk.batch_get_td_vecs(case["pixel_indices"], case["padded00"], case["padded90"],
                                    case["T0"], case["Tx"], int(case["M"]),
                                    int(case["n_coeffs"]), int(case["K"]), int(case["J"]))
        path = os.path.join(HERE, f"td_{case['name']}.npz")
        np.savez_compressed(path, **{k: v for k, v in case.items() if k != "name"},
                            out=np.asarray(out, np.float32))
        print(case["name"], out.shape, "->", os.path.relpath(path, REPO))


def main_subnet(ref_root):
    ref = load_reference(ref_root)
    snc = load_subnet(ref_root, ref[0])
    cases = [
        _subnet_case("hlv_o2_p60", ["L1", "H1", "V1"], 2, 60, 20, seed=31),
        _subnet_case("hlv_o3_p40_nocut", ["L1", "H1", "V1"], 3, 40, 20, seed=32, subcut=-1.0),
        _subnet_case("hlvk_o2_p50", ["L1", "H1", "V1", "K1"], 2, 50, 20, seed=33, snr=30.0),
        _subnet_case("hl_o2_p40", ["L1", "H1"], 2, 40, 20, seed=34),
        _subnet_case("hlv_o2_p60_cut0", ["L1", "H1", "V1"], 2, 60, 20, seed=35, subcut=0.0,
                     acore=1.2),
        _subnet_case("rand_s120_p30", ["L1", "H1", "V1"], None, 30, 20, seed=36,
                     random_tables=True, n_sky=120, subcut=-1.0, acore=1.0),
        _subnet_case("hlv_o2_p3_quiet", ["L1", "H1", "V1"], 2, 3, 20, seed=37, snr=4.0),
    ]
    for case in cases:
        res = run_subnet_case(snc, case)
        path = os.path.join(HERE, f"subnet_{case['name']}.npz")
        np.savez_compressed(path, **{k: v for k, v in case.items() if k != "name"}, **res)
        print(case["name"], res["out"], "->", os.path.relpath(path, REPO))


def load_skystat(ref_root):
    """pycwb/modules/likelihoodWP/sky_statistics.py (statistics at l_max) with
    packet_ops.py and typing.py under the stand-in; the xtalk type it imports
    for annotations only gets an empty module."""
    lwp = os.path.join(ref_root, "pycwb", "modules", "likelihoodWP")
    for name in ("pycwb", "pycwb.modules", "pycwb.modules.xtalk"):
        if name not in sys.modules:
            m = types.ModuleType(name)
            m.__path__ = []
            sys.modules[name] = m
    m = types.ModuleType("pycwb.modules.xtalk.type")
    m.XTalk = object
    sys.modules["pycwb.modules.xtalk.type"] = m
    _load("ref_lwp.typing", os.path.join(lwp, "typing.py"), "ref_lwp")
    _load("ref_lwp.packet_ops", os.path.join(lwp, "packet_ops.py"), "ref_lwp")
    return _load("ref_lwp.sky_statistics", os.path.join(lwp, "sky_statistics.py"), "ref_lwp")


def synthetic_xtalk(rng, n_pix, n_nbr=4, scale=0.05):
    """Packed xtalk rows for a cluster (the catalog itself is not in the
    reference checkout): each pixel overlaps itself with (1, 0, 0, 1) and up
    to n_nbr other pixels with small random coefficients."""
    rows, lookup = [], np.zeros((n_pix, 2), np.int64)
    for i in range(n_pix):
        start = len(rows)
        rows.append([i, 0, 0, 0, 1.0, 0.0, 0.0, 1.0])
        if n_pix > 1:
            for j in rng.choice(n_pix, size=min(n_nbr, n_pix), replace=False):
                if j != i:
                    rows.append([j, 0, 0, 0, *rng.normal(0.0, scale, 4)])
        lookup[i] = (start, len(rows))
    return np.asarray(rows, np.float32), lookup


SKYSTAT_SCALARS = ("Gn", "Ec", "Dc", "Rc", "Eh", "Es", "Np", "Em", "Lm", "norm", "cc", "rho",
                   "xrho", "Lo", "Eo")
SKYSTAT_ARRAYS = ("energy_array_plus", "energy_array_cross", "pixel_mask",
                  "gaussian_noise_correction", "coherent_energy", "noise_amplitude_00",
                  "noise_amplitude_90", "pd", "pD", "ps", "pS", "S_snr", "f", "F")


def main_skystat(ref_root):
    ref = load_reference(ref_root)
    ss = load_skystat(ref_root)
    cases = [
        ("hlv_o2_p40", _sky_case("hlv_o2_p40", ["L1", "H1", "V1"], 2, 40, 20, seed=41), {}),
        ("hlvk_o2_p30", _sky_case("hlvk_o2_p30", ["L1", "H1", "V1", "K1"], 2, 30, 20, seed=42,
                                  snr=25.0), {}),
        ("hl_o2_p32", _sky_case("hl_o2_p32", ["L1", "H1"], 2, 32, 20, seed=43), {}),
        ("hlv_o2_p60_xgb", _sky_case("hlv_o2_p60_xgb", ["L1", "H1", "V1"], 2, 60, 20, seed=44,
                                     snr=30.0), {"xgb_rho_mode": True}),
        ("hlv_o2_p40_offmax", _sky_case("hlv_o2_p40_offmax", ["L1", "H1", "V1"], 2, 40, 20,
                                        seed=45), {"direction": 17}),
        ("hlv_o2_p5_quiet", _sky_case("hlv_o2_p5_quiet", ["L1", "H1", "V1"], 2, 5, 20, seed=46,
                                      snr=6.0), {}),
    ]
    for name, case, opt in cases:
        res = run_sky_case(ref, case)
        rng = np.random.default_rng(zlib.crc32(name.encode()))
        xt, look = synthetic_xtalk(rng, case["n_pix"])
        l = int(opt.get("direction", res["l_max"]))
        out = ss.compute_statistics_at_sky_position(
            l, case["n_ifo"], case["n_pix"], case["FP"], case["FX"], case["rms"], case["td00"],
            case["td90"], case["ml"], res["REG"], case["network_energy_threshold"], xt, look,
            xgb_rho_mode=bool(opt.get("xgb_rho_mode", False)))
        arrays = {f"out_{k}": np.asarray(getattr(out, k)) for k in SKYSTAT_ARRAYS}
        arrays.update({f"out_{k}_r": np.asarray(getattr(out, k)[0]) for k in ("p00_POL", "p90_POL")})
        arrays.update({f"out_{k}_a": np.asarray(getattr(out, k)[1]) for k in ("p00_POL", "p90_POL")})
        dst = os.path.join(HERE, f"skystat_{name}.npz")
        np.savez_compressed(
            dst, n_ifo=case["n_ifo"], n_pix=case["n_pix"], FP=case["FP"], FX=case["FX"],
            rms=case["rms"], td00=case["td00"], td90=case["td90"], ml=case["ml"], REG=res["REG"],
            network_energy_threshold=case["network_energy_threshold"], sky_idx=l, xtalk=xt,
            xtalk_lookup=look, xgb_rho_mode=bool(opt.get("xgb_rho_mode", False)),
            scalars=np.array([float(getattr(out, k)) for k in SKYSTAT_SCALARS]),
            N_pix_effective=float(out.N_pix_effective), **arrays)
        print(dst, {k: float(getattr(out, k)) for k in ("Ec", "Lm", "rho", "Em")})


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PYCWB_REFERENCE", "")
    if len(sys.argv) > 2 and sys.argv[2] == "subnet":
        main_subnet(root)
    elif len(sys.argv) > 2 and sys.argv[2] == "skystat":
        main_skystat(root)
    else:
        main(root)
        main_subnet(root)
        main_skystat(root)
