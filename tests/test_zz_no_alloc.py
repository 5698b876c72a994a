"""pgw_sky_loop_noalloc: the sky loop for callers that cannot allocate.

Some callers cannot allocate device memory per call (cudaMalloc/cudaFree
may synchronise the device; a host framework that owns the device memory
may forbid allocations outside its pool).  pgw_sky_loop_noalloc takes no
workspace: its scratch is a static device array inside the library, shared
by every call and holding whatever the last call left there.  This test
calls it through the C ABI several times in a row on the same stream --
clusters of different detector counts and sizes, the same call twice, a
partial sky mask -- and compares each result with the workspace entry point
pgw_sky_loop on a fresh workspace, within the tolerance of tests/parity.py;
then it checks that a cluster too large for the array is refused with a
clear error instead of being run.

The file is named to be collected last, so that a run stopping at the first
failure has already run every other test.
"""

import ctypes
import math

import numpy as np
import pytest

from parity import RTOL, stat_errors

pytestmark = pytest.mark.gpu


RESULT = np.dtype([("l", "<i8"), ("s", "<f4"), ("f", "<i4"), ("st", "<i4"), ("r", "<f4"),
                   ("a", "<i8")])


def _case(ifos, P, order, seed, n_valid=None):
    """Inputs of one cluster on the device, in the reference's layouts."""
    import torch
    from pycwb_gb300 import sky
    from pycwb_gb300.synthetic import make_cluster, regulators

    K = 20
    dev = torch.device("cuda", torch.cuda.current_device())
    ml, FP, FX = sky.compute_sky_delay_and_patterns(list(ifos), ifos[0], 512.0, K,
                                                    healpix_order=order)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    rng = np.random.default_rng(seed)
    td00, td90, rms, _ = make_cluster(rng, ml, FP_t, FX_t, P, K, 18.0)
    n_sky = ml.shape[1]
    valid = np.arange(n_sky, dtype=np.int64)
    if n_valid is not None:
        valid = np.sort(rng.choice(n_sky, n_valid, replace=False)).astype(np.int64)
    reg = regulators(len(ifos))
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in dict(
        FP=FP_t, FX=FX_t, rms=rms, td00=td00, td90=td90, ml=ml, valid=valid).items()}
    common = (len(ifos), P, n_sky, t["FP"].data_ptr(), t["FX"].data_ptr(), t["rms"].data_ptr(),
              t["td00"].data_ptr(), t["td90"].data_ptr(), 2 * K + 1, t["ml"].data_ptr(),
              float(np.float32(reg["delta_regulator"] * math.sqrt(2))), reg["gamma_regulator"],
              reg["netCC"], reg["network_energy_threshold"], t["valid"].data_ptr(), valid.size,
              None)
    return dict(t=t, common=common, n_ifo=len(ifos), P=P, n_sky=n_sky, dev=dev)


def _outputs(c):
    import torch
    st = torch.full((11, c["n_sky"]), float("nan"), dtype=torch.float32, device=c["dev"])
    return (st, torch.zeros(32, dtype=torch.uint8, device=c["dev"]),
            torch.zeros(1, dtype=torch.float64, device=c["dev"]))


def _with_workspace(L, c, stream):
    """pgw_sky_loop with a fresh workspace of its own: the expected result."""
    import torch
    st, res, regv = _outputs(c)
    ws = torch.empty(L.pgw_workspace_bytes(c["n_ifo"], 41, c["P"], 1), dtype=torch.uint8,
                     device=c["dev"])
    rc = L.pgw_sky_loop(*c["common"], None, st.data_ptr(), res.data_ptr(), regv.data_ptr(), None,
                        ws.data_ptr(), ws.numel(), stream)
    assert rc == 0, L.pgw_last_error()
    torch.cuda.synchronize()
    return st.cpu().numpy(), res.cpu().numpy().view(RESULT)[0], float(regv.item())


def _noalloc(L, c, stream):
    import torch
    st, res, regv = _outputs(c)
    rc = L.pgw_sky_loop_noalloc(*c["common"], st.data_ptr(), res.data_ptr(), regv.data_ptr(),
                                stream)
    assert rc == 0, L.pgw_last_error()
    torch.cuda.synchronize()
    return st.cpu().numpy(), res.cpu().numpy().view(RESULT)[0], float(regv.item())


def _assert_same(got, ref, what):
    st, res, regv = got
    st_ref, res_ref, reg_ref = ref
    assert res["st"] == 0 and res_ref["st"] == 0, what
    assert res["l"] == res_ref["l"] and res["f"] == res_ref["f"], what
    assert abs(float(res["s"]) - float(res_ref["s"])) <= RTOL * abs(float(res_ref["s"])), what
    assert np.float32(regv) == np.float32(reg_ref), what
    errs = stat_errors(list(st), list(st_ref))
    assert max(errs) <= RTOL, (what, errs)


def test_noalloc_entry_point_matches_workspace_entry_point():
    """Calls in a row on the shared scratch array, each compared with
    pgw_sky_loop on a fresh workspace: a larger 4-detector cluster first, so
    that the smaller 3-detector calls after it run on scratch left behind by
    a different shape; the same 3-detector call twice; a call whose sky mask
    keeps only part of the sky (n_valid < n_sky)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pycwb_gb300 import _lib

    _lib.build()
    L = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    big = _case(("L1", "H1", "V1", "K1"), 1500, 4, seed=5)
    small = _case(("L1", "H1", "V1"), 300, 4, seed=77)
    masked = _case(("L1", "H1", "V1"), 200, 4, seed=9, n_valid=1000)
    expect = {"big": _with_workspace(L, big, stream), "small": _with_workspace(L, small, stream),
              "masked": _with_workspace(L, masked, stream)}
    for name, c in (("big", big), ("small", small), ("small", small), ("masked", masked),
                    ("small", small)):
        _assert_same(_noalloc(L, c, stream), expect[name], name)


def test_noalloc_refuses_a_cluster_larger_than_its_scratch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pycwb_gb300 import _lib

    _lib.build()
    L = _lib.load()
    cap = L.pgw_sky_loop_noalloc_max_scratch()
    too_many = cap // 100 + 1  # each pixel record alone exceeds 100 bytes at n_delay = 41
    one = torch.zeros(64, dtype=torch.float32, device="cuda")
    p = one.data_ptr()
    rc = L.pgw_sky_loop_noalloc(3, too_many, 12, p, p, p, p, p, 41, p, 0.7, 0.1, 0.5, 12.0, p, 12,
                                None, p, p, p, torch.cuda.current_stream().cuda_stream)
    assert rc == 4  # PGW_ERR_WORKSPACE, nothing launched
    msg = L.pgw_last_error().decode()
    assert "scratch" in msg and str(cap) in msg
