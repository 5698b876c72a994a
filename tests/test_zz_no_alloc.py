"""pgw_sky_loop_noalloc: the sky loop for callers that cannot allocate.

Some callers cannot allocate device memory per call (cudaMalloc/cudaFree
may synchronise the device; a host framework that owns the device memory
may forbid allocations outside its pool).  pgw_sky_loop_noalloc takes no
workspace: its scratch is a static device array inside the library.  This
test calls it through the C ABI twice in a row on the same stream and
compares each result with the workspace entry point pgw_sky_loop, within
the tolerance of tests/parity.py, then checks that a cluster too large for
the array is refused with a clear error instead of being run.

The file is named to be collected last, so that a run stopping at the first
failure has already run every other test.
"""

import ctypes
import math

import numpy as np
import pytest

from parity import RTOL, stat_errors

pytestmark = pytest.mark.gpu


def test_noalloc_entry_point_matches_workspace_entry_point_twice():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pycwb_gb300 import _lib, sky
    from pycwb_gb300.synthetic import make_cluster, regulators

    _lib.build()
    L = _lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    K, P = 20, 300
    ml, FP, FX = sky.compute_sky_delay_and_patterns(["L1", "H1", "V1"], "L1", 512.0, K,
                                                    healpix_order=4)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    td00, td90, rms, _ = make_cluster(np.random.default_rng(77), ml, FP_t, FX_t, P, K, 18.0)
    reg = regulators(3)
    REG0 = float(np.float32(reg["delta_regulator"] * math.sqrt(2)))
    n_sky = ml.shape[1]
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in dict(
        FP=FP_t, FX=FX_t, rms=rms, td00=td00, td90=td90, ml=ml,
        valid=np.arange(n_sky, dtype=np.int64)).items()}
    stream = torch.cuda.current_stream().cuda_stream

    def outputs():
        return (torch.empty((11, n_sky), dtype=torch.float32, device=dev),
                torch.zeros(32, dtype=torch.uint8, device=dev),
                torch.zeros(1, dtype=torch.float64, device=dev))

    common = (3, P, n_sky, t["FP"].data_ptr(), t["FX"].data_ptr(), t["rms"].data_ptr(),
              t["td00"].data_ptr(), t["td90"].data_ptr(), 2 * K + 1, t["ml"].data_ptr(), REG0,
              reg["gamma_regulator"], reg["netCC"], reg["network_energy_threshold"],
              t["valid"].data_ptr(), n_sky, None)

    # the entry point with a caller workspace
    st_ref, res_ref, reg_ref = outputs()
    ws = torch.empty(L.pgw_workspace_bytes(3, 2 * K + 1, P, 1), dtype=torch.uint8, device=dev)
    rc = L.pgw_sky_loop(*common, None, st_ref.data_ptr(), res_ref.data_ptr(), reg_ref.data_ptr(),
                        None, ws.data_ptr(), ws.numel(), stream)
    assert rc == 0, L.pgw_last_error()
    torch.cuda.synchronize()
    ref = res_ref.cpu().numpy().view(np.dtype([("l", "<i8"), ("s", "<f4"), ("f", "<i4"),
                                               ("st", "<i4"), ("r", "<f4"), ("a", "<i8")]))[0]
    assert ref["st"] == 0

    # the allocation-free entry point, twice in a row
    for _ in range(2):
        st, res, regv = outputs()
        st.fill_(float("nan"))
        rc = L.pgw_sky_loop_noalloc(*common, st.data_ptr(), res.data_ptr(), regv.data_ptr(),
                                    stream)
        assert rc == 0, L.pgw_last_error()
        torch.cuda.synchronize()
        got = res.cpu().numpy().view(ref.dtype)[0]
        assert got["st"] == 0
        assert got["l"] == ref["l"] and got["f"] == ref["f"]
        assert abs(float(got["s"]) - float(ref["s"])) <= RTOL * abs(float(ref["s"]))
        assert np.float32(regv.item()) == np.float32(reg_ref.item())
        errs = stat_errors(list(st.cpu().numpy()), list(st_ref.cpu().numpy()))
        assert max(errs) <= RTOL, errs


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
