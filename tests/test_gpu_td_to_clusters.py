"""td amplitudes built on the device straight into the batched scan's layout.

pgw_td_vecs_to_clusters must place, bit for bit, what the reference's
per-(plane, detector) batch_get_td_vecs (pycwb/utils/td_vector_kernels.py:
133-199, here the oracle) followed by the (D, I, P) rearrangement of
likelihood.py:303-304 would place; the sky loop run on those device-built
inputs must then give the same results as on host-built ones.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

K = 20
M, NC, L_LEVEL = 32, 6, 1
J = M * L_LEVEL
N_TIME = 160
SIZES = [7, 0, 30, 1, 12, 64]


@pytest.fixture(scope="module")
def env():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pycwb_gb300 import _lib, sky
    from pycwb_gb300.likelihoodWP.batched import SkyTables
    from pycwb_gb300.synthetic import regulators
    _lib.build()
    ifos = ["L1", "H1", "V1"]
    ml, FP, FX = sky.compute_sky_delay_and_patterns(ifos, "L1", 512.0, K, healpix_order=3)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    reg = regulators(3)
    tables = SkyTables.from_arrays(FP_t, FX_t, ml, None, **{k: reg[k] for k in (
        "network_energy_threshold", "gamma_regulator", "delta_regulator", "netCC")})
    return dict(tables=tables, n_ifo=len(ifos))


def _planes(rng, n_ifo):
    from pycwb_gb300.types.td_batch_inputs import TDBatchInputs
    rows = N_TIME + 2 * NC
    out = []
    for _ in range(n_ifo):
        p00 = np.zeros((rows, M + 1), np.float32)
        p90 = np.zeros((rows, M + 1), np.float32)
        p00[NC:NC + N_TIME] = rng.standard_normal((N_TIME, M + 1))
        p90[NC:NC + N_TIME] = rng.standard_normal((N_TIME, M + 1))
        T0 = rng.standard_normal((2 * J + 1, 2 * NC + 1))
        Tx = rng.standard_normal((2 * J + 1, 2 * NC + 1)) * 0.2
        out.append(TDBatchInputs(p00, p90, T0, Tx, M, NC, J))
    return out


def _layout(rng, n_ifo):
    """Per detector, the plane index of every cluster pixel (distinct within a
    cluster, as a cluster's pixels are), plus a shuffled scatter order."""
    idx = []
    for i in range(n_ifo):
        per = [rng.choice(N_TIME * (M + 1), size=P, replace=False).astype(np.int32)
               for P in SIZES]
        idx.append(per)
    cl = np.concatenate([np.full(P, c, np.int32) for c, P in enumerate(SIZES)])
    jj = np.concatenate([np.arange(P, dtype=np.int32) for P in SIZES])
    perm = rng.permutation(cl.size)
    return idx, cl[perm], jj[perm]


def _host_batch(oracle_mod, planes, idx, n_ifo):
    from pycwb_gb300.likelihoodWP.batched import ClusterBatch
    D = 2 * K + 1
    b = ClusterBatch(n_ifo, D, SIZES)
    rng = np.random.default_rng(5)
    for c, P in enumerate(SIZES):
        td00 = np.zeros((D, n_ifo, P), np.float32)
        td90 = np.zeros((D, n_ifo, P), np.float32)
        for i, t in enumerate(planes):
            if P == 0:
                continue
            v = oracle_mod.batch_get_td_vecs(idx[i][c], t.padded00, t.padded90, t.T0, t.Tx,
                                             M, NC, K, J)
            td00[:, i, :] = v[:, :D].T
            td90[:, i, :] = v[:, D:].T
        rms = rng.uniform(0.5, 2.0, size=(P, n_ifo)).astype(np.float32)
        b.set_cluster(c, td00, td90, rms)
    return b


def _bits(t):
    return t.detach().cpu().numpy().view(np.uint32)


def test_scatter_matches_oracle_layout(env, oracle_mod):
    import torch
    from pycwb_gb300.likelihoodWP.batched import BatchedSkyLoop
    from pycwb_gb300.utils.td_vector_kernels import td_vecs_to_clusters

    n_ifo = env["n_ifo"]
    rng = np.random.default_rng(2024)
    planes = _planes(rng, n_ifo)
    idx, cl, jj = _layout(rng, n_ifo)
    host = _host_batch(oracle_mod, planes, idx, n_ifo)

    loop = BatchedSkyLoop(env["tables"], host)
    loop.td00.fill_(float("nan"))
    loop.td90.fill_(float("nan"))
    offs = np.concatenate([[0], np.cumsum(SIZES)])
    for i, t in enumerate(planes):
        flat = np.concatenate(idx[i])             # cluster-major
        src = flat[offs[cl] + jj]                 # the shuffled scatter order
        td_vecs_to_clusters(loop, t, i, src, cl, jj, K)
    torch.cuda.synchronize()
    assert np.array_equal(_bits(loop.td00), host.td00.numpy().view(np.uint32))
    assert np.array_equal(_bits(loop.td90), host.td90.numpy().view(np.uint32))


def test_scan_on_device_built_inputs(env, oracle_mod):
    import torch
    from pycwb_gb300.likelihoodWP.batched import BatchedSkyLoop
    from pycwb_gb300.utils.td_vector_kernels import td_vecs_to_clusters

    n_ifo = env["n_ifo"]
    rng = np.random.default_rng(77)
    planes = _planes(rng, n_ifo)
    idx, cl, jj = _layout(rng, n_ifo)
    host = _host_batch(oracle_mod, planes, idx, n_ifo)

    ref = BatchedSkyLoop(env["tables"], host).run()
    ref_maps = ref.maps.cpu().numpy()

    dev = BatchedSkyLoop(env["tables"], host)
    offs = np.concatenate([[0], np.cumsum(SIZES)])
    for i, t in enumerate(planes):
        td_vecs_to_clusters(dev, t, i, np.concatenate(idx[i])[offs[cl] + jj], cl, jj, K)
    dev.upload(td=False)
    dev.launch()
    dev.download()
    dev.stream.synchronize()
    out = dev.results()
    torch.cuda.synchronize()
    assert np.array_equal(out.l_max, ref.l_max)
    assert np.array_equal(out.sky_stat_max.view(np.uint32), ref.sky_stat_max.view(np.uint32))
    assert np.array_equal(out.regulator, ref.regulator)
    assert np.array_equal(out.maps.cpu().numpy().view(np.uint32), ref_maps.view(np.uint32))


def test_bad_destinations_write_nothing(env):
    import torch
    from pycwb_gb300.likelihoodWP.batched import BatchedSkyLoop, ClusterBatch
    from pycwb_gb300.utils.td_vector_kernels import td_vecs_to_clusters

    n_ifo = env["n_ifo"]
    planes = _planes(np.random.default_rng(3), n_ifo)
    b = ClusterBatch(n_ifo, 2 * K + 1, SIZES)
    loop = BatchedSkyLoop(env["tables"], b)
    loop.td00.fill_(7.0)
    loop.td90.fill_(7.0)
    n_cl = len(SIZES)
    cl = np.array([-1, n_cl, n_cl + 5, 1, 0, 2, 3], np.int32)   # cluster 1 is empty
    jj = np.array([0, 0, 0, 0, SIZES[0], -1, 1], np.int32)       # cluster 3 has one pixel
    src = np.arange(cl.size, dtype=np.int32)
    td_vecs_to_clusters(loop, planes[0], 0, src, cl, jj, K)
    torch.cuda.synchronize()
    assert bool((loop.td00 == 7.0).all()) and bool((loop.td90 == 7.0).all())
    with pytest.raises(ValueError):
        td_vecs_to_clusters(loop, planes[0], 0, src, cl, jj, K + 1)
    with pytest.raises(ValueError):
        td_vecs_to_clusters(loop, planes[0], n_ifo, src, cl, jj, K)
