"""Batched sky loop (one persistent launch, work queue) against the oracle.

Each cluster of the batch must reproduce the single-cluster reference loop
(regulator then scan, likelihood.py:310-325) under the tolerance of
tests/parity.py; the batched maps must equal the plain per-cluster launch
exactly (same kernel, same arithmetic, same summation order).
"""

import math

import numpy as np
import pytest

from parity import assert_scan_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pycwb_gb300 import _lib, sky
    from pycwb_gb300.likelihoodWP.batched import SkyTables
    from pycwb_gb300.synthetic import regulators
    _lib.build()
    ml, FP, FX = sky.compute_sky_delay_and_patterns(["L1", "H1", "V1"], "L1", 512.0, 20,
                                                    healpix_order=4)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    reg = regulators(3)
    tables = SkyTables.from_arrays(FP_t, FX_t, ml, None, **{k: reg[k] for k in (
        "network_energy_threshold", "gamma_regulator", "delta_regulator", "netCC")})
    return dict(ml=ml, FP_t=FP_t, FX_t=FX_t, reg=reg, tables=tables)


def _clusters(env, sizes, seed):
    from pycwb_gb300.synthetic import make_cluster
    rng = np.random.default_rng(seed)
    out = []
    for P in sizes:
        td00, td90, rms, _ = make_cluster(rng, env["ml"], env["FP_t"], env["FX_t"], int(P), 20,
                                          float(rng.uniform(8, 40)))
        out.append((td00, td90, rms))
    return out


@pytest.mark.parametrize("spec", [None, (256, 2, 0, 3, 4, -1), (128, 1, 7, 2, 4, 1)])
def test_batched_matches_oracle_and_plain(env, oracle_mod, spec):
    from pycwb_gb300._lib import TileShape
    from pycwb_gb300.likelihoodWP import sky_loop
    from pycwb_gb300.likelihoodWP.batched import BatchedSkyLoop, ClusterBatch

    shape = None if spec is None else TileShape(*spec)
    sizes = [20, 350, 1, 77, 0, 130, 20, 512, 3]
    clusters = _clusters(env, sizes, seed=11)
    batch = ClusterBatch.from_clusters(clusters)
    loop = BatchedSkyLoop(env["tables"], batch, shape=shape)
    res = loop.run()
    reg, ml, FP_t, FX_t = env["reg"], env["ml"], env["FP_t"], env["FX_t"]
    n_sky = ml.shape[1]
    valid = np.arange(n_sky, dtype=np.int64)
    REG0 = np.float32(reg["delta_regulator"] * math.sqrt(2))
    for c, (td00, td90, rms) in enumerate(clusters):
        reg1 = oracle_mod.calculate_dpf(FP_t, FX_t, rms, n_sky, 3, reg["gamma_regulator"],
                                        reg["network_energy_threshold"], valid)
        assert np.float32(res.regulator[c]) == np.float32(reg1)
        REG = np.array([REG0, reg1, 0.0], np.float32)
        args = (3, rms.shape[0], n_sky, FP_t, FX_t, rms, td00, td90, ml)
        tail = (reg["netCC"], reg["delta_regulator"], reg["network_energy_threshold"], valid)
        ref = oracle_mod.scan_sky_for_best_fit(*args, REG, *tail, return_ellipticity=True)
        f64 = oracle_mod.scan_sky_for_best_fit(*args, REG.astype(np.float64), *tail,
                                               precision="f64", return_ellipticity=True)
        got = res.cluster_tuple(c)
        assert_scan_close(got, ref, f64, ref_cr=ref[13], netCC=reg["netCC"],
                          what=f"cluster {c} (P={rms.shape[0]}) shape {spec}")
        # the plain launch of the same kernel gives identical bits
        _, plain = sky_loop(*args, REG0, reg["gamma_regulator"], reg["netCC"],
                            reg["network_energy_threshold"], valid, shape=shape)
        assert plain[0] == got[0]
        for k in range(1, 12):
            np.testing.assert_array_equal(plain[k], got[k])


def test_batched_graph_replay_is_repeatable(env):
    from pycwb_gb300.likelihoodWP.batched import BatchedSkyLoop, ClusterBatch

    import torch

    batch = ClusterBatch.from_clusters(_clusters(env, [40, 300, 5, 999], seed=3))
    loop = BatchedSkyLoop(env["tables"], batch)
    first = loop.run()
    maps0 = loop.stats.clone()
    loop.capture()
    for _ in range(3):
        with torch.cuda.stream(loop.stream):   # wipe every output, then replay
            loop.stats.fill_(float("nan"))
            loop.res.zero_()
            loop.regs.zero_()
        loop.replay()
        loop.download()
        loop.stream.synchronize()
        again = loop.results()
        np.testing.assert_array_equal(first.l_max, again.l_max)
        np.testing.assert_array_equal(first.sky_stat_max, again.sky_stat_max)
        np.testing.assert_array_equal(first.regulator, again.regulator)
        assert bool((loop.stats == maps0).all())


def test_batched_regulators_only(env, oracle_mod):
    """pgw_calculate_dpf_batched gives the full loop's REG[1], bit for bit,
    and the oracle's regulator for every cluster."""
    from pycwb_gb300.likelihoodWP.batched import BatchedSkyLoop, ClusterBatch

    clusters = _clusters(env, [3, 250, 0, 1200, 64], seed=21)
    loop = BatchedSkyLoop(env["tables"], ClusterBatch.from_clusters(clusters))
    full = loop.run()
    only = loop.regulators()
    assert np.array_equal(only, full.regulator)
    reg, FP_t, FX_t = env["reg"], env["FP_t"], env["FX_t"]
    n_sky = FP_t.shape[0]
    valid = np.arange(n_sky, dtype=np.int64)
    for c, (_, _, rms) in enumerate(clusters):
        ref = oracle_mod.calculate_dpf(FP_t, FX_t, rms, n_sky, 3, reg["gamma_regulator"],
                                       reg["network_energy_threshold"], valid)
        assert np.float32(only[c]) == np.float32(ref), c


@pytest.mark.parametrize("gamma", [0.02, 0.12, 0.2, 0.35])
def test_regulator_early_decisions_are_exact(env, oracle_mod, gamma):
    """The regulator stops a direction once its pass (running sum over the
    threshold) or its fail (running sum plus a bound on the remaining
    pixels under it) is certain; the count must still equal the reference's
    for every cluster, at thresholds through the bulk of the directions."""
    from pycwb_gb300.likelihoodWP.batched import BatchedSkyLoop, ClusterBatch, SkyTables

    reg = env["reg"]
    FP_t, FX_t, ml = env["FP_t"], env["FX_t"], env["ml"]
    tables = SkyTables.from_arrays(FP_t, FX_t, ml, None,
                                   network_energy_threshold=reg["network_energy_threshold"],
                                   gamma_regulator=gamma, delta_regulator=reg["delta_regulator"],
                                   netCC=reg["netCC"])
    rng = np.random.default_rng(int(gamma * 1000))
    sizes = [1, 2, 17, 40, 333, 1500, 64, 900]
    clusters = []
    for k, P in enumerate(sizes):
        rms = rng.uniform(0.3, 2.0, size=(P, 3)).astype(np.float32)
        if k % 3 == 1 and P > 4:
            rms[: P // 2, 2] = 1e-4                       # a nearly deaf detector
        if k % 4 == 3:
            rms[0] = 0.0                                  # a pixel with no weight at all
        zero = np.zeros((41, 3, P), np.float32)
        clusters.append((zero, zero, rms))
    loop = BatchedSkyLoop(tables, ClusterBatch.from_clusters(clusters))
    loop.upload()
    got = loop.regulators()
    n_sky = FP_t.shape[0]
    valid = np.arange(n_sky, dtype=np.int64)
    for c, (_, _, rms) in enumerate(clusters):
        ref = oracle_mod.calculate_dpf(FP_t, FX_t, rms, n_sky, 3, gamma,
                                       reg["network_energy_threshold"], valid)
        assert np.float32(got[c]) == np.float32(ref), (gamma, c, got[c], ref)


@pytest.mark.parametrize("nbytes,offset", [(1 << 20, 0), ((1 << 22) + 13, 0), ((1 << 21) + 5, 3)])
def test_copy_from_host_is_exact(env, nbytes, offset):
    """pgw_copy_from_host (the upload path) moves bytes exactly, with
    16-byte words where both ends are aligned and a byte tail otherwise."""
    import torch
    from pycwb_gb300 import _lib
    src = torch.randint(0, 256, (nbytes + offset,), dtype=torch.uint8).pin_memory()
    dst = torch.zeros(nbytes + offset, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    rc = _lib.load().pgw_copy_from_host(dst.data_ptr() + offset, src.data_ptr() + offset, nbytes,
                                        s.cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    got = dst.cpu()
    assert torch.equal(got[offset:], src[offset:])
    assert int(got[:offset].sum()) == 0


def test_many_small_clusters_order_in_workspace(oracle_mod):
    """More clusters than the queue-order sort holds in shared memory (4,096):
    the sort keys then live in the workspace.  Every cluster's REG[1] and
    sky maximum must be the oracle's (checked on a spread of clusters)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pycwb_gb300 import _lib, sky
    from pycwb_gb300.likelihoodWP.batched import BatchedSkyLoop, ClusterBatch, SkyTables
    from pycwb_gb300.synthetic import make_cluster, regulators
    _lib.build()
    ml, FP, FX = sky.compute_sky_delay_and_patterns(["L1", "H1", "V1"], "L1", 512.0, 20,
                                                    healpix_order=1)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    reg = regulators(3)
    tables = SkyTables.from_arrays(FP_t, FX_t, ml, None, **{k: reg[k] for k in (
        "network_energy_threshold", "gamma_regulator", "delta_regulator", "netCC")})
    rng = np.random.default_rng(5000)
    sizes = rng.integers(1, 6, 5000)
    clusters = [make_cluster(rng, ml, FP_t, FX_t, int(P), 20, float(rng.uniform(8, 40)))[:3]
                for P in sizes]
    res = BatchedSkyLoop(tables, ClusterBatch.from_clusters(clusters)).run()
    n_sky = ml.shape[1]
    valid = np.arange(n_sky, dtype=np.int64)
    REG0 = np.float32(reg["delta_regulator"] * math.sqrt(2))
    for c in range(0, 5000, 97):
        td00, td90, rms = clusters[c]
        reg1 = oracle_mod.calculate_dpf(FP_t, FX_t, rms, n_sky, 3, reg["gamma_regulator"],
                                        reg["network_energy_threshold"], valid)
        assert np.float32(res.regulator[c]) == np.float32(reg1), c
        REG = np.array([REG0, reg1, 0.0], np.float32)
        ref = oracle_mod.scan_sky_for_best_fit(3, rms.shape[0], n_sky, FP_t, FX_t, rms, td00, td90,
                                               ml, REG, reg["netCC"], reg["delta_regulator"],
                                               reg["network_energy_threshold"], valid)
        if ref[12] > 0 and int(res.l_max[c]) != ref[0]:     # only a near-tie may differ
            a, b = float(ref[7][int(res.l_max[c])]), float(ref[7][ref[0]])
            assert abs(a - b) <= 1e-5 * abs(b), (c, a, b)


def test_run_many_streams_batches_like_run(env):
    """BatchedSkyLoop.run_many (double-buffered inputs, the next batch's copy
    overlapping the current launch) gives, batch by batch, the results of
    run() on each batch alone."""
    from pycwb_gb300.likelihoodWP.batched import BatchedSkyLoop, ClusterBatch
    from pycwb_gb300.synthetic import make_cluster
    e = env
    rng = np.random.default_rng(77)
    sizes = [40, 250, 7, 120]
    batches = []
    for _ in range(3):
        cl = []
        for P in sizes:
            td00, td90, rms, _ = make_cluster(rng, e["ml"], e["FP_t"], e["FX_t"], P, 20,
                                              float(rng.uniform(8, 40)))
            cl.append((td00, td90, rms))
        batches.append(ClusterBatch.from_clusters(cl))
    singles = []
    for b in batches:
        one = BatchedSkyLoop(e["tables"], b)
        r = one.run()
        singles.append((r.l_max.copy(), r.sky_stat_max.copy(), r.regulator.copy(),
                        r.maps.cpu().numpy()))
    loop = BatchedSkyLoop(e["tables"], batches[0])
    got = []
    for r in loop.run_many(batches):
        got.append((r.l_max.copy(), r.sky_stat_max.copy(), r.regulator.copy(),
                    r.maps.cpu().numpy()))
    assert len(got) == 3
    for (a, b, c, d), (A, B, C, D) in zip(singles, got):
        np.testing.assert_array_equal(a, A)
        np.testing.assert_array_equal(b, B)
        np.testing.assert_array_equal(c, C)
        np.testing.assert_array_equal(d, D)
    # the loop's own buffers are back, and a plain run still works
    r = loop.run()
    np.testing.assert_array_equal(r.l_max, singles[0][0])
