"""GPU td-amplitude vectors against the reference, bit for bit.

tests/golden/td_*.npz were produced by the reference's own
batch_get_td_vecs (pycwb/utils/td_vector_kernels.py:133-199); the kernel
accumulates in float64 in the same order with the same phase factors, so
the float32 outputs must be identical.  Larger random cases are checked
against the oracle (itself bit-exact to the reference).
"""

import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TD_CASES = sorted(glob.glob(os.path.join(GOLDEN, "td_*.npz")))


@pytest.fixture(scope="module")
def tdk():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pycwb_gb300 import _lib
    _lib.build()
    from pycwb_gb300.utils import td_vector_kernels
    return td_vector_kernels


def _bits(a):
    return np.asarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("path", TD_CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_td_vectors_equal_reference(tdk, path):
    z = np.load(path)
    out = tdk.batch_get_td_vecs(z["pixel_indices"], z["padded00"], z["padded90"], z["T0"],
                                z["Tx"], int(z["M"]), int(z["n_coeffs"]), int(z["K"]), int(z["J"]))
    assert np.array_equal(_bits(out), _bits(z["out"]))


@pytest.mark.parametrize("M,nc,L,K,n_time,n_pix", [
    (64, 10, 1, 20, 200, 3000),
    (32, 8, 2, 40, 120, 1000),
    (16, 6, 4, 90, 80, 500),     # K > J: whole-pixel shifts of both parities
    (8, 5, 1, 3, 30, 200),
])
def test_td_vectors_equal_oracle(tdk, oracle_mod, M, nc, L, K, n_time, n_pix):
    rng = np.random.default_rng(M * 1000 + K)
    J = M * L
    rows = n_time + 2 * nc
    p00 = np.zeros((rows, M + 1), np.float32)
    p90 = np.zeros((rows, M + 1), np.float32)
    p00[nc:nc + n_time] = rng.standard_normal((n_time, M + 1))
    p90[nc:nc + n_time] = rng.standard_normal((n_time, M + 1))
    T0 = rng.standard_normal((2 * J + 1, 2 * nc + 1))
    Tx = rng.standard_normal((2 * J + 1, 2 * nc + 1)) * 0.2
    # every time bin, including the first and last (rows outside the padded
    # plane read as zero in both implementations)
    n = rng.integers(0, n_time, size=n_pix)
    m = rng.integers(0, M + 1, size=n_pix)
    idx = (n * (M + 1) + m).astype(np.int32)
    ref = oracle_mod.batch_get_td_vecs(idx, p00, p90, T0, Tx, M, nc, K, J)
    out = tdk.batch_get_td_vecs(idx, p00, p90, T0, Tx, M, nc, K, J)
    assert np.array_equal(_bits(out), _bits(ref))


def test_td_batch_inputs_container(tdk):
    from pycwb_gb300.types.td_batch_inputs import TDBatchInputs
    z = np.load(TD_CASES[0])
    tdb = TDBatchInputs(z["padded00"], z["padded90"], z["T0"], z["Tx"], int(z["M"]),
                        int(z["n_coeffs"]), int(z["J"]))
    out = tdb.extract_td_vecs(z["pixel_indices"], int(z["K"]))
    assert out.shape == (len(z["pixel_indices"]), 4 * int(z["K"]) + 2)
    assert np.array_equal(_bits(out), _bits(z["out"]))


def test_td_vectors_bad_shapes(tdk):
    z = np.load(TD_CASES[0])
    with pytest.raises(ValueError):
        tdk.batch_get_td_vecs(z["pixel_indices"], z["padded00"][:, :-1], z["padded90"], z["T0"],
                              z["Tx"], int(z["M"]), int(z["n_coeffs"]), int(z["K"]), int(z["J"]))
