"""The C ABI: header declarations vs. library exports (no GPU needed)."""

import ctypes
import os
import re

import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "pycwb_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pgw_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_entry_points():
    names = declared_functions()
    for n in ("pgw_calculate_dpf", "pgw_scan_sky_for_best_fit", "pgw_sky_loop",
              "pgw_sky_loop_batched", "pgw_batch_get_td_vecs", "pgw_workspace_bytes"):
        assert n in names


def test_library_builds_loads_and_exports_every_declared_symbol():
    from pycwb_gb300 import _lib
    try:
        path = _lib.build()
    except (RuntimeError, FileNotFoundError) as e:  # no nvcc on this machine
        pytest.skip(f"nvcc unavailable: {e}")
    lib = ctypes.CDLL(path)  # loads without a GPU (no CUDA call at load time)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_workspace_size_is_pure_host_arithmetic():
    from pycwb_gb300 import _lib
    try:
        _lib.build()
    except (RuntimeError, FileNotFoundError) as e:
        pytest.skip(f"nvcc unavailable: {e}")
    L = _lib.load()
    a = L.pgw_workspace_bytes(3, 41, 1000, 1)
    b = L.pgw_workspace_bytes(3, 41, 2000, 1)
    assert a > 1000 * 252 * 4 and b > a
    assert L.pgw_workspace_bytes(0, 41, 10, 1) == 0
    assert L.pgw_workspace_bytes(9, 41, 10, 1) == 0


def test_regulator_order_is_a_permutation():
    """pgw_regulator_order runs on the host: a deterministic permutation of
    the valid positions, and out-of-range sky indices are rejected."""
    import numpy as np
    from pycwb_gb300 import _lib, sky
    try:
        _lib.build()
    except (RuntimeError, FileNotFoundError) as e:
        pytest.skip(f"nvcc unavailable: {e}")
    _, FP, FX = sky.compute_sky_delay_and_patterns(["L1", "H1", "V1"], "L1", 512.0, 20,
                                                   healpix_order=3)
    FP_t, FX_t = FP.T.astype(np.float32), FX.T.astype(np.float32)
    valid = np.arange(0, FP_t.shape[0], 3, dtype=np.int64)
    a = _lib.regulator_order(FP_t, FX_t, valid)
    b = _lib.regulator_order(FP_t, FX_t, valid)
    assert np.array_equal(a, b)
    assert np.array_equal(np.sort(a), np.arange(valid.size))
    with pytest.raises(ValueError):
        _lib.regulator_order(FP_t, FX_t, np.array([0, FP_t.shape[0]], np.int64))


def _struct_layout(struct, fields):
    """sizeof and offsetof of a header struct, from a small host C program."""
    import shutil
    import subprocess
    import tempfile
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    body = "".join(f'  printf("%zu\\n", offsetof({struct}, {f}));\n' for f in fields)
    src = ("#include <stddef.h>\n#include <stdio.h>\n#include <stdint.h>\n"
           "typedef void* cudaStream_t;\n"
           f'#include "{HEADER}"\n'
           f'int main(void) {{\n  printf("%zu\\n", sizeof({struct}));\n{body}  return 0;\n}}\n')
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "layout.c")
        exe = os.path.join(d, "layout")
        open(c, "w").write(src)
        subprocess.run([cc, "-std=c11", "-o", exe, c], check=True, capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    return int(out[0]), [int(x) for x in out[1:]]


def test_result_structs_match_the_python_dtypes():
    """The header's result structs and the numpy dtypes the Python layer reads
    them with agree field by field."""
    from pycwb_gb300._device import RESULT_DTYPE
    from pycwb_gb300.likelihoodWP.sky_statistics import SKYSTAT_DTYPE
    from pycwb_gb300.super_cluster.sub_net_cut import SUBNET_DTYPE
    for struct, dt in (("pgw_skystat_result", SKYSTAT_DTYPE), ("pgw_subnet_result", SUBNET_DTYPE),
                       ("pgw_scan_result", RESULT_DTYPE)):
        names = list(dt.names)
        size, offs = _struct_layout(struct, names)
        assert size == dt.itemsize, struct
        assert offs == [dt.fields[n][1] for n in names], struct


def test_pack_xtalk_offsets_rows():
    import numpy as np
    from pycwb_gb300.likelihoodWP.sky_statistics import pack_xtalk
    a = (np.arange(16, dtype=np.float32).reshape(2, 8), np.array([[0, 1], [1, 2]]))
    b = (np.ones((3, 8), np.float32), np.array([[0, 3]]))
    xt, lk = pack_xtalk([a, b])
    assert xt.shape == (5, 8) and lk.tolist() == [[0, 1], [1, 2], [2, 5]]
    xt0, lk0 = pack_xtalk([])
    assert xt0.shape == (0, 8) and lk0.shape == (0, 2)


def test_skystat_workspace_size_is_pure_host_arithmetic():
    from pycwb_gb300 import _lib
    try:
        _lib.build()
    except (RuntimeError, FileNotFoundError) as e:
        pytest.skip(f"nvcc unavailable: {e}")
    L = _lib.load()
    a = L.pgw_skystat_workspace_bytes(3, 1000)
    assert a >= 1000 * ((10 * 3 + 6) * 4 + (8 * 3 + 1) * 8)
    assert L.pgw_skystat_workspace_bytes(3, 2000) > a
    assert L.pgw_skystat_workspace_bytes(3, 0) > 0
    assert L.pgw_skystat_workspace_bytes(0, 10) == 0 and L.pgw_skystat_workspace_bytes(9, 10) == 0
    assert L.pgw_wdm_n_time(1000, 16) == 63 and L.pgw_wdm_n_time(10, 0) == -1


def test_probability_and_pixel_arrays_reject_bad_arguments_on_the_host():
    """pgw_sky_probability and pgw_skystat_pixel_arrays check their shapes
    and pointers before any CUDA call (and do nothing for empty inputs), so
    the error paths run without a GPU."""
    from pycwb_gb300 import _lib
    try:
        _lib.build()
    except (RuntimeError, FileNotFoundError) as e:
        pytest.skip(f"nvcc unavailable: {e}")
    L = _lib.load()
    ok = 0
    # n_select < 0, n_sky < 1, stride below 11 n_sky
    assert L.pgw_sky_probability(-1, 100, None, 1100, None, None, None, None) != 0
    assert L.pgw_sky_probability(2, 0, None, 1100, None, None, None, None) != 0
    assert L.pgw_sky_probability(2, 100, None, 1099, None, None, None, None) != 0
    # nothing selected: nothing to do
    assert L.pgw_sky_probability(0, 100, None, 1100, None, None, None, None) == ok
    # NULL device pointers
    assert L.pgw_sky_probability(2, 100, None, 1100, None, None, None, None) != 0
    assert "NULL" in L.pgw_last_error().decode()
    # per-pixel arrays: detector count, empty input, NULL pointers, workspace size
    assert L.pgw_skystat_pixel_arrays(1, 10, None, 0, None, None, None) != 0
    assert L.pgw_skystat_pixel_arrays(3, 0, None, 0, None, None, None) == ok
    assert L.pgw_skystat_pixel_arrays(3, 10, None, 0, None, None, None) != 0
    buf = ctypes.create_string_buffer(64)
    p = ctypes.cast(buf, ctypes.c_void_p)
    assert L.pgw_skystat_pixel_arrays(3, 10, p, 64, p, p, None) != 0
    assert "workspace" in L.pgw_last_error().decode()


def test_lpt_regulator_order_groups_the_sorted_directions():
    """pgw_regulator_order_lpt: a permutation made of the sorted order's
    groups of 32, the group where the key crosses the threshold first and
    then outward."""
    import numpy as np
    from pycwb_gb300 import _lib, sky
    try:
        _lib.build()
    except (RuntimeError, FileNotFoundError) as e:
        pytest.skip(f"nvcc unavailable: {e}")
    ml, FP, FX = sky.compute_sky_delay_and_patterns(["L1", "H1", "V1"], "L1", 512.0, 20,
                                                    healpix_order=3)
    FP_t, FX_t = FP.T.astype(np.float32).copy(), FX.T.astype(np.float32).copy()
    valid = np.arange(FP_t.shape[0], dtype=np.int64)
    plain = _lib.regulator_order(FP_t, FX_t, valid)
    for gamma in (0.05, 0.2, 0.5, 3.0):
        lpt = _lib.regulator_order(FP_t, FX_t, valid, gamma)
        assert sorted(lpt.tolist()) == list(range(valid.size))
        groups = [tuple(plain[g:g + 32]) for g in range(0, valid.size, 32)]
        got = [tuple(lpt[g:g + 32]) for g in range(0, valid.size, 32)]
        assert sorted(got) == sorted(groups)
        # distances from the first group taken never decrease
        idx = [groups.index(g) for g in got]
        d = [abs(i - idx[0]) for i in idx]
        assert all(d[k] <= d[k + 1] for k in range(len(d) - 1))
