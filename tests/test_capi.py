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
