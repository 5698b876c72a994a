"""Build and load the native library (libpycwb_gb300.so, CUDA sm_103a).

The library exports the C ABI declared in include/pycwb_gb300.h.  It is
built in-tree with nvcc; Python reaches it through ctypes and passes raw
device pointers and CUDA stream handles taken from torch tensors (torch is
used for device memory and streams only).  There is no fallback: if the
library is missing or CUDA is unavailable, the calls raise.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(REPO, "include")
LIB_PATH = os.path.join(PKG, "libpycwb_gb300.so")
# the sky-loop kernel's variants compile in five translation units of their
# own (skyloop_i*.cu), in parallel with the rest
SOURCES = ["skyloop.cu", "skyloop_i12.cu", "skyloop_i3.cu", "skyloop_i4.cu", "skyloop_i56.cu",
           "skyloop_i78.cu", "tdamp.cu", "probe.cu", "adjoint.cu", "subnet.cu", "skytables.cu",
           "wdm.cu", "skystat.cu", "skyprob.cu"]
HEADERS = ["common.cuh", "skyloop_kernel.cuh"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

_lock = threading.Lock()
_lib = None


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(INCLUDE, "pycwb_gb300.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every translation unit in parallel and link the shared library."""
    with _lock:
        if not force and not _stale():
            return LIB_PATH
        objs, procs = [], []
        for src in SOURCES:
            obj = os.path.join(CSRC, src.replace(".cu", ".o"))
            cmd = [nvcc(), ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-I", INCLUDE, "-c", os.path.join(CSRC, src), "-o", obj]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                                stderr=subprocess.STDOUT, text=True)))
            objs.append(obj)
        errors = []
        for src, p in procs:
            out, _ = p.communicate()
            if verbose and out:
                print(out)
            if p.returncode != 0:
                errors.append(f"{src}:\n{out}")
        if errors:
            raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
        tmp = LIB_PATH + ".tmp"
        subprocess.run([nvcc(), ARCH, "-shared", "-o", tmp] + objs + ["-lcudart"], check=True)
        os.replace(tmp, LIB_PATH)
        return LIB_PATH


def load():
    """The loaded library with argument types set (raises if it cannot load)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: run pycwb_gb300._lib.build() (needs nvcc)")
        L = ctypes.CDLL(LIB_PATH)
        P, i32, i64, f32, f64, sz = (ctypes.c_void_p, ctypes.c_int, ctypes.c_int64,
                                     ctypes.c_float, ctypes.c_double, ctypes.c_size_t)
        L.pgw_version.restype = ctypes.c_char_p
        L.pgw_last_error.restype = ctypes.c_char_p
        L.pgw_workspace_bytes.argtypes = [i32, i32, i64, i32]
        L.pgw_workspace_bytes.restype = sz
        L.pgw_calculate_dpf.argtypes = [P, P, P, i64, i32, i64, f64, f64, P, i64, P, P, P, sz, P]
        L.pgw_scan_sky_for_best_fit.argtypes = [i32, i64, i64, P, P, P, P, P, i32, P, P, f64, f64,
                                                f64, P, i64, P, P, P, P, sz, P]
        L.pgw_sky_loop.argtypes = [i32, i64, i64, P, P, P, P, P, i32, P, f32, f64, f64, f64, P,
                                   i64, P, P, P, P, P, P, P, sz, P]
        L.pgw_sky_loop_batched.argtypes = [i32, i32, P, P, i64, i64, P, P, P, P, P, i32, P, f32,
                                           f64, f64, f64, P, i64, P, P, P, P, P, P, P, sz, P]
        L.pgw_sky_order.argtypes = [P, i32, i64, P, i64, P, P]
        L.pgw_regulator_order.argtypes = [P, P, i32, i64, P, i64, P]
        L.pgw_regulator_order.restype = ctypes.c_int
        if hasattr(L, "pgw_regulator_order_lpt"):
            L.pgw_regulator_order_lpt.argtypes = [P, P, i32, i64, P, i64, f64, P]
            L.pgw_regulator_order_lpt.restype = ctypes.c_int
        L.pgw_td_vecs_to_clusters.argtypes = [P, i64, P, P, i32, P, P, i32, i32, P, P, i64, P, P, P, i32,
                                              i32, i32, i32, P, P, P]
        L.pgw_td_vecs_to_clusters.restype = ctypes.c_int
        L.pgw_sky_stat_grad.argtypes = [i32, i32, P, P, P, P, P, P, P, P, i32, P, f32, P, f64, P, P]
        L.pgw_sky_stat_grad.restype = ctypes.c_int
        L.pgw_refine_sky.argtypes = [i32, i32, P, P, P, P, P, P, P, P, i32, P, f32, P, f64, i32, f32,
                                     P, P, P, P, P]
        L.pgw_refine_sky.restype = ctypes.c_int
        L.pgw_sky_order.restype = ctypes.c_int
        L.pgw_batch_get_td_vecs.argtypes = [P, i64, P, P, i64, P, P, P, i32, i32, i32, i32, P, P]
        L.pgw_fp32_fma_peak.argtypes = [i32, P, P, P]
        L.pgw_calculate_dpf_batched.argtypes = [i32, i32, P, i64, i64, P, P, P, f64, f64, P, i64,
                                                P, P, P, P, P, sz, P]
        L.pgw_calculate_dpf_batched.restype = ctypes.c_int
        L.pgw_subnet_sky_batched.argtypes = [i32, i32, P, P, i64, i64, P, P, P, P, P, i32, P, f32,
                                             f64, f64, P, P]
        L.pgw_subnet_sky_batched.restype = ctypes.c_int
        L.pgw_sky_tables_healpix.argtypes = [i32, i32, P, P, f64, f64, i32, P, P, P, P]
        L.pgw_sky_tables_healpix.restype = ctypes.c_int
        L.pgw_skystat_workspace_bytes.argtypes = [i32, i64]
        L.pgw_skystat_workspace_bytes.restype = sz
        L.pgw_skystat_batched.argtypes = [i32, i32, P, P, i64, i64, P, P, P, P, P, i32, P, P, P,
                                          f32, f32, P, i64, P, i32, P, sz, P, P]
        L.pgw_skystat_batched.restype = ctypes.c_int
        L.pgw_wdm_t2w.argtypes = [P, i64, i32, P, i64, P, P, P, P, i32, P]
        L.pgw_wdm_t2w.restype = ctypes.c_int
        L.pgw_wdm_n_time.argtypes = [i64, i32]
        L.pgw_wdm_n_time.restype = i64
        L.pgw_copy_from_host.argtypes = [P, P, sz, P]
        L.pgw_copy_from_host.restype = ctypes.c_int
        L.pgw_fp64_mul_add_peak.argtypes = [i32, P, P, P]
        L.pgw_fp64_mul_add_peak.restype = ctypes.c_int
        L.pgw_sky_loop_noalloc.argtypes = [i32, i64, i64, P, P, P, P, P, i32, P, f32, f64, f64,
                                           f64, P, i64, P, P, P, P, P]
        L.pgw_sky_loop_noalloc.restype = ctypes.c_int
        L.pgw_sky_loop_noalloc_max_scratch.restype = sz
        L.pgw_sky_probability.argtypes = [i32, i64, P, i64, P, P, P, P]
        L.pgw_skystat_pixel_arrays.argtypes = [i32, i64, P, sz, P, P, P]
        L.pgw_skystat_pixel_arrays.restype = ctypes.c_int
        L.pgw_sky_probability.restype = ctypes.c_int
        for name in ("pgw_fp32_fma_peak", "pgw_calculate_dpf", "pgw_scan_sky_for_best_fit", "pgw_sky_loop",
                     "pgw_sky_loop_batched", "pgw_batch_get_td_vecs"):
            getattr(L, name).restype = ctypes.c_int
        _lib = L
        return _lib


class TileShape(ctypes.Structure):
    """pgw_tile_shape (include/pycwb_gb300.h); 0 in a field = automatic."""
    _fields_ = [("threads", ctypes.c_int), ("lanes_per_sky", ctypes.c_int),
                ("chunk_pix", ctypes.c_int), ("stages", ctypes.c_int),
                ("min_blocks", ctypes.c_int), ("fast_math", ctypes.c_int)]

    def key(self):
        return (self.threads, self.lanes_per_sky, self.chunk_pix, self.stages, self.min_blocks,
                self.fast_math)


def sky_order(ml, sky_valid_indices):
    """Scan order of the valid directions grouped by delay tuple (host int32)."""
    import numpy as np
    ml = np.ascontiguousarray(ml, dtype=np.int32)
    valid = np.ascontiguousarray(sky_valid_indices, dtype=np.int64)
    out = np.empty(valid.size, dtype=np.int32)
    n_t = ctypes.c_int64(0)
    rc = load().pgw_sky_order(ml.ctypes.data, ml.shape[0], ml.shape[1], valid.ctypes.data,
                              valid.size, out.ctypes.data, ctypes.byref(n_t))
    check(rc, "sky_order")
    return out, int(n_t.value)


def regulator_order(FP_t, FX_t, sky_valid_indices, gamma_regulator=None):
    """Regulator order of the valid directions (host int32): pgw_regulator_order,
    or with gamma_regulator its longest-tiles-first grouping
    (pgw_regulator_order_lpt)."""
    import numpy as np
    FP_t = np.ascontiguousarray(FP_t, dtype=np.float32)
    FX_t = np.ascontiguousarray(FX_t, dtype=np.float32)
    valid = np.ascontiguousarray(sky_valid_indices, dtype=np.int64)
    if FP_t.ndim != 2 or FX_t.shape != FP_t.shape:
        raise ValueError("FP/FX must both be (n_sky, n_ifo)")
    out = np.empty(valid.size, dtype=np.int32)
    L = load()
    if gamma_regulator is not None and hasattr(L, "pgw_regulator_order_lpt"):
        rc = L.pgw_regulator_order_lpt(FP_t.ctypes.data, FX_t.ctypes.data, FP_t.shape[1],
                                       FP_t.shape[0], valid.ctypes.data, valid.size,
                                       float(gamma_regulator), out.ctypes.data)
    else:
        rc = L.pgw_regulator_order(FP_t.ctypes.data, FX_t.ctypes.data, FP_t.shape[1],
                                   FP_t.shape[0], valid.ctypes.data, valid.size,
                                   out.ctypes.data)
    check(rc, "regulator_order")
    return out


STATUS_NAMES = {
    1: "bad shape", 2: "bad argument", 3: "CUDA error", 4: "workspace too small",
    5: "delay index outside the td window", 6: "bounded wait expired",
    7: "sky index outside [0, n_sky)",
}


def check(rc: int, what: str) -> None:
    """Turn a pgw_status into the reference's exception types."""
    if rc == 0:
        return
    msg = load().pgw_last_error().decode(errors="replace")
    if rc in (1, 2, 4):
        raise ValueError(f"{what}: {STATUS_NAMES.get(rc, rc)}: {msg}")
    raise RuntimeError(f"{what}: {STATUS_NAMES.get(rc, rc)}: {msg}")


def check_device_status(status: int, what: str) -> None:
    if status == 0:
        return
    names = [STATUS_NAMES.get(b, str(b)) for b in range(32) if status & (1 << b)]
    raise RuntimeError(f"{what}: device reported " + ", ".join(names))
