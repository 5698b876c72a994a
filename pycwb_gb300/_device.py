"""Device plumbing for the host layer: tensors, streams and workspaces.

torch provides device memory, pinned host memory and CUDA streams; the
compute is the native library's.  Every caller thread gets its own CUDA
stream and its own workspace, so concurrent callers (the reference runs lags
in a ThreadPoolExecutor, process_job_segment_native.py:351-389) never share
scratch memory.
"""

from __future__ import annotations

import threading

import numpy as np
import torch

RESULT_DTYPE = np.dtype([("l_max", "<i8"), ("sky_stat_max", "<f4"), ("found", "<i4"),
                         ("status", "<i4"), ("regulator", "<f4"), ("active_pairs", "<i8")])
assert RESULT_DTYPE.itemsize == 32

_tls = threading.local()


def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("pycwb_gb300 needs a CUDA GPU; no CPU fallback exists")
    return torch.device("cuda", torch.cuda.current_device())


def stream() -> torch.cuda.Stream:
    """This thread's CUDA stream (created on first use)."""
    s = getattr(_tls, "stream", None)
    if s is None:
        s = torch.cuda.Stream(device=require_cuda())
        _tls.stream = s
    return s


def begin() -> torch.cuda.Stream:
    """This thread's stream, ordered after the caller's current stream, so
    device inputs the caller produced on its stream are complete."""
    s = stream()
    s.wait_stream(torch.cuda.current_stream())
    return s


def end(s: torch.cuda.Stream, *outputs: torch.Tensor) -> None:
    """Order the caller's current stream after `s` and tie `outputs` to it."""
    cur = torch.cuda.current_stream()
    cur.wait_stream(s)
    for t in outputs:
        if isinstance(t, torch.Tensor) and t.is_cuda:
            t.record_stream(cur)


def workspace(nbytes: int) -> torch.Tensor:
    """This thread's scratch buffer, grown on demand (256-byte aligned)."""
    ws = getattr(_tls, "ws", None)
    if ws is None or ws.numel() < nbytes:
        with torch.cuda.stream(stream()):
            ws = torch.empty(max(int(nbytes), 1 << 16), dtype=torch.uint8, device=require_cuda())
        _tls.ws = ws
    return ws


def to_device(x, dtype: torch.dtype) -> torch.Tensor:
    """A contiguous CUDA tensor of `dtype` (no copy when x already is one)."""
    dev = require_cuda()
    if isinstance(x, torch.Tensor):
        if x.device.type == "cuda" and x.dtype == dtype and x.is_contiguous():
            x.record_stream(stream())  # used on this thread's stream from here on
            return x
        with torch.cuda.stream(stream()):
            return x.to(device=dev, dtype=dtype).contiguous()
    np_dtype = {torch.float32: np.float32, torch.float64: np.float64,
                torch.int32: np.int32, torch.int64: np.int64}[dtype]
    a = np.ascontiguousarray(np.asarray(x), dtype=np_dtype)
    with torch.cuda.stream(stream()):
        return torch.from_numpy(a).to(dev, non_blocking=False)


def ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def stream_handle(s: torch.cuda.Stream | None = None) -> int:
    return (s or stream()).cuda_stream


def shape_of(x) -> tuple:
    return tuple(x.shape)


def results_to_numpy(t: torch.Tensor) -> np.ndarray:
    """Device pgw_scan_result array -> numpy structured array."""
    return t.cpu().numpy().view(RESULT_DTYPE)
