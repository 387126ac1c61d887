"""PyTorch custom operator over the C ABI: ``torch.ops.sspmv.spmv_csr``.

    y = torch.ops.sspmv.spmv_csr(row_offset, col_index, values, num_cols, x)

row_offset / col_index are int32 CUDA tensors, values and x float32 or
float64 CUDA tensors of one dtype, all on one device; x is 1-D (num_cols) or
2-D (num_cols x k).  The result is a new tensor (num_rows) or
(num_rows x k).  The call runs on x's device and its current stream and
keeps no state between calls:

  1-D x: the merge-path CSR kernel through sspmv_LeSpMV_csr_noalloc, which
         allocates nothing (its scratch is a fixed device array shared by all
         calls: calls that overlap on the GPU race, so keep them on one
         stream, the current-stream rule of eager PyTorch);
  2-D x: the library's SpMM (sspmv_spmm_csr, one pass for up to 8 columns,
         the same merge-path kernel) on a matrix wrapped for this call; its
         plan is built in stream order and released in stream order after the
         call (sspmv_release_plan), nothing waits for the device.

A fake implementation gives shapes to tracing.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib

_VT = {torch.float64: _lib.F64, torch.float32: _lib.F32}


def _check(row_offset, col_index, values, num_cols, x):
    if row_offset.dtype != torch.int32 or col_index.dtype != torch.int32:
        raise TypeError("row_offset and col_index must be int32")
    if values.dtype not in _VT or x.dtype != values.dtype:
        raise TypeError("values and x must share dtype float32 or float64")
    for name, t in (("row_offset", row_offset), ("col_index", col_index), ("values", values), ("x", x)):
        if not t.is_cuda:
            raise ValueError(f"{name} must be a CUDA tensor")
        if t.device != x.device:
            raise ValueError(f"{name} is on {t.device}, x on {x.device}: all tensors must share one device")
    if row_offset.dim() != 1 or row_offset.numel() < 1:
        raise ValueError("row_offset must be 1-D with num_rows + 1 >= 1 entries")
    if col_index.dim() != 1 or values.dim() != 1 or values.numel() != col_index.numel():
        raise ValueError("col_index and values must be 1-D with num_nnzs entries each")
    if x.dim() not in (1, 2) or x.shape[0] != num_cols:
        raise ValueError("x must be (num_cols,) or (num_cols, k)")


@torch.library.custom_op("sspmv::spmv_csr", mutates_args=())
def spmv_csr(row_offset: torch.Tensor, col_index: torch.Tensor, values: torch.Tensor, num_cols: int,
             x: torch.Tensor) -> torch.Tensor:
    _check(row_offset, col_index, values, num_cols, x)
    m = row_offset.numel() - 1
    nnz = col_index.numel()
    rp, ci, cv = row_offset.contiguous(), col_index.contiguous(), values.contiguous()
    with torch.cuda.device(x.device):
        A = _lib.Csr()
        _lib.call("sspmv_csr_wrap", C.byref(A), _VT[values.dtype], m, int(num_cols), nnz, rp.data_ptr(),
                  ci.data_ptr() if nnz else rp.data_ptr(), cv.data_ptr() if nnz else rp.data_ptr())
        stream = C.c_void_p(torch.cuda.current_stream(x.device).cuda_stream)
        if x.dim() == 1:
            xc = x.contiguous()
            y = torch.empty(m, dtype=x.dtype, device=x.device)
            _lib.call("sspmv_LeSpMV_csr_noalloc", 1.0, C.byref(A), xc.data_ptr(), 0.0, y.data_ptr(), stream)
            return y
        X = x.contiguous()
        k = int(X.shape[1])
        Y = torch.empty((m, k), dtype=x.dtype, device=x.device)
        if k == 0 or m == 0:
            return Y
        _lib.call("sspmv_set_kernel", C.byref(A.f), 2, 0)  # merge-path: its plan builds without a host wait
        try:
            _lib.call("sspmv_spmm_csr", 1.0, C.byref(A), k, X.data_ptr(), k, 0.0, Y.data_ptr(), k, stream)
        finally:
            _lib.call("sspmv_release_plan", C.byref(A.f), stream)
        return Y


@spmv_csr.register_fake
def _(row_offset, col_index, values, num_cols, x):
    m = row_offset.shape[0] - 1
    return x.new_empty((m,) if x.dim() == 1 else (m, x.shape[1]))
