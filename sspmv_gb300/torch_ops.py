"""PyTorch custom operator over the C ABI: ``torch.ops.sspmv.spmv_csr``.

    y = torch.ops.sspmv.spmv_csr(row_offset, col_index, values, num_cols, x)

row_offset / col_index are int32 CUDA tensors, values and x float32 or
float64 CUDA tensors of one dtype; x is 1-D (num_cols) or 2-D (num_cols x k,
one SpMV per column).  The result is a new tensor (num_rows) or
(num_rows x k).  It runs the merge-path CSR kernel through
sspmv_LeSpMV_csr_noalloc on the current stream: nothing is allocated or
cached per matrix, so the operator is stateless; calls share one device
scratch array and must stay on one stream (the current-stream rule of
eager PyTorch).  A fake implementation gives shapes to tracing.
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
    if x.dim() not in (1, 2) or x.shape[0] != num_cols:
        raise ValueError("x must be (num_cols,) or (num_cols, k)")


@torch.library.custom_op("sspmv::spmv_csr", mutates_args=())
def spmv_csr(row_offset: torch.Tensor, col_index: torch.Tensor, values: torch.Tensor, num_cols: int,
             x: torch.Tensor) -> torch.Tensor:
    _check(row_offset, col_index, values, num_cols, x)
    m = row_offset.numel() - 1
    nnz = col_index.numel()
    rp, ci, cv = row_offset.contiguous(), col_index.contiguous(), values.contiguous()
    A = _lib.Csr()
    _lib.call("sspmv_csr_wrap", C.byref(A), _VT[values.dtype], m, int(num_cols), nnz, rp.data_ptr(),
              ci.data_ptr() if nnz else rp.data_ptr(), cv.data_ptr() if nnz else rp.data_ptr())
    stream = C.c_void_p(torch.cuda.current_stream(x.device).cuda_stream)
    cols = [x] if x.dim() == 1 else [x[:, j].contiguous() for j in range(x.shape[1])]
    outs = []
    for xc in cols:
        y = torch.empty(m, dtype=x.dtype, device=x.device)
        _lib.call("sspmv_LeSpMV_csr_noalloc", 1.0, C.byref(A), xc.data_ptr(), 0.0, y.data_ptr(), stream)
        outs.append(y)
    return outs[0] if x.dim() == 1 else torch.stack(outs, dim=1)


@spmv_csr.register_fake
def _(row_offset, col_index, values, num_cols, x):
    m = row_offset.shape[0] - 1
    return x.new_empty((m,) if x.dim() == 1 else (m, x.shape[1]))
