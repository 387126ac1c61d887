"""Reference-facing Python API: LeSpMV's names over the C ABI.

    reference (LeSpMV)                      here
    CSR_Matrix<I,V> / read_csr_matrix        CSR_Matrix / read_csr_matrix
    csr_to_<fmt>(csr, params...)             csr_to_<fmt>(csr, params...)
    LeSpMV_<fmt>(alpha, A, x, beta, y)       LeSpMV_<fmt>(alpha, A, x, beta, y)
    delete_host_matrix(A)                    A.delete() (or garbage collection)

Matrices live on the GPU; x and y are CUDA tensors (torch) or raw device
pointers.  Calls are ordered on the current torch stream unless a stream is
given.  Errors raise SSPMVError carrying the library's status.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import Csr, F32, F64, SSPMVError, call, lib
from .formats import FORMATS, bsr_block_for, feasible_host  # noqa: F401  (re-exported)
from .synth import HostCSR

RowMajor, ColMajor = _lib.ROW_MAJOR, _lib.COL_MAJOR


def _stream(stream) -> C.c_void_p:
    if stream is None:
        import torch
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if hasattr(stream, "cuda_stream"):
        return C.c_void_p(stream.cuda_stream)
    return C.c_void_p(int(stream))


def _dptr(t) -> C.c_void_p:
    if t is None:
        return C.c_void_p(None)
    if hasattr(t, "data_ptr"):
        return C.c_void_p(t.data_ptr())
    return C.c_void_p(int(t))


def _vt(dtype) -> int:
    return F64 if np.dtype(dtype) == np.float64 else F32


class Matrix:
    """Base of the format wrappers: owns one C struct and frees it."""
    fmt = ""
    struct = None

    def __init__(self, s):
        self.s = s
        self._alive = True

    @property
    def num_rows(self) -> int:
        return int(self.s.f.num_rows)

    @property
    def num_cols(self) -> int:
        return int(self.s.f.num_cols)

    @property
    def num_nnzs(self) -> int:
        return int(self.s.f.num_nnzs)

    @property
    def dtype(self):
        return np.float64 if self.s.f.value_type == F64 else np.float32

    @property
    def kernel_flag(self) -> int:
        return int(self.s.f.kernel_flag)

    @kernel_flag.setter
    def kernel_flag(self, v: int) -> None:
        self.s.f.kernel_flag = int(v)

    def ref(self):
        return C.byref(self.s)

    def set_kernel(self, kernel_flag: int, param: int = 0) -> None:
        """Selects the SpMV kernel (sspmv_set_kernel)."""
        call("sspmv_set_kernel", C.byref(self.s.f), int(kernel_flag), int(param))

    def delete(self) -> None:
        if self._alive:
            self._alive = False
            getattr(lib, f"sspmv_delete_{self.fmt}")(C.byref(self.s))

    def __del__(self):
        try:
            self.delete()
        except Exception:
            pass

    def algorithmic_bytes(self, k: int = 1, beta_nonzero: bool = False) -> float:
        return float(getattr(lib, f"sspmv_algorithmic_bytes_{self.fmt}")(self.ref(), k, int(beta_nonzero)))

    def reference_bytes(self) -> float:
        """The reference benchmark's bytes_per_spmv (include/spmv_benchmark.h:26-150)."""
        b = float(getattr(lib, f"sspmv_reference_bytes_{self.fmt}")(self.ref()))
        if b < 0:
            raise RuntimeError(f"reference_bytes({self.fmt}): malformed matrix")
        return b


class CSR_Matrix(Matrix):
    fmt = "csr"

    def export(self, stream=None) -> dict:
        rp = np.empty(self.num_rows + 1, np.int32)
        col = np.empty(self.num_nnzs, np.int32)
        val = np.empty(self.num_nnzs, self.dtype)
        call("sspmv_csr_export", self.ref(), rp.ctypes.data_as(C.c_void_p), col.ctypes.data_as(C.c_void_p),
             val.ctypes.data_as(C.c_void_p), _stream(stream))
        return {"row_offset": rp, "col": col, "val": val}


def _host(n, dtype):
    a = np.empty(max(int(n), 0), dtype)
    return a, a.ctypes.data_as(C.c_void_p)


class ELL_Matrix(Matrix):
    fmt = "ell"

    def export(self, stream=None) -> dict:
        n = self.num_rows * self.s.max_row_width
        col, pc = _host(n, np.int32)
        val, pv = _host(n, self.dtype)
        call("sspmv_ell_export", self.ref(), pc, pv, _stream(stream))
        return {"max_row_width": int(self.s.max_row_width), "col": col, "val": val}


class SELL_Matrix(Matrix):
    """S_ELL_Matrix (sliced ELLPACK)."""
    fmt = "sell"

    def export(self, stream=None) -> dict:
        rw, pr = _host(self.s.chunk_num, np.int32)
        col, pc = _host(self.s.total_slots, np.int32)
        val, pv = _host(self.s.total_slots, self.dtype)
        call("sspmv_sell_export", self.ref(), pr, pc, pv, _stream(stream))
        return {"chunk_num": int(self.s.chunk_num), "row_width": rw, "col": col, "val": val}


class _SellReordered(Matrix):
    def export(self, stream=None) -> dict:
        ro, pro = _host(self.num_rows, np.int32)
        cl, pcl = _host(self.s.validchunkNum, np.int32)
        col, pc = _host(self.s.total_slots, np.int32)
        val, pv = _host(self.s.total_slots, self.dtype)
        call(f"sspmv_{self.fmt}_export", self.ref(), pro, pcl, pc, pv, _stream(stream))
        return {"reorder": ro, "chunk_len": cl, "col": col, "val": val,
                "validchunkNum": int(self.s.validchunkNum)}


class SELL_C_Sigma_Matrix(_SellReordered):
    fmt = "sell_c_sigma"


class SELL_C_R_Matrix(_SellReordered):
    fmt = "sell_c_R"


class COO_Matrix(Matrix):
    fmt = "coo"

    def export(self, stream=None) -> dict:
        ri, pr = _host(self.num_nnzs, np.int32)
        ci, pc = _host(self.num_nnzs, np.int32)
        v, pv = _host(self.num_nnzs, self.dtype)
        call("sspmv_coo_export", self.ref(), pr, pc, pv, _stream(stream))
        return {"row": ri, "col": ci, "val": v}


class DIA_Matrix(Matrix):
    fmt = "dia"

    def export(self, stream=None) -> dict:
        nd, st = int(self.s.complete_ndiags), int(self.s.stride)
        off, po = _host(nd, np.int64)
        data, pd = _host(nd * st, self.dtype)
        call("sspmv_dia_export", self.ref(), po, pd, _stream(stream))
        return {"complete_ndiags": nd, "stride": st, "offsets": off, "data": data}


class BSR_Matrix(Matrix):
    fmt = "bsr"

    def export(self, stream=None) -> dict:
        s = self.s
        one = s.blockDim_r == 1 and s.blockDim_c == 1
        rp, prp = _host((self.num_rows if one else s.mb) + 1, np.int32)
        ci, pci = _host(s.nnzb, np.int32)
        data, pd = _host(s.nnzb * s.blockNNZ, self.dtype)
        call("sspmv_bsr_export", self.ref(), prp, pci, pd, _stream(stream))
        return {"mb": int(s.mb), "nb": int(s.nb), "nnzb": int(s.nnzb), "row_ptr": rp, "colindex": ci,
                "data": data, "r": int(s.blockDim_r), "c": int(s.blockDim_c)}


class CSR5_Matrix(Matrix):
    fmt = "csr5"

    def export(self, stream=None) -> dict:
        s = self.s
        p = int(s._p)
        tp, ptp = _host(p + 1, np.uint32)
        td, ptd = _host(p * s.omega * s.num_packets, np.uint32)
        tdp, ptdp = _host(p + 1, np.int32)
        tdo, ptdo = _host(s.num_offsets, np.int32)
        col, pc = _host(self.num_nnzs, np.int32)
        val, pv = _host(self.num_nnzs, self.dtype)
        call("sspmv_csr5_export", self.ref(), ptp, ptd, ptdp, ptdo, pc, pv, _stream(stream))
        return {"sigma": int(s.sigma), "omega": int(s.omega), "bit_y_offset": int(s.bit_y_offset),
                "bit_scansum_offset": int(s.bit_scansum_offset), "num_packets": int(s.num_packets), "p": p,
                "num_offsets": int(s.num_offsets), "tail_partition_start": int(s.tail_partition_start),
                "tile_ptr": tp, "tile_desc": td, "tile_desc_offset_ptr": tdp, "tile_desc_offset": tdo,
                "col": col, "val": val}


def csr_to_csr5(csr: CSR_Matrix, sigma: int = 0, omega: int = 0, stream=None) -> CSR5_Matrix:
    """csr_to_csr5 (include/sparse_conversion.h:939-1379); 0 = reference default."""
    s = _lib.Csr5()
    call("sspmv_csr_to_csr5", csr.ref(), int(sigma), int(omega), C.byref(s), _stream(stream))
    return CSR5_Matrix(s)


def csr_to_coo(csr: CSR_Matrix, stream=None) -> COO_Matrix:
    """csr_to_coo (include/sparse_conversion.h:145-168)."""
    s = _lib.Coo()
    call("sspmv_csr_to_coo", csr.ref(), C.byref(s), _stream(stream))
    return COO_Matrix(s)


def coo_from_host(num_rows, num_cols, row_index, col_index, values, stream=None) -> COO_Matrix:
    s = _lib.Coo()
    v = np.ascontiguousarray(values)
    ri = np.ascontiguousarray(row_index, np.int32)
    ci = np.ascontiguousarray(col_index, np.int32)
    call("sspmv_coo_create", C.byref(s), _vt(v.dtype), num_rows, num_cols, len(v), ri.ctypes.data_as(C.c_void_p),
         ci.ctypes.data_as(C.c_void_p), v.ctypes.data_as(C.c_void_p), 1, _stream(stream))
    return COO_Matrix(s)


def coo_to_csr(coo: COO_Matrix, stream=None) -> CSR_Matrix:
    """coo_to_csr (include/sparse_conversion.h:30-91, compact = false)."""
    s = Csr()
    call("sspmv_coo_to_csr", coo.ref(), C.byref(s), _stream(stream))
    return CSR_Matrix(s)


def coo_to_ell(coo: COO_Matrix, ld: int = RowMajor, stream=None) -> ELL_Matrix:
    """coo_to_ell (include/sparse_conversion.h:94-142): each row's entries in
    COO order; ld is ignored (RowMajor), as in the reference."""
    s = _lib.Ell()
    call("sspmv_coo_to_ell", coo.ref(), int(ld), C.byref(s), _stream(stream))
    return ELL_Matrix(s)


def csr_to_dia(csr: CSR_Matrix, max_diags: int = 0, alignment: int = 0, stream=None) -> DIA_Matrix:
    """csr_to_dia (include/sparse_conversion.h:612-766); SSPMVError status 2
    (SSPMV_INFEASIBLE) above max_diags."""
    s = _lib.Dia()
    call("sspmv_csr_to_dia", csr.ref(), int(max_diags), int(alignment), C.byref(s), _stream(stream))
    return DIA_Matrix(s)


def csr_to_bsr(csr: CSR_Matrix, blockDimRow: int = 0, blockDimCol: int = 0, stream=None) -> BSR_Matrix:
    """csr_to_bsr (include/sparse_conversion.h:769-926); 0 = reference default."""
    s = _lib.Bsr()
    call("sspmv_csr_to_bsr", csr.ref(), int(blockDimRow), int(blockDimCol), C.byref(s), _stream(stream))
    return BSR_Matrix(s)


def csr_to_ell(csr: CSR_Matrix, ld: int = RowMajor, stream=None) -> ELL_Matrix:
    """csr_to_ell (include/sparse_conversion.h:187-248)."""
    s = _lib.Ell()
    call("sspmv_csr_to_ell", csr.ref(), int(ld), C.byref(s), _stream(stream))
    return ELL_Matrix(s)


def csr_to_sell(csr: CSR_Matrix, chunkwidth: int = 0, alignment: int = 0, stream=None) -> SELL_Matrix:
    """csr_to_sell (include/sparse_conversion.h:258-334); 0 = reference default."""
    s = _lib.SEll()
    call("sspmv_csr_to_sell", csr.ref(), int(chunkwidth), int(alignment), C.byref(s), _stream(stream))
    return SELL_Matrix(s)


def csr_to_sell_c_sigma(csr: CSR_Matrix, slicewidth: int = 0, chunkwidth: int = 0, alignment: int = 0,
                        stream=None) -> SELL_C_Sigma_Matrix:
    """csr_to_sell_c_sigma (include/sparse_conversion.h:337-479)."""
    s = _lib.SellCSigma()
    call("sspmv_csr_to_sell_c_sigma", csr.ref(), int(slicewidth), int(chunkwidth), int(alignment), C.byref(s),
         _stream(stream))
    return SELL_C_Sigma_Matrix(s)


def csr_to_sell_c_R(csr: CSR_Matrix, chunkwidth: int = 0, alignment: int = 0, stream=None) -> SELL_C_R_Matrix:
    """csr_to_sell_c_R (include/sparse_conversion.h:483-598)."""
    s = _lib.SellCR()
    call("sspmv_csr_to_sell_c_R", csr.ref(), int(chunkwidth), int(alignment), C.byref(s), _stream(stream))
    return SELL_C_R_Matrix(s)


def csr_from_host(A: HostCSR, stream=None) -> CSR_Matrix:
    """Uploads a host CSR (the reference's CSR_Matrix) to the device."""
    s = Csr()
    vals = np.ascontiguousarray(A.values)
    call("sspmv_csr_create", C.byref(s), _vt(vals.dtype), A.num_rows, A.num_cols, A.nnz,
         A.row_offset.ctypes.data_as(C.c_void_p), A.col_index.ctypes.data_as(C.c_void_p),
         vals.ctypes.data_as(C.c_void_p), 1, _stream(stream))
    return CSR_Matrix(s)


FEATURE_NAMES = [lib.sspmv_feature_name(i).decode() for i in range(_lib.NUM_FEATURES)]


def features(csr: CSR_Matrix, tile_blocks: int = 256, arrays: bool = False, stream=None):
    """MTX feature extraction on the GPU (src/sparse_features.cpp): a vector of
    62 features (names in FEATURE_NAMES), and with arrays=True the per-tile
    nonzero / distinct-row / distinct-column counts (T*T each)."""
    F = np.zeros(_lib.NUM_FEATURES)
    TT = tile_blocks * tile_blocks
    t = np.zeros(TT, np.int32) if arrays else None
    u = np.zeros(TT, np.int32) if arrays else None
    v = np.zeros(TT, np.int32) if arrays else None
    ptr = (lambda a: a.ctypes.data_as(C.c_void_p) if a is not None else None)
    call("sspmv_csr_features", csr.ref(), int(tile_blocks), F.ctypes.data_as(C.c_void_p), ptr(t), ptr(u), ptr(v),
         _stream(stream))
    if arrays:
        return F, {"tiles": t, "urb": u, "ucb": v}
    return F


GRX_NAMES = ("GrX_uniqR", "GrX_uniqC", "GrX_potReuseR", "GrX_potReuseC")


def grx_features(csr: CSR_Matrix, tile_blocks: int = 256, group: int = 0, stream=None) -> np.ndarray:
    """GrX_uniqR, GrX_uniqC, GrX_potReuseR, GrX_potReuseC (tile group
    analysis, src/sparse_features.cpp:884-1065); group 0 = 64 / sizeof(value)."""
    out = np.zeros(4)
    call("sspmv_csr_grx_features", csr.ref(), int(tile_blocks), int(group), out.ctypes.data_as(C.c_void_p),
         _stream(stream))
    return out


def wait_timeouts() -> int:
    """Bounded device waits that gave up since the library was loaded (0 in
    every correct run)."""
    n = C.c_int64()
    call("sspmv_wait_timeouts", C.byref(n))
    return int(n.value)


def sum_csr_duplicates(A: HostCSR) -> HostCSR:
    """sum_csr_duplicates (include/sparse_operation.h:22-73) on a copy of A:
    equal columns of a row summed, columns in reverse order of first
    appearance, zero sums dropped."""
    rp = np.array(A.row_offset, np.int32)
    ci = np.array(A.col_index, np.int32)
    cv = np.array(A.values)
    nnz = C.c_int64(0)
    call("sspmv_sum_csr_duplicates", _vt(cv.dtype), A.num_rows, A.num_cols, rp.ctypes.data_as(C.c_void_p),
         ci.ctypes.data_as(C.c_void_p), cv.ctypes.data_as(C.c_void_p), C.byref(nnz))
    return HostCSR(A.num_rows, A.num_cols, rp, ci[:nnz.value].copy(), cv[:nnz.value].copy())


def read_csr_matrix(path: str, precision: int = 64, compact: bool = False) -> HostCSR:
    """read_csr_matrix (utils/sparse_io.cpp:180-204) on the host; compact:
    duplicates summed (sum_csr_duplicates)."""
    vt = F64 if precision == 64 else F32
    m, n, nnz = C.c_int64(), C.c_int64(), C.c_int64()
    call("sspmv_read_mtx", str(path).encode(), vt, C.byref(m), C.byref(n), C.byref(nnz), None, None, None)
    rp = np.empty(m.value + 1, np.int32)
    col = np.empty(nnz.value, np.int32)
    val = np.empty(nnz.value, np.float64 if vt == F64 else np.float32)
    call("sspmv_read_mtx", str(path).encode(), vt, C.byref(m), C.byref(n), C.byref(nnz),
         rp.ctypes.data_as(C.c_void_p), col.ctypes.data_as(C.c_void_p), val.ctypes.data_as(C.c_void_p))
    A = HostCSR(int(m.value), int(n.value), rp, col, val)
    return sum_csr_duplicates(A) if compact else A


def read_coo_triplets(path: str, precision: int = 64):
    """The .mtx triplets in file order (read_coo_matrix's order, symmetric
    mirrors right after their entries): (num_rows, num_cols, rows, cols, vals)."""
    vt = F64 if precision == 64 else F32
    m, n, nnz = C.c_int64(), C.c_int64(), C.c_int64()
    call("sspmv_read_mtx_coo", str(path).encode(), vt, C.byref(m), C.byref(n), C.byref(nnz), None, None, None)
    ri = np.empty(nnz.value, np.int32)
    ci = np.empty(nnz.value, np.int32)
    val = np.empty(nnz.value, np.float64 if vt == F64 else np.float32)
    call("sspmv_read_mtx_coo", str(path).encode(), vt, C.byref(m), C.byref(n), C.byref(nnz),
         ri.ctypes.data_as(C.c_void_p), ci.ctypes.data_as(C.c_void_p), val.ctypes.data_as(C.c_void_p))
    return int(m.value), int(n.value), ri, ci, val


# Readers of the reference's sparse_io.h: .mtx -> device matrix of a format
# (utils/sparse_io.cpp: CSR then csr_to_<fmt>; ELL through COO).
def read_coo_matrix(path: str, precision: int = 64, stream=None) -> COO_Matrix:
    """read_coo_matrix (utils/sparse_io.cpp:27-163): entries in file order."""
    return coo_from_host(*read_coo_triplets(path, precision), stream=stream)


def read_csr_device(path: str, precision: int = 64, stream=None) -> CSR_Matrix:
    """read_csr_matrix (utils/sparse_io.cpp:180-204) onto the device."""
    return csr_from_host(read_csr_matrix(path, precision), stream)


def _read_then(path, precision, convert, stream):
    csr = read_csr_device(path, precision, stream)
    try:
        return convert(csr)
    finally:
        csr.delete()


def read_ell_matrix(path: str, ld: int = RowMajor, precision: int = 64, stream=None) -> ELL_Matrix:
    """read_ell_matrix (utils/sparse_io.cpp:273-299): read_coo_matrix, then coo_to_ell."""
    coo = read_coo_matrix(path, precision, stream)
    try:
        return coo_to_ell(coo, ld, stream)
    finally:
        coo.delete()


def read_dia_matrix(path: str, max_diags: int = 0, alignment: int = 0, precision: int = 64, stream=None):
    """read_dia_matrix (utils/sparse_io.cpp:315-329)."""
    return _read_then(path, precision, lambda c: csr_to_dia(c, max_diags, alignment, stream), stream)


def read_bsr_matrix(path: str, blockDimRow: int = 0, blockDimCol: int = 0, precision: int = 64, stream=None):
    """read_bsr_matrix (utils/sparse_io.cpp:213-227)."""
    return _read_then(path, precision, lambda c: csr_to_bsr(c, blockDimRow, blockDimCol, stream), stream)


def read_csr5_matrix(path: str, precision: int = 64, stream=None):
    """read_csr5_matrix (utils/sparse_io.cpp:243-258)."""
    return _read_then(path, precision, lambda c: csr_to_csr5(c, 0, 0, stream), stream)


def read_sell_matrix(path: str, chunkwidth: int = 0, alignment: int = 0, precision: int = 64, stream=None):
    """read_sell_matrix (utils/sparse_io.cpp:347-362)."""
    return _read_then(path, precision, lambda c: csr_to_sell(c, chunkwidth, alignment, stream), stream)


def read_sell_c_sigma_matrix(path: str, slicewidth: int = 0, chunkwidth: int = 0, alignment: int = 0,
                             precision: int = 64, stream=None):
    """read_sell_c_sigma_matrix (utils/sparse_io.cpp:370-384)."""
    return _read_then(path, precision, lambda c: csr_to_sell_c_sigma(c, slicewidth, chunkwidth, alignment, stream),
                      stream)


def read_sell_c_R_matrix(path: str, chunkwidth: int = 0, alignment: int = 0, precision: int = 64, stream=None):
    """read_sell_c_R_matrix (utils/sparse_io.cpp:393-407)."""
    return _read_then(path, precision, lambda c: csr_to_sell_c_R(c, chunkwidth, alignment, stream), stream)


def write_mtx(path: str, A: HostCSR) -> None:
    vals = np.ascontiguousarray(A.values, dtype=np.float64)
    call("sspmv_write_mtx", str(path).encode(), A.num_rows, A.num_cols, A.row_offset.ctypes.data_as(C.c_void_p),
         A.col_index.ctypes.data_as(C.c_void_p), vals.ctypes.data_as(C.c_void_p))


def LeSpMV(alpha: float, A: Matrix, x, beta: float, y, stream=None) -> None:
    """y = alpha*A*x + beta*y for any format (LeSpMV_<fmt>)."""
    call(f"sspmv_LeSpMV_{A.fmt}", float(alpha), A.ref(), _dptr(x), float(beta), _dptr(y), _stream(stream))


def spmm(alpha: float, A: Matrix, X, beta: float, Y, k: int | None = None, ldx: int | None = None,
         ldy: int | None = None, stream=None) -> None:
    """Y = alpha*A*X + beta*Y, X row-major num_cols x k, Y num_rows x k."""
    if k is None:
        k = int(X.shape[1]) if hasattr(X, "shape") and len(X.shape) == 2 else 1
    ldx = ldx or (int(X.stride(0)) if hasattr(X, "stride") and len(X.shape) == 2 else k)
    ldy = ldy or (int(Y.stride(0)) if hasattr(Y, "stride") and len(Y.shape) == 2 else k)
    call(f"sspmv_spmm_{A.fmt}", float(alpha), A.ref(), int(k), _dptr(X), int(ldx), float(beta), _dptr(Y), int(ldy),
         _stream(stream))


def LeSpMV_csr(alpha, A: CSR_Matrix, x, beta, y, stream=None) -> None:
    LeSpMV(alpha, A, x, beta, y, stream)


# Smoke-check formats converted from CSR (besides CSR itself).
SMOKE_FORMATS: list[str] = ["coo", "ell", "sell", "sell_c_sigma", "sell_c_R", "bsr", "csr5"]


def count_blocks(csr: CSR_Matrix, r: int, c: int, stream=None) -> int:
    """Distinct r x c blocks of a device CSR (no block data allocated)."""
    n = C.c_int64()
    call("sspmv_csr_count_blocks", csr.ref(), int(r), int(c), C.byref(n), _stream(stream))
    return int(n.value)


def build_format(csr: CSR_Matrix, fmt: str, A: HostCSR | None = None):
    """Converts a device CSR to `fmt`; returns (matrix, None) or (None, why).
    Formats whose padding or block fill exceeds 4x the CSR size are skipped;
    DIA over 10240 diagonals is reported by the converter itself."""
    if fmt == "ell" and A is not None:
        ok, why = feasible_host(fmt, A)
        if not ok:
            return None, why
    if fmt == "bsr":
        r, c = bsr_block_for(A) if A is not None else (4, 4)
        nnzb = count_blocks(csr, r, c)
        if nnzb * r * c > 4 * max(csr.num_nnzs, 1):
            return None, f"BSR {r}x{c} fill {nnzb * r * c / max(csr.num_nnzs, 1):.1f}x"
    if fmt == "csr":
        return csr, None
    fn = globals().get(f"csr_to_{fmt}")
    if fn is None:
        return None, "not built"
    try:
        if fmt == "bsr" and A is not None:
            r, c = bsr_block_for(A)
            return fn(csr, r, c), None
        return fn(csr), None
    except SSPMVError as e:
        return None, str(e)


__all__ = ["CSR_Matrix", "csr_from_host", "read_csr_matrix", "write_mtx", "LeSpMV", "LeSpMV_csr", "spmm",
           "RowMajor", "ColMajor", "SSPMVError"]
