"""ctypes binding of libsspmv.so (include/sspmv.h).

The library is built in-tree (sspmv_gb300/lib/libsspmv.so).  Importing this
module fails loudly when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "lib" / "libsspmv.so"

F32, F64 = 0, 1
ROW_MAJOR, COL_MAJOR = 0, 1

STATUS = {0: "SSPMV_OK", 1: "SSPMV_INVALID_ARG", 2: "SSPMV_INFEASIBLE", 3: "SSPMV_OUT_OF_MEMORY",
          4: "SSPMV_BUDGET_EXCEEDED", 5: "SSPMV_DEVICE_TIMEOUT", 6: "SSPMV_CUDA_ERROR",
          7: "SSPMV_NOT_SUPPORTED"}


class SSPMVError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str):
        super().__init__(f"{where}: {STATUS.get(status, status)}: {detail}")
        self.status = status


class Features(C.Structure):
    _fields_ = [("num_rows", C.c_int64), ("num_cols", C.c_int64), ("num_nnzs", C.c_int64),
                ("sparsity", C.c_double), ("time", C.c_double), ("gflops", C.c_double),
                ("gbytes", C.c_double), ("tag", C.c_int32), ("kernel_flag", C.c_int32),
                ("value_type", C.c_int32), ("owns", C.c_int32), ("priv", C.c_void_p)]


P32 = C.POINTER(C.c_int32)


class Coo(C.Structure):
    _fields_ = [("f", Features), ("row_index", P32), ("col_index", P32), ("values", C.c_void_p),
                ("row_sorted", C.c_int32)]


class Csr(C.Structure):
    _fields_ = [("f", Features), ("row_offset", P32), ("col_index", P32), ("values", C.c_void_p)]


P64 = C.POINTER(C.c_int64)


class Ell(C.Structure):
    _fields_ = [("f", Features), ("ld", C.c_int32), ("max_row_width", C.c_int32), ("min_row_width", C.c_int32),
                ("col_index", P32), ("values", C.c_void_p)]


class SEll(C.Structure):
    _fields_ = [("f", Features), ("sliceWidth", C.c_int32), ("chunk_num", C.c_int32), ("alignment", C.c_int32),
                ("row_width", P32), ("chunk_ptr", P64), ("total_slots", C.c_int64), ("col_index", P32),
                ("values", C.c_void_p)]


class SellCSigma(C.Structure):
    _fields_ = [("f", Features), ("sliceWidth_Sigma", C.c_int32), ("chunkWidth_C", C.c_int32),
                ("sliceNum", C.c_int32), ("chunkNum", C.c_int32), ("validchunkNum", C.c_int32),
                ("chunk_num_per_slice", C.c_int32), ("alignment", C.c_int32), ("reorder", P32),
                ("chunk_len", P32), ("chunk_ptr", P64), ("total_slots", C.c_int64), ("col_index", P32),
                ("values", C.c_void_p)]


class SellCR(C.Structure):
    _fields_ = [("f", Features), ("chunkWidth_C", C.c_int32), ("validchunkNum", C.c_int32),
                ("alignment", C.c_int32), ("reorder", P32), ("chunk_len", P32), ("chunk_ptr", P64),
                ("total_slots", C.c_int64), ("col_index", P32), ("values", C.c_void_p)]


class Dia(C.Structure):
    _fields_ = [("f", Features), ("stride", C.c_int32), ("complete_ndiags", C.c_int32), ("diag_offsets", P64),
                ("diag_data", C.c_void_p)]


class Bsr(C.Structure):
    _fields_ = [("f", Features), ("blockDim_r", C.c_int64), ("blockDim_c", C.c_int64), ("blockNNZ", C.c_int64),
                ("mb", C.c_int64), ("nb", C.c_int64), ("nnzb", C.c_int64), ("row_ptr", P32),
                ("block_colindex", P32), ("block_data", C.c_void_p)]


PU32 = C.POINTER(C.c_uint32)


class Csr5(C.Structure):
    _fields_ = [("f", Features), ("row_offset", P32), ("col_index", P32), ("values", C.c_void_p),
                ("sigma", C.c_int32), ("omega", C.c_int32), ("bit_y_offset", C.c_int32),
                ("bit_scansum_offset", C.c_int32), ("num_packets", C.c_int32), ("num_offsets", C.c_int32),
                ("_p", C.c_int32), ("tail_partition_start", C.c_int32), ("tile_ptr", PU32), ("tile_desc", PU32),
                ("tile_desc_offset_ptr", P32), ("tile_desc_offset", P32)]


from .synth import SynthParams  # noqa: E402  (argument type of the sspmv_synth_* exports)


def _load():
    if not _LIB_PATH.exists():
        raise ImportError(f"libsspmv.so is not built ({_LIB_PATH}); run __graft_entry__.build() "
                          "or python -m sspmv_gb300.build")
    return C.CDLL(str(_LIB_PATH))


lib = _load()

_st = C.c_int
_vp = C.c_void_p
_i64 = C.c_int64
_i32 = C.c_int32
_d = C.c_double

_SIGS = {
    "sspmv_status_string": (C.c_char_p, [_st]),
    "sspmv_last_error": (C.c_char_p, []),
    "sspmv_version": (C.c_char_p, []),
    "sspmv_launch_count": (_i64, []),
    "sspmv_set_kernel": (_st, [C.POINTER(Features), _i32, _i32]),
    "sspmv_csr_create": (_st, [C.POINTER(Csr), _i32, _i64, _i64, _i64, _vp, _vp, _vp, _i32, _vp]),
    "sspmv_csr_wrap": (_st, [C.POINTER(Csr), _i32, _i64, _i64, _i64, _vp, _vp, _vp]),
    "sspmv_csr_export": (_st, [C.POINTER(Csr), _vp, _vp, _vp, _vp]),
    "sspmv_delete_csr": (_st, [C.POINTER(Csr)]),
    "sspmv_LeSpMV_csr": (_st, [_d, C.POINTER(Csr), _vp, _d, _vp, _vp]),
    "sspmv_spmm_csr": (_st, [_d, C.POINTER(Csr), _i32, _vp, _i64, _d, _vp, _i64, _vp]),
    "sspmv_LeSpMV_csr_noalloc": (_st, [_d, C.POINTER(Csr), _vp, _d, _vp, _vp]),
    "sspmv_wait_timeouts": (_st, [C.POINTER(_i64)]),
    "sspmv_release_plan": (_st, [C.POINTER(Features), _vp]),
    "sspmv_algorithmic_bytes_csr": (_d, [C.POINTER(Csr), _i32, _i32]),
    "sspmv_reference_bytes_csr": (_d, [C.POINTER(Csr)]),
    "sspmv_read_mtx": (_st, [C.c_char_p, _i32, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_i64), _vp, _vp, _vp]),
    "sspmv_write_mtx": (_st, [C.c_char_p, _i64, _i64, _vp, _vp, _vp]),
    "sspmv_synth_row_offsets": (_i64, [C.POINTER(SynthParams), C.c_uint64, _vp]),
    "sspmv_synth_fill_f64": (C.c_int, [C.POINTER(SynthParams), C.c_uint64, _vp, _vp, _vp]),
    "sspmv_synth_fill_f32": (C.c_int, [C.POINTER(SynthParams), C.c_uint64, _vp, _vp, _vp]),
    "sspmv_synth_vector_f64": (None, [_i64, C.c_uint64, _vp]),
    "sspmv_synth_vector_f32": (None, [_i64, C.c_uint64, _vp]),
}


def register(name: str, restype, argtypes) -> None:
    fn = getattr(lib, name)
    fn.restype = restype
    fn.argtypes = argtypes


def _format_sigs(fmt: str, struct, convert_args, export_args):
    P = C.POINTER(struct)
    sigs = {
        f"sspmv_LeSpMV_{fmt}": (_st, [_d, P, _vp, _d, _vp, _vp]),
        f"sspmv_spmm_{fmt}": (_st, [_d, P, _i32, _vp, _i64, _d, _vp, _i64, _vp]),
        f"sspmv_delete_{fmt}": (_st, [P]),
        f"sspmv_algorithmic_bytes_{fmt}": (_d, [P, _i32, _i32]),
        f"sspmv_reference_bytes_{fmt}": (_d, [P]),
        f"sspmv_{fmt}_export": (_st, [P, *export_args, _vp]),
    }
    if convert_args is not None:
        sigs[f"sspmv_csr_to_{fmt}"] = (_st, [C.POINTER(Csr), *convert_args, P, _vp])
    return sigs


_SIGS.update(_format_sigs("ell", Ell, [_i32], [_vp, _vp]))
_SIGS.update(_format_sigs("sell", SEll, [_i32, _i32], [_vp, _vp, _vp]))
_SIGS.update(_format_sigs("sell_c_sigma", SellCSigma, [_i32, _i32, _i32], [_vp, _vp, _vp, _vp]))
_SIGS.update(_format_sigs("sell_c_R", SellCR, [_i32, _i32], [_vp, _vp, _vp, _vp]))
_SIGS.update(_format_sigs("coo", Coo, [], [_vp, _vp, _vp]))
_SIGS.update(_format_sigs("dia", Dia, [_i32, _i32], [_vp, _vp]))
_SIGS.update(_format_sigs("bsr", Bsr, [_i32, _i32], [_vp, _vp, _vp]))
_SIGS.update(_format_sigs("csr5", Csr5, [_i32, _i32], [_vp, _vp, _vp, _vp, _vp, _vp]))
_SIGS["sspmv_coo_create"] = (_st, [C.POINTER(Coo), _i32, _i64, _i64, _i64, _vp, _vp, _vp, _i32, _vp])
_SIGS["sspmv_coo_to_csr"] = (_st, [C.POINTER(Coo), C.POINTER(Csr), _vp])
_SIGS["sspmv_coo_to_ell"] = (_st, [C.POINTER(Coo), _i32, C.POINTER(Ell), _vp])
_SIGS["sspmv_sum_csr_duplicates"] = (_st, [_i32, _i64, _i64, _vp, _vp, _vp, C.POINTER(_i64)])
_SIGS["sspmv_read_mtx_coo"] = (_st, [C.c_char_p, _i32, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_i64), _vp, _vp,
                                     _vp])
_SIGS["sspmv_csr_count_blocks"] = (_st, [C.POINTER(Csr), _i32, _i32, C.POINTER(_i64), _vp])
_SIGS["sspmv_csr_features"] = (_st, [C.POINTER(Csr), _i32, _vp, _vp, _vp, _vp, _vp])
_SIGS["sspmv_feature_name"] = (C.c_char_p, [_i32])
_SIGS["sspmv_csr_grx_features"] = (_st, [C.POINTER(Csr), _i32, _i32, _vp, _vp])
NUM_FEATURES = 62


class ServerConfig(C.Structure):
    _fields_ = [("mode", C.c_int32), ("max_batch_requests", C.c_int32), ("max_batch_tiles", C.c_int64),
                ("arena_bytes", C.c_int64), ("stage_limit_bytes", C.c_int64), ("hbm_budget_bytes", C.c_int64),
                ("num_inflight", C.c_int32), ("use_graphs", C.c_int32)]


class Request(C.Structure):
    _fields_ = [("matrix_id", C.c_int32), ("k", C.c_int32), ("alpha", C.c_double), ("beta", C.c_double),
                ("x", C.c_void_p), ("ldx", C.c_int64), ("y", C.c_void_p), ("ldy", C.c_int64),
                ("flags", C.c_int32), ("reserved", C.c_int32)]


class RequestInfo(C.Structure):
    _fields_ = [("status", C.c_int32), ("batch_size", C.c_int32), ("batch_id", C.c_int64),
                ("arrival_ns", C.c_int64), ("launch_ns", C.c_int64), ("done_ns", C.c_int64)]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("requests_done", "requests_failed", "batches", "batched_requests",
                                         "batched_tiles", "graph_launches", "loads", "evictions",
                                         "resident_matrices", "resident_bytes")]


_f = C.c_float
_SIGS.update({
    "sspmv_nn_linear_forward": (_st, [_i32, _i32, _i32, _vp, _i32, _vp, _vp, _i32, _vp, _i32, _vp]),
    "sspmv_nn_linear_backward": (_st, [_i32, _i32, _i32, _vp, _i32, _vp, _vp, _i32, _vp, _i32, _vp, _i32, _vp, _vp,
                                       _vp]),
    "sspmv_nn_softmax_xent": (_st, [_i32, _i32, _vp, _i32, _vp, _vp, _i32, _vp, _vp]),
    "sspmv_nn_masked_mse": (_st, [_i32, _i32, _vp, _i32, _vp, _vp, _f, _f, _vp, _i32, _vp, _vp]),
    "sspmv_nn_adam": (_st, [_i64, _vp, _vp, _vp, _vp, _f, _f, _f, _f, _i32, _f, _vp]),
})
_SIGS.update({
    "sspmv_server_create": (_st, [C.POINTER(ServerConfig), C.POINTER(_vp)]),
    "sspmv_server_destroy": (_st, [_vp]),
    "sspmv_server_add_matrix": (_st, [_vp, _i32, _i32, _i64, _i64, _i64, _vp, _vp, _vp, _i32, _vp]),
    "sspmv_server_preload": (_st, [_vp, _i32]),
    "sspmv_server_submit": (_st, [_vp, C.POINTER(Request), C.POINTER(_i64)]),
    "sspmv_server_wait": (_st, [_vp, _i64, _d, C.POINTER(RequestInfo)]),
    "sspmv_server_replay": (_st, [_vp, _i64, _vp, _vp, _vp]),
    "sspmv_server_get_stats": (_st, [_vp, C.POINTER(ServerStats)]),
})

for _n, (_r, _a) in _SIGS.items():
    register(_n, _r, _a)


def check(status: int, where: str) -> None:
    if status != 0:
        detail = lib.sspmv_last_error().decode(errors="replace")
        raise SSPMVError(status, where, detail)


def call(name: str, *args) -> None:
    check(getattr(lib, name)(*args), name)
