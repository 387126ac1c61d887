"""Python front end of the CPU oracle.  TEST INFRASTRUCTURE ONLY.

Two back ends with one output shape:
  * `Oracle`    -- the C restatement (oracle/liboracle.so, built from oracle.c);
  * `Reference` -- the reference's own code (oracle/_ref/libref.so, built by
                   `make -C oracle ref` from the LeSpMV sources; present only
                   where those sources are).
Each converter returns a dict of numpy arrays and ints in the reference's
logical layout (sliced formats flattened chunk by chunk, row-major in a chunk).

Only tests/, the smoke check and the benchmark's CPU-baseline leg use this
module.  The product (sspmv_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_vp = C.c_void_p
_i32 = C.c_int32
_i64 = C.c_int64


def _ptr(a) -> C.c_void_p:
    return C.c_void_p(None if a is None else a.ctypes.data)


def _sfx(dtype) -> str:
    return "f64" if np.dtype(dtype) == np.float64 else "f32"


def default_alignment(dtype) -> int:
    return 64 // np.dtype(dtype).itemsize


class Geom(C.Structure):
    _fields_ = [("sigma", _i32), ("omega", _i32), ("bit_y_offset", _i32), ("bit_scansum_offset", _i32),
                ("num_packets", _i32), ("p", _i32), ("num_offsets", _i32), ("tail_partition_start", _i32)]


class Oracle:
    """C restatement of the reference algorithms (oracle.c)."""

    def __init__(self, path: Path | None = None):
        path = path or HERE / "liboracle.so"
        if not path.exists():
            raise ImportError(f"{path} is not built (make -C oracle)")
        self.lib = C.CDLL(str(path))
        L = self.lib
        L.oracle_ell_width.restype = _i32
        L.oracle_sell_row_width.restype = _i64
        L.oracle_sell_cs_reorder.restype = C.c_int
        L.oracle_sell_cs_chunk_len.restype = _i64
        L.oracle_dia_map.restype = _i32
        L.oracle_bsr_row_ptr.restype = _i32
        L.oracle_csr5_geometry.restype = C.c_int
        L.oracle_max_threads.restype = C.c_int
        for s, V in (("f64", C.c_double), ("f32", C.c_float)):
            getattr(L, f"oracle_max_rel_error_{s}").restype = V
            for fn, args in {
                "oracle_spmv_csr": [_i32, _vp, _vp, _vp, V, _vp, V, _vp, C.c_int],
                "oracle_spmv_coo": [_i32, _i32, _vp, _vp, _vp, V, _vp, V, _vp, C.c_int],
                "oracle_spmv_ell": [_i32, _i32, _i32, _vp, _vp, V, _vp, V, _vp, C.c_int],
                "oracle_spmv_sell": [_i32, _i32, _vp, _vp, _vp, V, _vp, V, _vp, C.c_int],
                "oracle_spmv_sell_cs": [_i32, _i32, _vp, _vp, _vp, _vp, V, _vp, V, _vp, C.c_int],
                "oracle_spmv_dia": [_i32, _i32, _i32, _i32, _vp, _vp, V, _vp, V, _vp, C.c_int],
                "oracle_spmv_bsr": [_i32, _i32, _i32, _i32, _vp, _vp, _vp, V, _vp, V, _vp, C.c_int],
                "oracle_spmm_ref": [_i32, _vp, _vp, _vp, _i32, _vp, _i64, C.c_double, C.c_double, _vp, _i64,
                                    _vp, _vp, C.c_int],
            }.items():
                getattr(L, f"{fn}_{s}").argtypes = args

    # ------------------------------------------------------------ converters
    def coo_to_csr(self, m, ri, ci, v):
        nnz = len(ri)
        rp = np.empty(m + 1, np.int32)
        col = np.empty(nnz, np.int32)
        val = np.empty(nnz, v.dtype)
        getattr(self.lib, f"oracle_coo_to_csr_{_sfx(v.dtype)}")(
            _i32(m), _i32(nnz), _ptr(ri), _ptr(ci), _ptr(v), _ptr(rp), _ptr(col), _ptr(val))
        return {"row_offset": rp, "col": col, "val": val}

    def csr_to_coo(self, csr):
        m, nnz = csr.num_rows, csr.nnz
        ri, ci = np.empty(nnz, np.int32), np.empty(nnz, np.int32)
        v = np.empty(nnz, csr.values.dtype)
        getattr(self.lib, f"oracle_csr_to_coo_{_sfx(v.dtype)}")(
            _i32(m), _ptr(csr.row_offset), _ptr(csr.col_index), _ptr(csr.values), _ptr(ri), _ptr(ci), _ptr(v))
        return {"row": ri, "col": ci, "val": v}

    def csr_to_ell(self, csr, ld=0):
        m = csr.num_rows
        w = self.lib.oracle_ell_width(_i32(m), _ptr(csr.row_offset))
        col = np.empty(m * w, np.int32)
        val = np.empty(m * w, csr.values.dtype)
        getattr(self.lib, f"oracle_csr_to_ell_{_sfx(val.dtype)}")(
            _i32(m), _ptr(csr.row_offset), _ptr(csr.col_index), _ptr(csr.values), _i32(w), _i32(ld),
            _ptr(col), _ptr(val))
        return {"max_row_width": w, "col": col, "val": val}

    def csr_to_sell(self, csr, C_=4, align=None):
        align = align or default_alignment(csr.values.dtype)
        m = csr.num_rows
        nch = (m + C_ - 1) // C_
        rw = np.empty(nch, np.int32)
        tot = self.lib.oracle_sell_row_width(_i32(m), _ptr(csr.row_offset), _i32(C_), _i32(align), _ptr(rw))
        col = np.empty(tot, np.int32)
        val = np.empty(tot, csr.values.dtype)
        getattr(self.lib, f"oracle_csr_to_sell_{_sfx(val.dtype)}")(
            _i32(m), _ptr(csr.row_offset), _ptr(csr.col_index), _ptr(csr.values), _i32(C_), _ptr(rw),
            _ptr(col), _ptr(val))
        return {"chunk_num": nch, "row_width": rw, "col": col, "val": val}

    def csr_to_sell_c_sigma(self, csr, sigma=16384, C_=4, align=None):
        """sigma <= 0 reorders all rows at once (SELL-c-R)."""
        align = align or default_alignment(csr.values.dtype)
        m = csr.num_rows
        reorder = np.empty(m, np.int32)
        if self.lib.oracle_sell_cs_reorder(_i32(m), _ptr(csr.row_offset), _i32(sigma), _i32(C_),
                                           _ptr(reorder)) != 0:
            raise ValueError("sigma must be a multiple of C")
        nch = (m + C_ - 1) // C_
        cl = np.empty(nch, np.int32)
        tot = self.lib.oracle_sell_cs_chunk_len(_i32(m), _ptr(csr.row_offset), _ptr(reorder), _i32(C_),
                                                _i32(align), _ptr(cl))
        col = np.empty(tot, np.int32)
        val = np.empty(tot, csr.values.dtype)
        getattr(self.lib, f"oracle_csr_to_sell_cs_{_sfx(val.dtype)}")(
            _i32(m), _ptr(csr.row_offset), _ptr(csr.col_index), _ptr(csr.values), _ptr(reorder), _i32(C_),
            _ptr(cl), _ptr(col), _ptr(val))
        return {"reorder": reorder, "chunk_len": cl, "col": col, "val": val, "validchunkNum": nch}

    def csr_to_sell_c_R(self, csr, C_=4, align=None):
        return self.csr_to_sell_c_sigma(csr, 0, C_, align)

    def csr_to_dia(self, csr, max_diags=10240, align=None):
        align = align or default_alignment(csr.values.dtype)
        m, n = csr.num_rows, csr.num_cols
        dmap = np.empty(m + n, np.int32)
        nd = self.lib.oracle_dia_map(_i32(m), _i32(n), _ptr(csr.row_offset), _ptr(csr.col_index), _ptr(dmap))
        if nd > max_diags:
            return None
        stride = align * ((m + align - 1) // align)
        offs = np.empty(nd, np.int64)
        data = np.empty(nd * stride, csr.values.dtype)
        getattr(self.lib, f"oracle_csr_to_dia_{_sfx(data.dtype)}")(
            _i32(m), _i32(n), _ptr(csr.row_offset), _ptr(csr.col_index), _ptr(csr.values), _ptr(dmap),
            _i32(nd), _i32(stride), _ptr(offs), _ptr(data))
        return {"complete_ndiags": nd, "stride": stride, "offsets": offs, "data": data}

    def csr_to_bsr(self, csr, r=16, c=None):
        c = c or default_alignment(csr.values.dtype)
        m, n = csr.num_rows, csr.num_cols
        mb, nb = (m + r - 1) // r, (n + c - 1) // c
        rp = np.empty(mb + 1 if not (r == 1 and c == 1) else m + 1, np.int32)
        nnzb = self.lib.oracle_bsr_row_ptr(_i32(m), _i32(n), _ptr(csr.row_offset), _ptr(csr.col_index),
                                           _i32(r), _i32(c), _ptr(rp))
        ci = np.empty(nnzb, np.int32)
        self.lib.oracle_bsr_colindex(_i32(m), _i32(n), _ptr(csr.row_offset), _ptr(csr.col_index), _i32(r),
                                     _i32(c), _ptr(rp), _ptr(ci))
        data = np.empty(nnzb * r * c, csr.values.dtype)
        getattr(self.lib, f"oracle_csr_to_bsr_{_sfx(data.dtype)}")(
            _i32(m), _i32(n), _ptr(csr.row_offset), _ptr(csr.col_index), _ptr(csr.values), _i32(r), _i32(c),
            _ptr(rp), _ptr(ci), _ptr(data))
        return {"mb": mb, "nb": nb, "nnzb": nnzb, "row_ptr": rp[:mb + 1], "colindex": ci, "data": data,
                "r": r, "c": c}

    def csr_to_csr5(self, csr, sigma=16, omega=None):
        omega = omega or default_alignment(csr.values.dtype)
        m, nnz = csr.num_rows, csr.nnz
        g = Geom()
        if self.lib.oracle_csr5_geometry(_i32(nnz), _i32(sigma), _i32(omega), C.byref(g)) != 0:
            raise ValueError("CSR5 bit fields do not fit")
        tp = np.empty(g.p + 1, np.uint32)
        td = np.empty(g.p * omega * g.num_packets, np.uint32)
        tdo_ptr = np.empty(g.p + 1, np.int32)
        self.lib.oracle_csr5_descriptors(_i32(m), _ptr(csr.row_offset), C.byref(g), _ptr(tp), _ptr(td),
                                         _ptr(tdo_ptr))
        tdo = np.zeros(g.num_offsets, np.int32)
        self.lib.oracle_csr5_offsets(_i32(m), _ptr(csr.row_offset), C.byref(g), _ptr(tp), _ptr(td),
                                     _ptr(tdo_ptr), _ptr(tdo))
        col = csr.col_index.copy()
        val = csr.values.copy()
        self.lib.oracle_csr5_transpose(_i32(nnz), C.byref(g), _ptr(tp), _ptr(col), _i32(4))
        self.lib.oracle_csr5_transpose(_i32(nnz), C.byref(g), _ptr(tp), _ptr(val), _i32(val.itemsize))
        return {"sigma": g.sigma, "omega": g.omega, "bit_y_offset": g.bit_y_offset,
                "bit_scansum_offset": g.bit_scansum_offset, "num_packets": g.num_packets, "p": g.p,
                "num_offsets": g.num_offsets, "tail_partition_start": g.tail_partition_start,
                "tile_ptr": tp, "tile_desc": td, "tile_desc_offset_ptr": tdo_ptr, "tile_desc_offset": tdo,
                "col": col, "val": val}

    # ------------------------------------------------------------------ spmv
    def spmv(self, fmt: str, A: dict, csr, alpha, x, beta, y, nthreads=0):
        """y <- alpha*A*x + beta*y with the restated CPU kernel of `fmt`."""
        s = _sfx(y.dtype)
        V = C.c_double if s == "f64" else C.c_float
        L = self.lib
        m, n = csr.num_rows, csr.num_cols
        a, b = V(alpha), V(beta)
        if fmt == "csr":
            getattr(L, f"oracle_spmv_csr_{s}")(m, _ptr(csr.row_offset), _ptr(csr.col_index), _ptr(csr.values),
                                              a, _ptr(x), b, _ptr(y), nthreads)
        elif fmt == "coo":
            getattr(L, f"oracle_spmv_coo_{s}")(m, len(A["row"]), _ptr(A["row"]), _ptr(A["col"]), _ptr(A["val"]),
                                              a, _ptr(x), b, _ptr(y), nthreads)
        elif fmt == "ell":
            getattr(L, f"oracle_spmv_ell_{s}")(m, A["max_row_width"], A.get("ld", 0), _ptr(A["col"]),
                                              _ptr(A["val"]), a, _ptr(x), b, _ptr(y), nthreads)
        elif fmt == "sell":
            getattr(L, f"oracle_spmv_sell_{s}")(m, A["C"], _ptr(A["row_width"]), _ptr(A["col"]), _ptr(A["val"]),
                                               a, _ptr(x), b, _ptr(y), nthreads)
        elif fmt in ("sell_c_sigma", "sell_c_R"):
            getattr(L, f"oracle_spmv_sell_cs_{s}")(m, A["C"], _ptr(A["reorder"]), _ptr(A["chunk_len"]),
                                                  _ptr(A["col"]), _ptr(A["val"]), a, _ptr(x), b, _ptr(y),
                                                  nthreads)
        elif fmt == "dia":
            getattr(L, f"oracle_spmv_dia_{s}")(m, n, A["complete_ndiags"], A["stride"], _ptr(A["offsets"]),
                                              _ptr(A["data"]), a, _ptr(x), b, _ptr(y), nthreads)
        elif fmt == "bsr":
            getattr(L, f"oracle_spmv_bsr_{s}")(m, A["r"], A["c"], A["mb"], _ptr(A["row_ptr"]),
                                              _ptr(A["colindex"]), _ptr(A["data"]), a, _ptr(x), b, _ptr(y),
                                              nthreads)
        else:
            raise ValueError(fmt)
        return y

    def spmm_ref(self, csr, X, alpha, beta, Y0=None, nthreads=0):
        """FP64 CSR result on the given (possibly FP32) inputs and per-row
        sum_j |a_ij x_j|.  X: (n,) or (n,k) row-major."""
        X2 = X.reshape(csr.num_cols, -1)
        k = X2.shape[1]
        m = csr.num_rows
        y = np.empty((m, k), np.float64)
        ab = np.empty((m, k), np.float64)
        Y0c = None if Y0 is None else np.ascontiguousarray(Y0.reshape(m, -1))
        getattr(self.lib, f"oracle_spmm_ref_{_sfx(csr.values.dtype)}")(
            m, _ptr(csr.row_offset), _ptr(csr.col_index), _ptr(csr.values), k, _ptr(np.ascontiguousarray(X2)), k,
            float(alpha), float(beta), _ptr(Y0c), k, _ptr(y), _ptr(ab), nthreads)
        return (y.reshape(m), ab.reshape(m)) if X.ndim == 1 else (y, ab)

    def features(self, csr, T=256):
        """MTX features (62, library order) and per-tile counts of a CSR."""
        L = self.lib
        L.oracle_features.argtypes = [_i32, _i32, _vp, _vp, _vp, _i32, _vp, _vp, _vp, _vp]
        F = np.zeros(62)
        t, u, v = (np.zeros(T * T, np.int32) for _ in range(3))
        val = np.ascontiguousarray(csr.values, np.float64)
        L.oracle_features(csr.num_rows, csr.num_cols, _ptr(csr.row_offset), _ptr(csr.col_index), _ptr(val), T,
                          _ptr(F), _ptr(t), _ptr(u), _ptr(v))
        return F, {"tiles": t, "urb": u, "ucb": v}

    def grx(self, csr, T=256, X=8):
        """GrX_uniqR, GrX_uniqC, GrX_potReuseR, GrX_potReuseC of a CSR."""
        L = self.lib
        L.oracle_grx.argtypes = [_i32, _i32, _vp, _vp, _vp, _i32, _i32, _vp]
        out = np.zeros(4)
        val = np.ascontiguousarray(csr.values, np.float64)
        L.oracle_grx(csr.num_rows, csr.num_cols, _ptr(csr.row_offset), _ptr(csr.col_index), _ptr(val), T, X, _ptr(out))
        return out

    def max_rel_error(self, a, b):
        return float(getattr(self.lib, f"oracle_max_rel_error_{_sfx(a.dtype)}")(
            _ptr(a), _ptr(b), _i64(a.size)))


def csr5_unwritten_slots(tile_ptr, tile_desc_offset_ptr, p):
    """Slots of tile_desc_offset that the reference never writes: one per
    tile with empty rows, the last of its range (lane 0's leading segment is
    counted in the range size but not recorded, include/sparse_conversion.h:
    1203-1206 vs :1282-1290).  The reference leaves them uninitialised; the
    oracle and the GPU converter write 0 there."""
    slots = [int(tile_desc_offset_ptr[t + 1]) - 1 for t in range(p - 1)
             if (int(tile_ptr[t]) >> 31) & 1 and tile_desc_offset_ptr[t + 1] > tile_desc_offset_ptr[t]]
    return np.asarray(slots, dtype=np.int64)


class RefOut(C.Structure):
    _fields_ = [("ints", _i64 * 16), ("arrays", _vp * 8), ("lens", _i64 * 8)]


class Reference:
    """The reference's own converters and kernels (oracle/_ref/libref.so)."""

    def __init__(self, path: Path | None = None, threads: int = 1):
        path = path or HERE / "_ref" / "libref.so"
        if not path.exists():
            raise ImportError(f"{path} is not built (make -C oracle ref)")
        self.lib = C.CDLL(str(path))
        self.lib.ref_set_threads(threads)

    def _take(self, o: RefOut, specs):
        out = {}
        for i, (name, dt) in enumerate(specs):
            n = o.lens[i]
            p = o.arrays[i]
            if p:
                arr = np.ctypeslib.as_array(C.cast(p, C.POINTER(np.ctypeslib.as_ctypes_type(dt))), shape=(max(n, 1),))
                out[name] = arr[:n].copy()
                self.lib.ref_free(C.c_void_p(p))
            else:
                out[name] = np.empty(0, dt)
        return out

    def _csr_args(self, csr):
        return (_i32(csr.num_rows), _i32(csr.num_cols), _ptr(csr.row_offset), _ptr(csr.col_index),
                _ptr(csr.values))

    def coo_to_csr(self, m, n, ri, ci, v):
        o = RefOut()
        getattr(self.lib, f"ref_coo_to_csr_{_sfx(v.dtype)}")(_i32(m), _i32(n), _i32(len(ri)), _ptr(ri), _ptr(ci),
                                                           _ptr(v), C.byref(o))
        return self._take(o, [("row_offset", np.int32), ("col", np.int32), ("val", v.dtype)])

    def csr_to_ell(self, csr, ld=0):
        o = RefOut()
        getattr(self.lib, f"ref_csr_to_ell_{_sfx(csr.values.dtype)}")(*self._csr_args(csr), _i32(ld), C.byref(o))
        d = self._take(o, [("col", np.int32), ("val", csr.values.dtype)])
        d["max_row_width"] = int(o.ints[0])
        return d

    def csr_to_sell(self, csr, C_=4, align=None):
        align = align or default_alignment(csr.values.dtype)
        o = RefOut()
        getattr(self.lib, f"ref_csr_to_sell_{_sfx(csr.values.dtype)}")(*self._csr_args(csr), _i32(C_), _i32(align),
                                                                       C.byref(o))
        d = self._take(o, [("row_width", np.int32), ("col", np.int32), ("val", csr.values.dtype)])
        d["chunk_num"] = int(o.ints[0])
        return d

    def csr_to_sell_c_sigma(self, csr, sigma=16384, C_=4, align=None):
        align = align or default_alignment(csr.values.dtype)
        o = RefOut()
        getattr(self.lib, f"ref_csr_to_sell_c_sigma_{_sfx(csr.values.dtype)}")(
            *self._csr_args(csr), _i32(sigma), _i32(C_), _i32(align), C.byref(o))
        d = self._take(o, [("reorder", np.int32), ("chunk_len", np.int32), ("col", np.int32),
                           ("val", csr.values.dtype)])
        d.update(sliceNum=int(o.ints[0]), chunkNum=int(o.ints[1]), validchunkNum=int(o.ints[2]),
                 chunk_num_per_slice=int(o.ints[3]))
        return d

    def csr_to_sell_c_R(self, csr, C_=4, align=None):
        align = align or default_alignment(csr.values.dtype)
        o = RefOut()
        getattr(self.lib, f"ref_csr_to_sell_c_R_{_sfx(csr.values.dtype)}")(*self._csr_args(csr), _i32(C_),
                                                                          _i32(align), C.byref(o))
        d = self._take(o, [("reorder", np.int32), ("chunk_len", np.int32), ("col", np.int32),
                           ("val", csr.values.dtype)])
        d["validchunkNum"] = int(o.ints[2])
        return d

    def csr_to_dia(self, csr, max_diags=10240, align=None):
        align = align or default_alignment(csr.values.dtype)
        o = RefOut()
        getattr(self.lib, f"ref_csr_to_dia_{_sfx(csr.values.dtype)}")(*self._csr_args(csr), _i32(max_diags),
                                                                      _i32(align), C.byref(o))
        d = self._take(o, [("offsets", np.int64), ("data", csr.values.dtype)])
        d.update(complete_ndiags=int(o.ints[0]), stride=int(o.ints[1]))
        return d

    def csr_to_bsr(self, csr, r=16, c=None):
        c = c or default_alignment(csr.values.dtype)
        o = RefOut()
        getattr(self.lib, f"ref_csr_to_bsr_{_sfx(csr.values.dtype)}")(*self._csr_args(csr), _i32(r), _i32(c),
                                                                      C.byref(o))
        d = self._take(o, [("row_ptr", np.int32), ("colindex", np.int32), ("data", csr.values.dtype)])
        d.update(mb=int(o.ints[0]), nb=int(o.ints[1]), nnzb=int(o.ints[2]), r=r, c=c)
        return d

    def csr_to_csr5(self, csr):
        o = RefOut()
        getattr(self.lib, f"ref_csr_to_csr5_{_sfx(csr.values.dtype)}")(*self._csr_args(csr), C.byref(o))
        d = self._take(o, [("tile_ptr", np.uint32), ("tile_desc", np.uint32), ("tile_desc_offset_ptr", np.int32),
                           ("tile_desc_offset", np.int32), ("col", np.int32), ("val", csr.values.dtype)])
        keys = ["sigma", "omega", "bit_y_offset", "bit_scansum_offset", "num_packets", "p", "num_offsets",
                "tail_partition_start"]
        d.update({k: int(o.ints[i]) for i, k in enumerate(keys)})
        d["tile_desc_offset"][csr5_unwritten_slots(d["tile_ptr"], d["tile_desc_offset_ptr"], d["p"])] = 0
        return d

    def spmv(self, fmt, flag, csr, alpha, x, beta, y, p0=0, p1=0, p2=0):
        s = _sfx(y.dtype)
        V = C.c_double if s == "f64" else C.c_float
        fn = getattr(self.lib, f"ref_spmv_{s}")
        fn.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, V, _vp,
                       V, _vp]
        rc = fn(fmt.encode(), flag, p0, p1, p2, csr.num_rows, csr.num_cols, _ptr(csr.row_offset),
                _ptr(csr.col_index), _ptr(csr.values), alpha, _ptr(x), beta, _ptr(y))
        if rc != 0:
            raise ValueError(fmt)
        return y

    def read_csr(self, path: str, dtype=np.float64):
        o = RefOut()
        getattr(self.lib, f"ref_read_csr_{_sfx(dtype)}")(str(path).encode(), C.byref(o))
        d = self._take(o, [("row_offset", np.int32), ("col", np.int32), ("val", dtype)])
        d.update(num_rows=int(o.ints[0]), num_cols=int(o.ints[1]), num_nnzs=int(o.ints[2]))
        return d


def tolerance_ok(y, y_ref64, absum, nnz_per_row, dtype, alpha=1.0, beta=0.0, y0=None, factor=8.0):
    """Per-row bound |y_i - y_ref_i| <= factor*nnz_i*eps*|alpha|*sum_j|a_ij x_j|
    (+ 2*eps*|beta*y0_i| for the beta term).  Returns (ok, max_norm, median_norm)
    where norm = |err| / bound (rows with bound 0 must match exactly)."""
    eps = np.finfo(dtype).eps
    y = np.asarray(y, np.float64)
    err = np.abs(y - y_ref64)
    nz = np.asarray(nnz_per_row, np.float64)
    if y.ndim == 2:
        nz = nz[:, None]
    bound = factor * np.maximum(nz, 1.0) * eps * abs(alpha) * absum
    if beta != 0 and y0 is not None:
        bound = bound + 2.0 * eps * np.abs(beta * np.asarray(y0, np.float64))
    bound = bound + np.finfo(np.float64).tiny
    norm = err / bound
    return bool(np.all(norm <= 1.0)), float(norm.max(initial=0.0)), float(np.median(norm) if norm.size else 0.0)
