"""Seeded synthetic matrices (host side).

The generator is sspmv_gb300/csrc/synth.cpp.  It is exported by libsspmv.so
(the C ABI's sspmv_synth_*) and also built on its own, host-only, as
lib/libsspmv_synth.so, which is what this module loads: the CPU legs of the
benchmark generate their inputs without loading the GPU library.

The suite's workloads, by name and size:
  laplacian_1024   2-D 5-point Laplacian on a 1024 x 1024 grid (N=1,048,576)
  banded_2M        N=2^21, 9 diagonals at 0, +-1, +-2, +-1024, +-2048
  powerlaw_4M      N=2^22, Zipf(1.8) row lengths scaled to mean 16, cap 50k
  block4_2M        N=2^21, 500k distinct dense 4x4 blocks
  uniform_4M       N=2^22, 32 distinct uniform columns per row
  powerlaw_16M     N=2^24, Zipf(2.0) row lengths scaled to mean 16, cap 50k
Values are U[-1,1) (the Laplacian uses 4 / -1); x is U[-1,1) from seed 0.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "lib" / "libsspmv_synth.so"

LAPLACIAN2D, BANDED, POWERLAW, BLOCK, UNIFORM = range(5)


class SynthParams(C.Structure):
    """sspmv_synth_params (include/sspmv.h)."""
    _fields_ = [("family", C.c_int32), ("num_offsets", C.c_int32), ("num_rows", C.c_int64),
                ("num_cols", C.c_int64), ("grid", C.c_int64), ("offsets", C.c_int64 * 32),
                ("alpha", C.c_double), ("mean", C.c_double), ("cap", C.c_int64),
                ("block_dim", C.c_int64), ("num_blocks", C.c_int64), ("per_row", C.c_int64),
                ("empty_row_frac", C.c_double)]


def _load():
    if not _LIB_PATH.exists():
        raise ImportError(f"libsspmv_synth.so is not built ({_LIB_PATH}); run __graft_entry__.build() "
                          "or python -m sspmv_gb300.build")
    h = C.CDLL(str(_LIB_PATH))
    vp = C.c_void_p
    for name, res, args in (("sspmv_synth_row_offsets", C.c_int64, [C.POINTER(SynthParams), C.c_uint64, vp]),
                            ("sspmv_synth_fill_f64", C.c_int, [C.POINTER(SynthParams), C.c_uint64, vp, vp, vp]),
                            ("sspmv_synth_fill_f32", C.c_int, [C.POINTER(SynthParams), C.c_uint64, vp, vp, vp]),
                            ("sspmv_synth_vector_f64", None, [C.c_int64, C.c_uint64, vp]),
                            ("sspmv_synth_vector_f32", None, [C.c_int64, C.c_uint64, vp])):
        f = getattr(h, name)
        f.restype, f.argtypes = res, args
    return h


lib = _load()


def laplacian2d(grid: int) -> SynthParams:
    p = SynthParams()
    p.family, p.grid = LAPLACIAN2D, grid
    return p


def banded(n: int, offsets=(0, 1, -1, 2, -2, 1024, -1024, 2048, -2048), num_cols: int = 0) -> SynthParams:
    p = SynthParams()
    p.family, p.num_rows, p.num_cols = BANDED, n, num_cols
    p.num_offsets = len(offsets)
    for i, o in enumerate(offsets):
        p.offsets[i] = o
    return p


def powerlaw(n: int, alpha: float = 1.8, mean: float = 16.0, cap: int = 50000, empty_frac: float = 0.0,
             num_cols: int = 0) -> SynthParams:
    p = SynthParams()
    p.family, p.num_rows, p.num_cols = POWERLAW, n, num_cols
    p.alpha, p.mean, p.cap, p.empty_row_frac = alpha, mean, cap, empty_frac
    return p


def block(n: int, b: int = 4, num_blocks: int = 500_000, num_cols: int = 0) -> SynthParams:
    p = SynthParams()
    p.family, p.num_rows, p.num_cols = BLOCK, n, num_cols
    p.block_dim, p.num_blocks = b, num_blocks
    return p


def uniform(n: int, per_row: int = 32, empty_frac: float = 0.0, num_cols: int = 0) -> SynthParams:
    p = SynthParams()
    p.family, p.num_rows, p.num_cols = UNIFORM, n, num_cols
    p.per_row, p.empty_row_frac = per_row, empty_frac
    return p


WORKLOADS = {
    "laplacian_1024": lambda: laplacian2d(1024),
    "banded_2M": lambda: banded(1 << 21),
    "powerlaw_4M": lambda: powerlaw(1 << 22, 1.8, 16.0, 50000),
    "block4_2M": lambda: block(1 << 21, 4, 500_000),
    "uniform_4M": lambda: uniform(1 << 22, 32),
    "powerlaw_16M": lambda: powerlaw(1 << 24, 2.0, 16.0, 50000),
}


@dataclass
class HostCSR:
    num_rows: int
    num_cols: int
    row_offset: np.ndarray
    col_index: np.ndarray
    values: np.ndarray

    @property
    def nnz(self) -> int:
        return int(self.row_offset[-1]) if self.num_rows else 0

    def astype(self, dtype) -> "HostCSR":
        return HostCSR(self.num_rows, self.num_cols, self.row_offset, self.col_index,
                       self.values.astype(dtype))


def _shape(p: SynthParams) -> tuple[int, int]:
    m = p.grid * p.grid if p.family == LAPLACIAN2D else p.num_rows
    n = p.num_cols if p.num_cols > 0 else m
    return int(m), int(n)


def generate(p: SynthParams, seed: int = 1, dtype=np.float64) -> HostCSR:
    m, n = _shape(p)
    rp = np.empty(m + 1, dtype=np.int32)
    nnz = lib.sspmv_synth_row_offsets(C.byref(p), seed, rp.ctypes.data)
    if nnz < 0:
        raise ValueError("synthetic matrix does not fit int32 indices")
    col = np.empty(max(nnz, 1), dtype=np.int32)[:nnz]
    val = np.empty(max(nnz, 1), dtype=dtype)[:nnz]
    fill = lib.sspmv_synth_fill_f64 if np.dtype(dtype) == np.float64 else lib.sspmv_synth_fill_f32
    fill(C.byref(p), seed, rp.ctypes.data, col.ctypes.data, val.ctypes.data)
    return HostCSR(m, n, rp, col, val)


def vector(n: int, seed: int = 0, dtype=np.float64, k: int = 1) -> np.ndarray:
    """x_i ~ U[-1,1); for k > 1 a row-major n x k block (column r from seed+r)."""
    out = np.empty((n, k), dtype=dtype)
    f = lib.sspmv_synth_vector_f64 if np.dtype(dtype) == np.float64 else lib.sspmv_synth_vector_f32
    col = np.empty(n, dtype=dtype)
    for r in range(k):
        f(n, seed + r, col.ctypes.data)
        out[:, r] = col
    return out.reshape(n) if k == 1 else out


def load(name: str, seed: int = 1, dtype=np.float64) -> HostCSR:
    return generate(WORKLOADS[name](), seed, dtype)


__all__ = ["laplacian2d", "banded", "powerlaw", "block", "uniform", "generate", "vector", "load",
           "WORKLOADS", "HostCSR", "SynthParams"]
