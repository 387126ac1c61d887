"""Format names and host-side feasibility rules (numpy only; loads no
native library, so the CPU baseline can use it without the GPU library).

The reference exits where a format cannot hold a matrix (DIA beyond
MAX_DIAG_NUM = 10240 diagonals, include/sparse_conversion.h:651-656; ELL and
BSR have no limit there but pad without bound).  Here a format is built only
when its padding or block fill stays within 4x the CSR size.
"""
from __future__ import annotations

import numpy as np

# Formats the library builds, in benchmark order.
FORMATS = ["csr", "coo", "ell", "sell", "sell_c_sigma", "sell_c_R", "dia", "bsr", "csr5"]

MAX_DIAGS = 10240
MAX_FILL = 4.0


def bsr_block_for(A) -> tuple[int, int]:
    """Block shape used for a host matrix when none is given: 4x4."""
    return 4, 4


def feasible_host(fmt: str, A) -> tuple[bool, str]:
    """Whether `fmt` is worth building for the host CSR `A` (padding within
    4x the CSR size, DIA within the reference's 10240-diagonal limit)."""
    if fmt in ("csr", "coo", "csr5", "sell", "sell_c_sigma", "sell_c_R"):
        return True, ""
    m, nnz = A.num_rows, max(A.nnz, 1)
    lens = np.diff(A.row_offset)
    if fmt == "ell":
        w = int(lens.max()) if m else 0
        return (m * w <= MAX_FILL * nnz, f"ELL width {w} pads {m * w / nnz:.1f}x")
    if fmt == "dia":
        rows = np.repeat(np.arange(m, dtype=np.int64), lens)
        nd = int(np.count_nonzero(np.bincount(A.col_index.astype(np.int64) - rows + m, minlength=1)))
        return (nd <= MAX_DIAGS, f"{nd} diagonals > {MAX_DIAGS}")
    if fmt == "bsr":
        r, c = bsr_block_for(A)
        rows = np.repeat(np.arange(m, dtype=np.int64), lens) // r
        keys = np.sort(rows * ((A.num_cols + c - 1) // c) + A.col_index // c, kind="stable")  # radix sort
        nnzb = int(keys.size > 0) + int(np.count_nonzero(keys[1:] != keys[:-1]))
        return (nnzb * r * c <= MAX_FILL * nnz, f"BSR {r}x{c} fill {nnzb * r * c / nnz:.1f}x")
    return False, "unknown format"
