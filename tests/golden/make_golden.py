"""Writes the golden fixtures in tests/golden/*.npz from the REFERENCE's own
code (LeSpMV converters and LeSpMV_<fmt> kernels, compiled from its sources by
`make -C oracle ref` into oracle/_ref/libref.so).

Run in a checkout that has the reference sources:
    make -C oracle ref && python tests/golden/make_golden.py

Each fixture holds one small seeded matrix (inputs stored verbatim, so the
fixture does not depend on the generator's libm), x and y0, and for every
converter variant the SHA-256 of each output array (logical layout: sliced
formats flattened chunk by chunk, row-major inside a chunk) plus the scalar
fields, and the reference SpMV results y = 0.8*A*x + 0.7*y0 per format and
kernel_flag.  The reference runs single-threaded (its CSR->BSR converter has
a data race on a shared counter under OpenMP).
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

from oracle import Reference  # noqa: E402
from sspmv_gb300 import synth  # noqa: E402

OUT = Path(__file__).resolve().parent
ALPHA, BETA = 0.8, 0.7


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def long_row_matrix(dtype):
    """Short uniform rows plus one row of 5000 nonzeros and a run of empty rows."""
    base = synth.generate(synth.uniform(1200, 6, 0.0, num_cols=6000), 11, np.float64)
    rows = [base.col_index[base.row_offset[i]:base.row_offset[i + 1]] for i in range(base.num_rows)]
    vals = [base.values[base.row_offset[i]:base.row_offset[i + 1]] for i in range(base.num_rows)]
    rng = np.random.default_rng(3)
    rows[517] = np.sort(rng.choice(6000, 5000, replace=False)).astype(np.int32)
    vals[517] = rng.uniform(-1, 1, 5000)
    for i in range(800, 860):
        rows[i] = np.zeros(0, np.int32)
        vals[i] = np.zeros(0)
    rp = np.zeros(base.num_rows + 1, np.int32)
    rp[1:] = np.cumsum([len(r) for r in rows])
    return synth.HostCSR(base.num_rows, 6000, rp, np.concatenate(rows).astype(np.int32),
                         np.concatenate(vals).astype(dtype))


def duplicate_matrix(dtype, ref: Reference):
    """COO triplets with duplicates and unsorted columns, through coo_to_csr."""
    rng = np.random.default_rng(5)
    m = n = 400
    nnz = 3000
    ri = rng.integers(0, m, nnz).astype(np.int32)
    ci = rng.integers(0, n, nnz).astype(np.int32)
    ri[100:200] = ri[0:100]
    ci[100:200] = ci[0:100]  # exact duplicates
    v = rng.uniform(-1, 1, nnz).astype(dtype)
    out = ref.coo_to_csr(m, n, ri, ci, v)
    csr = synth.HostCSR(m, n, out["row_offset"], out["col"], out["val"])
    return csr, {"coo_row": ri, "coo_col": ci, "coo_val": v}, out


CASES = {
    "lap16": lambda dt: synth.generate(synth.laplacian2d(16), 1, dt),
    "band5000": lambda dt: synth.generate(synth.banded(5000), 1, dt),
    "pl1500": lambda dt: synth.generate(synth.powerlaw(1500, 1.8, 16.0, 600, 0.05), 1, dt),
    "blk1000": lambda dt: synth.generate(synth.block(1000, 4, 200), 1, dt),
    "uni1000": lambda dt: synth.generate(synth.uniform(1000, 16, 0.03), 1, dt),
    "nsq300x500": lambda dt: synth.generate(synth.uniform(300, 20, 0.1, num_cols=500), 1, dt),
    "tiny1x1": lambda dt: synth.HostCSR(1, 1, np.array([0, 1], np.int32), np.array([0], np.int32),
                                        np.array([2.5], dt)),
    "empty10": lambda dt: synth.HostCSR(10, 10, np.zeros(11, np.int32), np.zeros(0, np.int32), np.zeros(0, dt)),
    "longrow": long_row_matrix,
}

CONVERTERS = [
    ("ell_row", "csr_to_ell", dict(ld=0)),
    ("ell_col", "csr_to_ell", dict(ld=1)),
    ("sell", "csr_to_sell", dict()),
    ("sell_c8_a4", "csr_to_sell", dict(C_=8, align=4)),
    ("scs", "csr_to_sell_c_sigma", dict()),
    ("scs_s64_c8", "csr_to_sell_c_sigma", dict(sigma=64, C_=8)),
    ("scs_s256_c32_a1", "csr_to_sell_c_sigma", dict(sigma=256, C_=32, align=1)),
    ("scr", "csr_to_sell_c_R", dict()),
    ("scr_c8", "csr_to_sell_c_R", dict(C_=8)),
    ("dia", "csr_to_dia", dict()),
    ("bsr", "csr_to_bsr", dict()),
    ("bsr_4x4", "csr_to_bsr", dict(r=4, c=4)),
    ("bsr_3x5", "csr_to_bsr", dict(r=3, c=5)),
    ("bsr_1x1", "csr_to_bsr", dict(r=1, c=1)),
    ("csr5", "csr_to_csr5", dict()),
]

# (format, kernel_flag) pairs run through the reference's LeSpMV_<fmt>.
SPMV = [("csr", 1), ("csr", 2), ("coo", 1), ("ell", 1), ("ell", 2), ("sell", 1), ("sell", 2),
        ("sell_c_sigma", 1), ("sell_c_sigma", 2), ("sell_c_R", 1), ("sell_c_R", 2), ("dia", 0), ("dia", 1),
        ("bsr", 1), ("bsr", 2)]


def main() -> None:
    ref = Reference(threads=1)
    index = {}
    for dt in (np.float64, np.float32):
        tag = "f64" if dt == np.float64 else "f32"
        cases = dict(CASES)
        cases["dups"] = None
        for name, make in cases.items():
            extra = {}
            if name == "dups":
                A, coo, coo_out = duplicate_matrix(dt, ref)
                extra.update({f"in_{k}": v for k, v in coo.items()})
            else:
                A = make(dt)
            rec: dict = {"num_rows": A.num_rows, "num_cols": A.num_cols, "nnz": A.nnz, "conv": {}, "spmv": []}
            arrays = {"row_offset": A.row_offset, "col_index": A.col_index, "values": A.values, **extra}
            x = synth.vector(A.num_cols, 0, dt)
            y0 = synth.vector(A.num_rows, 5, dt)
            arrays["x"], arrays["y0"] = x, y0
            for key, fn, kw in CONVERTERS:
                if fn == "csr_to_csr5" and A.nnz == 0:
                    continue  # the reference indexes tile_ptr[-1] when nnz == 0
                out = getattr(ref, fn)(A, **kw)
                rec["conv"][key] = {
                    "fn": fn, "kw": kw,
                    "digests": {k: digest(v) for k, v in out.items() if isinstance(v, np.ndarray)},
                    "shapes": {k: list(v.shape) for k, v in out.items() if isinstance(v, np.ndarray)},
                    "scalars": {k: int(v) for k, v in out.items() if not isinstance(v, np.ndarray)},
                }
            # The reference's BSR kernel reads x up to the end of the last block
            # column (src/spmv_bsr.cpp:148), past num_cols when it is not a
            # multiple of the block width: give it zero padding to read.
            x_pad = np.zeros(A.num_cols + 64, dt)
            x_pad[:A.num_cols] = x
            for fmt, flag in SPMV:
                if fmt == "dia" and ref_dia_too_wide(ref, A):
                    continue
                y = y0.copy()
                ref.spmv(fmt, flag, A, ALPHA, x_pad, BETA, y)
                arrays[f"y_{fmt}_{flag}"] = y
                rec["spmv"].append([fmt, flag])
            if name == "dups":
                rec["coo_to_csr"] = {k: digest(v) for k, v in coo_out.items()}
            if A.nnz > 0:
                F, arrs = ref_features(ref, A)
                arrays["features"] = F
                rec["feature_arrays"] = {k: digest(v) for k, v in arrs.items()}
            fname = f"{name}_{tag}.npz"
            np.savez_compressed(OUT / fname, **arrays, meta=np.frombuffer(json.dumps(rec).encode(), np.uint8))
            index[fname] = {"num_rows": A.num_rows, "nnz": A.nnz}
            print(fname, A.num_rows, A.nnz)
    (OUT / "INDEX.json").write_text(json.dumps(index, indent=1, sort_keys=True) + "\n")


def ref_features(ref: Reference, A):
    """The reference's MTX features (double build, T = 256) of A written as a
    Matrix Market file (row-major order = CSR order), in the library's
    feature order, plus its per-tile nonzero / distinct-row / distinct-column
    counts."""
    import ctypes as C
    import tempfile
    from oracle import RefOut
    from sspmv_gb300.lespmv import write_mtx
    with tempfile.TemporaryDirectory() as d:
        path = Path(d) / "m.mtx"
        write_mtx(str(path), A)
        F = np.zeros(62)
        o = RefOut()
        rc = ref.lib.ref_features_f64(str(path).encode(), C.c_void_p(F.ctypes.data), C.byref(o))
        assert rc == 0
        arrs = ref._take(o, [("tiles", np.int32), ("urb", np.int32), ("ucb", np.int32)])
    return F, arrs


def ref_dia_too_wide(ref, A) -> bool:
    """The reference exits the process when DIA needs more than 10240
    diagonals; such cases are skipped (the library reports SSPMV_INFEASIBLE)."""
    rows = np.repeat(np.arange(A.num_rows), np.diff(A.row_offset))
    return len(np.unique(A.col_index.astype(np.int64) - rows)) > 10240


if __name__ == "__main__":
    main()
