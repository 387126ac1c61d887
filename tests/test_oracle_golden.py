"""Pins the CPU oracle (oracle/oracle.c) to the reference's own outputs stored
in tests/golden (written by tests/golden/make_golden.py from LeSpMV itself):
every converter array bit-exact, every SpMV within the per-row bound."""
import numpy as np
import pytest

from golden_util import ALPHA, BETA, digest, files, load
from oracle import tolerance_ok

CASES = files()


@pytest.mark.parametrize("path", CASES, ids=[p.stem for p in CASES])
def test_converters_bit_exact(path, oracle_lib):
    z, meta, A = load(path)
    assert meta["conv"], "fixture without converter records"
    for key, rec in meta["conv"].items():
        out = getattr(oracle_lib, rec["fn"])(A, **rec["kw"])
        assert out is not None, key
        for name, d in rec["digests"].items():
            assert list(out[name].shape) == rec["shapes"][name], (key, name)
            assert digest(out[name]) == d, f"{path.stem}:{key}:{name} differs from the reference"
        for name, v in rec["scalars"].items():
            if name in out:
                assert int(out[name]) == v, (key, name)


@pytest.mark.parametrize("path", [p for p in CASES if "dups" in p.stem], ids=lambda p: p.stem)
def test_coo_to_csr_bit_exact(path, oracle_lib):
    z, meta, A = load(path)
    out = oracle_lib.coo_to_csr(A.num_rows, z["in_coo_row"], z["in_coo_col"], z["in_coo_val"])
    for k, d in meta["coo_to_csr"].items():
        assert digest(out[k]) == d, k


FMT_CONV = {
    "coo": ("csr_to_coo", {}),
    "ell": ("csr_to_ell", {"ld": 0}),
    "sell": ("csr_to_sell", {}),
    "sell_c_sigma": ("csr_to_sell_c_sigma", {}),
    "sell_c_R": ("csr_to_sell_c_R", {}),
    "dia": ("csr_to_dia", {}),
    "bsr": ("csr_to_bsr", {}),
}


@pytest.mark.parametrize("path", CASES, ids=[p.stem for p in CASES])
def test_spmv_matches_reference(path, oracle_lib):
    z, meta, A = load(path)
    x, y0 = z["x"], z["y0"]
    dt = A.values.dtype
    yref64, absum = oracle_lib.spmm_ref(A, x, ALPHA, BETA, y0)
    nnz_row = np.diff(A.row_offset)
    has_dups = "in_coo_row" in z.files
    for fmt, flag in meta["spmv"]:
        y_ref = z[f"y_{fmt}_{flag}"]
        # DIA and BSR keep the last of duplicate entries where CSR sums them
        # (include/sparse_conversion.h:758,921): no CSR bound for those.
        overwrite = has_dups and fmt in ("dia", "bsr")
        # The reference's DIA kernels bound the row loop by num_rows - offset
        # (src/spmv_dia.cpp:30,62) instead of num_cols - offset, so on a
        # non-square matrix they drop entries; the oracle and the library use
        # the column bound.  Their result is only checked when square.
        wrong_ref = fmt == "dia" and A.num_rows != A.num_cols
        if not overwrite and not wrong_ref:
            # the reference's own result against the FP64 bound (oracle self-check)
            ok, mx, _ = tolerance_ok(y_ref, yref64, absum, nnz_row, dt, ALPHA, BETA, y0)
            assert ok, f"reference {fmt}/{flag} outside the bound ({mx})"
        if fmt == "csr":
            A_fmt = None
        else:
            fn, kw = FMT_CONV[fmt]
            A_fmt = getattr(oracle_lib, fn)(A, **kw)
            if fmt in ("sell", "sell_c_sigma", "sell_c_R"):
                A_fmt["C"] = 4
            if fmt == "ell":
                A_fmt["ld"] = 0
        y = y0.copy()
        oracle_lib.spmv(fmt, A_fmt, A, ALPHA, x, BETA, y)
        if not overwrite:
            ok, mx, _ = tolerance_ok(y, yref64, absum, nnz_row, dt, ALPHA, BETA, y0)
            assert ok, f"oracle {fmt} outside the bound ({mx})"
        if not wrong_ref:
            assert oracle_lib.max_rel_error(y, y_ref) < 5 * np.sqrt(np.finfo(dt).eps)
