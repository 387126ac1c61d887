"""Parity at the benchmark's full-size workloads, every row, through the C ABI.

  laplacian_1024  2-D 5-point Laplacian, N = 1,048,576, written as a Matrix
                  Market file and read back through sspmv_read_mtx, CSR FP64
                  with alpha = 1, beta = 0 (every CSR kernel)
  suite           banded_2M, powerlaw_4M, block4_2M, uniform_4M x every
                  feasible format x FP64 / FP32, alpha = 1, beta = 0
  powerlaw_16M    N = 16,777,216, ~268M nonzeros, FP32: CSR and SELL-c-sigma
                  (C = 32, sigma = N and C = 8, sigma = 256) with k = 1 and
                  k = 8 right-hand sides

Each y is compared on every row with the FP64 CSR product of the oracle on
the same (FP32-rounded where FP32) inputs, within the per-row bound
|y_i - y64_i| <= 8 * nnz_i * eps * sum_j |a_ij x_j| (eps = 2^-52 / 2^-23),
the metric of the reference's benchmark check (include/sparse_operation.h:
76-164) made per row.  The max and median normalised error of every case
are recorded (record_property) and printed.
"""
import tempfile
from pathlib import Path

import numpy as np
import pytest

from gpu_util import to_dev, to_host
from oracle import tolerance_ok

pytestmark = pytest.mark.gpu

SUITE = ["banded_2M", "powerlaw_4M", "block4_2M", "uniform_4M"]


def _check(name, yg, y64, absum, A, dt, record_property):
    ok, mx, med = tolerance_ok(yg, y64, absum, np.diff(A.row_offset), dt)
    record_property(name, f"max {mx:.4g} median {med:.4g}")
    print(f"{name}: max normalised error {mx:.4g}, median {med:.4g}")
    assert ok, f"{name}: max normalised error {mx}"


def test_laplacian_1024_from_mtx_every_row(oracle_lib, record_property):
    from sspmv_gb300 import synth
    from sspmv_gb300 import lespmv as L
    A0 = synth.load("laplacian_1024", 1, np.float64)
    with tempfile.TemporaryDirectory() as d:
        path = str(Path(d) / "laplacian_1024.mtx")
        L.write_mtx(path, A0)
        A = L.read_csr_matrix(path, 64)
    assert A.num_rows == 1 << 20 and A.nnz == 5_238_784
    assert np.array_equal(A.row_offset, A0.row_offset) and np.array_equal(A.col_index, A0.col_index)
    x = synth.vector(A.num_cols, 0, np.float64)
    y64, absum = oracle_lib.spmm_ref(A, x, 1.0, 0.0)
    M = L.csr_from_host(A)
    for flag, param in ((0, 0), (1, 2), (2, 0), (3, 0)):
        M.set_kernel(flag, param)
        y = to_dev(np.full(A.num_rows, np.nan))
        L.LeSpMV(1.0, M, to_dev(x), 0.0, y)
        _check(f"laplacian_1024/csr/f64/flag{flag}", to_host(y), y64, absum, A, np.float64, record_property)
    assert L.wait_timeouts() == 0


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("fam", SUITE)
def test_suite_every_format_every_row(fam, dt, oracle_lib, record_property):
    from sspmv_gb300 import synth
    from sspmv_gb300 import lespmv as L
    A = synth.load(fam, 1, dt)
    x = synth.vector(A.num_cols, 0, dt)
    y64, absum = oracle_lib.spmm_ref(A, x, 1.0, 0.0)
    csr = L.csr_from_host(A)
    xd = to_dev(x)
    built = 0
    for fmt in L.FORMATS:
        M, why = L.build_format(csr, fmt, A)
        if M is None:  # padding or block fill above 4x the CSR size, or DIA over 10240 diagonals
            assert fmt in ("ell", "bsr", "dia") and any(w in why for w in ("pads", "fill", "INFEASIBLE")), \
                f"{fam}/{fmt}: {why}"
            continue
        y = to_dev(np.full(A.num_rows, np.nan, dt))
        L.LeSpMV(1.0, M, xd, 0.0, y)
        _check(f"{fam}/{fmt}/{np.dtype(dt).name}", to_host(y), y64, absum, A, dt, record_property)
        if M is not csr:
            M.delete()
        built += 1
    csr.delete()
    assert built >= 6


def test_powerlaw_16M_sell_c_sigma_and_csr(oracle_lib, record_property):
    import torch
    from sspmv_gb300 import synth
    from sspmv_gb300 import lespmv as L
    A = synth.load("powerlaw_16M", 1, np.float32)
    n, m = A.num_cols, A.num_rows
    assert m == 1 << 24 and A.nnz > 200_000_000
    csr = L.csr_from_host(A)
    sig_n = -(-m // 32) * 32
    mats = [("csr", csr), ("sell_c_sigma_C32_sN", L.csr_to_sell_c_sigma(csr, sig_n, 32)),
            ("sell_c_sigma_C8_s256", L.csr_to_sell_c_sigma(csr, 256, 8))]
    for k in (1, 8):
        X = synth.vector(n, 0, np.float32, k).reshape(n, k) if k > 1 else synth.vector(n, 0, np.float32)
        y64, absum = oracle_lib.spmm_ref(A, X, 1.0, 0.0)
        Xd = to_dev(X)
        for name, M in mats:
            Y = torch.full((m, k) if k > 1 else (m,), float("nan"), dtype=torch.float32, device="cuda")
            L.spmm(1.0, M, Xd, 0.0, Y)
            _check(f"powerlaw_16M/{name}/f32/k{k}", to_host(Y), y64, absum, A, np.float32, record_property)
            del Y
        del Xd, y64, absum
    for _, M in mats:
        M.delete()
