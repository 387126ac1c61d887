"""The autotuner (sspmv_gb300/autotune.py), which replaces the reference's
compile-time tuning macros (SELL_SIGMA, CHUNK_SIZE, CSR5_SIGMA,
BSR_BlockDimRow: include/general_config.h:17-26) by measurement.

On a mid-size power-law matrix and a banded matrix: the tuned configuration
(CSR kernel, SELL-c-sigma C / sigma, BSR block shape and kernel) passes the
oracle's per-row bound, and its time, measured again after tuning, is no
worse than the library default's time x 1.05 (medians of 30 L2-flushed
runs, the default measured the same way)."""
import numpy as np
import pytest

from gpu_util import to_dev, to_host
from oracle import tolerance_ok

pytestmark = pytest.mark.gpu

MATS = {
    "powerlaw": lambda s: s.powerlaw(1_000_000, 1.8, 16.0, 50000),
    "banded": lambda s: s.banded(1_000_000),
}


def _check(L, M, A, x, y64, absum, what):
    y = to_dev(np.full(A.num_rows, np.nan, A.values.dtype))
    L.LeSpMV(1.0, M, to_dev(x), 0.0, y)
    ok, mx, _ = tolerance_ok(to_host(y), y64, absum, np.diff(A.row_offset), A.values.dtype)
    assert ok, f"{what}: max normalised error {mx}"


def _no_slower(tuned_ms, default_ms, what):
    assert tuned_ms <= default_ms * 1.05, f"{what}: tuned {tuned_ms:.4f} ms > default {default_ms:.4f} ms x 1.05"


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("fam", list(MATS))
def test_tuned_csr_kernel(fam, dt, oracle_lib):
    import torch
    from sspmv_gb300 import autotune, synth
    from sspmv_gb300 import lespmv as L
    A = synth.generate(MATS[fam](synth), 5, dt)
    x = synth.vector(A.num_cols, 0, dt)
    y64, absum = oracle_lib.spmm_ref(A, x, 1.0, 0.0)
    M = L.csr_from_host(A)
    xd, yd = to_dev(x), torch.zeros(A.num_rows, dtype=torch.from_numpy(x).dtype, device="cuda")
    flush = autotune.L2Flush("cuda")
    default_ms = autotune.time_spmv(M, xd, yd, reps=30, flush=flush)
    res = autotune.tune_csr(M, xd, yd)
    best = res["best"]
    assert M.kernel_flag == best["kernel_flag"]
    _check(L, M, A, x, y64, absum, f"{fam} csr {best}")
    _no_slower(autotune.time_spmv(M, xd, yd, reps=30, flush=flush), default_ms, f"{fam} csr {best}")


@pytest.mark.parametrize("fmt", ["sell_c_sigma", "bsr"])
@pytest.mark.parametrize("fam", list(MATS))
def test_tuned_conversion(fam, fmt, oracle_lib):
    import torch
    from sspmv_gb300 import autotune, synth
    from sspmv_gb300 import lespmv as L
    dt = np.float64
    A = synth.generate(MATS[fam](synth), 5, dt)
    x = synth.vector(A.num_cols, 0, dt)
    y64, absum = oracle_lib.spmm_ref(A, x, 1.0, 0.0)
    csr = L.csr_from_host(A)
    xd, yd = to_dev(x), torch.zeros(A.num_rows, dtype=torch.float64, device="cuda")
    flush = autotune.L2Flush("cuda")
    if fmt == "bsr":
        if not L.feasible_host("bsr", A)[0]:
            pytest.skip("BSR fill above 4x on this matrix")
        D = L.csr_to_bsr(csr, 4, 4)  # the library's default block for these families
    else:
        D = L.csr_to_sell_c_sigma(csr)
    default_ms = autotune.time_spmv(D, xd, yd, reps=30, flush=flush)
    D.delete()
    M, rec = autotune.tune_conversion(csr, fmt, xd, yd)
    assert M is not None and rec["params"] in [c["params"] for c in rec["table"]]
    _check(L, M, A, x, y64, absum, f"{fam} {fmt} {rec['params']}")
    _no_slower(autotune.time_spmv(M, xd, yd, reps=30, flush=flush), default_ms, f"{fam} {fmt} {rec['params']}")
    M.delete()
