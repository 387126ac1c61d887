"""CSR SpMV / SpMM on the GPU against the reference's own results (golden
fixtures) and the FP64 oracle, through the C ABI.

Tolerance (per row, FP64 and FP32): |y_i - y_ref_i| <= 8*nnz_i*eps*|alpha|*
sum_j|a_ij x_j| + 2*eps*|beta*y0_i|, y_ref the FP64 CSR result on the same
(possibly FP32-rounded) inputs."""
import numpy as np
import pytest

from golden_util import ALPHA, BETA, files, load
from gpu_util import to_dev, to_host
from oracle import tolerance_ok

pytestmark = pytest.mark.gpu

CASES = files()


def _csr(A):
    from sspmv_gb300.lespmv import csr_from_host
    return csr_from_host(A)


@pytest.mark.parametrize("flag", [0, 1, 3, 4])
@pytest.mark.parametrize("path", CASES, ids=[p.stem for p in CASES])
def test_csr_golden(path, flag, oracle_lib):
    from sspmv_gb300.lespmv import LeSpMV_csr
    z, meta, A = load(path)
    dt = A.values.dtype
    x, y0 = z["x"], z["y0"]
    M = _csr(A)
    M.kernel_flag = flag
    y = to_dev(y0)
    LeSpMV_csr(ALPHA, M, to_dev(x), BETA, y)
    yg = to_host(y)
    y64, absum = oracle_lib.spmm_ref(A, x, ALPHA, BETA, y0)
    ok, mx, med = tolerance_ok(yg, y64, absum, np.diff(A.row_offset), dt, ALPHA, BETA, y0)
    assert ok, f"max normalised error {mx}"
    assert oracle_lib.max_rel_error(yg, z["y_csr_2"]) < 5 * np.sqrt(np.finfo(dt).eps)


FAMILIES = {
    "powerlaw": lambda s: s.powerlaw(60000, 1.8, 16.0, 50000, 0.02),
    "uniform": lambda s: s.uniform(50000, 32, 0.01),
    "laplacian": lambda s: s.laplacian2d(300),
    "banded": lambda s: s.banded(40000),
    "block": lambda s: s.block(40000, 4, 9000),
}


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("fam", list(FAMILIES))
@pytest.mark.parametrize("k", [1, 2, 3, 8])
def test_csr_spmm_families(fam, k, dt, oracle_lib):
    from sspmv_gb300 import synth
    from sspmv_gb300.lespmv import spmm
    A = synth.generate(FAMILIES[fam](synth), 2, dt)
    X = synth.vector(A.num_cols, 0, dt, k).reshape(A.num_cols, k)
    Y0 = synth.vector(A.num_rows, 7, dt, k).reshape(A.num_rows, k)
    M = _csr(A)
    for flag in (0, 1, 3, 4):
        M.kernel_flag = flag
        Y = to_dev(Y0)
        spmm(ALPHA, M, to_dev(X), BETA, Y)
        Yg = to_host(Y)
        y64, absum = oracle_lib.spmm_ref(A, X, ALPHA, BETA, Y0)
        ok, mx, med = tolerance_ok(Yg, y64, absum, np.diff(A.row_offset), dt, ALPHA, BETA, Y0)
        assert ok, f"{fam} k={k} flag={flag}: max normalised error {mx}"


def _short_rows(s, case):
    """Matrices for the row-block kernel: rows of at most 64 nonzeros, runs
    of empty rows (more than one 1024-row block of them), rows of exactly 64,
    blocks that end on a window boundary."""
    if case == "uniform64_empty":
        return s.uniform(30000, 64, 0.3)
    if case == "uniform1":
        return s.uniform(70000, 1)
    if case == "lap":
        return s.laplacian2d(257)
    if case == "banded":
        return s.banded(50000)
    if case == "block":
        return s.block(50000, 4, 12000)
    return s.powerlaw(40000, 1.8, 8.0, 64, 0.05)


def _empty_runs(dt):
    """Runs of 2500 and 3000 empty rows between rows of 1..64 nonzeros, and
    empty last rows."""
    rng = np.random.default_rng(11)
    lens = np.concatenate([np.zeros(2500, np.int64), rng.integers(1, 65, 4000), np.zeros(3000, np.int64),
                           rng.integers(0, 4, 5000), np.zeros(700, np.int64)])
    m = n = len(lens)
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    col = np.concatenate([np.sort(rng.choice(n, int(k), replace=False)) for k in lens if k] or
                         [np.zeros(0, np.int64)]).astype(np.int32)
    from sspmv_gb300.synth import HostCSR
    return HostCSR(m, n, rp, col, rng.uniform(-1, 1, int(rp[-1])).astype(dt))


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("window", [0, 512, 1024, 2048, 4096])
@pytest.mark.parametrize("case", ["uniform64_empty", "uniform1", "lap", "banded", "block", "powerlaw_cap64",
                                  "empty_runs"])
def test_csr_rowblock(case, window, dt, oracle_lib):
    """kernel_flag 3 (row-block kernel) on every window, with alpha/beta and
    with alpha = 1, beta = 0 (the y = sum instantiation, y filled with NaN)."""
    from sspmv_gb300 import synth
    from sspmv_gb300.lespmv import LeSpMV_csr
    A = _empty_runs(dt) if case == "empty_runs" else synth.generate(_short_rows(synth, case), 3, dt)
    assert np.diff(A.row_offset).max() <= 64
    x = synth.vector(A.num_cols, 0, dt)
    y0 = synth.vector(A.num_rows, 5, dt)
    M = _csr(A)
    M.set_kernel(3, window)
    for alpha, beta, init in ((ALPHA, BETA, y0), (1.0, 0.0, np.full(A.num_rows, np.nan, dt))):
        y = to_dev(init)
        LeSpMV_csr(alpha, M, to_dev(x), beta, y)
        yg = to_host(y)
        y64, absum = oracle_lib.spmm_ref(A, x, alpha, beta, y0 if beta else None)
        ok, mx, _ = tolerance_ok(yg, y64, absum, np.diff(A.row_offset), dt, alpha, beta, y0 if beta else None)
        assert ok, f"{case} window {window} alpha {alpha}: max normalised error {mx}"
    from sspmv_gb300.lespmv import wait_timeouts
    assert wait_timeouts() == 0


def test_csr_rowblock_falls_back_on_long_rows(oracle_lib):
    """A row longer than 64 nonzeros: kernel_flag 3 runs the default kernel."""
    from sspmv_gb300 import synth
    from sspmv_gb300.lespmv import LeSpMV_csr
    A = synth.generate(synth.powerlaw(20000, 1.8, 16, 5000), 4)
    x = synth.vector(A.num_cols, 0)
    M = _csr(A)
    M.set_kernel(3, 0)
    y = to_dev(np.zeros(A.num_rows))
    LeSpMV_csr(1.0, M, to_dev(x), 0.0, y)
    y64, absum = oracle_lib.spmm_ref(A, x, 1.0, 0.0)
    ok, mx, _ = tolerance_ok(to_host(y), y64, absum, np.diff(A.row_offset), np.float64)
    assert ok, mx


def _rows_up_to(dt, longest, m, seed):
    """m rows of 0..longest nonzeros (every length present), random columns."""
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, longest + 1, m)
    k = min(m, longest + 1)
    lens[:k] = np.arange(longest + 1 - k, longest + 1)
    n = max(m, 64)
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    col = np.concatenate([np.sort(rng.choice(n, int(k), replace=False)) for k in lens if k] or
                         [np.zeros(0, np.int64)]).astype(np.int32)
    from sspmv_gb300.synth import HostCSR
    return HostCSR(m, n, rp, col, rng.uniform(-1, 1, int(rp[-1])).astype(dt))


_PIPE_CACHE = {}


def _pipe_matrix(case, dt):
    """The test matrices of test_csr_pipe, built once per (case, dtype)."""
    key = (case, np.dtype(dt).name)
    if key in _PIPE_CACHE:
        return _PIPE_CACHE[key]
    from sspmv_gb300 import synth
    if case.startswith("rows"):
        h = int(case[4:])
        A = _rows_up_to(dt, h, 50000 + 17 * h if h <= 12 else 20000 + h, h)
    elif case == "m5":
        A = _rows_up_to(dt, 7, 5, 1)
    elif case == "m40":
        A = _rows_up_to(dt, 12, 40, 2)
    elif case == "empty_runs_12":
        A = _empty_runs(dt)
        lens = np.minimum(np.diff(A.row_offset), 12)
        keep = np.concatenate([np.arange(A.row_offset[i], A.row_offset[i] + lens[i]) for i in range(A.num_rows)])
        from sspmv_gb300.synth import HostCSR
        A = HostCSR(A.num_rows, A.num_cols, np.concatenate([[0], np.cumsum(lens)]).astype(np.int32),
                    A.col_index[keep], A.values[keep])
    elif case == "block":
        A = synth.generate(synth.block(50000, 4, 3000), 3, dt)
    else:
        A = synth.generate(_short_rows(synth, case), 3, dt)
    _PIPE_CACHE[key] = A
    return A


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("param", list(range(16)))
@pytest.mark.parametrize("case", ["lap", "banded", "block", "uniform1", "empty_runs_12"] +
                         [f"rows{h}" for h in (1, 2, 3, 4, 5, 6, 7, 8, 10, 12, 16, 32, 64)] + ["m5", "m40"])
def test_csr_pipe(case, param, dt, oracle_lib):
    """kernel_flag 4 (pipelined row kernel) with each param (bit 0: value-load
    point; bits 1-2: 1, 2, 4 or 8 lanes per row; bit 3: 1024-thread CTAs) on
    every template row length
    (rows of up to 1..12, 16, 32, 64 nonzeros, every length present; rows
    longer than a lane count takes run the default kernel), the short-row
    families, runs of empty rows, fewer rows than a warp, with alpha/beta and
    with alpha = 1, beta = 0 (the y = sum instantiation, y filled with NaN)."""
    from sspmv_gb300 import synth
    from sspmv_gb300.lespmv import LeSpMV_csr
    A = _pipe_matrix(case, dt)
    x = synth.vector(A.num_cols, 0, dt)
    y0 = synth.vector(A.num_rows, 5, dt)
    M = _csr(A)
    M.set_kernel(4, param)
    for alpha, beta, init in ((ALPHA, BETA, y0), (1.0, 0.0, np.full(A.num_rows, np.nan, dt))):
        y = to_dev(init)
        LeSpMV_csr(alpha, M, to_dev(x), beta, y)
        yg = to_host(y)
        y64, absum = oracle_lib.spmm_ref(A, x, alpha, beta, y0 if beta else None)
        ok, mx, _ = tolerance_ok(yg, y64, absum, np.diff(A.row_offset), dt, alpha, beta, y0 if beta else None)
        assert ok, f"{case} param {param} alpha {alpha}: max normalised error {mx}"


@pytest.mark.parametrize("flag,param", [(3, 1024), (4, 0), (4, 1), (4, 7)])
def test_csr_short_row_kernels_strided_single_rhs(flag, param, oracle_lib):
    """One right-hand side read from and written to every third column of
    row-major blocks (ldx = ldy = 3): the row-block and pipelined kernels
    index x and y by their leading dimensions; the other columns stay as
    they were."""
    from sspmv_gb300 import synth
    from sspmv_gb300.lespmv import spmm
    A = synth.generate(synth.banded(30000), 3, np.float64)
    X3 = synth.vector(A.num_cols * 3, 0).reshape(A.num_cols, 3)
    Y3 = synth.vector(A.num_rows * 3, 5).reshape(A.num_rows, 3)
    M = _csr(A)
    M.set_kernel(flag, param)
    Yd = to_dev(Y3)
    spmm(ALPHA, M, to_dev(X3)[:, 1:2], BETA, Yd[:, 2:3], k=1, ldx=3, ldy=3)
    Yg = to_host(Yd)
    y64, absum = oracle_lib.spmm_ref(A, np.ascontiguousarray(X3[:, 1]), ALPHA, BETA, np.ascontiguousarray(Y3[:, 2]))
    ok, mx, _ = tolerance_ok(Yg[:, 2], y64, absum, np.diff(A.row_offset), np.float64, ALPHA, BETA,
                             np.ascontiguousarray(Y3[:, 2]))
    assert ok, mx
    assert np.array_equal(Yg[:, :2], Y3[:, :2])


def test_csr_pipe_falls_back_on_long_rows(oracle_lib):
    """A row of 13 nonzeros: kernel_flag 4 runs the default kernel."""
    from sspmv_gb300 import synth
    from sspmv_gb300.lespmv import LeSpMV_csr
    A = _rows_up_to(np.float64, 13, 30000, 5)
    x = synth.vector(A.num_cols, 0)
    M = _csr(A)
    M.set_kernel(4, 0)
    y = to_dev(np.full(A.num_rows, np.nan))
    LeSpMV_csr(1.0, M, to_dev(x), 0.0, y)
    y64, absum = oracle_lib.spmm_ref(A, x, 1.0, 0.0)
    ok, mx, _ = tolerance_ok(to_host(y), y64, absum, np.diff(A.row_offset), np.float64)
    assert ok, mx


def test_csr_beta_zero_ignores_nan_y(oracle_lib):
    from sspmv_gb300 import synth
    from sspmv_gb300.lespmv import LeSpMV_csr
    A = synth.generate(synth.powerlaw(20000, 1.8, 16, 20000, 0.05), 4)
    x = synth.vector(A.num_cols, 0)
    M = _csr(A)
    y = to_dev(np.full(A.num_rows, np.nan))
    LeSpMV_csr(1.0, M, to_dev(x), 0.0, y)
    yg = to_host(y)
    y64, absum = oracle_lib.spmm_ref(A, x, 1.0, 0.0)
    ok, mx, _ = tolerance_ok(yg, y64, absum, np.diff(A.row_offset), np.float64)
    assert ok and np.isfinite(yg).all()


def test_csr_deterministic():
    from sspmv_gb300 import synth
    from sspmv_gb300.lespmv import LeSpMV_csr
    A = synth.generate(synth.powerlaw(100000, 1.8, 16, 50000), 6)
    x = to_dev(synth.vector(A.num_cols, 0))
    M = _csr(A)
    outs = []
    for _ in range(3):
        y = to_dev(np.zeros(A.num_rows))
        LeSpMV_csr(1.0, M, x, 0.0, y)
        outs.append(to_host(y))
    assert all(np.array_equal(outs[0], o) for o in outs[1:])


def test_csr_rowblock_window_changes_and_unaligned_arrays(oracle_lib):
    """The row-block plan is rebuilt when the window changes (back and forth
    on one matrix), and arrays that are not 16-byte aligned (a CSR wrapped
    over offset device buffers) run the default kernel instead."""
    import ctypes as C
    import torch
    from sspmv_gb300 import _lib, synth
    from sspmv_gb300.lespmv import CSR_Matrix, LeSpMV_csr
    A = synth.generate(synth.banded(40000), 3, np.float64)
    x = synth.vector(A.num_cols, 0)
    y64, absum = oracle_lib.spmm_ref(A, x, 1.0, 0.0)
    M = _csr(A)
    for w in (512, 4096, 1024, 512, 2048):
        M.set_kernel(3, w)
        y = to_dev(np.full(A.num_rows, np.nan))
        LeSpMV_csr(1.0, M, to_dev(x), 0.0, y)
        ok, mx, _ = tolerance_ok(to_host(y), y64, absum, np.diff(A.row_offset), np.float64)
        assert ok, f"window {w}: {mx}"
    # the same arrays one element into larger buffers: 4-byte and 8-byte aligned only
    rp = torch.zeros(A.num_rows + 2, dtype=torch.int32, device="cuda")
    ci = torch.zeros(A.nnz + 1, dtype=torch.int32, device="cuda")
    cv = torch.zeros(A.nnz + 1, dtype=torch.float64, device="cuda")
    rp[1:].copy_(torch.from_numpy(A.row_offset))
    ci[1:].copy_(torch.from_numpy(A.col_index))
    cv[1:].copy_(torch.from_numpy(A.values))
    s = _lib.Csr()
    _lib.call("sspmv_csr_wrap", C.byref(s), _lib.F64, A.num_rows, A.num_cols, A.nnz, C.c_void_p(rp[1:].data_ptr()),
              C.c_void_p(ci[1:].data_ptr()), C.c_void_p(cv[1:].data_ptr()))
    W = CSR_Matrix(s)
    W.set_kernel(3, 0)
    y = to_dev(np.full(A.num_rows, np.nan))
    LeSpMV_csr(1.0, W, to_dev(x), 0.0, y)
    ok, mx, _ = tolerance_ok(to_host(y), y64, absum, np.diff(A.row_offset), np.float64)
    assert ok, mx
    _lib.call("sspmv_release_plan", C.byref(W.s.f), None)
