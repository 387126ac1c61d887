"""The allocation-free CSR SpMV entry point, sspmv_LeSpMV_csr_noalloc, called
through the C ABI.

It exists for callers that cannot allocate device memory at SpMV time -- a
solver or serving loop whose device heap belongs to its own pool allocator,
a latency-bound loop that cannot take cudaMalloc's implicit synchronisation,
a component held to a device-memory budget enforced outside this library.
Instead of a per-matrix plan it uses one fixed device array for its scratch.

Checked here: on two calls in a row its output matches the FP64 oracle and
the regular entry point (sspmv_LeSpMV_csr) within the per-row bound the
other GPU tests use, 8*nnz_i*eps*|alpha|*sum_j|a_ij x_j| + 2*eps*|beta*y0_i|;
it builds no plan on the matrix; and a matrix past its size limit is refused
with SSPMV_INVALID_ARG before anything runs.  This file is collected last, and
passes alone in a fresh process as well as after the other tests."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(alpha, M, x, beta, y):
    import torch
    from sspmv_gb300 import _lib
    stream = torch.cuda.current_stream().cuda_stream
    return _lib.lib.sspmv_LeSpMV_csr_noalloc(alpha, C.byref(M.s), C.c_void_p(x.data_ptr()), beta,
                                            C.c_void_p(y.data_ptr()), C.c_void_p(stream))


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["f64", "f32"])
def test_noalloc_matches_regular_entry_point(dt, oracle_lib):
    import torch
    from oracle import tolerance_ok
    from sspmv_gb300 import _lib, synth
    from sspmv_gb300 import lespmv as L

    A = synth.generate(synth.powerlaw(300000, 1.8, 16.0, 40000, 0.02), 4, dt)
    xh = synth.vector(A.num_cols, 0, dt)
    x = torch.from_numpy(xh).cuda()
    y0 = synth.vector(A.num_rows, 3, dt)
    nnz_row = np.diff(A.row_offset)
    y64, absum = oracle_lib.spmm_ref(A, xh, 0.8, 0.7, y0)  # FP64 oracle on the same inputs

    regular = L.csr_from_host(A)
    y_reg = torch.from_numpy(y0.copy()).cuda()
    L.LeSpMV(0.8, regular, x, 0.7, y_reg)
    torch.cuda.synchronize()
    ref = y_reg.cpu().numpy()
    ok, mx, _ = tolerance_ok(ref, y64, absum, nnz_row, dt, 0.8, 0.7, y0)
    assert ok, f"regular entry point: max normalised error {mx}"

    M = L.csr_from_host(A)  # a fresh matrix: the no-alloc call must not give it a plan
    for call in range(2):
        y = torch.from_numpy(y0.copy()).cuda()
        st = _noalloc(0.8, M, x, 0.7, y)
        assert st == 0, _lib.lib.sspmv_last_error().decode()
        torch.cuda.synchronize()
        yg = y.cpu().numpy()
        ok, mx, _ = tolerance_ok(yg, y64, absum, nnz_row, dt, 0.8, 0.7, y0)
        assert ok, f"call {call + 1}: max normalised error {mx} against the FP64 oracle"
        # and against the existing entry point's output, the same bound with
        # that output in the reference's place
        ok, mx, _ = tolerance_ok(yg, ref.astype(np.float64), absum, nnz_row, dt, 0.8, 0.7, y0)
        assert ok, f"call {call + 1}: max normalised error {mx} against sspmv_LeSpMV_csr"
    assert not M.s.f.priv, "the allocation-free entry point built a plan"


def test_noalloc_rejects_matrices_past_its_limit():
    import torch
    from sspmv_gb300 import _lib
    from sspmv_gb300 import lespmv as L

    # a CSR header claiming 300M rows over a tiny buffer: refused before any launch
    buf = torch.zeros(16, dtype=torch.int32, device="cuda")
    s = _lib.Csr()
    _lib.call("sspmv_csr_wrap", C.byref(s), _lib.F64, 300_000_000, 300_000_000, 0, C.c_void_p(buf.data_ptr()),
              C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()))
    M = L.CSR_Matrix(s)
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    st = _noalloc(1.0, M, x, 0.0, x)
    assert st == 1  # SSPMV_INVALID_ARG
    assert b"limit" in _lib.lib.sspmv_last_error()


@pytest.mark.gpu
def test_torch_custom_op_matches_library_call():
    """torch.ops.sspmv.spmv_csr (stateless: 1-D x on the no-allocation entry
    point, 2-D x on the library's SpMM with its plan released after the call)
    equals sspmv_LeSpMV_csr with the merge-path kernel bit for bit, and
    rejects CPU tensors and mismatched lengths before any launch."""
    import torch
    import sspmv_gb300.torch_ops  # noqa: F401  (registers the operator)
    from sspmv_gb300 import synth
    from sspmv_gb300.lespmv import LeSpMV_csr, csr_from_host
    for dt in (np.float64, np.float32):
        A = synth.generate(synth.powerlaw(30000, 1.8, 16.0, 20000, 0.05), 9, dt)
        rp = torch.from_numpy(A.row_offset).cuda()
        ci = torch.from_numpy(A.col_index).cuda()
        cv = torch.from_numpy(A.values).cuda()
        X = torch.from_numpy(synth.vector(A.num_cols, 0, dt, 3).reshape(A.num_cols, 3)).cuda()
        Y = torch.ops.sspmv.spmv_csr(rp, ci, cv, A.num_cols, X)
        y1 = torch.ops.sspmv.spmv_csr(rp, ci, cv, A.num_cols, X[:, 1].contiguous())
        M = csr_from_host(A)
        M.kernel_flag = 2  # the merge-path kernel the allocation-free entry point runs
        for j in range(3):
            ref = torch.zeros(A.num_rows, dtype=cv.dtype, device="cuda")
            LeSpMV_csr(1.0, M, X[:, j].contiguous(), 0.0, ref)
            assert torch.equal(Y[:, j], ref)
        assert torch.equal(y1, Y[:, 1])
    with pytest.raises(ValueError):
        torch.ops.sspmv.spmv_csr(rp, ci, cv[:-1], A.num_cols, X[:, 0].contiguous())
    with pytest.raises(ValueError):
        torch.ops.sspmv.spmv_csr(rp.cpu(), ci, cv, A.num_cols, X[:, 0].contiguous())
